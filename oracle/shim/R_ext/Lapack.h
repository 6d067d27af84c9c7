#ifndef NNGP_SHIM_LAPACK_H
#define NNGP_SHIM_LAPACK_H
#include "BLAS.h"
#ifdef __cplusplus
extern "C" {
#endif
void dpotrf_(const char *uplo, const int *n, double *a, const int *lda, int *info);
void dpotri_(const char *uplo, const int *n, double *a, const int *lda, int *info);
#ifdef __cplusplus
}
#endif
#endif
