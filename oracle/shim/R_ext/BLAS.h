/* BLAS subset used by the reference hot path; implemented in this project's
 * oracle/linalg.c (reference-BLAS semantics, column-major, LP64 ints). */
#ifndef NNGP_SHIM_BLAS_H
#define NNGP_SHIM_BLAS_H
#include "RS.h"
#ifdef __cplusplus
extern "C" {
#endif
double ddot_(const int *n, const double *x, const int *incx, const double *y, const int *incy);
void dcopy_(const int *n, const double *x, const int *incx, double *y, const int *incy);
void daxpy_(const int *n, const double *a, const double *x, const int *incx, double *y, const int *incy);
void dgemv_(const char *trans, const int *m, const int *n, const double *alpha, const double *a,
            const int *lda, const double *x, const int *incx, const double *beta, double *y, const int *incy);
void dsymv_(const char *uplo, const int *n, const double *alpha, const double *a, const int *lda,
            const double *x, const int *incx, const double *beta, double *y, const int *incy);
void dtrmv_(const char *uplo, const char *trans, const char *diag, const int *n, const double *a,
            const int *lda, double *x, const int *incx);
#ifdef __cplusplus
}
#endif
#endif
