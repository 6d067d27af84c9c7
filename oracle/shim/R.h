/* Minimal stand-in for R's <R.h>, written for this project so that the
 * reference package's own C++ sources compile outside R (test oracle only).
 * Only the entry points the NNGP hot-path files use are declared. */
#ifndef NNGP_SHIM_R_H
#define NNGP_SHIM_R_H
#include <stdlib.h>
#include <stdio.h>
#include <stddef.h>
#include <math.h>
#include "R_ext/RS.h"
#include "R_ext/Utils.h"
#ifdef __cplusplus
extern "C" {
#endif
void Rprintf(const char *fmt, ...);
void Rf_error(const char *fmt, ...);
void Rf_warning(const char *fmt, ...);
char *R_alloc(size_t n, int size);
void R_FlushConsole(void);
void GetRNGstate(void);
void PutRNGstate(void);
#ifdef __cplusplus
}
#endif
#endif
