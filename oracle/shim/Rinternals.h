/* Minimal stand-in for R's <Rinternals.h> (test oracle only): a SEXP is a
 * plain tagged buffer; PROTECT/UNPROTECT are no-ops. */
#ifndef NNGP_SHIM_RINTERNALS_H
#define NNGP_SHIM_RINTERNALS_H
#include "R.h"
#ifdef __cplusplus
extern "C" {
#endif
typedef struct shim_sexp *SEXP;
struct shim_sexp {
  int type;
  long length;
  int nrow, ncol;
  void *data;
  SEXP *elts;
  SEXP names;
  const char *chr;
};
#define CHARSXP 9
#define INTSXP 13
#define REALSXP 14
#define VECSXP 19
extern SEXP R_NilValue;
double *REAL(SEXP x);
int *INTEGER(SEXP x);
SEXP Rf_allocMatrix(int type, int nrow, int ncol);
SEXP Rf_allocVector(int type, long n);
SEXP SET_VECTOR_ELT(SEXP x, long i, SEXP v);
SEXP Rf_mkChar(const char *s);
SEXP Rf_namesgets(SEXP x, SEXP names);
#define PROTECT(x) (x)
#define UNPROTECT(n) ((void)(n))
#ifdef __cplusplus
}
#endif
#endif
