// Registration of the .Call routines (the table of src/init.cpp:11-22 in the reference, plus the
// three neighbor routines R/nn.R calls by name).  The five routines of the latent, logit and
// SLGP models are outside the GB300 build: they keep their names and arities, so the package's
// R code loads unchanged, and raise an error when called.
#ifndef R_NO_REMAP
#define R_NO_REMAP
#endif
#include <R.h>
#include <Rinternals.h>
#include <R_ext/Rdynload.h>

extern "C" {
SEXP rNNGP(SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP,
           SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP);
SEXP cNNGP(SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP);
SEXP rNNGPPredict(SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP,
                  SEXP);
SEXP rNNGPReplicated(SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP);
SEXP mkNNIndx(SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP);
SEXP mkNNIndxCB(SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP);
SEXP mkUIndx(SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP);
void nngp_call_release(void);

static SEXP out_of_scope(const char *routine) {
  Rf_error("c++ Rf_error: %s is not part of the GB300 build of spNNGP (its latent, logit and SLGP models are "
           "outside it)\n", routine);
  return R_NilValue;
}
#define S SEXP
SEXP sNNGP(S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S) {
  return out_of_scope("sNNGP");
}
SEXP sNNGPLogit(S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S) {
  return out_of_scope("sNNGPLogit");
}
SEXP cSLGP(S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S) { return out_of_scope("cSLGP"); }
SEXP sNNGPPredict(S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S, S) { return out_of_scope("sNNGPPredict"); }
SEXP PGLogit(S, S, S, S, S, S, S, S, S) { return out_of_scope("PGLogit"); }
#undef S

static const R_CallMethodDef CallEntries[] = {
    {"rNNGP", (DL_FUNC)&rNNGP, 28},
    {"sNNGP", (DL_FUNC)&sNNGP, 29},
    {"sNNGPLogit", (DL_FUNC)&sNNGPLogit, 27},
    {"cNNGP", (DL_FUNC)&cNNGP, 18},
    {"cSLGP", (DL_FUNC)&cSLGP, 21},
    {"rNNGPPredict", (DL_FUNC)&rNNGPPredict, 17},
    {"sNNGPPredict", (DL_FUNC)&sNNGPPredict, 19},
    {"PGLogit", (DL_FUNC)&PGLogit, 9},
    {"rNNGPReplicated", (DL_FUNC)&rNNGPReplicated, 14},
    {"mkNNIndx", (DL_FUNC)&mkNNIndx, 7},
    {"mkNNIndxCB", (DL_FUNC)&mkNNIndxCB, 7},
    {"mkUIndx", (DL_FUNC)&mkUIndx, 8},
    {NULL, NULL, 0}};

void R_init_spNNGP(DllInfo *dll) {
  R_registerRoutines(dll, NULL, CallEntries, NULL, NULL);
  R_useDynamicSymbols(dll, FALSE);
}

void R_unload_spNNGP(DllInfo *dll) {
  (void)dll;
  nngp_call_release();
}
}
