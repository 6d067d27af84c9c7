/*
 * TEST ORACLE ONLY.  Runtime for the R-API stand-in headers in this folder,
 * plus extern "C" drivers that wrap plain pointers into shim SEXPs and call
 * the reference package's own .Call entry points (compiled unmodified from the
 * reference's src/ folder by oracle/Makefile).  Nothing here is part of the
 * product; it exists so the reference's C++ can serve as a checker.
 *
 * Rf_error records the message and RETURNS (R's longjmp cannot cross the
 * reference's OpenMP regions safely); every driver reports a recorded error
 * through its return value.  rnorm/runif read the host-fed streams of
 * oracle/rmath.c.
 *
 * Compiled with -DSHIM_CALL_ONLY (oracle/Makefile rcall) the file leaves out
 * the four drivers that reach the reference's internal helpers (updateBF,
 * updateConjBF, Q, spCor), so the remaining drivers -- which only call the
 * .Call routines by name -- can be linked against any implementation of the
 * .Call layer, such as this project's src/.  R_registerRoutines keeps the
 * registered table for inspection.
 */
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <mutex>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "R.h"
#include "Rinternals.h"
#include "Rmath.h"
#include "R_ext/Rdynload.h"

extern "C" {
double or_bessel_k(double x, double nu);
double or_gammafn(double x);
void or_rsort_with_index(double *x, int *idx, int n);
void or_stream_set(const double *normals, long n_norm, const double *unifs, long n_unif);
void or_stream_used(long *n_norm, long *n_unif, int *overrun);
double or_rnorm(double mu, double sd);
double or_runif(double a, double b);
double or_next_normal(void);
double or_next_unif(void);
}

/* ------------------------------------------------------------------ R runtime */
static std::vector<void *> g_allocs;
static std::mutex g_alloc_mu;
static std::string g_error;
static int g_verbose = 0;

static void track(void *p) {
  std::lock_guard<std::mutex> lk(g_alloc_mu);
  g_allocs.push_back(p);
}

extern "C" {

static struct shim_sexp g_nil = {0, 0, 0, 0, nullptr, nullptr, nullptr, nullptr};
SEXP R_NilValue = &g_nil;

void Rprintf(const char *fmt, ...) {
  if (!g_verbose) return;
  va_list ap;
  va_start(ap, fmt);
  vfprintf(stderr, fmt, ap);
  va_end(ap);
}
void Rf_error(const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  std::lock_guard<std::mutex> lk(g_alloc_mu);
  if (g_error.empty()) g_error = buf;
}
void Rf_warning(const char *fmt, ...) { (void)fmt; }
char *R_alloc(size_t n, int size) {
  size_t bytes = n * (size_t)size;
  void *p = calloc(bytes ? bytes : 1, 1);
  track(p);
  return (char *)p;
}
void R_FlushConsole(void) {}
void R_CheckUserInterrupt(void) {}
void GetRNGstate(void) {}
void PutRNGstate(void) {}

double *REAL(SEXP x) { return (double *)x->data; }
int *INTEGER(SEXP x) { return (int *)x->data; }

static SEXP new_sexp(int type, long n) {
  SEXP s = (SEXP)calloc(1, sizeof(struct shim_sexp));
  track(s);
  s->type = type;
  s->length = n;
  if (type == REALSXP) s->data = calloc(n ? n : 1, sizeof(double));
  else if (type == INTSXP) s->data = calloc(n ? n : 1, sizeof(int));
  else if (type == VECSXP) s->elts = (SEXP *)calloc(n ? n : 1, sizeof(SEXP));
  if (s->data) track(s->data);
  if (s->elts) track(s->elts);
  return s;
}
SEXP Rf_allocVector(int type, long n) { return new_sexp(type, n); }
SEXP Rf_allocMatrix(int type, int nrow, int ncol) {
  SEXP s = new_sexp(type, (long)nrow * ncol);
  s->nrow = nrow;
  s->ncol = ncol;
  return s;
}
SEXP SET_VECTOR_ELT(SEXP x, long i, SEXP v) {
  x->elts[i] = v;
  return v;
}
SEXP Rf_mkChar(const char *str) {
  SEXP s = new_sexp(CHARSXP, 0);
  s->chr = str;
  return s;
}
SEXP Rf_namesgets(SEXP x, SEXP names) {
  x->names = names;
  return x;
}

/* Rmath / sort / RNG, R argument conventions */
double rnorm(double mu, double sd) { return or_rnorm(mu, sd); }
double runif(double a, double b) { return or_runif(a, b); }
double norm_rand(void) { return or_next_normal(); }
double unif_rand(void) { return or_next_unif(); }
double gammafn(double x) { return or_gammafn(x); }
double bessel_k_ex(double x, double alpha, double expo, double *bk) {
  (void)bk;
  const double k = or_bessel_k(x, alpha);
  return (expo == 2.0) ? exp(x) * k : k;
}
void rsort_with_index(double *x, int *indx, int n) { or_rsort_with_index(x, indx, n); }

/* routine registration */
static const R_CallMethodDef *g_routines = nullptr;
int R_registerRoutines(DllInfo *info, const void *croutines, const R_CallMethodDef *callRoutines,
                       const void *fortranRoutines, const void *externalRoutines) {
  (void)info;
  (void)croutines;
  (void)fortranRoutines;
  (void)externalRoutines;
  g_routines = callRoutines;
  return 1;
}
int R_useDynamicSymbols(DllInfo *info, Rboolean value) {
  (void)info;
  (void)value;
  return 1;
}
const R_CallMethodDef *shim_call_routines(void) { return g_routines; }

} /* extern "C" */

/* ------------------------------------------------------------ reference entry points */
extern "C" {
SEXP mkNNIndx(SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP);
SEXP mkNNIndxCB(SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP);
SEXP mkUIndx(SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP);
SEXP rNNGP(SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP,
           SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP);
SEXP cNNGP(SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP,
           SEXP, SEXP, SEXP, SEXP);
SEXP rNNGPPredict(SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP,
                  SEXP, SEXP, SEXP, SEXP);
SEXP rNNGPReplicated(SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP, SEXP,
                     SEXP, SEXP);
}
#ifndef SHIM_CALL_ONLY
/* C++-linkage helpers of the reference (src/rNNGP.cpp:46, src/cNNGP.cpp:24, src/util.cpp:208,261) */
double updateBF(double *B, double *F, double *c, double *C, double *coords, int *nnIndx,
                int *nnIndxLU, int n, int m, double *theta, int tauSqIndx, int sigmaSqIndx,
                int phiIndx, int nuIndx, int covModel, double *bk, double nuUnifb);
void updateConjBF(double *B, double *F, double *c, double *C, double *coords, int *nnIndx,
                  int *nnIndxLU, int n, int m, double phi, double alpha, double nu, int covModel,
                  double *bk, double nuMax);
double spCor(double &D, double &phi, double &nu, int &covModel, double *bk);
double Q(double *B, double *F, double *u, double *v, int n, int *nnIndx, int *nnIndxLU);
#endif

/* wrap caller memory (no copy) */
static SEXP wrap_real(const double *p, long n) {
  SEXP s = (SEXP)calloc(1, sizeof(struct shim_sexp));
  track(s);
  s->type = REALSXP;
  s->length = n;
  s->data = (void *)p;
  return s;
}
static SEXP wrap_int(const int *p, long n) {
  SEXP s = (SEXP)calloc(1, sizeof(struct shim_sexp));
  track(s);
  s->type = INTSXP;
  s->length = n;
  s->data = (void *)p;
  return s;
}
static SEXP int1(int v) {
  SEXP s = new_sexp(INTSXP, 1);
  INTEGER(s)[0] = v;
  return s;
}
static SEXP real1(double v) {
  SEXP s = new_sexp(REALSXP, 1);
  REAL(s)[0] = v;
  return s;
}
static SEXP list_get(SEXP list, const char *name) {
  if (!list || list->type != VECSXP || !list->names) return nullptr;
  for (long i = 0; i < list->length; i++)
    if (strcmp(list->names->elts[i]->chr, name) == 0) return list->elts[i];
  return nullptr;
}
static void begin_call() {
  g_error.clear();
}
static int end_call() {
  std::lock_guard<std::mutex> lk(g_alloc_mu);
  for (void *p : g_allocs) free(p);
  g_allocs.clear();
  return g_error.empty() ? 0 : -1;
}
static void copy_out(SEXP v, double *dst) {
  if (v && dst) memcpy(dst, REAL(v), sizeof(double) * v->length);
}

extern "C" {

const char *ref_last_error(void) { return g_error.c_str(); }
void ref_clear_error(void) {
  std::lock_guard<std::mutex> lk(g_alloc_mu);
  g_error.clear();
}
void ref_set_verbose(int v) { g_verbose = v; }
void ref_stream_set(const double *normals, long n_norm, const double *unifs, long n_unif) {
  or_stream_set(normals, n_norm, unifs, n_unif);
}
void ref_stream_used(long *n_norm, long *n_unif, int *overrun) { or_stream_used(n_norm, n_unif, overrun); }

int ref_mkNNIndx(int n, int m, const double *coords, int *nnIndx, double *nnDist, int *nnIndxLU,
                 int nThreads) {
  begin_call();
  long nIndx = (long)((double)(1 + m) / 2 * m + (double)(n - m - 1) * m);
  mkNNIndx(int1(n), int1(m), wrap_real(coords, 2L * n), wrap_int(nnIndx, nIndx),
           wrap_real(nnDist, nIndx), wrap_int(nnIndxLU, 2L * n), int1(nThreads));
  return end_call();
}

int ref_mkNNIndxCB(int n, int m, const double *coords, int *nnIndx, double *nnDist, int *nnIndxLU,
                   int nThreads) {
  begin_call();
  long nIndx = (long)((double)(1 + m) / 2 * m + (double)(n - m - 1) * m);
  mkNNIndxCB(int1(n), int1(m), wrap_real(coords, 2L * n), wrap_int(nnIndx, nIndx),
             wrap_real(nnDist, nIndx), wrap_int(nnIndxLU, 2L * n), int1(nThreads));
  return end_call();
}

int ref_mkUIndx(int n, int m, const int *nnIndx, int *uIndx, int *uIndxLU, int *uiIndx,
                const int *nnIndxLU, int searchType) {
  begin_call();
  long nIndx = (long)((double)(1 + m) / 2 * m + (double)(n - m - 1) * m);
  mkUIndx(int1(n), int1(m), wrap_int(nnIndx, nIndx), wrap_int(uIndx, nIndx),
          wrap_int(uIndxLU, 2L * n), wrap_int(uiIndx, nIndx), wrap_int(nnIndxLU, 2L * n),
          int1(searchType));
  return end_call();
}

#ifndef SHIM_CALL_ONLY
double ref_spCor(double D, double phi, double nu, int covModel) {
  double bk[64];
  return spCor(D, phi, nu, covModel, bk);
}

/* theta = (sigma^2, tau^2, phi[, nu]) as in src/rNNGP.cpp:182-190 */
int ref_updateBF(int n, int m, const double *coords, const int *nnIndx, const int *nnIndxLU,
                 const double *theta, int covModel, double nuUnifb, int nThreads, double *B,
                 double *F, double *logDet) {
  begin_call();
#ifdef _OPENMP
  omp_set_num_threads(nThreads);
#else
  nThreads = 1;
#endif
  double *c = (double *)R_alloc((size_t)m * nThreads, sizeof(double));
  double *C = (double *)R_alloc((size_t)m * m * nThreads, sizeof(double));
  int nb = 1 + (int)floor(nuUnifb);
  double *bk = (double *)R_alloc((size_t)nThreads * nb, sizeof(double));
  *logDet = updateBF(B, F, c, C, (double *)coords, (int *)nnIndx, (int *)nnIndxLU, n, m,
                     (double *)theta, 1, 0, 2, 3, covModel, bk, nuUnifb);
  return end_call();
}

int ref_updateConjBF(int n, int m, const double *coords, const int *nnIndx, const int *nnIndxLU,
                     double phi, double alpha, double nu, int covModel, int nThreads, double *B,
                     double *F) {
  begin_call();
#ifdef _OPENMP
  omp_set_num_threads(nThreads);
#else
  nThreads = 1;
#endif
  double *c = (double *)R_alloc((size_t)m * nThreads, sizeof(double));
  double *C = (double *)R_alloc((size_t)m * m * nThreads, sizeof(double));
  int nb = 1 + (int)floor(nu);
  double *bk = (double *)R_alloc((size_t)nThreads * nb, sizeof(double));
  updateConjBF(B, F, c, C, (double *)coords, (int *)nnIndx, (int *)nnIndxLU, n, m, phi, alpha,
               nu, covModel, bk, nu);
  return end_call();
}

double ref_Q(const double *B, const double *F, const double *u, const double *v, int n,
             const int *nnIndx, const int *nnIndxLU) {
  return Q((double *)B, (double *)F, (double *)u, (double *)v, n, (int *)nnIndx, (int *)nnIndxLU);
}

/* src/rNNGP.cpp:105-109 argument order; outputs p x nSamples, nTheta x nSamples, n x nRep */
#endif

int ref_rNNGP(const double *y, const double *X, int p, int n, int m, const double *coords,
              int covModel, const int *nnIndx, const int *nnIndxLU, const double *sigmaSqIG,
              const double *tauSqIG, const double *phiUnif, const double *nuUnif,
              const double *betaStarting, double sigmaSqStarting, double tauSqStarting,
              double phiStarting, double nuStarting, double sigmaSqTuning, double tauSqTuning,
              double phiTuning, double nuTuning, int nSamples, int nThreads, int nRep,
              const int *repIndx, double *betaSamples, double *thetaSamples, double *repSamples) {
  begin_call();
  long nIndx = (long)((double)(1 + m) / 2 * m + (double)(n - m - 1) * m);
  SEXP out = rNNGP(wrap_real(y, n), wrap_real(X, (long)n * p), int1(p), int1(n), int1(m),
                   wrap_real(coords, 2L * n), int1(covModel), wrap_int(nnIndx, nIndx),
                   wrap_int(nnIndxLU, 2L * n), wrap_real(sigmaSqIG, 2), wrap_real(tauSqIG, 2),
                   wrap_real(phiUnif, 2), wrap_real(nuUnif, 2), wrap_real(betaStarting, p),
                   real1(sigmaSqStarting), real1(tauSqStarting), real1(phiStarting),
                   real1(nuStarting), real1(sigmaSqTuning), real1(tauSqTuning), real1(phiTuning),
                   real1(nuTuning), int1(nSamples), int1(nThreads), int1(0), int1(100),
                   int1(nRep), wrap_int(repIndx, nRep ? nSamples : 1));
  copy_out(list_get(out, "p.beta.samples"), betaSamples);
  copy_out(list_get(out, "p.theta.samples"), thetaSamples);
  if (nRep) copy_out(list_get(out, "y.rep.samples"), repSamples);
  return end_call();
}

/* src/cNNGP.cpp:73-75 argument order; ab is written as 2 x g (see the stride note there) */
int ref_cNNGP(const double *y, const double *X, int p, int n, const double *coords,
              const double *thetaAlpha, const int *nnIndx, const int *nnIndxLU, const double *X0,
              const double *coords0, int n0, const int *nnIndx0, int g, int m,
              const double *sigmaSqIG, int covModel, int nThreads, double *betaHat, double *ab,
              double *bBInv, double *bb, double *y0Hat, double *y0HatVar) {
  begin_call();
  long nIndx = (long)((double)(1 + m) / 2 * m + (double)(n - m - 1) * m);
  const int nTheta = covModel == 2 ? 3 : 2;
  SEXP out = cNNGP(wrap_real(y, n), wrap_real(X, (long)n * p), int1(p), int1(n),
                   wrap_real(coords, 2L * n), wrap_real(thetaAlpha, (long)nTheta * g),
                   wrap_int(nnIndx, nIndx), wrap_int(nnIndxLU, 2L * n),
                   wrap_real(X0, (long)n0 * p), wrap_real(coords0, 2L * n0), int1(n0),
                   wrap_int(nnIndx0, (long)n0 * m), int1(g), int1(m), wrap_real(sigmaSqIG, 2),
                   int1(covModel), int1(nThreads), int1(0));
  copy_out(list_get(out, "beta.hat"), betaHat);
  SEXP abv = list_get(out, "ab");
  if (abv && ab) memcpy(ab, REAL(abv), sizeof(double) * 2 * g);
  copy_out(list_get(out, "bB.inv"), bBInv);
  copy_out(list_get(out, "bb"), bb);
  if (n0 > 0) {
    copy_out(list_get(out, "y.0.hat"), y0Hat);
    copy_out(list_get(out, "y.0.hat.var"), y0HatVar);
  }
  return end_call();
}

/* src/rNNGPPredict.cpp:25-26 argument order; output q x nSamples */
int ref_rNNGPPredict(const double *X, const double *y, const double *coords, int n, int p, int m,
                     const double *X0, const double *coords0, int q, const int *nnIndx0,
                     const double *betaSamples, const double *thetaSamples, int nSamples,
                     int covModel, int nThreads, double *y0) {
  begin_call();
  const int nTheta = covModel == 2 ? 4 : 3;
  SEXP out = rNNGPPredict(wrap_real(X, (long)n * p), wrap_real(y, n), wrap_real(coords, 2L * n),
                          int1(n), int1(p), int1(m), wrap_real(X0, (long)q * p),
                          wrap_real(coords0, 2L * q), int1(q), wrap_int(nnIndx0, (long)q * m),
                          wrap_real(betaSamples, (long)p * nSamples),
                          wrap_real(thetaSamples, (long)nTheta * nSamples), int1(nSamples),
                          int1(covModel), int1(nThreads), int1(0), int1(100));
  copy_out(list_get(out, "p.y.0"), y0);
  return end_call();
}

/* src/rNNGPReplicated.cpp:74-76 argument order; beta is nSamples x p, theta nTheta x nSamples */
int ref_rNNGPReplicated(const double *X, int p, int n, int m, const double *coords, int covModel,
                        const int *nnIndx, const int *nnIndxLU, const double *beta,
                        const double *theta, int nSamples, int nThreads, double *yRep) {
  begin_call();
  long nIndx = (long)((double)(1 + m) / 2 * m + (double)(n - m - 1) * m);
  const int nTheta = covModel == 2 ? 4 : 3;
  SEXP out = rNNGPReplicated(wrap_real(X, (long)n * p), int1(p), int1(n), int1(m),
                             wrap_real(coords, 2L * n), int1(covModel), wrap_int(nnIndx, nIndx),
                             wrap_int(nnIndxLU, 2L * n), wrap_real(beta, (long)nSamples * p),
                             wrap_real(theta, (long)nTheta * nSamples), int1(nSamples),
                             int1(nThreads), int1(0), int1(100));
  copy_out(list_get(out, "y.rep.samples"), yRep);
  return end_call();
}

} /* extern "C" */
