// The R package's .Call layer over the GB300 library: the routines R/spNNGP.R,
// R/spConjNNGP.R, R/generics.R and R/nn.R call by name, with the reference's
// arities, argument order, in-place outputs and named result lists, each
// unwrapping its SEXP arguments and calling the C ABI of include/spnngp_gb300.h.
//
//   rNNGP (28)            src/spNNGP.h:10-14   -> nngp_rNNGP
//   cNNGP (18)            src/spNNGP.h:22-24   -> nngp_cNNGP
//   rNNGPPredict (17)     src/spNNGP.h:36-37   -> nngp_rNNGPPredict
//   rNNGPReplicated (14)  src/spNNGP.h:44-46   -> nngp_rNNGPReplicated
//   mkNNIndx (7), mkNNIndxCB (7), mkUIndx (8)  src/nn.h:18,25,38 -> nngp_mkNNIndx,
//                         nngp_mkNNIndxCB, nngp_mkUIndx (written into their argument
//                         vectors, as R/nn.R expects)
//
// Random numbers: the library reads host-fed streams.  Each routine that samples
// draws them here, before the call, from R's generator (norm_rand / unif_rand
// between GetRNGstate and PutRNGstate) in exactly the order the reference consumes
// it, so a seeded R session gets the reference's draws.  rNNGP per iteration: p
// normals for beta (mvrnorm, src/util.cpp:28-41), n for a replicate when
// repIndx[s] != 0 (src/rNNGP.cpp:309-313), one per Metropolis proposal whose tuning
// is non-zero in the order phi, sigma^2, tau^2[, nu] (rnorm(mu, 0) draws nothing),
// then one uniform (src/rNNGP.cpp:327-349).  rNNGPPredict: q x nSamples normals up
// front (src/rNNGPPredict.cpp:134-136).  rNNGPReplicated: n per sample, sample by
// sample (src/rNNGPReplicated.cpp:183-189).
//
// Errors: a library status other than NNGP_OK becomes Rf_error with the library's
// message, raised on the calling (host) thread.  n.omp.threads is accepted and
// ignored (the device does the parallel work).  The library's device context is
// created on first use, on the device named by the environment variable
// SPNNGP_GB300_DEVICE (default 0), and kept for the session.
#ifndef R_NO_REMAP
#define R_NO_REMAP
#endif
#include <R.h>
#include <Rinternals.h>
#include <Rmath.h>

#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "spnngp_gb300.h"

namespace {

nngp_ctx *g_ctx = nullptr;

nngp_ctx *context() {
  if (!g_ctx) {
    const char *dev = getenv("SPNNGP_GB300_DEVICE");
    if (nngp_create(dev ? atoi(dev) : 0, &g_ctx) != NNGP_OK) {
      g_ctx = nullptr;
      Rf_error("c++ Rf_error: no usable GB300 device for spNNGP\n");
    }
  }
  return g_ctx;
}

// Raises the library's error; returns true when the caller must return (the stand-in R runtime
// used by the tests records the error and returns instead of jumping).
bool failed(int status, const char *routine) {
  if (status == NNGP_OK) return false;
  const char *msg = g_ctx ? nngp_error_message(g_ctx) : "no device";
  if (strncmp(msg, routine, strlen(routine)) == 0) Rf_error("c++ Rf_error: %s\n", msg);
  else Rf_error("c++ Rf_error: %s: %s\n", routine, msg);
  return true;
}

int int1(SEXP x) { return INTEGER(x)[0]; }
double real1(SEXP x) { return REAL(x)[0]; }

// A named list in the reference's construction (names as a list of CHARSXP).
SEXP named_list(const std::vector<SEXP> &vals, const std::vector<const char *> &names) {
  SEXP res = PROTECT(Rf_allocVector(VECSXP, (long)vals.size()));
  SEXP nm = PROTECT(Rf_allocVector(VECSXP, (long)vals.size()));
  for (size_t k = 0; k < vals.size(); k++) {
    SET_VECTOR_ELT(res, (long)k, vals[k]);
    SET_VECTOR_ELT(nm, (long)k, Rf_mkChar(names[k]));
  }
  Rf_namesgets(res, nm);
  UNPROTECT(2);
  return res;
}

}  // namespace

extern "C" {

SEXP mkNNIndx(SEXP n_r, SEXP m_r, SEXP coords_r, SEXP nnIndx_r, SEXP nnDist_r, SEXP nnIndxLU_r, SEXP nThreads_r) {
  (void)nThreads_r;
  nngp_ctx *ctx = context();
  if (!ctx) return R_NilValue;
  failed(nngp_mkNNIndx(ctx, int1(n_r), int1(m_r), REAL(coords_r), INTEGER(nnIndx_r), REAL(nnDist_r),
                       INTEGER(nnIndxLU_r)),
         "mkNNIndx");
  return R_NilValue;
}

SEXP mkNNIndxCB(SEXP n_r, SEXP m_r, SEXP coords_r, SEXP nnIndx_r, SEXP nnDist_r, SEXP nnIndxLU_r, SEXP nThreads_r) {
  (void)nThreads_r;
  nngp_ctx *ctx = context();
  if (!ctx) return R_NilValue;
  failed(nngp_mkNNIndxCB(ctx, int1(n_r), int1(m_r), REAL(coords_r), INTEGER(nnIndx_r), REAL(nnDist_r),
                         INTEGER(nnIndxLU_r)),
         "mkNNIndxCB");
  return R_NilValue;
}

SEXP mkUIndx(SEXP n_r, SEXP m_r, SEXP nnIndx_r, SEXP uIndx_r, SEXP uIndxLU_r, SEXP uiIndx_r, SEXP nnIndxLU_r,
             SEXP searchType_r) {
  nngp_ctx *ctx = context();
  if (!ctx) return R_NilValue;
  failed(nngp_mkUIndx(ctx, int1(n_r), int1(m_r), INTEGER(nnIndx_r), INTEGER(uIndx_r), INTEGER(uIndxLU_r),
                      INTEGER(uiIndx_r), INTEGER(nnIndxLU_r), int1(searchType_r)),
         "mkUIndx");
  return R_NilValue;
}

SEXP rNNGP(SEXP y_r, SEXP X_r, SEXP p_r, SEXP n_r, SEXP m_r, SEXP coords_r, SEXP covModel_r, SEXP nnIndx_r,
           SEXP nnIndxLU_r, SEXP sigmaSqIG_r, SEXP tauSqIG_r, SEXP phiUnif_r, SEXP nuUnif_r, SEXP betaStarting_r,
           SEXP sigmaSqStarting_r, SEXP tauSqStarting_r, SEXP phiStarting_r, SEXP nuStarting_r,
           SEXP sigmaSqTuning_r, SEXP tauSqTuning_r, SEXP phiTuning_r, SEXP nuTuning_r, SEXP nSamples_r,
           SEXP nThreads_r, SEXP verbose_r, SEXP nReport_r, SEXP nRep_r, SEXP repIndx_r) {
  (void)nThreads_r;
  (void)nReport_r;
  nngp_ctx *ctx = context();
  if (!ctx) return R_NilValue;
  const int p = int1(p_r), n = int1(n_r), m = int1(m_r), covModel = int1(covModel_r);
  const int nSamples = int1(nSamples_r), nRep = int1(nRep_r);
  const int *repIndx = INTEGER(repIndx_r);
  const bool matern = covModel == 2;
  const int nTheta = matern ? 4 : 3;
  const double theta0[4] = {real1(sigmaSqStarting_r), real1(tauSqStarting_r), real1(phiStarting_r),
                            matern ? real1(nuStarting_r) : 0.0};
  const double tuning[4] = {real1(sigmaSqTuning_r), real1(tauSqTuning_r), real1(phiTuning_r),
                            matern ? real1(nuTuning_r) : 0.0};
  const double nuUnif[2] = {matern ? REAL(nuUnif_r)[0] : 0.0, matern ? REAL(nuUnif_r)[1] : 0.0};
  if (int1(verbose_r))
    Rprintf("NNGP response model: %i observations, %i covariates, %i neighbors, %i samples on a GB300.\n", n, p,
            m, nSamples);
  // the streams, in the reference's consumption order
  std::vector<double> normals, unifs;
  int perIter = p;
  for (int k : {2, 0, 1, 3})
    if (k < nTheta && tuning[k] > 0.0) perIter++;
  normals.reserve((size_t)nSamples * perIter + (size_t)nRep * n);
  unifs.reserve(nSamples);
  GetRNGstate();
  for (int s = 0; s < nSamples; s++) {
    for (int i = 0; i < p; i++) normals.push_back(norm_rand());
    if (nRep && repIndx[s])
      for (int i = 0; i < n; i++) normals.push_back(norm_rand());
    for (int k : {2, 0, 1, 3})  // proposals: phi, sigma^2, tau^2, nu
      if (k < nTheta && tuning[k] > 0.0) normals.push_back(norm_rand());
    unifs.push_back(unif_rand());
  }
  PutRNGstate();
  SEXP beta_r = PROTECT(Rf_allocMatrix(REALSXP, p, nSamples));
  SEXP theta_r = PROTECT(Rf_allocMatrix(REALSXP, nTheta, nSamples));
  SEXP rep_r = nRep ? PROTECT(Rf_allocMatrix(REALSXP, n, nRep)) : R_NilValue;
  int accept = 0;
  const int st = nngp_rNNGP(ctx, REAL(y_r), REAL(X_r), p, n, m, REAL(coords_r), covModel, INTEGER(nnIndx_r),
                            INTEGER(nnIndxLU_r), REAL(sigmaSqIG_r), REAL(tauSqIG_r), REAL(phiUnif_r), nuUnif,
                            REAL(betaStarting_r), theta0, tuning, nSamples, nRep, repIndx, normals.data(),
                            (int64_t)normals.size(), unifs.data(), (int64_t)unifs.size(), NNGP_FP64, REAL(beta_r),
                            REAL(theta_r), nRep ? REAL(rep_r) : nullptr, &accept);
  if (failed(st, "rNNGP")) {
    UNPROTECT(nRep ? 3 : 2);
    return R_NilValue;
  }
  if (int1(verbose_r))
    Rprintf("Overall Metrop. Acceptance rate: %3.2f%%\n", nSamples ? 100.0 * accept / nSamples : 0.0);
  SEXP res = nRep ? named_list({beta_r, theta_r, rep_r}, {"p.beta.samples", "p.theta.samples", "y.rep.samples"})
                  : named_list({beta_r, theta_r}, {"p.beta.samples", "p.theta.samples"});
  UNPROTECT(nRep ? 3 : 2);
  return res;
}

SEXP cNNGP(SEXP y_r, SEXP X_r, SEXP p_r, SEXP n_r, SEXP coords_r, SEXP thetaAlpha_r, SEXP nnIndx_r,
           SEXP nnIndxLU_r, SEXP X0_r, SEXP coords0_r, SEXP n0_r, SEXP nnIndx0_r, SEXP g_r, SEXP m_r,
           SEXP sigmaSqIG_r, SEXP covModel_r, SEXP nThreads_r, SEXP verbose_r) {
  (void)nThreads_r;
  nngp_ctx *ctx = context();
  if (!ctx) return R_NilValue;
  const int p = int1(p_r), n = int1(n_r), n0 = int1(n0_r), g = int1(g_r), m = int1(m_r);
  const int covModel = int1(covModel_r);
  const int nTheta = covModel == 2 ? 3 : 2;  // (phi, alpha[, nu]) per grid point
  if (int1(verbose_r))
    Rprintf("Conjugate NNGP: %i observations, %i covariates, %i neighbors, %i parameter sets on a GB300.\n", n, p,
            m, g);
  SEXP beta_r = PROTECT(Rf_allocMatrix(REALSXP, p, g));
  SEXP ab_r = PROTECT(Rf_allocMatrix(REALSXP, nTheta, g));  // a, b packed in the first 2 g entries
  SEXP bBInv_r = PROTECT(Rf_allocMatrix(REALSXP, p * p, g));
  SEXP bb_r = PROTECT(Rf_allocMatrix(REALSXP, p, g));
  SEXP y0_r = PROTECT(Rf_allocMatrix(REALSXP, n0, g));
  SEXP y0var_r = PROTECT(Rf_allocMatrix(REALSXP, n0, g));
  memset(REAL(ab_r), 0, sizeof(double) * (size_t)nTheta * g);
  const int st = nngp_cNNGP(ctx, REAL(y_r), REAL(X_r), p, n, REAL(coords_r), REAL(thetaAlpha_r), INTEGER(nnIndx_r),
                            INTEGER(nnIndxLU_r), n0 ? REAL(X0_r) : nullptr, n0 ? REAL(coords0_r) : nullptr, n0,
                            n0 ? INTEGER(nnIndx0_r) : nullptr, g, m, REAL(sigmaSqIG_r), covModel, NNGP_FP64,
                            REAL(beta_r), REAL(ab_r), REAL(bBInv_r), REAL(bb_r), n0 ? REAL(y0_r) : nullptr,
                            n0 ? REAL(y0var_r) : nullptr);
  if (failed(st, "cNNGP")) {
    UNPROTECT(6);
    return R_NilValue;
  }
  SEXP res = n0 ? named_list({beta_r, ab_r, bBInv_r, bb_r, y0_r, y0var_r},
                             {"beta.hat", "ab", "bB.inv", "bb", "y.0.hat", "y.0.hat.var"})
                : named_list({beta_r, ab_r, bBInv_r, bb_r}, {"beta.hat", "ab", "bB.inv", "bb"});
  UNPROTECT(6);
  return res;
}

SEXP rNNGPPredict(SEXP X_r, SEXP y_r, SEXP coords_r, SEXP n_r, SEXP p_r, SEXP m_r, SEXP X0_r, SEXP coords0_r,
                  SEXP q_r, SEXP nnIndx0_r, SEXP betaSamples_r, SEXP thetaSamples_r, SEXP nSamples_r,
                  SEXP covModel_r, SEXP nThreads_r, SEXP verbose_r, SEXP nReport_r) {
  (void)nThreads_r;
  (void)nReport_r;
  nngp_ctx *ctx = context();
  if (!ctx) return R_NilValue;
  const int n = int1(n_r), p = int1(p_r), m = int1(m_r), q = int1(q_r), nSamples = int1(nSamples_r);
  if (int1(verbose_r)) Rprintf("Predicting at %i locations from %i samples on a GB300.\n", q, nSamples);
  std::vector<double> z((size_t)q * nSamples);
  GetRNGstate();
  for (double &v : z) v = norm_rand();
  PutRNGstate();
  SEXP y0_r = PROTECT(Rf_allocMatrix(REALSXP, q, nSamples));
  const int st = nngp_rNNGPPredict(ctx, REAL(X_r), REAL(y_r), REAL(coords_r), n, p, m, REAL(X0_r), REAL(coords0_r),
                                   q, INTEGER(nnIndx0_r), REAL(betaSamples_r), REAL(thetaSamples_r), nSamples,
                                   int1(covModel_r), z.data(), NNGP_FP64, REAL(y0_r));
  if (failed(st, "rNNGPPredict")) {
    UNPROTECT(1);
    return R_NilValue;
  }
  SEXP res = named_list({y0_r}, {"p.y.0"});
  UNPROTECT(1);
  return res;
}

SEXP rNNGPReplicated(SEXP X_r, SEXP p_r, SEXP n_r, SEXP m_r, SEXP coords_r, SEXP covModel_r, SEXP nnIndx_r,
                     SEXP nnIndxLU_r, SEXP beta_r, SEXP theta_r, SEXP nSamples_r, SEXP nThreads_r, SEXP verbose_r,
                     SEXP nReport_r) {
  (void)nThreads_r;
  (void)nReport_r;
  nngp_ctx *ctx = context();
  if (!ctx) return R_NilValue;
  const int p = int1(p_r), n = int1(n_r), m = int1(m_r), nSamples = int1(nSamples_r);
  if (int1(verbose_r)) Rprintf("Replicating %i samples at %i locations on a GB300.\n", nSamples, n);
  std::vector<double> z((size_t)n * nSamples);
  GetRNGstate();
  for (double &v : z) v = norm_rand();
  PutRNGstate();
  SEXP rep_r = PROTECT(Rf_allocMatrix(REALSXP, n, nSamples));
  const int st = nngp_rNNGPReplicated(ctx, REAL(X_r), p, n, m, REAL(coords_r), int1(covModel_r), INTEGER(nnIndx_r),
                                      INTEGER(nnIndxLU_r), REAL(beta_r), REAL(theta_r), nSamples, z.data(), NNGP_FP64,
                                      REAL(rep_r));
  if (failed(st, "rNNGPReplicated")) {
    UNPROTECT(1);
    return R_NilValue;
  }
  SEXP res = named_list({rep_r}, {"y.rep.samples"});
  UNPROTECT(1);
  return res;
}

// Releases the device context (R_unload_spNNGP calls it when the package is unloaded).
void nngp_call_release(void) {
  if (g_ctx) nngp_destroy(g_ctx);
  g_ctx = nullptr;
}

}  // extern "C"
