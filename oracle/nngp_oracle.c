/*
 * TEST ORACLE ONLY -- a CPU restatement of the spNNGP (v1.0.1) response /
 * conjugate NNGP hot path.  It is the checker for the CUDA product library
 * and the timed CPU baseline; the product never links, loads or calls it.
 *
 * Each function follows the reference routine cited beside it (paths are
 * relative to the spNNGP source tree).  The arithmetic order of the
 * reference is kept where results depend on it:
 *   - neighbor search: FP64 squared distances dx*dx + dy*dy and the
 *     mean-distance key ((x_i + y_i) - x_j) - y_j, no FMA contraction
 *     (build with -ffp-contract=off), strict '<' acceptance, Shell-sort list
 *     maintenance (R's rsort_with_index, oracle/rmath.c);
 *   - B/F: potrf -> potri (explicit inverse) -> symv, as LAPACK is called in
 *     src/rNNGP.cpp:86-89;
 *   - Q: serial sum over locations when run on one thread.
 * Random numbers come from host-fed streams (oracle/rmath.c) consumed in the
 * reference's order, so MCMC runs can be replayed draw for draw.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <limits.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* BLAS/LAPACK subset (oracle/linalg.c) */
double ddot_(const int *n, const double *x, const int *incx, const double *y, const int *incy);
void dcopy_(const int *n, const double *x, const int *incx, double *y, const int *incy);
void daxpy_(const int *n, const double *a, const double *x, const int *incx, double *y, const int *incy);
void dgemv_(const char *trans, const int *m, const int *n, const double *alpha, const double *a,
            const int *lda, const double *x, const int *incx, const double *beta, double *y, const int *incy);
void dsymv_(const char *uplo, const int *n, const double *alpha, const double *a, const int *lda,
            const double *x, const int *incx, const double *beta, double *y, const int *incy);
void dtrmv_(const char *uplo, const char *trans, const char *diag, const int *n, const double *a,
            const int *lda, double *x, const int *incx);
void dpotrf_(const char *uplo, const int *n, double *a, const int *lda, int *info);
void dpotri_(const char *uplo, const int *n, double *a, const int *lda, int *info);
/* Rmath stand-ins (oracle/rmath.c) */
double or_bessel_k(double x, double nu);
double or_gammafn(double x);
void or_rsort_with_index(double *x, int *idx, int n);
double or_rnorm(double mu, double sd);
double or_runif(double a, double b);

static const int ONE_I = 1;
static const double ONE_D = 1.0, ZERO_D = 0.0, NEG_ONE_D = -1.0;

static int set_threads(int t) {
#ifdef _OPENMP
  if (t < 1) t = 1;
  omp_set_num_threads(t);
  return t;
#else
  (void)t;
  return 1;
#endif
}
static int thread_id(void) {
#ifdef _OPENMP
  return omp_get_thread_num();
#else
  return 0;
#endif
}

/* ------------------------------------------------------------------ indexing */

/* Offset and length of location i's block in the packed neighbor arrays
 * (src/util.cpp:55-70). */
void or_get_nn_indx(int i, int m, int *off, int *cnt) {
  if (i == 0) { *off = 0; *cnt = 0; return; }
  if (i < m) { *off = (int)((double)i / 2 * (i - 1)); *cnt = i; return; }
  *off = (int)((double)m / 2 * (m - 1) + (i - m) * m);
  *cnt = m;
}

/* Length of the packed neighbor arrays (src/rNNGP.cpp:218). */
long or_n_indx(int n, int m) { return (long)((double)(1 + m) / 2 * m + (double)(n - m - 1) * m); }

/* ---------------------------------------------------------------- correlation */

/* Euclidean distance as src/util.cpp:51-53 forms it. */
static double dist2(double ax, double ay, double bx, double by) {
  const double dx = ax - bx, dy = ay - by;
  return sqrt(dx * dx + dy * dy);
}

/* Correlation rho(D) for covModel 0 exponential, 1 spherical, 2 matern, 3 gaussian
 * (src/util.cpp:208-245). */
double or_spcor(double d, double phi, double nu, int model) {
  if (model == 0) return exp(-phi * d);
  if (model == 1) {
    if (d > 0 && d <= 1.0 / phi) {
      const double t = phi * d;
      return 1.0 - 1.5 * t + 0.5 * (t * t * t);
    }
    if (d >= 1.0 / phi) return 0.0;
    return 1.0;
  }
  if (model == 2) {
    const double x = d * phi;
    if (x > 0.0) return pow(x, nu) / (pow(2.0, nu - 1.0) * or_gammafn(nu)) * or_bessel_k(x, nu);
    return 1.0;
  }
  if (model == 3) {
    const double t = phi * d;
    return exp(-1.0 * (t * t));
  }
  return NAN;
}

/* ------------------------------------------------------------- neighbor search */

/* Brute-force ordered kNN: for each i, scan j = 0..i-1 and keep the m smallest
 * Euclidean distances, replacing the current worst on a strict '<' and re-sorting
 * the list (src/nn.cpp:63-111).  nnIndxLU = [offsets | counts]. */
void or_mkNNIndx(int n, int m, const double *coords, int *nnIndx, double *nnDist, int *nnIndxLU,
                 int nthreads) {
  const long nIndx = or_n_indx(n, m);
  for (long k = 0; k < nIndx; k++) nnDist[k] = INFINITY;
  set_threads(nthreads);
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (int i = 0; i < n; i++) {
    int off, cnt;
    or_get_nn_indx(i, m, &off, &cnt);
    nnIndxLU[i] = off;
    nnIndxLU[n + i] = cnt;
    if (i == 0) continue;
    double *dl = nnDist + off;
    int *il = nnIndx + off;
    for (int j = 0; j < i; j++) {
      const double d = dist2(coords[i], coords[n + i], coords[j], coords[n + j]);
      if (d < dl[cnt - 1]) {
        dl[cnt - 1] = d;
        il[cnt - 1] = j;
        or_rsort_with_index(dl, il, cnt);
      }
    }
  }
}

/* Mean-distance-ordered search of Ra & Kim (1993) for one location (src/nn.cpp:128-211):
 * walk the u = x+y sorted order alternately down and up from the query's own position,
 * stop a direction once (u_q - u_j)^2 > 2*worst, accept predecessors (original index
 * below the query's) whose squared distance beats the current worst. */
static void cb_one(int cnt, int n, const double *coords, int qpos, const int *sidx, int *outIdx,
                   double *outDist) {
  for (int k = 0; k < cnt; k++) outDist[k] = INFINITY;
  const int q = sidx[qpos];
  const double qx = coords[q], qy = coords[n + q];
  int lo = qpos, hi = qpos;
  int down = 1, up = 1;
  while (down || up) {
    if (lo == 0) down = 0;
    if (hi == n - 1) up = 0;
    if (down) {
      lo--;
      const int j = sidx[lo];
      const double du = ((qx + qy) - coords[j]) - coords[n + j];
      const double dm = du * du;
      if (dm > 2 * outDist[cnt - 1]) {
        down = 0;
      } else {
        const double dx = qx - coords[j], dy = qy - coords[n + j];
        const double de = dx * dx + dy * dy;
        if (de < outDist[cnt - 1] && j < q) {
          outDist[cnt - 1] = de;
          outIdx[cnt - 1] = j;
          or_rsort_with_index(outDist, outIdx, cnt);
        }
      }
    }
    if (up) {
      hi++;
      const int j = sidx[hi];
      const double du = ((qx + qy) - coords[j]) - coords[n + j];
      const double dm = du * du;
      if (dm > 2 * outDist[cnt - 1]) {
        up = 0;
      } else {
        const double dx = qx - coords[j], dy = qy - coords[n + j];
        const double de = dx * dx + dy * dy;
        if (de < outDist[cnt - 1] && j < q) {
          outDist[cnt - 1] = de;
          outIdx[cnt - 1] = j;
          or_rsort_with_index(outDist, outIdx, cnt);
        }
      }
    }
  }
  for (int k = 0; k < cnt; k++) outDist[k] = sqrt(outDist[k]);
}

/* Ordered kNN by the code-book search (src/nn.cpp:213-258): sort u = x+y with its
 * index by R's Shell sort, then search every location from its sorted position. */
void or_mkNNIndxCB(int n, int m, const double *coords, int *nnIndx, double *nnDist, int *nnIndxLU,
                   int nthreads) {
  int *sidx = (int *)malloc(sizeof(int) * (size_t)n);
  double *u = (double *)malloc(sizeof(double) * (size_t)n);
  for (int i = 0; i < n; i++) {
    sidx[i] = i;
    u[i] = coords[i] + coords[n + i];
  }
  or_rsort_with_index(u, sidx, n);
  set_threads(nthreads);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256)
#endif
  for (int s = 0; s < n; s++) {
    int off, cnt;
    const int i = sidx[s];
    or_get_nn_indx(i, m, &off, &cnt);
    nnIndxLU[i] = off;
    nnIndxLU[n + i] = cnt;
    /* location 0 owns no slot; the reference still runs the search with a zero-length list */
    if (cnt > 0) cb_one(cnt, n, coords, s, sidx, nnIndx + off, nnDist + off);
  }
  free(sidx);
  free(u);
}

/* "Who has i as a neighbor": counting-sort transpose of the packed lists (CSR -> CSC,
 * src/util.cpp:115-185) for search types 0 and 2 (rows in increasing order); type 1
 * lists them in decreasing order (src/util.cpp:93-112).  uiIndx holds the position of i
 * inside each such list (src/nn.cpp:48-53, first match as src/util.cpp:248-258). */
void or_mkUIndx(int n, int m, const int *nnIndx, const int *nnIndxLU, int *uIndx, int *uIndxLU,
                int *uiIndx, int searchType) {
  (void)m;
  int *fill = (int *)calloc((size_t)n + 1, sizeof(int));
  for (int i = 0; i < n; i++)
    for (int k = 0; k < nnIndxLU[n + i]; k++) fill[nnIndx[nnIndxLU[i] + k]]++;
  int run = 0;
  for (int c = 0; c < n; c++) {
    uIndxLU[c] = run;
    uIndxLU[n + c] = fill[c];
    run += fill[c];
    fill[c] = 0;
  }
  for (int r = 0; r < n; r++) {
    for (int k = 0; k < nnIndxLU[n + r]; k++) {
      const int c = nnIndx[nnIndxLU[r] + k];
      uIndx[uIndxLU[c] + fill[c]++] = r;
    }
  }
  if (searchType == 1) {
    for (int c = 0; c < n; c++) {
      int *a = uIndx + uIndxLU[c];
      for (int lo = 0, hi = uIndxLU[n + c] - 1; lo < hi; lo++, hi--) {
        const int t = a[lo];
        a[lo] = a[hi];
        a[hi] = t;
      }
    }
  }
  for (int i = 0; i < n; i++) {
    for (int j = 0; j < uIndxLU[n + i]; j++) {
      const int k = uIndx[uIndxLU[i] + j];
      int pos = -1;
      for (int t = 0; t < nnIndxLU[n + k]; t++)
        if (nnIndx[nnIndxLU[k] + t] == i) { pos = t; break; }
      uiIndx[uIndxLU[i] + j] = pos;
    }
  }
  free(fill);
}

/* Exact kNN of prediction points among all training points: the role RANN::nn2 plays at
 * R/spConjNNGP.R:158,311 and R/generics.R:642.  Ordered by FP64 squared distance, ties by
 * the smaller training index.  nnIdx is n0 x k column-major, 0-based. */
void or_nn2(int n, const double *coords, int n0, const double *coords0, int k, int *nnIdx,
            double *nnDist, int nthreads) {
  set_threads(nthreads);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64)
#endif
  for (int q = 0; q < n0; q++) {
    double bd[64];
    int bi[64];
    int cnt = 0;
    const double qx = coords0[q], qy = coords0[n0 + q];
    for (int j = 0; j < n; j++) {
      const double dx = qx - coords[j], dy = qy - coords[n + j];
      const double de = dx * dx + dy * dy;
      if (cnt == k && !(de < bd[k - 1])) continue;
      int pos = (cnt < k) ? cnt++ : k - 1;
      while (pos > 0 && bd[pos - 1] > de) {
        bd[pos] = bd[pos - 1];
        bi[pos] = bi[pos - 1];
        pos--;
      }
      bd[pos] = de;
      bi[pos] = j;
    }
    for (int t = 0; t < k; t++) {
      nnIdx[(long)t * n0 + q] = bi[t];
      if (nnDist) nnDist[(long)t * n0 + q] = sqrt(bd[t]);
    }
  }
}

/* ------------------------------------------------------------------ B and F */

/* B_i = C_NN^-1 c_iN, F_i = sigma^2 + tau^2 - B_i'c_iN for every location, with the
 * neighborhood covariance built from spCor and factored potrf -> potri -> symv
 * (src/rNNGP.cpp:46-101).  sigmaSq multiplies the correlations and tauSq is the nugget;
 * the conjugate form (src/cNNGP.cpp:24-69) is sigmaSq = 1, tauSq = alpha.
 * Returns 0, or -(i+1) for the first location whose neighborhood is not SPD. */
int or_updateBF(int n, int m, const double *coords, const int *nnIndx, const int *nnIndxLU,
                int model, double sigmaSq, double tauSq, double phi, double nu, double *B,
                double *F, double *logDet, int nthreads) {
  const int T = set_threads(nthreads);
  double *cbuf = (double *)malloc(sizeof(double) * (size_t)m * T);
  double *Cbuf = (double *)malloc(sizeof(double) * (size_t)m * m * T);
  int bad = INT_MAX;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (int i = 0; i < n; i++) {
    const int t = thread_id();
    double *c = cbuf + (size_t)m * t;
    double *C = Cbuf + (size_t)m * m * t;
    if (i == 0) {
      B[0] = 0;
      F[0] = sigmaSq + tauSq;
      continue;
    }
    const int mi = nnIndxLU[n + i];
    const int *nb = nnIndx + nnIndxLU[i];
    for (int k = 0; k < mi; k++) {
      const int a = nb[k];
      c[k] = sigmaSq * or_spcor(dist2(coords[i], coords[n + i], coords[a], coords[n + a]), phi, nu, model);
      for (int l = 0; l <= k; l++) {
        const int b = nb[l];
        double v = sigmaSq * or_spcor(dist2(coords[a], coords[n + a], coords[b], coords[n + b]), phi, nu, model);
        if (l == k) v += tauSq;
        C[l * mi + k] = v;
      }
    }
    int info = 0;
    dpotrf_("L", &mi, C, &mi, &info);
    if (info == 0) dpotri_("L", &mi, C, &mi, &info);
    if (info != 0) {
#ifdef _OPENMP
#pragma omp critical
#endif
      { if (i < bad) bad = i; }
    }
    double *Bi = B + nnIndxLU[i];
    dsymv_("L", &mi, &ONE_D, C, &mi, c, &ONE_I, &ZERO_D, Bi, &ONE_I);
    F[i] = sigmaSq - ddot_(&mi, Bi, &ONE_I, c, &ONE_I) + tauSq;
  }
  double s = 0;
  for (int i = 0; i < n; i++) s += log(F[i]);
  *logDet = s;
  free(cbuf);
  free(Cbuf);
  return bad == INT_MAX ? 0 : -(bad + 1);
}

/* u'(I-B)'F^-1(I-B)v (src/util.cpp:261-280). */
double or_Q(const double *B, const double *F, const double *u, const double *v, int n,
            const int *nnIndx, const int *nnIndxLU, int nthreads) {
  set_threads(nthreads);
  double q = 0;
#ifdef _OPENMP
#pragma omp parallel for reduction(+ : q) schedule(static)
#endif
  for (int i = 0; i < n; i++) {
    double a = 0, b = 0;
    for (int j = 0; j < nnIndxLU[n + i]; j++) {
      a += B[nnIndxLU[i] + j] * u[nnIndx[nnIndxLU[i] + j]];
      b += B[nnIndxLU[i] + j] * v[nnIndx[nnIndxLU[i] + j]];
    }
    q += (u[i] - a) * (v[i] - b) / F[i];
  }
  return q;
}

/* ----------------------------------------------------------------- MCMC */

/* beta ~ N(mu, L L') with L lower (src/util.cpp:28-41). */
static void mvrnorm(double *des, const double *mu, const double *L, int dim) {
  for (int i = 0; i < dim; i++) des[i] = or_rnorm(0, 1);
  dtrmv_("L", "N", "N", &dim, L, &dim, des, &ONE_I);
  daxpy_(&dim, &ONE_D, mu, &ONE_I, des, &ONE_I);
}
static double logit_(double t, double a, double b) { return log((t - a) / (b - t)); }
static double logit_inv(double z, double a, double b) { return b - (b - a) / (1 + exp(z)); }

/* Replicate draw v_i = B_i v_N(i) + sqrt(F_i) z_i, sequential over i (src/rNNGP.cpp:24-42). */
static void update_rep(const double *B, const double *F, int n, double *out, const int *nnIndx,
                       const int *nnIndxLU) {
  for (int i = 0; i < n; i++) {
    const double z = or_rnorm(0.0, 1.0);
    if (i == 0) {
      out[i] = sqrt(F[i]) * z;
    } else {
      double s = 0;
      for (int j = 0; j < nnIndxLU[n + i]; j++) s += B[nnIndxLU[i] + j] * out[nnIndx[nnIndxLU[i] + j]];
      out[i] = s + sqrt(F[i]) * z;
    }
  }
}

/* Log target of the response model: -0.5 logdet - 0.5 Q plus the priors and the Jacobians of
 * the logit / log proposal scales (src/rNNGP.cpp:317-324,340-347). theta = (s2, t2, phi[, nu]). */
static double log_post(double logDet, double q, const double *th, int matern, const double *sIG,
                       const double *tIG, const double *pU, const double *nU) {
  double lp = -0.5 * logDet - 0.5 * q;
  lp += log(th[2] - pU[0]) + log(pU[1] - th[2]);
  lp += -1.0 * (1.0 + sIG[0]) * log(th[0]) - sIG[1] / th[0] + log(th[0]);
  lp += -1.0 * (1.0 + tIG[0]) * log(th[1]) - tIG[1] / th[1] + log(th[1]);
  if (matern) lp += log(th[3] - nU[0]) + log(nU[1] - th[3]);
  return lp;
}

/* Response-model Metropolis-within-Gibbs (src/rNNGP.cpp:103-421). y n, X n x p, coords n x 2,
 * all column-major and already in the NNGP order.  Outputs betaSamples p x nSamples,
 * thetaSamples nTheta x nSamples (s2, t2, phi[, nu]), repSamples n x nRep; acceptance count in
 * *nAccept.  Returns 0, or a negative status (-(i+1): location i not SPD; -1000000000: the
 * beta Gram was not SPD). */
int or_rNNGP(const double *y, const double *X, int p, int n, int m, const double *coords,
             int covModel, const int *nnIndx, const int *nnIndxLU, const double *sigmaSqIG,
             const double *tauSqIG, const double *phiUnif, const double *nuUnif,
             const double *betaStarting, const double *thetaStarting, const double *tuningIn,
             int nSamples, int nthreads, int nRep, const int *repIndx, double *betaSamples,
             double *thetaSamples, double *repSamples, int *nAccept) {
  const int matern = covModel == 2;
  const int nTheta = matern ? 4 : 3;
  double theta[4] = {0}, cand[4] = {0}, tuning[4] = {0};
  for (int k = 0; k < nTheta; k++) { theta[k] = thetaStarting[k]; tuning[k] = tuningIn[k]; }
  const long nIndx = or_n_indx(n, m);
  double *beta = (double *)malloc(sizeof(double) * p);
  memcpy(beta, betaStarting, sizeof(double) * p);
  double *B = (double *)malloc(sizeof(double) * nIndx);
  double *F = (double *)malloc(sizeof(double) * n);
  double *tmp_n = (double *)malloc(sizeof(double) * n);
  double *rep = nRep ? (double *)malloc(sizeof(double) * n) : NULL;
  double *Gxx = (double *)calloc((size_t)p * p, sizeof(double));
  double *gxy = (double *)malloc(sizeof(double) * p);
  double *mean = (double *)malloc(sizeof(double) * p);
  if (nRep) memset(repSamples, 0, sizeof(double) * (size_t)n * nRep);
  int st = 0, accept = 0, repCnt = 0, info = 0;
  double logDet;
  const double nu0 = matern ? theta[3] : 0;
  st = or_updateBF(n, m, coords, nnIndx, nnIndxLU, covModel, theta[0], theta[1], theta[2], nu0, B,
                   F, &logDet, nthreads);
  if (st) goto done;
  int thetaUpdate = 1;
  for (int s = 0; s < nSamples; s++) {
    if (thetaUpdate) {
      thetaUpdate = 0;
      for (int i = 0; i < p; i++) {
        gxy[i] = or_Q(B, F, X + (size_t)n * i, y, n, nnIndx, nnIndxLU, nthreads);
        for (int j = 0; j <= i; j++)
          Gxx[j * p + i] = or_Q(B, F, X + (size_t)n * j, X + (size_t)n * i, n, nnIndx, nnIndxLU, nthreads);
      }
      dpotrf_("L", &p, Gxx, &p, &info);
      if (info == 0) dpotri_("L", &p, Gxx, &p, &info);
      if (info != 0) { st = -1000000000; goto done; }
      dsymv_("L", &p, &ONE_D, Gxx, &p, gxy, &ONE_I, &ZERO_D, mean, &ONE_I);
      dpotrf_("L", &p, Gxx, &p, &info);
      if (info != 0) { st = -1000000000; goto done; }
    }
    mvrnorm(beta, mean, Gxx, p);
    dgemv_("N", &n, &p, &ONE_D, X, &n, beta, &ONE_I, &ZERO_D, tmp_n, &ONE_I);
    if (nRep && repIndx[s]) dcopy_(&n, tmp_n, &ONE_I, repSamples + (size_t)repCnt * n, &ONE_I);
    daxpy_(&n, &NEG_ONE_D, y, &ONE_I, tmp_n, &ONE_I);

    st = or_updateBF(n, m, coords, nnIndx, nnIndxLU, covModel, theta[0], theta[1], theta[2],
                     matern ? theta[3] : 0, B, F, &logDet, nthreads);
    if (st) goto done;
    if (nRep && repIndx[s]) {
      update_rep(B, F, n, rep, nnIndx, nnIndxLU);
      daxpy_(&n, &ONE_D, rep, &ONE_I, repSamples + (size_t)repCnt * n, &ONE_I);
      repCnt++;
    }
    double q = or_Q(B, F, tmp_n, tmp_n, n, nnIndx, nnIndxLU, nthreads);
    const double lpCur = log_post(logDet, q, theta, matern, sigmaSqIG, tauSqIG, phiUnif, nuUnif);

    cand[2] = logit_inv(or_rnorm(logit_(theta[2], phiUnif[0], phiUnif[1]), tuning[2]), phiUnif[0], phiUnif[1]);
    cand[0] = exp(or_rnorm(log(theta[0]), tuning[0]));
    cand[1] = exp(or_rnorm(log(theta[1]), tuning[1]));
    if (matern) cand[3] = logit_inv(or_rnorm(logit_(theta[3], nuUnif[0], nuUnif[1]), tuning[3]), nuUnif[0], nuUnif[1]);

    st = or_updateBF(n, m, coords, nnIndx, nnIndxLU, covModel, cand[0], cand[1], cand[2],
                     matern ? cand[3] : 0, B, F, &logDet, nthreads);
    if (st) goto done;
    q = or_Q(B, F, tmp_n, tmp_n, n, nnIndx, nnIndxLU, nthreads);
    const double lpCand = log_post(logDet, q, cand, matern, sigmaSqIG, tauSqIG, phiUnif, nuUnif);
    if (or_runif(0.0, 1.0) <= exp(lpCand - lpCur)) {
      thetaUpdate = 1;
      memcpy(theta, cand, sizeof(double) * nTheta);
      accept++;
    }
    memcpy(betaSamples + (size_t)s * p, beta, sizeof(double) * p);
    memcpy(thetaSamples + (size_t)s * nTheta, theta, sizeof(double) * nTheta);
  }
done:
  if (nAccept) *nAccept = accept;
  free(beta); free(B); free(F); free(tmp_n); free(rep); free(Gxx); free(gxy); free(mean);
  return st;
}

/* --------------------------------------------------------------- conjugate */

/* Conjugate NNGP fit over g (phi, alpha[, nu]) sets and prediction at n0 points
 * (src/cNNGP.cpp:73-358).  thetaAlpha is nTheta x g; nnIndx0 n0 x m column-major.  Outputs:
 * betaHat p x g, ab 2 x g (a*, b*), bBInv p*p x g (lower triangle valid, as dpotri leaves it),
 * bb p x g, y0Hat n0 x g, y0HatVar n0 x g. */
int or_cNNGP(const double *y, const double *X, int p, int n, const double *coords,
             const double *thetaAlpha, const int *nnIndx, const int *nnIndxLU, const double *X0,
             const double *coords0, int n0, const int *nnIndx0, int g, int m,
             const double *sigmaSqIG, int covModel, int nthreads, double *betaHat, double *ab,
             double *bBInv, double *bb, double *y0Hat, double *y0HatVar) {
  const int nTheta = covModel == 2 ? 3 : 2;
  const int T = set_threads(nthreads);
  const long nIndx = or_n_indx(n, m);
  double *B = (double *)malloc(sizeof(double) * nIndx);
  double *F = (double *)malloc(sizeof(double) * n);
  double *V = (double *)calloc((size_t)p * p, sizeof(double)); /* upper triangle stays 0, as R_alloc'd scratch is never written there */
  double *v = (double *)malloc(sizeof(double) * p);
  double *C0 = (double *)malloc(sizeof(double) * (size_t)m * m * T);
  double *c0 = (double *)malloc(sizeof(double) * (size_t)m * T);
  double *w = (double *)malloc(sizeof(double) * (size_t)m * T);
  double *r = (double *)malloc(sizeof(double) * (size_t)m * T);
  double *u = (double *)malloc(sizeof(double) * (size_t)p * T);
  double *Vu = (double *)malloc(sizeof(double) * (size_t)p * T);
  int st = 0, info = 0;
  for (int k = 0; k < g; k++) {
    const double phi = thetaAlpha[k * nTheta], alpha = thetaAlpha[k * nTheta + 1];
    const double nu = covModel == 2 ? thetaAlpha[k * nTheta + 2] : 0;
    double ld;
    st = or_updateBF(n, m, coords, nnIndx, nnIndxLU, covModel, 1.0, alpha, phi, nu, B, F, &ld, nthreads);
    if (st) break;
    for (int i = 0; i < p; i++) {
      v[i] = or_Q(B, F, X + (size_t)n * i, y, n, nnIndx, nnIndxLU, nthreads);
      for (int j = 0; j <= i; j++)
        V[j * p + i] = or_Q(B, F, X + (size_t)n * j, X + (size_t)n * i, n, nnIndx, nnIndxLU, nthreads);
    }
    dpotrf_("L", &p, V, &p, &info);
    if (info == 0) dpotri_("L", &p, V, &p, &info);
    if (info != 0) { st = -1000000000; break; }
    double *bk = betaHat + (size_t)k * p;
    dsymv_("L", &p, &ONE_D, V, &p, v, &ONE_I, &ZERO_D, bk, &ONE_I);
    const double a = sigmaSqIG[0] + 1.0 * n / 2.0;
    const double b = sigmaSqIG[1] + 0.5 * (or_Q(B, F, y, y, n, nnIndx, nnIndxLU, nthreads) -
                                           ddot_(&p, bk, &ONE_I, v, &ONE_I));
    ab[2 * k] = a;
    ab[2 * k + 1] = b;
    memcpy(bBInv + (size_t)k * p * p, V, sizeof(double) * p * p);
    memcpy(bb + (size_t)k * p, v, sizeof(double) * p);
    int bad = INT_MAX;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int i = 0; i < n0; i++) {
      const int t = thread_id();
      double *C = C0 + (size_t)m * m * t, *c = c0 + (size_t)m * t, *wt = w + (size_t)m * t;
      double *rt = r + (size_t)m * t, *ut = u + (size_t)p * t, *vut = Vu + (size_t)p * t;
      for (int j = 0; j < m; j++) {
        const int a1 = nnIndx0[(size_t)j * n0 + i];
        c[j] = or_spcor(dist2(coords0[i], coords0[n0 + i], coords[a1], coords[n + a1]), phi, nu, covModel);
        for (int l = 0; l <= j; l++) {
          const int b1 = nnIndx0[(size_t)l * n0 + i];
          double e = or_spcor(dist2(coords[a1], coords[n + a1], coords[b1], coords[n + b1]), phi, nu, covModel);
          if (l == j) e += alpha;
          C[l * m + j] = e;
        }
      }
      int inf = 0;
      dpotrf_("L", &m, C, &m, &inf);
      if (inf == 0) dpotri_("L", &m, C, &m, &inf);
      if (inf != 0) {
#ifdef _OPENMP
#pragma omp critical
#endif
        { if (i < bad) bad = i; }
      }
      dsymv_("L", &m, &ONE_D, C, &m, c, &ONE_I, &ZERO_D, wt, &ONE_I);
      for (int j = 0; j < m; j++) {
        const int a1 = nnIndx0[(size_t)j * n0 + i];
        rt[j] = y[a1] - ddot_(&p, X + a1, &n, bk, &ONE_I);
      }
      y0Hat[(size_t)k * n0 + i] = ddot_(&p, X0 + i, &n0, bk, &ONE_I) + ddot_(&m, wt, &ONE_I, rt, &ONE_I);
      /* u = x0 - X_N' w */
      for (int j = 0; j < p; j++) {
        double s = 0;
        for (int l = 0; l < m; l++) s += X[(size_t)j * n + nnIndx0[(size_t)l * n0 + i]] * wt[l];
        ut[j] = X0[(size_t)j * n0 + i] - s;
      }
      dsymv_("L", &p, &ONE_D, V, &p, ut, &ONE_I, &ZERO_D, vut, &ONE_I);
      y0HatVar[(size_t)k * n0 + i] =
          b * (ddot_(&p, ut, &ONE_I, vut, &ONE_I) + 1.0 + alpha - ddot_(&m, wt, &ONE_I, c, &ONE_I)) / (a - 1.0);
    }
    if (bad != INT_MAX) { st = -(bad + 1); break; }
  }
  free(B); free(F); free(V); free(v); free(C0); free(c0); free(w); free(r); free(u); free(Vu);
  return st;
}

/* ------------------------------------------------------------ response predict */

/* Posterior predictive draws at q points (src/rNNGPPredict.cpp:25-223): for every location i
 * and kept sample s, the full m x m neighborhood covariance with tau^2 on the diagonal,
 * w = C^-1 c, y0 = x0'beta + w'(y_N - X_N beta) + sqrt(s2 + t2 - w'c) z.  z is q*nSamples
 * standard normals with z[i*nSamples + s] used for (i, s) (the single-thread pairing of
 * src/rNNGPPredict.cpp:176-181).  beta p x nSamples, theta nTheta x nSamples; y0 q x nSamples. */
int or_rNNGPPredict(const double *X, const double *y, const double *coords, int n, int p, int m,
                    const double *X0, const double *coords0, int q, const int *nnIndx0,
                    const double *beta, const double *theta, int nSamples, int covModel,
                    const double *z, int nthreads, double *y0) {
  const int nTheta = covModel == 2 ? 4 : 3;
  const int T = set_threads(nthreads);
  double *Cb = (double *)malloc(sizeof(double) * (size_t)m * m * T);
  double *cb = (double *)malloc(sizeof(double) * (size_t)m * T);
  double *wb = (double *)malloc(sizeof(double) * (size_t)m * T);
  int bad = INT_MAX;
  for (int i = 0; i < q; i++) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int s = 0; s < nSamples; s++) {
      const int t = thread_id();
      double *C = Cb + (size_t)m * m * t, *c = cb + (size_t)m * t, *w = wb + (size_t)m * t;
      const double *th = theta + (size_t)s * nTheta;
      const double s2 = th[0], t2 = th[1], phi = th[2], nu = covModel == 2 ? th[3] : 0;
      for (int k = 0; k < m; k++) {
        const int a = nnIndx0[i + (size_t)q * k];
        c[k] = s2 * or_spcor(dist2(coords[a], coords[n + a], coords0[i], coords0[q + i]), phi, nu, covModel);
        for (int l = 0; l < m; l++) {
          const int b = nnIndx0[i + (size_t)q * l];
          C[l * m + k] = s2 * or_spcor(dist2(coords[a], coords[n + a], coords[b], coords[n + b]), phi, nu, covModel);
          if (k == l) C[l * m + k] += t2;
        }
      }
      int info = 0;
      dpotrf_("L", &m, C, &m, &info);
      if (info == 0) dpotri_("L", &m, C, &m, &info);
      if (info != 0) {
#ifdef _OPENMP
#pragma omp critical
#endif
        { if (i < bad) bad = i; }
      }
      dsymv_("L", &m, &ONE_D, C, &m, c, &ONE_I, &ZERO_D, w, &ONE_I);
      const double *bs = beta + (size_t)s * p;
      double d = 0;
      for (int k = 0; k < m; k++) {
        const int a = nnIndx0[i + (size_t)q * k];
        d += w[k] * (y[a] - ddot_(&p, X + a, &n, bs, &ONE_I));
      }
      y0[(size_t)s * q + i] = ddot_(&p, X0 + i, &q, bs, &ONE_I) + d +
                              sqrt(s2 + t2 - ddot_(&m, w, &ONE_I, c, &ONE_I)) * z[(size_t)i * nSamples + s];
    }
  }
  free(Cb); free(cb); free(wb);
  return bad == INT_MAX ? 0 : -(bad + 1);
}

/* Replicated data y_rep = X beta_s + v_s with v_s drawn by the sequential recurrence at every
 * sample's theta (src/rNNGPReplicated.cpp:24-244).  beta is nSamples x p (column-major),
 * theta nTheta x nSamples; normals are consumed n per sample from the host stream. */
int or_rNNGPReplicated(const double *X, int p, int n, int m, const double *coords, int covModel,
                       const int *nnIndx, const int *nnIndxLU, const double *beta,
                       const double *theta, int nSamples, int nthreads, double *yRep) {
  const int nTheta = covModel == 2 ? 4 : 3;
  const long nIndx = or_n_indx(n, m);
  double *B = (double *)malloc(sizeof(double) * nIndx);
  double *F = (double *)malloc(sizeof(double) * n);
  double *v = (double *)calloc((size_t)n, sizeof(double));
  int st = 0;
  for (int s = 0; s < nSamples; s++) {
    const double *th = theta + (size_t)s * nTheta;
    double ld;
    st = or_updateBF(n, m, coords, nnIndx, nnIndxLU, covModel, th[0], th[1], th[2],
                     covModel == 2 ? th[3] : 0, B, F, &ld, nthreads);
    if (st) break;
    update_rep(B, F, n, v, nnIndx, nnIndxLU);
    double *out = yRep + (size_t)s * n;
    memcpy(out, v, sizeof(double) * n);
    dgemv_("N", &n, &p, &ONE_D, X, &n, beta + s, &nSamples, &ONE_D, out, &ONE_I);
  }
  free(B); free(F); free(v);
  return st;
}
