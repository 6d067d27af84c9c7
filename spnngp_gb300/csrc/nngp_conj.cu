// Model drivers other than the MCMC: the conjugate fit + prediction
// (reference cNNGP, src/cNNGP.cpp:73-358), response prediction (rNNGPPredict,
// src/rNNGPPredict.cpp:25-223) and replicated data (rNNGPReplicated,
// src/rNNGPReplicated.cpp:74-244).
//
// cNNGP runs all g parameter sets in one fused likelihood pass (g jobs over the
// same dataset), then one thread per set does the p x p algebra
// (src/cNNGP.cpp:226-249), then one thread per (set, prediction point) solves
// the prediction neighborhood.  rNNGPReplicated runs the standalone B/F pass
// for all kept samples at once and one thread per sample walks the sequential
// recurrence.
#include <cuda_runtime.h>
#include <cmath>
#include <vector>
#include "nngp_internal.h"
#include "nngp_rep.h"
#include "nngp_pred.h"
#include "nngp_small.cuh"

using nngp_pred::KIND_CONJ;
using nngp_pred::KIND_RESP;
using nngp_pred::PredArgs;

namespace {

__global__ void interleave_kernel3(const double *__restrict__ cm, int n, double *__restrict__ xy) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    xy[2 * i] = cm[i];
    xy[2 * i + 1] = cm[n + i];
  }
}

__global__ void build_v_kernel3(const double *__restrict__ X, const double *__restrict__ y, int n, int p,
                                double *__restrict__ V) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int nv = p + 1;
  if (t < (long)n * nv) {
    const int i = (int)(t / nv), v = (int)(t % nv);
    V[t] = (v < p) ? X[(size_t)v * n + i] : (y ? y[i] : 0.0);
  }
}

// Per parameter set: beta-hat, a*, b*, bB^-1 (lower), bb from the Gram (src/cNNGP.cpp:226-249).
__global__ void conj_fit_kernel(const double *__restrict__ out, int ng, int g, int p, int n, double aIG,
                                double bIG, double *__restrict__ betaHat, double *__restrict__ ab,
                                double *__restrict__ bBInv, double *__restrict__ bb,
                                unsigned long long *__restrict__ status) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= g) return;
  const int nv = p + 1;
  const double *o = out + (size_t)k * ng;
  double G[NNGP_MAX_NV * NNGP_MAX_NV];
  int t = 1;
  for (int a = 0; a < nv; a++)
    for (int b = a; b < nv; b++) {
      G[b * nv + a] = o[t];
      G[a * nv + b] = o[t];
      t++;
    }
  double V[(NNGP_MAX_NV - 1) * (NNGP_MAX_NV - 1)], v[NNGP_MAX_NV - 1], bh[NNGP_MAX_NV - 1];
  for (int i = 0; i < p; i++) {
    v[i] = G[p * nv + i];
    for (int j = 0; j < p; j++) V[j * p + i] = (j <= i) ? G[j * nv + i] : 0.0;
  }
  if (!small_potrf(V, p)) {
    atomicMin(status, (2ull << 48) | (unsigned long long)k);
    return;
  }
  small_potri(V, p);
  small_symv(V, p, v, bh);
  double bv = 0.0;
  for (int i = 0; i < p; i++) bv += bh[i] * v[i];
  ab[2 * k] = aIG + 1.0 * n / 2.0;
  ab[2 * k + 1] = bIG + 0.5 * (G[p * nv + p] - bv);
  for (int i = 0; i < p; i++) {
    betaHat[(size_t)k * p + i] = bh[i];
    bb[(size_t)k * p + i] = v[i];
  }
  for (int i = 0; i < p * p; i++) bBInv[(size_t)k * p * p + i] = V[i];
}

// Batched form of conj_fit_kernel: evaluation e belongs to a dataset of size ns[e].
__global__ void conj_fit_multi_kernel(const double *__restrict__ out, int ng, int E, int p, const int *__restrict__ ns,
                                      double aIG, double bIG, double *__restrict__ betaHat, double *__restrict__ ab,
                                      double *__restrict__ bBInv, double *__restrict__ bb,
                                      unsigned long long *__restrict__ status) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= E) return;
  const int nv = p + 1;
  const double *o = out + (size_t)k * ng;
  double G[NNGP_MAX_NV * NNGP_MAX_NV];
  int t = 1;
  for (int a = 0; a < nv; a++)
    for (int b = a; b < nv; b++) {
      G[b * nv + a] = o[t];
      G[a * nv + b] = o[t];
      t++;
    }
  double V[(NNGP_MAX_NV - 1) * (NNGP_MAX_NV - 1)], v[NNGP_MAX_NV - 1], bh[NNGP_MAX_NV - 1];
  for (int i = 0; i < p; i++) {
    v[i] = G[p * nv + i];
    for (int j = 0; j < p; j++) V[j * p + i] = (j <= i) ? G[j * nv + i] : 0.0;
  }
  if (!small_potrf(V, p)) {
    atomicMin(status, (2ull << 48) | (unsigned long long)k);
    return;
  }
  small_potri(V, p);
  small_symv(V, p, v, bh);
  double bv = 0.0;
  for (int i = 0; i < p; i++) bv += bh[i] * v[i];
  ab[2 * k] = aIG + 1.0 * ns[k] / 2.0;
  ab[2 * k + 1] = bIG + 0.5 * (G[p * nv + p] - bv);
  for (int i = 0; i < p; i++) {
    betaHat[(size_t)k * p + i] = bh[i];
    bb[(size_t)k * p + i] = v[i];
  }
  for (int i = 0; i < p * p; i++) bBInv[(size_t)k * p * p + i] = V[i];
}

// CRPS and RMSPE of one parameter set's predictions (R/util.R:247-255); block j scores
// column j of the n0 x g prediction matrices, summing in a fixed order.
__global__ void conj_score_kernel(const double *__restrict__ yTrue, const double *__restrict__ yHat,
                                  const double *__restrict__ yVar, int n0, double *__restrict__ crps,
                                  double *__restrict__ rmspe) {
  const int j = blockIdx.x;
  __shared__ double s1[256], s2[256];
  double a = 0.0, b = 0.0;
  for (int i = threadIdx.x; i < n0; i += 256) {
    const double yh = yHat[(size_t)j * n0 + i];
    const double sd = sqrt(yVar[(size_t)j * n0 + i]);
    const double z = (yTrue[i] - yh) / sd;
    const double pdf = 0.3989422804014327 * exp(-0.5 * z * z);
    a += -sd * (0.5641895835477563 - 2.0 * pdf - z * (2.0 * normcdf(z) - 1.0));
    const double e = yTrue[i] - yh;
    b += e * e;
  }
  s1[threadIdx.x] = a;
  s2[threadIdx.x] = b;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      s1[threadIdx.x] += s1[threadIdx.x + w];
      s2[threadIdx.x] += s2[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    crps[j] = s1[0] / n0;
    rmspe[j] = sqrt(s2[0] / n0);
  }
}

inline unsigned nb(long cnt, int tpb) { return (unsigned)((cnt + tpb - 1) / tpb); }

struct Tmp {
  nngp_ctx *ctx;
  std::vector<void *> v;
  bool bad = false;
  explicit Tmp(nngp_ctx *c) : ctx(c) {}
  void *up(const void *h, size_t bytes) {
    void *d = nngp_malloc_async(ctx, bytes ? bytes : 16);
    if (!d) bad = true;
    else if (h && bytes) cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, ctx->stream);
    v.push_back(d);
    return d;
  }
  ~Tmp() {
    for (void *q : v) nngp_free_async(ctx, q);
    cudaStreamSynchronize(ctx->stream);
  }
};

int launch_pred_any(nngp_ctx *ctx, int precision, int kind, const PredArgs &a) {
  using namespace nngp_pred;
  const bool r32 = precision == NNGP_FP32R;
  if (a.m <= 16) {
    if (kind == KIND_CONJ) return r32 ? launch_pred<16, true, KIND_CONJ>(ctx, a) : launch_pred<16, false, KIND_CONJ>(ctx, a);
    return r32 ? launch_pred<16, true, KIND_RESP>(ctx, a) : launch_pred<16, false, KIND_RESP>(ctx, a);
  }
  if (kind == KIND_CONJ) return r32 ? launch_pred<32, true, KIND_CONJ>(ctx, a) : launch_pred<32, false, KIND_CONJ>(ctx, a);
  return r32 ? launch_pred<32, true, KIND_RESP>(ctx, a) : launch_pred<32, false, KIND_RESP>(ctx, a);
}

// Runs the prediction kernel; an FP32R factor failure reruns the whole launch in FP64.
int run_pred(nngp_ctx *ctx, int precision, int kind, PredArgs a, const char *what) {
  int st = nngp_reset_status(ctx, a.status);
  if (!st) st = launch_pred_any(ctx, precision, kind, a);
  if (st) return st;
  unsigned long long h = 0;
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(&h, a.status, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
  NNGP_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  if (h != NNGP_STATUS_OK && (h >> 48) == 4 && precision == NNGP_FP32R) {
    if ((st = nngp_reset_status(ctx, a.status))) return st;
    if ((st = launch_pred_any(ctx, NNGP_FP64, kind, a))) return st;
  }
  return nngp_check_status(ctx, a.status, what);
}

CovParams params(int model, double s2, double t2, double phi, double nu) {
  CovParams c{};
  c.model = model;
  c.sigmaSq = s2;
  c.tauSq = t2;
  c.phi = phi;
  c.nu = nu;
  cov_prepare(c);
  return c;
}

}  // namespace

extern "C" {

int nngp_cNNGP(nngp_ctx *ctx, const double *y, const double *X, int p, int n, const double *coords,
               const double *thetaAlpha, const int *nnIndx, const int *nnIndxLU, const double *X0,
               const double *coords0, int n0, const int *nnIndx0, int g, int m, const double *sigmaSqIG,
               int covModel, int precision, double *betaHat, double *ab, double *bBInv, double *bb,
               double *y0Hat, double *y0HatVar) {
  if (!ctx) return NNGP_ERR_ARG;
  if (p < 1 || p > NNGP_MAX_NV - 1) return nngp_fail(ctx, NNGP_ERR_ARG, "1 <= p <= 7 required");
  if (n < 1 || m < 1 || m > NNGP_MAX_M || n < m) return nngp_fail(ctx, NNGP_ERR_ARG, "n >= m and 1 <= m <= 32 required");
  if (covModel < 0 || covModel > 3) return nngp_fail(ctx, NNGP_ERR_ARG, "cov.model is not correctly specified");
  if (g < 1 || n0 < 0) return nngp_fail(ctx, NNGP_ERR_ARG, "g >= 1 and n0 >= 0 required");
  cudaSetDevice(ctx->device);
  const int nTheta = covModel == 2 ? 3 : 2, nv = p + 1, ng = 1 + nv * (nv + 1) / 2;
  const int64_t nI = nngp_nindx(n, m);
  Tmp T(ctx);
  const double *dcm = (const double *)T.up(coords, sizeof(double) * 2 * n);
  const int *dnn = (const int *)T.up(nnIndx, sizeof(int) * (nI > 0 ? nI : 0));
  const int *dlu = (const int *)T.up(nnIndxLU, sizeof(int) * 2 * n);
  const double *dX = (const double *)T.up(X, sizeof(double) * (size_t)n * p);
  const double *dy = (const double *)T.up(y, sizeof(double) * n);
  double *xy = (double *)T.up(nullptr, sizeof(double) * 2 * n);
  float *xyf = (float *)T.up(nullptr, sizeof(float) * 4 * n);
  double *V = (double *)T.up(nullptr, sizeof(double) * (size_t)n * nv);
  std::vector<CovParams> th(g);
  for (int k = 0; k < g; k++)
    th[k] = params(covModel, 1.0, thetaAlpha[k * nTheta + 1], thetaAlpha[k * nTheta],
                   covModel == 2 ? thetaAlpha[k * nTheta + 2] : 0.0);
  CovParams *dth = (CovParams *)T.up(th.data(), sizeof(CovParams) * g);
  double *out = (double *)T.up(nullptr, sizeof(double) * 2 * (size_t)g * ng);
  double *dbeta = (double *)T.up(nullptr, sizeof(double) * (size_t)p * g);
  double *dab = (double *)T.up(nullptr, sizeof(double) * 2 * (size_t)g);
  double *dV = (double *)T.up(nullptr, sizeof(double) * (size_t)p * p * g);
  double *dbb = (double *)T.up(nullptr, sizeof(double) * (size_t)p * g);
  unsigned long long *dst = (unsigned long long *)T.up(nullptr, sizeof(unsigned long long));
  if (T.bad) return nngp_fail(ctx, NNGP_ERR_NO_MEMORY, "device allocation failed");
  nngp_prepare_coords(ctx, dcm, n, xy, xyf);
  build_v_kernel3<<<nb((long)n * nv, 256), 256, 0, ctx->stream>>>(dX, dy, n, p, V);
  ctx->launches += 1;
  int st = nngp_reset_status(ctx, dst);
  if (st) return st;
  BFData d{};
  d.n = n;
  d.m = m;
  d.nv = nv;
  d.xy = xy;
  d.xyf = xyf;
  d.nnIndx = dnn;
  d.nnLU = dlu;
  d.V = V;
  std::vector<PassEval> ev(g);
  for (int k = 0; k < g; k++) ev[k] = PassEval{0, k};
  BFPlan plan;
  st = nngp_bf_plan(ctx, &plan, precision, 1, nv, {d}, dth, ev, dst, nngp_plan_cov(th.data(), g));
  if (!st) st = nngp_bf_run(ctx, &plan, out);
  if (!st) {
    conj_fit_kernel<<<nb(g, 64), 64, 0, ctx->stream>>>(out, ng, g, p, n, sigmaSqIG[0], sigmaSqIG[1], dbeta, dab,
                                                       dV, dbb, dst);
    ctx->launches++;
  }
  nngp_bf_plan_free(ctx, &plan);
  if (st) return st;
  if ((st = nngp_check_status(ctx, dst, "cNNGP"))) return st;
  if (n0 > 0) {
    PredArgs a{};
    a.n = n;
    a.m = m;
    a.p = p;
    a.n0 = n0;
    a.npar = g;
    a.xy = xy;
    a.V = V;
    a.c0 = (const double *)T.up(coords0, sizeof(double) * 2 * n0);
    a.X0 = (const double *)T.up(X0, sizeof(double) * (size_t)n0 * p);
    a.nn0 = (const int *)T.up(nnIndx0, sizeof(int) * (size_t)n0 * m);
    a.par = dth;
    a.beta = dbeta;
    a.Vinv = dV;
    a.ab = dab;
    a.out0 = (double *)T.up(nullptr, sizeof(double) * (size_t)n0 * g);
    a.out1 = (double *)T.up(nullptr, sizeof(double) * (size_t)n0 * g);
    a.status = dst;
    if (T.bad) return nngp_fail(ctx, NNGP_ERR_NO_MEMORY, "device allocation failed");
    if ((st = run_pred(ctx, precision, KIND_CONJ, a, "cNNGP prediction"))) return st;
    NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(y0Hat, a.out0, sizeof(double) * (size_t)n0 * g, cudaMemcpyDeviceToHost, ctx->stream));
    NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(y0HatVar, a.out1, sizeof(double) * (size_t)n0 * g, cudaMemcpyDeviceToHost, ctx->stream));
  }
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(betaHat, dbeta, sizeof(double) * (size_t)p * g, cudaMemcpyDeviceToHost, ctx->stream));
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(ab, dab, sizeof(double) * 2 * (size_t)g, cudaMemcpyDeviceToHost, ctx->stream));
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(bBInv, dV, sizeof(double) * (size_t)p * p * g, cudaMemcpyDeviceToHost, ctx->stream));
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(bb, dbb, sizeof(double) * (size_t)p * g, cudaMemcpyDeviceToHost, ctx->stream));
  NNGP_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return NNGP_OK;
}

int nngp_rNNGPPredict(nngp_ctx *ctx, const double *X, const double *y, const double *coords, int n, int p,
                      int m, const double *X0, const double *coords0, int q, const int *nnIndx0,
                      const double *betaSamples, const double *thetaSamples, int nSamples, int covModel,
                      const double *z, int precision, double *y0) {
  if (!ctx) return NNGP_ERR_ARG;
  if (p < 1 || p > NNGP_MAX_NV - 1) return nngp_fail(ctx, NNGP_ERR_ARG, "1 <= p <= 7 required");
  if (n < 1 || m < 1 || m > NNGP_MAX_M || n < m) return nngp_fail(ctx, NNGP_ERR_ARG, "n >= m and 1 <= m <= 32 required");
  if (covModel < 0 || covModel > 3) return nngp_fail(ctx, NNGP_ERR_ARG, "cov.model is not correctly specified");
  if (q < 0 || nSamples < 0) return nngp_fail(ctx, NNGP_ERR_ARG, "q >= 0 and n.samples >= 0 required");
  if (q == 0 || nSamples == 0) return NNGP_OK;
  cudaSetDevice(ctx->device);
  const int nTheta = covModel == 2 ? 4 : 3;
  Tmp T(ctx);
  std::vector<CovParams> th(nSamples);
  for (int s = 0; s < nSamples; s++) {
    const double *t = thetaSamples + (size_t)s * nTheta;
    th[s] = params(covModel, t[0], t[1], t[2], covModel == 2 ? t[3] : 0.0);
  }
  PredArgs a{};
  a.n = n;
  a.m = m;
  a.p = p;
  a.n0 = q;
  a.npar = nSamples;
  const double *dcm = (const double *)T.up(coords, sizeof(double) * 2 * n);
  const double *dX = (const double *)T.up(X, sizeof(double) * (size_t)n * p);
  const double *dy = (const double *)T.up(y, sizeof(double) * n);
  double *xy = (double *)T.up(nullptr, sizeof(double) * 2 * n);
  double *V = (double *)T.up(nullptr, sizeof(double) * (size_t)n * (p + 1));
  a.c0 = (const double *)T.up(coords0, sizeof(double) * 2 * q);
  a.X0 = (const double *)T.up(X0, sizeof(double) * (size_t)q * p);
  a.nn0 = (const int *)T.up(nnIndx0, sizeof(int) * (size_t)q * m);
  a.par = (const CovParams *)T.up(th.data(), sizeof(CovParams) * nSamples);
  a.beta = (const double *)T.up(betaSamples, sizeof(double) * (size_t)p * nSamples);
  a.z = (const double *)T.up(z, sizeof(double) * (size_t)q * nSamples);
  a.out0 = (double *)T.up(nullptr, sizeof(double) * (size_t)q * nSamples);
  a.status = (unsigned long long *)T.up(nullptr, sizeof(unsigned long long));
  if (T.bad) return nngp_fail(ctx, NNGP_ERR_NO_MEMORY, "device allocation failed");
  interleave_kernel3<<<nb(n, 256), 256, 0, ctx->stream>>>(dcm, n, xy);
  build_v_kernel3<<<nb((long)n * (p + 1), 256), 256, 0, ctx->stream>>>(dX, dy, n, p, V);
  ctx->launches += 2;
  a.xy = xy;
  a.V = V;
  int st = run_pred(ctx, precision, KIND_RESP, a, "rNNGPPredict");
  if (st) return st;
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(y0, a.out0, sizeof(double) * (size_t)q * nSamples, cudaMemcpyDeviceToHost, ctx->stream));
  NNGP_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return NNGP_OK;
}

namespace {
// Exact posterior draws of the conjugate model at one parameter set (R/spConjNNGP.R:423-436 and
// R/util.R:1-11): sigma^2 = b / g with g ~ Gamma(a, 1) host-fed (rigamma's 1 / rgamma(a, rate b)),
// beta = B^-1 bb + sigma L z with L the lower Cholesky factor of B^-1 (rmvn's z'chol(V),
// V = sigma^2 B^-1), tau^2 = alpha sigma^2.  Every block recomputes the p x p factor and mean in
// shared memory (p <= 8); then one thread per sample.  out is nSamples x (p + 2), column-major
// (the rows of R's p.beta.theta.samples: beta, sigma.sq, tau.sq).
__global__ void conj_posterior_kernel(int p, const double *__restrict__ bb, const double *__restrict__ Binv, double b,
                                      double alpha, int nSamples, const double *__restrict__ gam,
                                      const double *__restrict__ z, double *__restrict__ out, int *__restrict__ bad) {
  __shared__ double L[NNGP_MAX_NV * NNGP_MAX_NV], mu[NNGP_MAX_NV];
  if (threadIdx.x == 0) {
    for (int j = 0; j < p; j++)
      for (int i = 0; i < p; i++) L[j * p + i] = (i >= j) ? Binv[j * p + i] : 0.0;
    small_symv(L, p, bb, mu);  // B^-1 bb from the lower triangle
    if (!small_potrf(L, p)) *bad = 1;
    for (int j = 0; j < p; j++)
      for (int i = 0; i < j; i++) L[j * p + i] = 0.0;  // the strict upper part is not the factor's
  }
  __syncthreads();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nSamples) return;
  const double s2 = b / gam[s];
  const double sd = sqrt(s2);
  const double *zs = z + (size_t)s * p;
  for (int j = 0; j < p; j++) {
    double acc = 0.0;
    for (int i = 0; i <= j; i++) acc += L[i * p + j] * zs[i];
    out[(size_t)j * nSamples + s] = mu[j] + sd * acc;
  }
  out[(size_t)p * nSamples + s] = s2;
  out[(size_t)(p + 1) * nSamples + s] = alpha * s2;
}
}  // namespace

int nngp_conj_posterior_samples(nngp_ctx *ctx, int p, const double *bb, const double *bBInv, double a, double b,
                                double alpha, int nSamples, const double *gammas, const double *normals,
                                double *samples) {
  if (!ctx) return NNGP_ERR_ARG;
  if (p < 1 || p > NNGP_MAX_NV) return nngp_fail(ctx, NNGP_ERR_ARG, "1 <= p <= 8 required");
  if (nSamples <= 0) return NNGP_OK;
  if (!(a > 0.0) || !(b > 0.0)) return nngp_fail(ctx, NNGP_ERR_ARG, "the inverse-gamma parameters must be positive");
  cudaSetDevice(ctx->device);
  Tmp T(ctx);
  const double *dbb = (const double *)T.up(bb, sizeof(double) * p);
  const double *dB = (const double *)T.up(bBInv, sizeof(double) * p * p);
  const double *dg = (const double *)T.up(gammas, sizeof(double) * (size_t)nSamples);
  const double *dz = (const double *)T.up(normals, sizeof(double) * (size_t)nSamples * p);
  double *dout = (double *)T.up(nullptr, sizeof(double) * (size_t)nSamples * (p + 2));
  int *dbad = (int *)T.up(nullptr, sizeof(int));
  if (T.bad) return nngp_fail(ctx, NNGP_ERR_NO_MEMORY, "device allocation failed");
  NNGP_CUDA_TRY(ctx, cudaMemsetAsync(dbad, 0, sizeof(int), ctx->stream));
  conj_posterior_kernel<<<nb(nSamples, 128), 128, 0, ctx->stream>>>(p, dbb, dB, b, alpha, nSamples, dg, dz, dout, dbad);
  NNGP_LAUNCH_CHECK(ctx);
  int hbad = 0;
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(&hbad, dbad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(samples, dout, sizeof(double) * (size_t)nSamples * (p + 2),
                                     cudaMemcpyDeviceToHost, ctx->stream));
  NNGP_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  if (hbad) return nngp_fail(ctx, NNGP_ERR_NOT_SPD, "conjugate posterior: bB.inv is not positive definite");
  return NNGP_OK;
}

int nngp_rNNGPReplicated(nngp_ctx *ctx, const double *X, int p, int n, int m, const double *coords,
                         int covModel, const int *nnIndx, const int *nnIndxLU, const double *beta,
                         const double *theta, int nSamples, const double *normals, int precision,
                         double *yRep) {
  if (!ctx) return NNGP_ERR_ARG;
  if (p < 1 || n < 1 || m < 1 || m > NNGP_MAX_M || n < m) return nngp_fail(ctx, NNGP_ERR_ARG, "invalid sizes");
  if (covModel < 0 || covModel > 3) return nngp_fail(ctx, NNGP_ERR_ARG, "cov.model is not correctly specified");
  if (nSamples <= 0) return NNGP_OK;
  cudaSetDevice(ctx->device);
  const int nTheta = covModel == 2 ? 4 : 3;
  const int64_t nI = nngp_nindx(n, m);
  Tmp T(ctx);
  const double *dcm = (const double *)T.up(coords, sizeof(double) * 2 * n);
  const int *dnn = (const int *)T.up(nnIndx, sizeof(int) * (nI > 0 ? nI : 0));
  const int *dlu = (const int *)T.up(nnIndxLU, sizeof(int) * 2 * n);
  const double *dX = (const double *)T.up(X, sizeof(double) * (size_t)n * p);
  const double *dbeta = (const double *)T.up(beta, sizeof(double) * (size_t)nSamples * p);
  const double *dz = (const double *)T.up(normals, sizeof(double) * (size_t)n * nSamples);
  double *dy = (double *)T.up(nullptr, sizeof(double) * (size_t)n * nSamples);
  double *xy = (double *)T.up(nullptr, sizeof(double) * 2 * n);
  float *xyf = (float *)T.up(nullptr, sizeof(float) * 4 * n);
  std::vector<CovParams> th(nSamples);
  for (int s = 0; s < nSamples; s++) {
    const double *t = theta + (size_t)s * nTheta;
    th[s] = params(covModel, t[0], t[1], t[2], covModel == 2 ? t[3] : 0.0);
  }
  CovParams *dth = (CovParams *)T.up(th.data(), sizeof(CovParams) * nSamples);
  unsigned long long *dst = (unsigned long long *)T.up(nullptr, sizeof(unsigned long long));
  std::vector<long long> zoff(nSamples);
  for (int s = 0; s < nSamples; s++) zoff[s] = (long long)s * n;
  const long long *dzoff = (const long long *)T.up(zoff.data(), sizeof(long long) * nSamples);
  if (T.bad) return nngp_fail(ctx, NNGP_ERR_NO_MEMORY, "device allocation failed");
  nngp_prepare_coords(ctx, dcm, n, xy, xyf);
  int st = nngp_reset_status(ctx, dst);
  if (st) return st;
  // the dataflow solve of every sample's recurrence (nngp_rep.cu)
  RepSpec rs{};
  rs.n = n;
  rs.m = m;
  rs.p = p;
  rs.nRep = nSamples;
  rs.precision = precision;
  rs.cov = nngp_plan_cov(th.data(), nSamples);
  rs.xb_first = 0;  // v, then + beta_j X_j in order (src/rNNGPReplicated.cpp:204 dgemv)
  rs.xy = xy;
  rs.xyf = xyf;
  rs.nnIndx = dnn;
  rs.nnLU = dlu;
  rs.X = dX;
  rs.d_theta = dth;
  rs.beta = dbeta;
  rs.bs_r = 1;
  rs.bs_j = nSamples;
  rs.z = dz;
  rs.d_zoff = dzoff;
  rs.yRep = dy;
  rs.d_status = dst;
  if ((st = nngp_replicate_solve(ctx, rs))) return st;
  if ((st = nngp_check_status(ctx, dst, "rNNGPReplicated"))) return st;
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(yRep, dy, sizeof(double) * (size_t)n * nSamples, cudaMemcpyDeviceToHost, ctx->stream));
  NNGP_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return NNGP_OK;
}

int nngp_cNNGP_multi(nngp_ctx *ctx, int nprob, const nngp_conj_problem *probs, int p, int m,
                     const double *sigmaSqIG, int covModel, int precision, int resident) {
  if (!ctx) return NNGP_ERR_ARG;
  if (nprob < 1) return NNGP_OK;
  if (p < 1 || p > NNGP_MAX_NV - 1) return nngp_fail(ctx, NNGP_ERR_ARG, "1 <= p <= 7 required");
  if (m < 1 || m > NNGP_MAX_M) return nngp_fail(ctx, NNGP_ERR_ARG, "1 <= m <= 32 required");
  if (covModel < 0 || covModel > 3) return nngp_fail(ctx, NNGP_ERR_ARG, "cov.model is not correctly specified");
  for (int k = 0; k < nprob; k++)
    if (probs[k].n < m || probs[k].g < 1 || probs[k].n0 < 0)
      return nngp_fail(ctx, NNGP_ERR_ARG, "every problem needs n >= m, g >= 1 and n0 >= 0");
  cudaSetDevice(ctx->device);
  const int nTheta = covModel == 2 ? 3 : 2, nv = p + 1, ng = 1 + nv * (nv + 1) / 2;
  Tmp T(ctx);
  auto dev = [&](const void *h, size_t bytes) -> const void * { return resident ? h : T.up(h, bytes); };
  std::vector<BFData> datas(nprob);
  std::vector<CovParams> th;
  std::vector<PassEval> ev;
  std::vector<int> eoff(nprob), ns;
  struct Dev {
    const double *cm, *X, *y, *X0, *c0, *y0t;
    const int *nn0;
  };
  std::vector<Dev> dv(nprob);
  for (int k = 0; k < nprob; k++) {
    const nngp_conj_problem &P = probs[k];
    const int64_t nI = nngp_nindx(P.n, m);
    Dev &D = dv[k];
    D.cm = (const double *)dev(P.coords, sizeof(double) * 2 * P.n);
    D.X = (const double *)dev(P.X, sizeof(double) * (size_t)P.n * p);
    D.y = (const double *)dev(P.y, sizeof(double) * P.n);
    const int *dnn = (const int *)dev(P.nnIndx, sizeof(int) * (nI > 0 ? nI : 0));
    const int *dlu = (const int *)dev(P.nnIndxLU, sizeof(int) * 2 * P.n);
    if (P.n0 > 0) {
      D.X0 = (const double *)dev(P.X0, sizeof(double) * (size_t)P.n0 * p);
      D.c0 = (const double *)dev(P.coords0, sizeof(double) * 2 * P.n0);
      D.nn0 = (const int *)dev(P.nnIndx0, sizeof(int) * (size_t)P.n0 * m);
      D.y0t = P.y0True ? (const double *)dev(P.y0True, sizeof(double) * P.n0) : nullptr;
    }
    double *xy = (double *)T.up(nullptr, sizeof(double) * 2 * P.n);
    float *xyf = (float *)T.up(nullptr, sizeof(float) * 4 * P.n);
    double *V = (double *)T.up(nullptr, sizeof(double) * (size_t)P.n * nv);
    if (T.bad) return nngp_fail(ctx, NNGP_ERR_NO_MEMORY, "device allocation failed");
    nngp_prepare_coords(ctx, D.cm, P.n, xy, xyf);
    build_v_kernel3<<<nb((long)P.n * nv, 256), 256, 0, ctx->stream>>>(D.X, D.y, P.n, p, V);
    ctx->launches++;
    BFData d{};
    d.n = P.n;
    d.m = m;
    d.nv = nv;
    d.xy = xy;
    d.xyf = xyf;
    d.nnIndx = dnn;
    d.nnLU = dlu;
    d.V = V;
    datas[k] = d;
    eoff[k] = (int)th.size();
    for (int j = 0; j < P.g; j++) {
      const double *ta = P.thetaAlpha + (size_t)j * nTheta;
      th.push_back(params(covModel, 1.0, ta[1], ta[0], covModel == 2 ? ta[2] : 0.0));
      ev.push_back(PassEval{k, (int)th.size() - 1});
      ns.push_back(P.n);
    }
  }
  const int E = (int)th.size();
  CovParams *dth = (CovParams *)T.up(th.data(), sizeof(CovParams) * E);
  int *dns = (int *)T.up(ns.data(), sizeof(int) * E);
  double *out = (double *)T.up(nullptr, sizeof(double) * 2 * (size_t)E * ng);
  double *dbeta = (double *)T.up(nullptr, sizeof(double) * (size_t)p * E);
  double *dab = (double *)T.up(nullptr, sizeof(double) * 2 * (size_t)E);
  double *dV = (double *)T.up(nullptr, sizeof(double) * (size_t)p * p * E);
  double *dbb = (double *)T.up(nullptr, sizeof(double) * (size_t)p * E);
  unsigned long long *dst = (unsigned long long *)T.up(nullptr, sizeof(unsigned long long));
  if (T.bad) return nngp_fail(ctx, NNGP_ERR_NO_MEMORY, "device allocation failed");
  int st = nngp_reset_status(ctx, dst);
  if (st) return st;
  BFPlan plan;
  st = nngp_bf_plan(ctx, &plan, precision, 1, nv, datas, dth, ev, dst, nngp_plan_cov(th.data(), E));
  if (!st) st = nngp_bf_run(ctx, &plan, out);
  if (!st) {
    conj_fit_multi_kernel<<<nb(E, 64), 64, 0, ctx->stream>>>(out, ng, E, p, dns, sigmaSqIG[0], sigmaSqIG[1], dbeta,
                                                             dab, dV, dbb, dst);
    ctx->launches++;
  }
  nngp_bf_plan_free(ctx, &plan);
  if (st) return st;
  if ((st = nngp_check_status(ctx, dst, "cNNGP"))) return st;
  const cudaMemcpyKind back = resident ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  for (int k = 0; k < nprob; k++) {
    const nngp_conj_problem &P = probs[k];
    const int g = P.g, e0 = eoff[k];
    if (P.n0 > 0 && (P.y0Hat || P.y0HatVar || (P.y0True && (P.crps || P.rmspe)))) {
      PredArgs a{};
      a.n = P.n;
      a.m = m;
      a.p = p;
      a.n0 = P.n0;
      a.npar = g;
      a.xy = datas[k].xy;
      a.V = datas[k].V;
      a.c0 = dv[k].c0;
      a.X0 = dv[k].X0;
      a.nn0 = dv[k].nn0;
      a.par = dth + e0;
      a.beta = dbeta + (size_t)e0 * p;
      a.Vinv = dV + (size_t)e0 * p * p;
      a.ab = dab + 2 * (size_t)e0;
      a.out0 = (double *)T.up(nullptr, sizeof(double) * (size_t)P.n0 * g);
      a.out1 = (double *)T.up(nullptr, sizeof(double) * (size_t)P.n0 * g);
      a.status = dst;
      if (T.bad) return nngp_fail(ctx, NNGP_ERR_NO_MEMORY, "device allocation failed");
      if ((st = run_pred(ctx, precision, KIND_CONJ, a, "cNNGP prediction"))) return st;
      if (P.y0True && (P.crps || P.rmspe)) {
        double *sc = (double *)T.up(nullptr, sizeof(double) * 2 * (size_t)g);
        if (T.bad) return nngp_fail(ctx, NNGP_ERR_NO_MEMORY, "device allocation failed");
        conj_score_kernel<<<g, 256, 0, ctx->stream>>>(dv[k].y0t, a.out0, a.out1, P.n0, sc, sc + g);
        ctx->launches++;
        if (P.crps) NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(P.crps, sc, sizeof(double) * g, back, ctx->stream));
        if (P.rmspe) NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(P.rmspe, sc + g, sizeof(double) * g, back, ctx->stream));
      }
      if (P.y0Hat)
        NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(P.y0Hat, a.out0, sizeof(double) * (size_t)P.n0 * g, back, ctx->stream));
      if (P.y0HatVar)
        NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(P.y0HatVar, a.out1, sizeof(double) * (size_t)P.n0 * g, back, ctx->stream));
    }
    if (P.betaHat)
      NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(P.betaHat, dbeta + (size_t)e0 * p, sizeof(double) * p * g, back, ctx->stream));
    if (P.ab) NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(P.ab, dab + 2 * (size_t)e0, sizeof(double) * 2 * g, back, ctx->stream));
    if (P.bBInv)
      NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(P.bBInv, dV + (size_t)e0 * p * p, sizeof(double) * p * p * g, back, ctx->stream));
    if (P.bb) NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(P.bb, dbb + (size_t)e0 * p, sizeof(double) * p * g, back, ctx->stream));
  }
  NNGP_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return NNGP_OK;
}

}  // extern "C"

