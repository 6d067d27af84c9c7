// Response-model MCMC (reference rNNGP, src/rNNGP.cpp:103-421) on the device.
//
// The chain stays sequential over iterations; everything inside an iteration
// runs on the GPU, for one or many independent instances at once:
//   mc_pre    (one thread per instance) beta | theta from the cached Gram of the
//             current theta (p x p potrf/potri/symv/potrf, src/rNNGP.cpp:274-292),
//             beta draw (src/util.cpp:28-41), log target at the current theta,
//             Metropolis proposals (src/rNNGP.cpp:327-333) written as the
//             candidate's CovParams;
//   B/F pass  the fused likelihood pass at the candidate for all instances
//             (log F and the Gram of [X y], no B written);
//   mc_post   (one thread per instance) log target at the candidate, accept /
//             reject on the next uniform (src/rNNGP.cpp:349-354), samples saved.
// The reference recomputes updateBF at the current theta every iteration
// (src/rNNGP.cpp:306); that recomputation is deterministic, so the current
// theta's log-determinant and Gram are cached instead, which halves the solves
// without changing any value.  Q(X beta - y) comes from the Gram:
// beta'Gxx beta - 2 beta'Gxy + Gyy.  An iteration with a replicate draw
// (fit.rep, src/rNNGP.cpp:300-303,309-313) records the current theta, the beta
// draw and where its n normals start in the stream; the draws do not feed back
// into the chain, so after the last iteration all of them are made at once by
// the dataflow solve of nngp_rep.cu (the recurrence of
// src/rNNGP.cpp:24-42 for every recorded theta).
// Random numbers come from host-fed streams in the reference's order.  Each
// iteration is captured once as a CUDA graph and replayed.
#include <cuda_runtime.h>
#include <cmath>
#include <vector>
#include "nngp_internal.h"
#include "nngp_rep.h"
#include "nngp_small.cuh"

namespace {

constexpr int PMAX = NNGP_MAX_NV - 1;

struct MCConst {
  int n, p, model, nTheta, nSamples;
  double sIG[2], tIG[2], pU[2], nU[2], tuning[4];
  const double *normals;
  long long nNormals;
  const double *unifs;
  long long nUnifs;
  const int *repIndx;  // may be null
  double *betaOut;     // p x nSamples
  double *thetaOut;    // nTheta x nSamples
  double *repOut;      // n x nRep
  const double *X;     // n x p column-major
  // replicate records, one per draw: the current theta, the beta draw, the normals' offset
  CovParams *repTheta;
  double *repBeta;     // nRep x p
  long long *repZoff;
  const double *out;   // this instance's (log F, Gram) sums in its size class's output buffer
};

struct MCState {
  double theta[4], cand[4];
  double beta[PMAX], mean[PMAX], L[PMAX * PMAX];
  double G[NNGP_MAX_NV * NNGP_MAX_NV];
  double ld, lpCur;
  long long npos, upos, repStart;
  int thetaUpdate, accept, s, repCnt, status, doRep;
};

__device__ inline bool next_normal(const MCConst &c, MCState &st, double &z) {
  if (st.npos >= c.nNormals) {
    st.status = 3;
    z = 0.0;
    return false;
  }
  z = c.normals[st.npos++];
  return true;
}
// R's rnorm(mu, sd): consumes a draw only when sd > 0 and mu is finite.
__device__ inline double r_rnorm(const MCConst &c, MCState &st, double mu, double sd) {
  if (isnan(mu) || !isfinite(sd) || sd < 0.0) return nan("");
  if (sd == 0.0 || !isfinite(mu)) return mu;
  double z;
  next_normal(c, st, z);
  return mu + sd * z;
}
__device__ inline double logit(double t, double a, double b) { return log((t - a) / (b - t)); }
__device__ inline double logit_inv(double z, double a, double b) { return b - (b - a) / (1 + exp(z)); }

__device__ inline double log_post(const MCConst &c, double ld, double q, const double *th) {
  double lp = -0.5 * ld - 0.5 * q;
  lp += log(th[2] - c.pU[0]) + log(c.pU[1] - th[2]);
  lp += -1.0 * (1.0 + c.sIG[0]) * log(th[0]) - c.sIG[1] / th[0] + log(th[0]);
  lp += -1.0 * (1.0 + c.tIG[0]) * log(th[1]) - c.tIG[1] / th[1] + log(th[1]);
  if (c.model == 2) lp += log(th[3] - c.nU[0]) + log(c.nU[1] - th[3]);
  return lp;
}

// Q(X beta - y) from the Gram G of V = [X y] (nv = p + 1, column-major).
__device__ inline double quad_from_gram(const double *G, int p, const double *beta) {
  const int nv = p + 1;
  double q = G[p * nv + p];
  for (int a = 0; a < p; a++) {
    q -= 2.0 * beta[a] * G[p * nv + a];
    for (int b = 0; b < p; b++) q += beta[a] * G[b * nv + a] * beta[b];
  }
  return q;
}

__device__ inline void set_params(CovParams &cp, int model, const double *th) {
  cp.model = model;
  cp.sigmaSq = th[0];
  cp.tauSq = th[1];
  cp.phi = th[2];
  cp.nu = model == 2 ? th[3] : 0.0;
  cov_prepare(cp);
}

// Unpacks nngp_bf_run's (log F, upper-triangle Gram) sums.
__device__ inline void unpack(const double *o, int nv, double &ld, double *G) {
  ld = o[0];
  int k = 1;
  for (int a = 0; a < nv; a++)
    for (int b = a; b < nv; b++) {
      G[b * nv + a] = o[k];
      G[a * nv + b] = o[k];
      k++;
    }
}

__global__ void mc_init_kernel(const MCConst *__restrict__ cs, MCState *__restrict__ sts, int ninst) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= ninst) return;
  MCState &st = sts[k];
  unpack(cs[k].out, cs[k].p + 1, st.ld, st.G);
  st.thetaUpdate = 1;
}

__global__ void mc_pre_kernel(const MCConst *__restrict__ cs, MCState *__restrict__ sts,
                              CovParams *__restrict__ thetas, int ninst) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= ninst) return;
  const MCConst &c = cs[k];
  MCState &st = sts[k];
  if (st.status || st.s >= c.nSamples) return;
  const int p = c.p, nv = p + 1;
  if (st.thetaUpdate) {
    st.thetaUpdate = 0;
    double V[PMAX * PMAX], g[PMAX];
    for (int i = 0; i < p; i++) {
      g[i] = st.G[p * nv + i];
      for (int j = 0; j < p; j++) V[j * p + i] = (j <= i) ? st.G[j * nv + i] : 0.0;
    }
    if (!small_potrf(V, p)) {
      st.status = 2;
      return;
    }
    small_potri(V, p);
    small_symv(V, p, g, st.mean);
    if (!small_potrf(V, p)) {
      st.status = 2;
      return;
    }
    for (int i = 0; i < p * p; i++) st.L[i] = V[i];
  }
  // beta ~ N(mean, L L'): z then L z + mean
  double z[PMAX];
  for (int i = 0; i < p; i++) z[i] = r_rnorm(c, st, 0.0, 1.0);
  for (int i = 0; i < p; i++) {
    double s = st.mean[i];
    for (int j = 0; j <= i; j++) s += st.L[j * p + i] * z[j];
    st.beta[i] = s;
  }
  // replicate draw at the current theta consumes n normals here; it is recorded and made
  // after the chain
  st.doRep = (c.repIndx && c.repIndx[st.s]) ? 1 : 0;
  if (st.doRep) {
    st.repStart = st.npos;
    if (st.npos + c.n > c.nNormals) st.status = 3;
    set_params(c.repTheta[st.repCnt], c.model, st.theta);
    for (int i = 0; i < p; i++) c.repBeta[(size_t)st.repCnt * p + i] = st.beta[i];
    c.repZoff[st.repCnt] = st.npos;
    st.repCnt++;
    st.npos += c.n;
  }
  const double q = quad_from_gram(st.G, p, st.beta);
  st.lpCur = log_post(c, st.ld, q, st.theta);
  // proposals in the reference's order: phi, sigma^2, tau^2, nu
  st.cand[2] = logit_inv(r_rnorm(c, st, logit(st.theta[2], c.pU[0], c.pU[1]), c.tuning[2]), c.pU[0], c.pU[1]);
  st.cand[0] = exp(r_rnorm(c, st, log(st.theta[0]), c.tuning[0]));
  st.cand[1] = exp(r_rnorm(c, st, log(st.theta[1]), c.tuning[1]));
  if (c.model == 2)
    st.cand[3] = logit_inv(r_rnorm(c, st, logit(st.theta[3], c.nU[0], c.nU[1]), c.tuning[3]), c.nU[0], c.nU[1]);
  set_params(thetas[2 * k + 1], c.model, st.cand);
}

__global__ void mc_post_kernel(const MCConst *__restrict__ cs, MCState *__restrict__ sts,
                               CovParams *__restrict__ thetas, int ninst) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= ninst) return;
  const MCConst &c = cs[k];
  MCState &st = sts[k];
  if (st.status || st.s >= c.nSamples) return;
  const int p = c.p, nv = p + 1;
  double ld, G[NNGP_MAX_NV * NNGP_MAX_NV];
  unpack(c.out, nv, ld, G);
  const double q = quad_from_gram(G, p, st.beta);
  const double lpCand = log_post(c, ld, q, st.cand);
  double u = 0.5;
  if (st.upos >= c.nUnifs) st.status = 3;
  else u = c.unifs[st.upos++];
  if (u <= exp(lpCand - st.lpCur)) {
    st.thetaUpdate = 1;
    for (int t = 0; t < 4; t++) st.theta[t] = st.cand[t];
    st.ld = ld;
    for (int t = 0; t < nv * nv; t++) st.G[t] = G[t];
    thetas[2 * k] = thetas[2 * k + 1];
    st.accept++;
  }
  for (int i = 0; i < p; i++) c.betaOut[(size_t)st.s * p + i] = st.beta[i];
  for (int t = 0; t < c.nTheta; t++) c.thetaOut[(size_t)st.s * c.nTheta + t] = st.theta[t];
  st.s++;
}

__global__ void build_v_kernel(const double *__restrict__ X, const double *__restrict__ y, int n, int p,
                               double *__restrict__ V) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int nv = p + 1;
  if (t < (long)n * nv) {
    const int i = (int)(t / nv), v = (int)(t % nv);
    V[t] = (v < p) ? X[(size_t)v * n + i] : y[i];
  }
}

inline unsigned nblk(long cnt, int tpb) { return (unsigned)((cnt + tpb - 1) / tpb); }

}  // namespace

// One instance of the response model as the batched driver takes it (device pointers).
struct MCInstance {
  int n, m, p, model;
  const double *coords_cm;  // n x 2 column-major
  const int *nnIndx, *nnLU;
  const double *X, *y;      // X n x p column-major
  double sIG[2], tIG[2], pU[2], nU[2];
  double betaStart[PMAX], thetaStart[4], tuning[4];
  int nSamples;
  const double *normals;
  long long nNormals;
  const double *unifs;
  long long nUnifs;
  const int *repIndx;       // device, nSamples entries, or null
  double *betaOut, *thetaOut, *repOut;
};

// Runs nSamples iterations for every instance (all instances share p).
int nngp_run_mcmc(nngp_ctx *ctx, const std::vector<MCInstance> &insts, int precision,
                  const std::vector<int> *host_rep, int *accept_out) {
  const int ninst = (int)insts.size();
  if (ninst == 0) return NNGP_OK;
  const int p = insts[0].p, nv = p + 1, ng = 1 + nv * (nv + 1) / 2;
  int nS = 0;
  for (const auto &I : insts) nS = I.nSamples > nS ? I.nSamples : nS;
  std::vector<void *> owned;
  auto own = [&](size_t bytes) {
    void *q = nngp_malloc_async(ctx, bytes);
    owned.push_back(q);
    return q;
  };
  auto release = [&]() {
    for (void *q : owned) nngp_free_async(ctx, q);
  };
  std::vector<BFData> datas(ninst);
  std::vector<MCConst> consts(ninst);
  std::vector<MCState> states(ninst);
  std::vector<CovParams> th(2 * ninst);
  const bool anyRep = host_rep != nullptr;
  for (int k = 0; k < ninst; k++) {
    const MCInstance &I = insts[k];
    if (I.p != p) return nngp_fail(ctx, NNGP_ERR_ARG, "instances of one batch must share p");
    double *xy = (double *)own(sizeof(double) * 2 * I.n);
    float *xyf = precision == NNGP_FP32R ? (float *)own(sizeof(float) * 4 * I.n) : nullptr;
    double *V = (double *)own(sizeof(double) * (size_t)I.n * nv);
    if (!xy || !V || (precision == NNGP_FP32R && !xyf)) {
      release();
      return nngp_fail(ctx, NNGP_ERR_NO_MEMORY, "device allocation failed");
    }
    nngp_prepare_coords(ctx, I.coords_cm, I.n, xy, xyf);
    build_v_kernel<<<nblk((long)I.n * nv, 256), 256, 0, ctx->stream>>>(I.X, I.y, I.n, p, V);
    ctx->launches += 1;
    BFData d{};
    d.n = I.n;
    d.m = I.m;
    d.nv = nv;
    d.xy = xy;
    d.xyf = xyf;
    d.nnIndx = I.nnIndx;
    d.nnLU = I.nnLU;
    d.V = V;
    datas[k] = d;
    MCConst &c = consts[k];
    c = MCConst{};
    c.n = I.n;
    c.p = p;
    c.model = I.model;
    c.nTheta = I.model == 2 ? 4 : 3;
    c.nSamples = I.nSamples;
    for (int t = 0; t < 2; t++) {
      c.sIG[t] = I.sIG[t];
      c.tIG[t] = I.tIG[t];
      c.pU[t] = I.pU[t];
      c.nU[t] = I.nU[t];
    }
    for (int t = 0; t < 4; t++) c.tuning[t] = I.tuning[t];
    c.normals = I.normals;
    c.nNormals = I.nNormals;
    c.unifs = I.unifs;
    c.nUnifs = I.nUnifs;
    c.repIndx = I.repIndx;
    c.betaOut = I.betaOut;
    c.thetaOut = I.thetaOut;
    c.repOut = I.repOut;
    c.X = I.X;
    if (anyRep && I.repIndx) {
      int nrep = 0;
      for (int v : *host_rep) nrep += v != 0;
      c.repTheta = (CovParams *)own(sizeof(CovParams) * (nrep > 0 ? nrep : 1));
      c.repBeta = (double *)own(sizeof(double) * (size_t)(nrep > 0 ? nrep : 1) * p);
      c.repZoff = (long long *)own(sizeof(long long) * (nrep > 0 ? nrep : 1));
      if (!c.repTheta || !c.repBeta || !c.repZoff) {
        release();
        return nngp_fail(ctx, NNGP_ERR_NO_MEMORY, "device allocation failed");
      }
    }
    MCState &s = states[k];
    s = MCState{};
    for (int t = 0; t < 4; t++) s.theta[t] = s.cand[t] = I.thetaStart[t];
    for (int t = 0; t < p; t++) s.beta[t] = I.betaStart[t];
    CovParams cp{};
    cp.model = I.model;
    cp.sigmaSq = I.thetaStart[0];
    cp.tauSq = I.thetaStart[1];
    cp.phi = I.thetaStart[2];
    cp.nu = I.model == 2 ? I.thetaStart[3] : 0.0;
    cov_prepare(cp);
    th[2 * k] = th[2 * k + 1] = cp;
  }
  // Instances are split into classes by neighbor bound and by correlation code -- the model,
  // with Matern needing the general-nu kernel when nu is sampled or starts off the
  // half-integers -- so each class runs the kernel instantiation it needs and no other.  The
  // bounds are those the kernels are built for: FP32R 10 / 15 / 16 (register kernel), 24 and
  // 32; FP64 16, 24 and 32.
  constexpr int NCLS = 25;
  auto bound_class = [&](int m) {
    if (m > 24) return 4;
    if (m > 16) return 3;
    if (precision != NNGP_FP32R) return 2;
    return m <= 10 ? 0 : (m <= 15 ? 1 : 2);
  };
  std::vector<int> cls(ninst), pos(ninst);
  std::vector<std::vector<BFData>> cdatas(NCLS);
  std::vector<std::vector<PassEval>> cevCand(NCLS);
  for (int k = 0; k < ninst; k++) {
    const MCInstance &I = insts[k];
    const bool gen = I.model == 2 && (I.tuning[3] != 0.0 || th[2 * k].halfk < 0);
    const int cov = gen ? NNGP_COV_ANY : I.model;
    cls[k] = 5 * bound_class(I.m) + cov;
    pos[k] = (int)cdatas[cls[k]].size();
    cdatas[cls[k]].push_back(datas[k]);
    cevCand[cls[k]].push_back(PassEval{pos[k], 2 * k + 1});
  }
  double *d_outc[NCLS] = {};
  for (int c = 0; c < NCLS; c++) {
    const size_t cnt = cdatas[c].size();
    if (!cnt) continue;
    d_outc[c] = (double *)own(sizeof(double) * 2 * cnt * ng);
    if (!d_outc[c]) {
      release();
      return nngp_fail(ctx, NNGP_ERR_NO_MEMORY, "device allocation failed");
    }
  }
  for (int k = 0; k < ninst; k++) consts[k].out = d_outc[cls[k]] + (size_t)pos[k] * ng;
  MCConst *d_c = (MCConst *)own(sizeof(MCConst) * ninst);
  MCState *d_s = (MCState *)own(sizeof(MCState) * ninst);
  CovParams *d_th = (CovParams *)own(sizeof(CovParams) * 2 * ninst);
  unsigned long long *d_status = (unsigned long long *)own(sizeof(unsigned long long));
  if (!d_c || !d_s || !d_th || !d_status) {
    release();
    return nngp_fail(ctx, NNGP_ERR_NO_MEMORY, "device allocation failed");
  }
  int st = NNGP_OK;
#define MC_TRY(expr)                                                  \
  do {                                                                \
    cudaError_t e_ = (expr);                                          \
    if (e_ != cudaSuccess) {                                          \
      release();                                                      \
      return nngp_fail(ctx, NNGP_ERR_CUDA, std::string(#expr ": ") + cudaGetErrorString(e_)); \
    }                                                                 \
  } while (0)
  MC_TRY(cudaMemcpyAsync(d_c, consts.data(), sizeof(MCConst) * ninst, cudaMemcpyHostToDevice, ctx->stream));
  MC_TRY(cudaMemcpyAsync(d_s, states.data(), sizeof(MCState) * ninst, cudaMemcpyHostToDevice, ctx->stream));
  MC_TRY(cudaMemcpyAsync(d_th, th.data(), sizeof(CovParams) * 2 * ninst, cudaMemcpyHostToDevice, ctx->stream));
  if ((st = nngp_reset_status(ctx, d_status))) {
    release();
    return st;
  }
  BFPlan planCand[NCLS];
  bool haveCand[NCLS] = {};
  auto free_plans = [&]() {
    for (int c = 0; c < NCLS; c++)
      if (haveCand[c]) nngp_bf_plan_free(ctx, &planCand[c]);
  };
  for (int c = 0; c < NCLS && !st; c++) {
    if (cdatas[c].empty()) continue;
    const int cov = c % 5;
    st = nngp_bf_plan(ctx, &planCand[c], precision, 1, nv, cdatas[c], d_th, cevCand[c], d_status, cov);
    haveCand[c] = true;
  }
  if (st) {
    free_plans();
    release();
    return st;
  }
  auto run_cand = [&]() -> int {
    for (int c = 0; c < NCLS; c++)
      if (haveCand[c]) {
        const int r = nngp_bf_run(ctx, &planCand[c], d_outc[c]);
        if (r) return r;
      }
    return NNGP_OK;
  };
  // initial state: likelihood pass at the starting theta (candidate slot = start)
  st = run_cand();
  if (!st) {
    mc_init_kernel<<<nblk(ninst, 64), 64, 0, ctx->stream>>>(d_c, d_s, ninst);
    ctx->launches++;
  }
  // one iteration as a graph.  The classes' passes are
  // independent: each class runs on its own branch (side streams forked from and joined back
  // to the capturing stream), so small classes overlap instead of queueing.
  int nclasses = 0;
  for (int c = 0; c < NCLS; c++) nclasses += haveCand[c] ? 1 : 0;
  const int nside = nclasses > 1 ? (nclasses < 4 ? nclasses : 4) : 0;
  cudaStream_t side[4] = {};
  cudaEvent_t evFork = nullptr, evJoin[NCLS] = {};
  bool branches_ok = nside > 0;
  for (int k = 0; k < nside && branches_ok; k++)
    branches_ok = cudaStreamCreateWithFlags(&side[k], cudaStreamNonBlocking) == cudaSuccess;
  if (branches_ok) branches_ok = cudaEventCreateWithFlags(&evFork, cudaEventDisableTiming) == cudaSuccess;
  for (int c = 0; c < NCLS && branches_ok; c++)
    if (haveCand[c]) branches_ok = cudaEventCreateWithFlags(&evJoin[c], cudaEventDisableTiming) == cudaSuccess;
  // runs run_one(c) for every class, on parallel branches when they are available
  auto fan_out = [&](auto run_one) -> int {
    if (!branches_ok) {
      for (int c = 0; c < NCLS; c++)
        if (haveCand[c]) {
          const int r = run_one(c);
          if (r) return r;
        }
      return NNGP_OK;
    }
    cudaStream_t main_stream = ctx->stream;
    if (cudaEventRecord(evFork, main_stream) != cudaSuccess) return nngp_fail(ctx, NNGP_ERR_CUDA, "graph fork");
    int r = NNGP_OK, k = 0;
    for (int c = 0; c < NCLS && !r; c++) {
      if (!haveCand[c]) continue;
      cudaStream_t sc = side[k++ % nside];
      cudaStreamWaitEvent(sc, evFork, 0);
      ctx->stream = sc;
      r = run_one(c);
      ctx->stream = main_stream;
      cudaEventRecord(evJoin[c], sc);
      cudaStreamWaitEvent(main_stream, evJoin[c], 0);
    }
    return r;
  };
  auto capture = [&](cudaGraphExec_t *exec) -> int {
    cudaGraph_t g;
    const cudaError_t eb = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
    if (eb != cudaSuccess) return nngp_fail(ctx, NNGP_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(eb));
    int s2 = NNGP_OK;
    mc_pre_kernel<<<nblk(ninst, 64), 64, 0, ctx->stream>>>(d_c, d_s, d_th, ninst);
    s2 = fan_out([&](int c) { return nngp_bf_run(ctx, &planCand[c], d_outc[c]); });
    mc_post_kernel<<<nblk(ninst, 64), 64, 0, ctx->stream>>>(d_c, d_s, d_th, ninst);
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    if (s2) return s2;
    if (e != cudaSuccess) return nngp_fail(ctx, NNGP_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return nngp_fail(ctx, NNGP_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    return NNGP_OK;
  };
  cudaGraphExec_t gPlain = nullptr;
  const bool timing = ctx->timing;
  ctx->timing = false;  // no per-pass events inside a captured graph
  const int64_t launches_before = ctx->launches;
  if (!st) st = capture(&gPlain);
  const int64_t per_plain = ctx->launches - launches_before;
  ctx->launches = launches_before;  // captured launches are counted when replayed below
  ctx->timing = timing;
  for (int s = 0; !st && s < nS; s++) {
    cudaError_t e = cudaGraphLaunch(gPlain, ctx->stream);
    if (e != cudaSuccess) st = nngp_fail(ctx, NNGP_ERR_CUDA, std::string("graph launch: ") + cudaGetErrorString(e));
    ctx->launches += per_plain;
  }
  if (!st) {
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) st = nngp_fail(ctx, NNGP_ERR_CUDA, std::string("mcmc: ") + cudaGetErrorString(e));
  }
  for (int k = 0; k < nside; k++)
    if (side[k]) cudaStreamDestroy(side[k]);
  if (evFork) cudaEventDestroy(evFork);
  for (int c = 0; c < NCLS; c++)
    if (evJoin[c]) cudaEventDestroy(evJoin[c]);
  if (gPlain) cudaGraphExecDestroy(gPlain);
  if (!st) st = nngp_check_status(ctx, d_status, "rNNGP");
  if (!st) {
    MC_TRY(cudaMemcpy(states.data(), d_s, sizeof(MCState) * ninst, cudaMemcpyDeviceToHost));
    for (int k = 0; k < ninst && !st; k++) {
      if (accept_out) accept_out[k] = states[k].accept;
      if (states[k].status == 2) st = nngp_fail(ctx, NNGP_ERR_NOT_SPD, "rNNGP: beta Gram matrix not positive definite (dpotrf failed)");
      if (states[k].status == 3) st = nngp_fail(ctx, NNGP_ERR_STREAM, "rNNGP: a host-fed random stream ran out");
    }
  }
  // the recorded replicate draws, every one of an instance in one dataflow solve
  for (int k = 0; k < ninst && !st; k++) {
    const MCConst &c = consts[k];
    if (!c.repTheta || states[k].repCnt == 0) continue;
    RepSpec rs{};
    rs.n = c.n;
    rs.m = insts[k].m;
    rs.p = p;
    rs.nRep = states[k].repCnt;
    rs.precision = precision;
    rs.cov = cls[k] % 5;
    rs.xb_first = 1;  // X beta (dgemv), then + v (daxpy): src/rNNGP.cpp:300-303,311
    rs.xy = datas[k].xy;
    rs.xyf = datas[k].xyf;
    rs.nnIndx = insts[k].nnIndx;
    rs.nnLU = insts[k].nnLU;
    rs.X = insts[k].X;
    rs.d_theta = c.repTheta;
    rs.beta = c.repBeta;
    rs.bs_r = p;
    rs.bs_j = 1;
    rs.z = c.normals;
    rs.d_zoff = c.repZoff;
    rs.yRep = c.repOut;
    rs.d_status = d_status;
    if ((st = nngp_reset_status(ctx, d_status))) break;
    st = nngp_replicate_solve(ctx, rs);
    if (!st) st = nngp_check_status(ctx, d_status, "rNNGP replicates");
  }
  free_plans();
  release();
  cudaStreamSynchronize(ctx->stream);
#undef MC_TRY
  return st;
}

extern "C" int nngp_rNNGP(nngp_ctx *ctx, const double *y, const double *X, int p, int n, int m,
                          const double *coords, int covModel, const int *nnIndx, const int *nnIndxLU,
                          const double *sigmaSqIG, const double *tauSqIG, const double *phiUnif,
                          const double *nuUnif, const double *betaStarting, const double *thetaStarting,
                          const double *tuning, int nSamples, int nRep, const int *repIndx,
                          const double *normals, int64_t nNormals, const double *unifs, int64_t nUnifs,
                          int precision, double *betaSamples, double *thetaSamples, double *repSamples,
                          int *nAccept) {
  if (!ctx) return NNGP_ERR_ARG;
  if (p < 1 || p > PMAX) return nngp_fail(ctx, NNGP_ERR_ARG, "1 <= p <= 7 required");
  if (n < 1 || m < 1 || m > NNGP_MAX_M || n < m) return nngp_fail(ctx, NNGP_ERR_ARG, "n >= m and 1 <= m <= 32 required");
  if (covModel < 0 || covModel > 3) return nngp_fail(ctx, NNGP_ERR_ARG, "cov.model is not correctly specified");
  if (nSamples < 0) return nngp_fail(ctx, NNGP_ERR_ARG, "n.samples must be >= 0");
  cudaSetDevice(ctx->device);
  const int nTheta = covModel == 2 ? 4 : 3;
  const int64_t nI = nngp_nindx(n, m);
  std::vector<void *> tmp;
  auto up = [&](const void *h, size_t bytes) -> void * {
    void *d = nngp_malloc_async(ctx, bytes ? bytes : 16);
    if (d && bytes && h) cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, ctx->stream);
    tmp.push_back(d);
    return d;
  };
  auto fin = [&](int status) {
    for (void *q : tmp) nngp_free_async(ctx, q);
    cudaStreamSynchronize(ctx->stream);
    return status;
  };
  MCInstance I{};
  I.n = n;
  I.m = m;
  I.p = p;
  I.model = covModel;
  I.coords_cm = (const double *)up(coords, sizeof(double) * 2 * n);
  I.nnIndx = (const int *)up(nnIndx, sizeof(int) * (nI > 0 ? nI : 0));
  I.nnLU = (const int *)up(nnIndxLU, sizeof(int) * 2 * n);
  I.X = (const double *)up(X, sizeof(double) * (size_t)n * p);
  I.y = (const double *)up(y, sizeof(double) * n);
  for (int t = 0; t < 2; t++) {
    I.sIG[t] = sigmaSqIG[t];
    I.tIG[t] = tauSqIG[t];
    I.pU[t] = phiUnif[t];
    I.nU[t] = covModel == 2 ? nuUnif[t] : 0.0;
  }
  for (int t = 0; t < p; t++) I.betaStart[t] = betaStarting[t];
  for (int t = 0; t < 4; t++) {
    I.thetaStart[t] = t < nTheta ? thetaStarting[t] : 0.0;
    I.tuning[t] = t < nTheta ? tuning[t] : 0.0;
  }
  I.nSamples = nSamples;
  I.normals = (const double *)up(normals, sizeof(double) * (size_t)nNormals);
  I.nNormals = nNormals;
  I.unifs = (const double *)up(unifs, sizeof(double) * (size_t)nUnifs);
  I.nUnifs = nUnifs;
  std::vector<int> hrep;
  if (nRep > 0) {
    I.repIndx = (const int *)up(repIndx, sizeof(int) * nSamples);
    hrep.assign(repIndx, repIndx + nSamples);
  }
  I.betaOut = (double *)up(nullptr, sizeof(double) * (size_t)p * (nSamples ? nSamples : 1));
  I.thetaOut = (double *)up(nullptr, sizeof(double) * (size_t)nTheta * (nSamples ? nSamples : 1));
  I.repOut = nRep > 0 ? (double *)up(nullptr, sizeof(double) * (size_t)n * nRep) : nullptr;
  for (void *q : tmp)
    if (!q) return fin(nngp_fail(ctx, NNGP_ERR_NO_MEMORY, "device allocation failed"));
  if (nSamples == 0) {
    if (nAccept) *nAccept = 0;
    return fin(NNGP_OK);
  }
  int acc = 0;
  int st = nngp_run_mcmc(ctx, {I}, precision, nRep > 0 ? &hrep : nullptr, &acc);
  if (st) return fin(st);
  if (nAccept) *nAccept = acc;
  cudaMemcpyAsync(betaSamples, I.betaOut, sizeof(double) * (size_t)p * nSamples, cudaMemcpyDeviceToHost, ctx->stream);
  cudaMemcpyAsync(thetaSamples, I.thetaOut, sizeof(double) * (size_t)nTheta * nSamples, cudaMemcpyDeviceToHost,
                  ctx->stream);
  if (nRep > 0 && repSamples)
    cudaMemcpyAsync(repSamples, I.repOut, sizeof(double) * (size_t)n * nRep, cudaMemcpyDeviceToHost, ctx->stream);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return fin(nngp_fail(ctx, NNGP_ERR_CUDA, cudaGetErrorString(e)));
  return fin(NNGP_OK);
}

extern "C" int nngp_rNNGP_batch(nngp_ctx *ctx, int nprob, nngp_mcmc_problem *probs, int p, int precision,
                                int resident) {
  if (!ctx) return NNGP_ERR_ARG;
  if (nprob < 0 || (nprob > 0 && !probs)) return nngp_fail(ctx, NNGP_ERR_ARG, "nprob >= 0 and probs required");
  if (p < 1 || p > PMAX) return nngp_fail(ctx, NNGP_ERR_ARG, "1 <= p <= 7 required");
  if (precision != NNGP_FP64 && precision != NNGP_FP32R) return nngp_fail(ctx, NNGP_ERR_ARG, "unknown precision");
  for (int k = 0; k < nprob; k++) {
    const nngp_mcmc_problem &P = probs[k];
    if (P.n < 1 || P.m < 1 || P.m > NNGP_MAX_M || P.n < P.m)
      return nngp_fail(ctx, NNGP_ERR_ARG, "n >= m and 1 <= m <= 32 required in every chain");
    if (P.covModel < 0 || P.covModel > 3) return nngp_fail(ctx, NNGP_ERR_ARG, "cov.model is not correctly specified");
    if (P.nSamples < 0) return nngp_fail(ctx, NNGP_ERR_ARG, "n.samples must be >= 0");
    if (!P.sigmaSqIG || !P.tauSqIG || !P.phiUnif || (P.covModel == 2 && !P.nuUnif) || !P.betaStarting ||
        !P.thetaStarting || !P.tuning)
      return nngp_fail(ctx, NNGP_ERR_ARG, "priors, starting values and tuning are required");
  }
  if (nprob == 0) return NNGP_OK;
  cudaSetDevice(ctx->device);
  std::vector<void *> tmp;
  auto up = [&](const void *h, size_t bytes) -> void * {
    if (resident) return const_cast<void *>(h);
    void *d = nngp_malloc_async(ctx, bytes ? bytes : 16);
    if (d && bytes && h) cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, ctx->stream);
    tmp.push_back(d);
    return d;
  };
  auto fin = [&](int status) {
    for (void *q : tmp) nngp_free_async(ctx, q);
    cudaStreamSynchronize(ctx->stream);
    return status;
  };
  std::vector<MCInstance> insts;
  std::vector<int> which;
  for (int k = 0; k < nprob; k++) {
    nngp_mcmc_problem &P = probs[k];
    P.nAccept = 0;
    if (P.nSamples == 0) continue;
    const int n = P.n, m = P.m, nTheta = P.covModel == 2 ? 4 : 3;
    const int64_t nI = nngp_nindx(n, m);
    MCInstance I{};
    I.n = n;
    I.m = m;
    I.p = p;
    I.model = P.covModel;
    I.coords_cm = (const double *)up(P.coords, sizeof(double) * 2 * n);
    I.nnIndx = (const int *)up(P.nnIndx, sizeof(int) * (nI > 0 ? nI : 0));
    I.nnLU = (const int *)up(P.nnIndxLU, sizeof(int) * 2 * n);
    I.X = (const double *)up(P.X, sizeof(double) * (size_t)n * p);
    I.y = (const double *)up(P.y, sizeof(double) * n);
    for (int t = 0; t < 2; t++) {
      I.sIG[t] = P.sigmaSqIG[t];
      I.tIG[t] = P.tauSqIG[t];
      I.pU[t] = P.phiUnif[t];
      I.nU[t] = P.covModel == 2 ? P.nuUnif[t] : 0.0;
    }
    for (int t = 0; t < p; t++) I.betaStart[t] = P.betaStarting[t];
    for (int t = 0; t < 4; t++) {
      I.thetaStart[t] = t < nTheta ? P.thetaStarting[t] : 0.0;
      I.tuning[t] = t < nTheta ? P.tuning[t] : 0.0;
    }
    I.nSamples = P.nSamples;
    I.normals = (const double *)up(P.normals, sizeof(double) * (size_t)P.nNormals);
    I.nNormals = P.nNormals;
    I.unifs = (const double *)up(P.unifs, sizeof(double) * (size_t)P.nUnifs);
    I.nUnifs = P.nUnifs;
    I.repIndx = nullptr;
    I.betaOut = resident ? P.betaSamples : (double *)up(nullptr, sizeof(double) * (size_t)p * P.nSamples);
    I.thetaOut = resident ? P.thetaSamples : (double *)up(nullptr, sizeof(double) * (size_t)nTheta * P.nSamples);
    I.repOut = nullptr;
    insts.push_back(I);
    which.push_back(k);
  }
  for (void *q : tmp)
    if (!q) return fin(nngp_fail(ctx, NNGP_ERR_NO_MEMORY, "device allocation failed"));
  if (insts.empty()) return fin(NNGP_OK);
  std::vector<int> acc(insts.size(), 0);
  int st = nngp_run_mcmc(ctx, insts, precision, nullptr, acc.data());
  if (st) return fin(st);
  for (size_t j = 0; j < insts.size(); j++) {
    nngp_mcmc_problem &P = probs[which[j]];
    P.nAccept = acc[j];
    if (!resident) {
      const int nTheta = P.covModel == 2 ? 4 : 3;
      cudaMemcpyAsync(P.betaSamples, insts[j].betaOut, sizeof(double) * (size_t)p * P.nSamples,
                      cudaMemcpyDeviceToHost, ctx->stream);
      cudaMemcpyAsync(P.thetaSamples, insts[j].thetaOut, sizeof(double) * (size_t)nTheta * P.nSamples,
                      cudaMemcpyDeviceToHost, ctx->stream);
    }
  }
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return fin(nngp_fail(ctx, NNGP_ERR_CUDA, cudaGetErrorString(e)));
  return fin(NNGP_OK);
}
