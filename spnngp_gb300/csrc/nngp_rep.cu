// Replicated data by a level-scheduled sparse triangular solve.
//
// The reference draws one replicate v at parameter set s by the sequential recurrence
//   v_0 = sqrt(F_0) z_0,   v_i = B_i . v_N(i) + sqrt(F_i) z_i    (i = 1 .. n-1)
// (updateRep, src/rNNGP.cpp:24-42, and the per-sample loop of src/rNNGPReplicated.cpp:
// 183-205), then y_rep = X beta_s + v.  That is the unit lower-triangular solve
// (I - B) v = F^(1/2) z, sequential only along the neighbor DAG: v_i waits for its m
// neighbors, nothing else.  Its depth is about 8.5 sqrt(n) for x-ordered uniform locations
// (8,454 levels at n = 1e6, ~118 locations per level), so the solve runs one launch per
// level over every (location in the level) x (sample) pair of a chunk of samples, instead of
// one thread walking all n locations per sample.
//
// The level schedule is built once per neighbor structure on the device:
//   level_kernel    lev[i] = 1 + max lev[N(i)] (lev[0] = 0).  Blocks take tickets in the
//                   order they start, so a location waits only on locations of blocks that
//                   are resident or done; each wait on a neighbor's level is bounded (an
//                   error flag and an early return after kSpinLimit polls);
//   level_count / level_scatter   a counting sort of the locations by level (order within
//                   a level is arbitrary: the locations of one level do not read each other).
// Per chunk of samples: the standalone B/F pass at every sample's parameter set (the same
// kernels as updateBF), the level launches, then y_rep = X beta + v in the reference's
// summation order (rNNGPReplicated: v, then + beta_j X_ij for j in order, as dgemv does;
// the response MCMC: X beta first, then + v, as its dgemv / daxpy do).
#include <cuda_runtime.h>
#include <algorithm>
#include <cstring>
#include <vector>
#include "nngp_internal.h"
#include "nngp_rep.h"

namespace {

constexpr int kSpinLimit = 1 << 21;  // polls of one neighbor's level (each >= 64 ns apart)

__device__ __forceinline__ int ld_relaxed(const int *p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed(int *p, int v) {
  asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// err bit 1: a neighbor index that is not a predecessor (k < 0 or k >= i); bit 2: a wait ran
// out of polls.  lev must hold -1 everywhere on entry; depth receives 1 + the largest level.
__global__ void level_kernel(int n, const int *__restrict__ nnIndx, const int *__restrict__ nnLU, int *lev,
                             unsigned *ticket, int *err, int *depth) {
  __shared__ unsigned blk;
  if (threadIdx.x == 0) blk = atomicAdd(ticket, 1u);
  __syncthreads();
  const long long i = (long long)blk * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int off = nnLU[i], cnt = nnLU[n + i];
  int l = 0;
  for (int j = 0; j < cnt; j++) {
    const int k = nnIndx[off + j];
    if (k < 0 || k >= i) {
      atomicOr(err, 1);
      continue;
    }
    int v = ld_relaxed(lev + k);
    int spins = 0;
    while (v < 0) {  // a short sleep between polls: polling flat out from every waiting thread
                     // crowds the memory system and slowed each level of the critical path
      if (++spins > kSpinLimit) {
        atomicOr(err, 2);
        break;
      }
      __nanosleep(64);
      v = ld_relaxed(lev + k);
    }
    if (v >= l) l = v + 1;
  }
  st_relaxed(lev + i, l);
  atomicMax(depth, l + 1);
}

__global__ void level_count_kernel(int n, const int *__restrict__ lev, int *__restrict__ count) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) atomicAdd(count + lev[i], 1);
}

__global__ void level_scatter_kernel(int n, const int *__restrict__ lev, int *__restrict__ cursor,
                                     int *__restrict__ order) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) order[atomicAdd(cursor + lev[i], 1)] = (int)i;
}

struct LevelArgs {
  int n, ns, r0;
  const int *nnIndx, *nnLU, *order;
  const double *B;  // ns x nI: sample t's packed B at B + t nI
  int64_t nI;
  const double *F;  // ns x n
  const double *z;  // sample r's normals at z + zoff[r]
  const long long *zoff;
  double *vbuf;     // n x ns, location-major (the ns samples of a location are contiguous)
};

// Locations order[lo .. lo + cnt) of one level, every sample of the chunk: thread (q, t),
// t fastest, so the samples of a neighbor are read as one contiguous run.  The sum is the
// reference's ddot order (j = 0 .. cnt - 1) without fused multiply-adds.
__global__ void rep_level_kernel(LevelArgs a, int lo, int cnt) {
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= (long long)cnt * a.ns) return;
  const int t = (int)(tid % a.ns);
  const int i = a.order[lo + (int)(tid / a.ns)];
  const double *Bt = a.B + (size_t)t * a.nI;
  const int off = a.nnLU[i], c = a.nnLU[a.n + i];
  double acc = 0.0;
  for (int j = 0; j < c; j++)
    acc = __dadd_rn(acc, __dmul_rn(Bt[off + j], a.vbuf[(size_t)a.nnIndx[off + j] * a.ns + t]));
  const double zz = a.z[a.zoff[a.r0 + t] + i];
  a.vbuf[(size_t)i * a.ns + t] = __dadd_rn(acc, __dmul_rn(sqrt(a.F[(size_t)t * a.n + i]), zz));
}

// y_rep of sample r0 + t at location i (i fastest: coalesced writes).
__global__ void rep_finish_kernel(LevelArgs a, int p, const double *__restrict__ X, const double *__restrict__ beta,
                                  int64_t bs_r, int64_t bs_j, int xb_first, double *__restrict__ yRep) {
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= (long long)a.n * a.ns) return;
  const int i = (int)(tid % a.n), t = (int)(tid / a.n);
  const int64_t r = a.r0 + t;
  const double v = a.vbuf[(size_t)i * a.ns + t];
  double acc = xb_first ? 0.0 : v;
  for (int j = 0; j < p; j++) acc = __dadd_rn(acc, __dmul_rn(beta[r * bs_r + j * bs_j], X[(size_t)j * a.n + i]));
  if (xb_first) acc = __dadd_rn(acc, v);
  yRep[(size_t)r * a.n + i] = acc;
}

long long nblocks(long long work, int tpb) { return (work + tpb - 1) / tpb; }

}  // namespace

int nngp_level_schedule(nngp_ctx *ctx, int n, const int *nnIndx, const int *nnLU, LevelSchedule *ls) {
  ls->n = n;
  ls->depth = 0;
  ls->start.clear();
  ls->order = (int *)nngp_malloc_async(ctx, sizeof(int) * (size_t)n);
  int *lev = (int *)nngp_malloc_async(ctx, sizeof(int) * (size_t)n);
  int *words = (int *)nngp_malloc_async(ctx, sizeof(int) * 4);  // ticket, err, depth
  if (!ls->order || !lev || !words) {
    nngp_free_async(ctx, ls->order);
    nngp_free_async(ctx, lev);
    nngp_free_async(ctx, words);
    ls->order = nullptr;
    return nngp_fail(ctx, NNGP_ERR_NO_MEMORY, "device allocation failed");
  }
  auto done = [&](int st) {
    nngp_free_async(ctx, lev);
    nngp_free_async(ctx, words);
    if (st) {
      nngp_free_async(ctx, ls->order);
      ls->order = nullptr;
    }
    return st;
  };
  if (cudaMemsetAsync(lev, 0xFF, sizeof(int) * (size_t)n, ctx->stream) != cudaSuccess ||
      cudaMemsetAsync(words, 0, sizeof(int) * 4, ctx->stream) != cudaSuccess)
    return done(nngp_fail(ctx, NNGP_ERR_CUDA, "level schedule: memset failed"));
  level_kernel<<<(unsigned)nblocks(n, 128), 128, 0, ctx->stream>>>(n, nnIndx, nnLU, lev, (unsigned *)words,
                                                                    words + 1, words + 2);
  ctx->launches++;
  int h[4] = {};
  cudaMemcpyAsync(h, words, sizeof(int) * 4, cudaMemcpyDeviceToHost, ctx->stream);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess)
    return done(nngp_fail(ctx, NNGP_ERR_CUDA, std::string("level schedule: ") + cudaGetErrorString(e)));
  if (h[1] & 1) return done(nngp_fail(ctx, NNGP_ERR_ARG, "nnIndx lists a neighbor that is not a predecessor"));
  if (h[1] & 2) return done(nngp_fail(ctx, NNGP_ERR_CUDA, "level schedule: a wait for a neighbor's level timed out"));
  const int depth = h[2];
  int *count = (int *)nngp_malloc_async(ctx, sizeof(int) * (size_t)(depth + 1));
  if (!count) return done(nngp_fail(ctx, NNGP_ERR_NO_MEMORY, "device allocation failed"));
  cudaMemsetAsync(count, 0, sizeof(int) * (size_t)(depth + 1), ctx->stream);
  level_count_kernel<<<(unsigned)nblocks(n, 256), 256, 0, ctx->stream>>>(n, lev, count);
  ctx->launches++;
  std::vector<int> hc(depth + 1, 0);
  cudaMemcpyAsync(hc.data(), count, sizeof(int) * (size_t)depth, cudaMemcpyDeviceToHost, ctx->stream);
  e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    nngp_free_async(ctx, count);
    return done(nngp_fail(ctx, NNGP_ERR_CUDA, std::string("level schedule: ") + cudaGetErrorString(e)));
  }
  ls->start.assign(depth + 1, 0);
  for (int l = 0; l < depth; l++) ls->start[l + 1] = ls->start[l] + hc[l];
  cudaMemcpyAsync(count, ls->start.data(), sizeof(int) * (size_t)depth, cudaMemcpyHostToDevice, ctx->stream);
  level_scatter_kernel<<<(unsigned)nblocks(n, 256), 256, 0, ctx->stream>>>(n, lev, count, ls->order);
  ctx->launches++;
  e = cudaStreamSynchronize(ctx->stream);  // the host start vector is read by the copy above
  nngp_free_async(ctx, count);
  if (e != cudaSuccess) return done(nngp_fail(ctx, NNGP_ERR_CUDA, std::string("level schedule: ") + cudaGetErrorString(e)));
  ls->depth = depth;
  return done(NNGP_OK);
}

void nngp_level_schedule_free(nngp_ctx *ctx, LevelSchedule *ls) {
  nngp_free_async(ctx, ls->order);
  ls->order = nullptr;
  ls->start.clear();
  ls->depth = 0;
}

int nngp_replicate_solve(nngp_ctx *ctx, const RepSpec &s) {
  if (s.nRep <= 0) return NNGP_OK;
  const int n = s.n;
  const int64_t nI = std::max<int64_t>(nngp_nindx(n, s.m), 1);
  LevelSchedule ls;
  int st = nngp_level_schedule(ctx, n, s.nnIndx, s.nnLU, &ls);
  if (st) return st;
  // samples per chunk: B, F and the location-major v of a chunk within a quarter of the free
  // memory (at most 32 GB)
  size_t freeb = 0, totalb = 0;
  cudaMemGetInfo(&freeb, &totalb);
  const size_t budget = std::min<size_t>(freeb / 4, (size_t)32 << 30);
  const size_t per = sizeof(double) * ((size_t)nI + 2 * (size_t)n);
  const int chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)s.nRep, budget / per));
  double *dB = (double *)nngp_malloc_async(ctx, sizeof(double) * (size_t)nI * chunk);
  double *dF = (double *)nngp_malloc_async(ctx, sizeof(double) * (size_t)n * chunk);
  double *vbuf = (double *)nngp_malloc_async(ctx, sizeof(double) * (size_t)n * chunk);
  double *out = (double *)nngp_malloc_async(ctx, sizeof(double) * 2 * (size_t)chunk);
  auto release = [&]() {
    nngp_free_async(ctx, dB);
    nngp_free_async(ctx, dF);
    nngp_free_async(ctx, vbuf);
    nngp_free_async(ctx, out);
    nngp_level_schedule_free(ctx, &ls);
  };
  if (!dB || !dF || !vbuf || !out) {
    release();
    return nngp_fail(ctx, NNGP_ERR_NO_MEMORY, "device allocation failed");
  }
  for (int r0 = 0; !st && r0 < s.nRep; r0 += chunk) {
    const int ns = std::min(chunk, s.nRep - r0);
    std::vector<BFData> datas(ns);
    std::vector<PassEval> ev(ns);
    for (int t = 0; t < ns; t++) {
      BFData d{};
      d.n = n;
      d.m = s.m;
      d.xy = s.xy;
      d.xyf = s.xyf;
      d.nnIndx = s.nnIndx;
      d.nnLU = s.nnLU;
      d.B = dB + (size_t)t * nI;
      d.F = dF + (size_t)t * n;
      datas[t] = d;
      ev[t] = PassEval{t, r0 + t};
    }
    BFPlan plan;
    st = nngp_bf_plan(ctx, &plan, s.precision, 0, 0, datas, s.d_theta, ev, s.d_status, s.cov);
    if (!st) st = nngp_bf_run(ctx, &plan, out);
    nngp_bf_plan_free(ctx, &plan);
    if (st) break;
    LevelArgs a{};
    a.n = n;
    a.ns = ns;
    a.r0 = r0;
    a.nnIndx = s.nnIndx;
    a.nnLU = s.nnLU;
    a.order = ls.order;
    a.B = dB;
    a.nI = nI;
    a.F = dF;
    a.z = s.z;
    a.zoff = s.d_zoff;
    a.vbuf = vbuf;
    for (int l = 0; l < ls.depth; l++) {
      const int lo = ls.start[l], cnt = ls.start[l + 1] - lo;
      rep_level_kernel<<<(unsigned)nblocks((long long)cnt * ns, 128), 128, 0, ctx->stream>>>(a, lo, cnt);
    }
    ctx->launches += ls.depth;
    rep_finish_kernel<<<(unsigned)nblocks((long long)n * ns, 256), 256, 0, ctx->stream>>>(
        a, s.p, s.X, s.beta, s.bs_r, s.bs_j, s.xb_first, s.yRep);
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) st = nngp_fail(ctx, NNGP_ERR_CUDA, std::string("replicate solve: ") + cudaGetErrorString(e));
  }
  release();
  return st;
}
