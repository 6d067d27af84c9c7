// Replicated data by a dataflow sparse triangular solve.
//
// The reference draws one replicate v at parameter set s by the sequential recurrence
//   v_0 = sqrt(F_0) z_0,   v_i = B_i . v_N(i) + sqrt(F_i) z_i    (i = 1 .. n-1)
// (updateRep, src/rNNGP.cpp:24-42, and the per-sample loop of src/rNNGPReplicated.cpp:
// 183-205), then y_rep = X beta_s + v.  That is the unit lower-triangular solve
// (I - B) v = F^(1/2) z, sequential only along the neighbor DAG: v_i waits for its m
// neighbors, nothing else.  The DAG's depth is about 8.5 sqrt(n) for x-ordered uniform
// locations (8,454 levels at n = 1e6, ~118 locations per level on average).
//
// rep_flow_kernel solves a chunk of samples in one launch without a level schedule: each warp
// takes the next location from a ticket counter (locations in index order, a topological
// order of the DAG since every neighbor precedes its location; for x-ordered data it is
// also close to level order), waits until its neighbors are published, computes v_i for
// every sample of the chunk (lane t: samples t, t + 32, ...), and publishes location i.  A
// location waits only on smaller tickets, held by warps already running, so the waits always
// end; each is bounded all the same (kSpinLimit polls, then an error bit; the host fails the
// call).  v is read through L2 only: an SM's L1 may hold a line from before another SM wrote
// it.  Per chunk of samples: the standalone B/F pass at every sample's parameter set (the
// same kernels as updateBF), the solve, then y_rep = X beta + v in the reference's summation
// order (rNNGPReplicated: v, then + beta_j X_ij for j in order, as dgemv does; the response
// MCMC: X beta first, then + v, as its dgemv / daxpy do).
#include <cuda_runtime.h>
#include <algorithm>
#include <cstring>
#include <vector>
#include "nngp_internal.h"
#include "nngp_rep.h"

namespace {

constexpr int kSpinLimit = 1 << 21;  // polls of one neighbor's flag (each >= 32 ns apart)

__device__ __forceinline__ int ld_acquire(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int *p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

struct LevelArgs {
  int n, ns, r0;
  const int *nnIndx, *nnLU;
  const double *B;  // ns x nI: sample t's packed B at B + t nI
  int64_t nI;
  const double *F;  // ns x n
  const double *z;  // sample r's normals at z + zoff[r]
  const long long *zoff;
  double *vbuf;     // n x ns, location-major (the ns samples of a location are contiguous)
};

// words[0]: the ticket counter; words[1]: error bits (1: a neighbor that is not a
// predecessor, 2: a wait ran out of polls); ready[i] != 0 once v_i of every sample is written.
// The sum is the reference's ddot order (j = 0 .. cnt - 1) without fused multiply-adds.
constexpr int kFlowWarps = 4;  // warps per block

__global__ void __launch_bounds__(32 * kFlowWarps) rep_flow_kernel(LevelArgs a, int *ready, int *words) {
  __shared__ int nbs[kFlowWarps][32];  // the current location's neighbors, per warp
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int *ticket = words, *err = words + 1;
  for (;;) {
    int k = 0;
    if (lane == 0) k = atomicAdd(ticket, 1);
    const int i = __shfl_sync(0xffffffffu, k, 0);
    if (i >= a.n) break;
    const int off = a.nnLU[i], c = a.nnLU[a.n + i];
    int nb = 0;
    if (lane < c) {  // c <= 32: one neighbor per lane
      nb = a.nnIndx[off + lane];
      if (nb < 0 || nb >= i) {
        atomicOr(err, 1);
        nb = 0;
      } else {
        int spins = 0;
        while (ld_acquire(ready + nb) == 0) {
          if (++spins > kSpinLimit) {
            atomicOr(err, 2);
            break;
          }
          __nanosleep(32);
        }
      }
    }
    if (lane < c) nbs[warp][lane] = nb;
    __syncwarp();
    for (int t = lane; t < a.ns; t += 32) {
      const double *Bt = a.B + (size_t)t * a.nI + off;
      double acc = 0.0;
      for (int j = 0; j < c; j++)
        acc = __dadd_rn(acc, __dmul_rn(Bt[j], __ldcg(a.vbuf + (size_t)nbs[warp][j] * a.ns + t)));
      const double zz = a.z[a.zoff[a.r0 + t] + i];
      a.vbuf[(size_t)i * a.ns + t] = __dadd_rn(acc, __dmul_rn(sqrt(a.F[(size_t)t * a.n + i]), zz));
    }
    __syncwarp();  // every lane's stores precede the flag; nbs is rewritten next round
    if (lane == 0) {
      __threadfence();
      st_release(ready + i, 1);
    }
    __syncwarp();
  }
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

int nngp_replicate_solve(nngp_ctx *ctx, const RepSpec &s) {
  if (s.nRep <= 0) return NNGP_OK;
  if (s.m > 32) return nngp_fail(ctx, NNGP_ERR_ARG, "replicate solve: m > 32");
  const int n = s.n;
  const int64_t nI = std::max<int64_t>(nngp_nindx(n, s.m), 1);
  int st = NNGP_OK;
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
  int *ready = (int *)nngp_malloc_async(ctx, sizeof(int) * (size_t)n);
  int *words = (int *)nngp_malloc_async(ctx, sizeof(int) * 2);  // ticket, error bits
  auto release = [&]() {
    nngp_free_async(ctx, dB);
    nngp_free_async(ctx, dF);
    nngp_free_async(ctx, vbuf);
    nngp_free_async(ctx, out);
    nngp_free_async(ctx, ready);
    nngp_free_async(ctx, words);
  };
  if (!dB || !dF || !vbuf || !out || !ready || !words) {
    release();
    return nngp_fail(ctx, NNGP_ERR_NO_MEMORY, "device allocation failed");
  }
  // one block of four warps per SM: about five levels' worth of locations in flight at
  // n = 1e6, so a warp seldom waits and few poll at once
  const int grid = ctx->sm_count > 0 ? ctx->sm_count : 1;
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
    a.B = dB;
    a.nI = nI;
    a.F = dF;
    a.z = s.z;
    a.zoff = s.d_zoff;
    a.vbuf = vbuf;
    if (cudaMemsetAsync(ready, 0, sizeof(int) * (size_t)n, ctx->stream) != cudaSuccess ||
        cudaMemsetAsync(words, 0, sizeof(int) * 2, ctx->stream) != cudaSuccess) {
      st = nngp_fail(ctx, NNGP_ERR_CUDA, "replicate solve: memset failed");
      break;
    }
    rep_flow_kernel<<<grid, 32 * kFlowWarps, 0, ctx->stream>>>(a, ready, words);
    ctx->launches++;
    int herr[2] = {};
    cudaMemcpyAsync(herr, words, sizeof(int) * 2, cudaMemcpyDeviceToHost, ctx->stream);
    if (cudaStreamSynchronize(ctx->stream) == cudaSuccess && herr[1] != 0) {
      st = nngp_fail(ctx, herr[1] & 1 ? NNGP_ERR_ARG : NNGP_ERR_CUDA,
                     herr[1] & 1 ? "nnIndx lists a neighbor that is not a predecessor"
                                 : "replicate solve: a wait for a neighbor timed out");
      break;
    }
    rep_finish_kernel<<<(unsigned)nblocks((long long)n * ns, 256), 256, 0, ctx->stream>>>(
        a, s.p, s.X, s.beta, s.bs_r, s.bs_j, s.xb_first, s.yRep);
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) st = nngp_fail(ctx, NNGP_ERR_CUDA, std::string("replicate solve: ") + cudaGetErrorString(e));
  }
  release();
  return st;
}
