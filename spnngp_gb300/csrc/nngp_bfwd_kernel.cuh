// FP64 B/F kernel for the 32-neighbor bound (24 < m <= 32): one warp per location
// (reference updateBF, src/rNNGP.cpp:46-101; updateConjBF, src/cNNGP.cpp:24-69; the
// likelihood sums of src/rNNGP.cpp:306-317 and Q, src/util.cpp:261-280).  It runs the FP64
// form's pass and the FP64 re-solve of the locations the FP32R kernels flag.
//
// With a thread per location, a 32-neighbor system needs 4.2 KB of shared memory per thread
// (the packed triangle in double), which leaves one warp per SM and the FP64 pipe mostly idle.
// Here lane r of a warp owns row r, as in the FP32R warp kernel (nngp_bfw_kernel.cuh): the
// covariance pairs are spread over the lanes by row pairs into the warp's 32 x 33-padded
// matrix, lane r loads row r, the right-looking Cholesky broadcasts pivots and columns by
// shuffles, L goes back to the matrix for the back substitution's column reads, and F and the
// V products are warp sums.  Every lane executes every step (rows past m_i are the identity),
// so about twice the minimal FP64 work is issued, but the FP64 pipe stays busy: at n = 1e6,
// m = 32 the pass takes 97 ms against 206 ms for the thread-per-location kernel.  At the
// 24-neighbor bound the thread-per-location kernel still holds two blocks per SM and is faster
// (38 against 67 ms), so it keeps that bound.
// Arithmetic follows the shared-memory kernel's expressions (distances, spCor, the diagonal
// sigma^2 rho(0) + tau^2, F = sigma^2 - B'c + tau^2); the factor's summation order differs,
// which moves results by O(kappa 2^-53).
#pragma once
#include <cuda_runtime.h>
#include "nngp_internal.h"
#include "nngp_math.cuh"

namespace nngp_bfwd {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kLD = 33;

// Per-warp shared memory (doubles): 32 neighbor coordinates (x, y), the 32 x 33 matrix (C,
// then L), the fused pass's residuals r_v.
constexpr int kGeo = 0;
constexpr int kMat = 64;
constexpr int kRV = kMat + 32 * kLD;
constexpr int kWarpDoubles = kRV + NNGP_MAX_NV;
constexpr int kWarpsPerBlock = 4;

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);  // commutative: same on every lane
  return v;
}

template <int M, int MODE, int COV>
__global__ void __launch_bounds__(128, 3) bfwd_kernel(const BFData *__restrict__ datas,
                                                   const CovParams *__restrict__ thetas,
                                                   const BFJob *__restrict__ jobs, int njobs, int tile_begin,
                                                   int tile_end, int nv, unsigned long long *__restrict__ status,
                                                   int only_flagged, const int *__restrict__ tile_list,
                                                   const int *__restrict__ tile_count) {
  extern __shared__ __align__(16) double smem_d[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  double *ws = smem_d + (size_t)warp * kWarpDoubles;
  double2 *geo = reinterpret_cast<double2 *>(ws + kGeo);
  double *mat = ws + kMat, *rvs = ws + kRV;
  const int ng = MODE == 0 ? 1 : 1 + nv * (nv + 1) / 2;
  const int rb = kLD * lane;
  for (int k = lane; k < 32 * kLD; k += 32) mat[k] = 0.0;  // entries outside M x M stay zero
  __syncwarp();

  // the FP64 re-solve walks the list of tiles the FP32R pass recorded; the other passes walk
  // tiles [tile_begin, tile_end)
  const int ntodo = tile_list ? *tile_count : tile_end - tile_begin;
  for (int kt = blockIdx.x * wpb + warp; kt < ntodo; kt += gridDim.x * wpb) {
    const int tile = tile_list ? tile_list[kt] : tile_begin + kt;
    const BFJob *jp = jobs + nngp_find_job(jobs, njobs, tile);
    const BFData *dp = datas + jp->data;
    const CovParams *cpp = thetas + jp->theta;
    const double sigmaSq = cpp->sigmaSq, tauSq = cpp->tauSq;
    const int tj = tile - jp->tile0;
    const int n = dp->n;
    const int i_end = min(n, (tj + 1) * 32);
    const double2 *xy = reinterpret_cast<const double2 *>(dp->xy);
    const int *nnLU = dp->nnLU;
    const unsigned char *flags = jp->flags;
    double acc0 = 0.0, acc1 = 0.0;

#pragma unroll 1
    for (int i = tj * 32; i < i_end; i++) {
      if (only_flagged && !flags[i]) continue;  // warp-uniform
      const int off = nnLU[i];
      const int mi = min(nnLU[n + i], M);
      const bool pad = lane >= mi;

      // ---- covariance: c_r on lane r, the strict lower triangle by row pairs, the diagonal
      const double2 pi = xy[i];
      int nbk = 0;
      double2 g = make_double2(0.0, 0.0);
      if (!pad) {
        nbk = dp->nnIndx[off + lane];
        g = xy[nbk];
      }
      geo[lane] = g;
      double cv = 0.0;
      if (!pad) {
        const double ax = pi.x - g.x, ay = pi.y - g.y;
        cv = sigmaSq * nngp_cor_d<COV>(sqrt(ax * ax + ay * ay), *cpp);
      }
      __syncwarp();
#pragma unroll 1
      for (int t = 0; t < M / 2; t++) {
        // rows t and M - 1 - t: t + (M - 1 - t) = M - 1 pairs on lanes 0 .. M - 2
        const int r = lane < t ? t : M - 1 - t;
        const int c = lane < t ? lane : min(lane - t, M - 1);
        if (lane < M - 1) {
          double e = 0.0;
          if (r < mi) {
            const double2 gr = geo[r], gc = geo[c];
            const double bx = gr.x - gc.x, by = gr.y - gc.y;
            e = sigmaSq * nngp_cor_d<COV>(sqrt(bx * bx + by * by), *cpp);
          }
          mat[kLD * r + c] = e;
          mat[kLD * c + r] = e;
        }
      }
      if (lane < M) mat[rb + lane] = pad ? 1.0 : sigmaSq * nngp_cor_d<COV>(0.0, *cpp) + tauSq;
      __syncwarp();

      // ---- Cholesky: lane r holds row r; step k broadcasts the pivot and column k
      double row[M];
#pragma unroll
      for (int c = 0; c < M; c++) row[c] = mat[rb + c];
      bool ok = true;
      double ivmine = 1.0;  // 1 / L_rr on lane r
#pragma unroll
      for (int k = 0; k < M; k++) {
        const double dk = __shfl_sync(kFull, row[k], k);
        ok = ok && (dk > 0.0);
        const double ik = 1.0 / sqrt(dk);
        if (lane == k) ivmine = ik;
        const double lk = row[k] * ik;  // L[r][k] on lane r > k
        row[k] = lk;
        if (k + 1 < M) {
#pragma unroll
          for (int j = k + 1; j < M; j++) row[j] = fma(-lk, __shfl_sync(kFull, lk, j), row[j]);
        }
      }
      // L's strict lower part (diagonal and upper part zero) back to the matrix for the column
      // reads of the back substitution; every lane has read its row above
#pragma unroll
      for (int c = 0; c < M; c++) {
        row[c] = c < lane ? row[c] : 0.0;
        mat[rb + c] = row[c];
      }
      __syncwarp();

      // ---- L z = c, L' B = z: lane k's numerator times its 1 / L_kk is broadcast at step k
      double t = cv;
#pragma unroll
      for (int k = 0; k < M; k++) t = fma(-row[k], __shfl_sync(kFull, t * ivmine, k), t);
      t = t * ivmine;
#pragma unroll 4
      for (int k = M - 1; k >= 0; k--) t = fma(-mat[kLD * k + lane], __shfl_sync(kFull, t * ivmine, k), t);
      const double bmine = t * ivmine;  // B_r on lane r (0 past m_i)
      if (!ok && lane == 0) nngp_record_status(status, 1, i);

      // ---- F = sigma^2 - B'c + tau^2, log F, likelihood terms
      const double Fi = sigmaSq - warp_sum_d(bmine * cv) + tauSq;
      const double logF = log(Fi);
      if constexpr (MODE == 0) {
        if (!pad) dp->B[off + lane] = bmine;
        if (lane == 0) {
          dp->F[i] = Fi;
          acc0 += logF;
        }
      } else {
        // r_v = V_iv - sum_k B_k V_nb(k)v
        const double *V = dp->V;
#pragma unroll 1
        for (int v = 0; v < nv; v++) {
          const double q = pad ? 0.0 : V[(size_t)nbk * nv + v];
          const double rv = V[(size_t)i * nv + v] - warp_sum_d(bmine * q);
          if (lane == 0) rvs[v] = rv;
        }
        __syncwarp();
        const double invF = 1.0 / Fi;
#pragma unroll
        for (int s = 0; s < 2; s++) {
          const int tt = lane + 32 * s;
          if (tt < ng) {
            double val = logF;
            if (tt > 0) {
              int rem = tt - 1, a = 0;
              while (rem >= nv - a) {
                rem -= nv - a;
                a++;
              }
              val = rvs[a] * rvs[a + rem] * invF;
            }
            if (s == 0) acc0 += val;
            else acc1 += val;
          }
        }
      }
      __syncwarp();  // the warp's buffers are rewritten by the next location
    }
    double *partial = jp->partial + (size_t)tj * ng;
    if (lane < ng) partial[lane] = acc0;
    if (lane + 32 < ng) partial[lane + 32] = acc1;
  }
}

// Launches the kernel on tiles [t0, t1) of the plan's primary jobs, or (fallback_pass) on the
// FP64 tiles the FP32R pass recorded: blocks of wpb (1 - 4) warps, `grid` blocks (0: one
// 32-location tile per warp; fewer: each warp loops over tiles).  Each warp reduces its own
// tiles, so the shape never changes a result.
template <int M, int MODE, int COV>
int launch_warp_d(nngp_ctx *ctx, const BFPlan *pl, bool fallback_pass, int t0, int t1, int wpb = kWarpsPerBlock,
                  int grid = 0) {
  static bool configured[64] = {};  // the attribute is per device (set for the largest block)
  const int dev = ctx->device & 63;
  if (!configured[dev]) {
    NNGP_CUDA_TRY(ctx, cudaFuncSetAttribute(bfwd_kernel<M, MODE, COV>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)(sizeof(double) * kWarpDoubles * kWarpsPerBlock)));
    configured[dev] = true;
  }
  if (wpb < 1 || wpb > kWarpsPerBlock) wpb = kWarpsPerBlock;
  const size_t smem = sizeof(double) * kWarpDoubles * wpb;
  const int tiles = fallback_pass ? pl->tiles_fb : t1 - t0;
  if (tiles <= 0) return NNGP_OK;
  const int full = (tiles + wpb - 1) / wpb;
  if (grid <= 0 || grid > full) grid = full;
  if (fallback_pass) {
    // the re-solve walks the recorded tiles (none recorded: every block returns at once)
    const int cap = 3 * (ctx->sm_count > 0 ? ctx->sm_count : 1);
    grid = grid < cap ? grid : cap;
  }
  bfwd_kernel<M, MODE, COV><<<grid, 32 * wpb, smem, ctx->stream>>>(
      pl->d_datas, pl->d_thetas, fallback_pass ? pl->d_jobs_fb : pl->d_jobs, pl->njobs, fallback_pass ? 0 : t0,
      fallback_pass ? pl->tiles_fb : t1, pl->nv, pl->d_status, fallback_pass ? 1 : 0,
      fallback_pass ? pl->d_fb64_list : nullptr, fallback_pass ? (const int *)pl->d_fb64_count : nullptr);
  NNGP_LAUNCH_CHECK(ctx);
  return NNGP_OK;
}

}  // namespace nngp_bfwd
