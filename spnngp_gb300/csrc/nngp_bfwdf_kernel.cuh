// Double-float re-solve of the locations the warp-per-location FP32R kernel (24 < m <= 32,
// nngp_bfw_kernel.cuh) flags -- typically a gaussian covariance with a small nugget, whose
// float factor cannot be certified.  A thread-per-location triangle at this bound needs
// ~5.4 KB of shared memory per thread (one 32-thread block per SM; the thread-per-location
// kernel of nngp_bfdf_kernel.cuh serves m <= 24), so this kernel keeps the warp-per-location
// layout of the FP32R kernel and factors in double-float arithmetic on the FP32 pipe instead of handing the
// locations to the FP64 kernel (reference updateBF, src/rNNGP.cpp:46-101, and the likelihood
// sums of src/rNNGP.cpp:306-317):
//   1. geometry and the covariance in double-float exactly as the FP32R warp kernel builds it
//      (lane k: c_k; the strict lower triangle by row pairs into the warp's padded hi / lo
//      matrices, stored at (r, c) and (c, r));
//   2. lane r loads row r (hi, lo) into registers; right-looking Cholesky in double-float, step
//      k broadcasting the pivot and column k by shuffles; z = L^-1 c by the same broadcasts;
//      F = sigma^2 + tau^2 - z'z; L back to shared memory so that the back substitution
//      B = L^-T z reads its columns;
//   3. in FP64: log F and, in the fused pass, r = (I - B) V and r_a r_b / F (warp sums); lane t
//      adds value t of each location in location order, so a tile's sums have a fixed order.
// The kernel walks the FP32R pass's list of flagged FP64 tiles (32 locations each); a tile with
// a location it cannot certify -- a non-positive double-float pivot, F < 1e-6 (sigma^2 + tau^2),
// or a squared pivot ratio above 1e10 -- goes whole to the FP64 kernel's list.
#pragma once
#include <cuda_runtime.h>
#include "nngp_cov_df.cuh"

namespace nngp_bfwdf {

using nngp_bfr::CorDF;
constexpr unsigned kFull = 0xffffffffu;
constexpr int kTile = 32;          // the FP64 tile for 16 < m <= 32 (the flagged-tile list's unit)
constexpr int kWarpsPerBlock = 4;
constexpr int kNGMax = 1 + NNGP_MAX_NV * (NNGP_MAX_NV + 1) / 2;
constexpr float kMaxPivotRatio2 = 1e10f;

// Per-warp shared memory (floats): geometry (32 float4), hi and lo parts of C (then of L) as 32 x 33
// padded matrices, the exp / Matern table.
constexpr int LD = 33;
constexpr int MAT = 32 * LD;
constexpr int OFF_CH = 4 * 32;
constexpr int OFF_CL = OFF_CH + MAT;
constexpr int OFF_TAB = OFF_CL + MAT;
constexpr int WARP_FLOATS = (OFF_TAB + nngp_bfr::kTabFloats + 3) & ~3;
constexpr size_t kSmemBytes = sizeof(float) * (size_t)WARP_FLOATS * kWarpsPerBlock;

__device__ __forceinline__ nngp_df::df shfl_df(nngp_df::df v, int src) {
  return nngp_df::df{__shfl_sync(kFull, v.h, src), __shfl_sync(kFull, v.l, src)};
}
__device__ __forceinline__ nngp_df::df warp_sum_df(nngp_df::df p) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) p = nngp_df::add(p, nngp_df::df{__shfl_xor_sync(kFull, p.h, o), __shfl_xor_sync(kFull, p.l, o)});
  return p;
}
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// Step K of the right-looking Cholesky on lane r's row (rh, rl): the pivot from lane K, L[r][K]
// on lanes r > K, then the update of entries K < j <= r.  Written as a recursion over K and j so
// that every row index is a compile-time constant (the row stays in registers).
template <int M, int J>
__device__ __forceinline__ void chol_update(float (&rh)[M], float (&rl)[M], nngp_df::df lk, int lane) {
  if constexpr (J < M) {
    const nngp_df::df ljk = shfl_df(lk, J);
    const nngp_df::df u = nngp_df::sub(nngp_df::df{rh[J], rl[J]}, nngp_df::mul(lk, ljk));
    if (lane >= J) {
      rh[J] = u.h;
      rl[J] = u.l;
    }
    chol_update<M, J + 1>(rh, rl, lk, lane);
  }
}
template <int M, int K>
__device__ __forceinline__ void chol_step(float (&rh)[M], float (&rl)[M], int lane, bool &ok, float &pmin,
                                          float &pmax, nngp_df::df &ivmine) {
  if constexpr (K < M) {
    namespace F = nngp_df;
    const F::df dk = shfl_df(F::df{rh[K], rl[K]}, K);
    ok = ok && (dk.h > 0.0f);
    const F::df lkk = F::sqrt(dk);
    const F::df ik = F::recip(lkk);
    pmin = fminf(pmin, lkk.h);
    pmax = fmaxf(pmax, lkk.h);
    if (lane == K) ivmine = ik;
    const F::df lk = lane > K ? F::mul(F::df{rh[K], rl[K]}, ik) : F::df{0.0f, 0.0f};  // L[r][K] on lane r > K
    rh[K] = lk.h;
    rl[K] = lk.l;
    chol_update<M, K + 1>(rh, rl, lk, lane);
    chol_step<M, K + 1>(rh, rl, lane, ok, pmin, pmax, ivmine);
  }
}

template <int M, int MODE, int COV>
__global__ void __launch_bounds__(32 * kWarpsPerBlock, 2) bfwdf_kernel(
    const BFData *__restrict__ datas, const CovParams *__restrict__ thetas, const BFJob *__restrict__ jobs_fb,
    int njobs, int nv, const int *__restrict__ tile_list, const int *__restrict__ tile_count, int *__restrict__ list64,
    int *__restrict__ count64, unsigned long long *__restrict__ locs64) {
  namespace F = nngp_df;
  namespace G = nngp_df2;
  extern __shared__ __align__(16) float smem_wd[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float *ws = smem_wd + (size_t)warp * WARP_FLOATS;
  float4 *geo = reinterpret_cast<float4 *>(ws);
  float *chs = ws + OFF_CH, *cls = ws + OFF_CL, *tab = ws + OFF_TAB;
  const int rb = LD * lane;
  const int ng = MODE == 0 ? 1 : 1 + nv * (nv + 1) / 2;
  for (int k = lane; k < 2 * MAT; k += 32) chs[k] = 0.0f;  // CH and CL are contiguous
  __syncwarp();

  static_assert(M % 2 == 0 && M <= 32, "the covariance fill walks row pairs of a warp-wide matrix");
  const int ntodo = *tile_count;
  for (int kt = blockIdx.x * kWarpsPerBlock + warp; kt < ntodo; kt += gridDim.x * kWarpsPerBlock) {
    const int tile = tile_list[kt];
    const BFJob *jp = jobs_fb + nngp_find_job(jobs_fb, njobs, tile);
    const BFData *dp = datas + jp->data;
    const CovParams *cpp = thetas + jp->theta;
    const int tj = tile - jp->tile0;
    const CorDF ck = nngp_bfr::cor_prepare<COV>(cpp);
    const F::df Sd{cpp->dfDiag[0], cpp->dfDiag[1]};
    nngp_bfr::fill_tab<COV>(tab, ck, cpp, lane);
    __syncwarp();
    const int n = dp->n;
    const int i_end = min(n, (tj + 1) * kTile);
    const float4 *xyf = reinterpret_cast<const float4 *>(dp->xyf);
    double acc0 = 0.0, acc1 = 0.0;
    bool tile_ok = true;
    int nflag = 0;

#pragma unroll 1
    for (int i = tj * kTile; i < i_end; i++) {
      if (!jp->flags[i]) continue;
      nflag++;
      const int off = dp->nnLU[i];
      const int mi = min(dp->nnLU[n + i], M);
      const bool pad = lane >= mi;

      // ---- 1. geometry and covariance (double-float; the FP32R warp kernel's construction)
      const float4 pi4 = xyf[i];
      F::df ox{0.0f, 0.0f}, oy{0.0f, 0.0f};
      int nbk = 0;
      if (!pad) {
        nbk = dp->nnIndx[off + lane];
        const float4 q = xyf[nbk];
        ox = F::diff(q.x, q.z, pi4.x, pi4.z);
        oy = F::diff(q.y, q.w, pi4.y, pi4.w);
      }
      const float omax = fmaxf(1e-30f, __int_as_float((int)__reduce_max_sync(
                                           kFull, (unsigned)__float_as_int(fmaxf(fabsf(ox.h), fabsf(oy.h))))));
      float4 g = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      {
        const int eb = ((__float_as_int(omax) >> 23) & 0xff) - 22;
        const float grid = __int_as_float(max(eb, 1) << 23), inv = __int_as_float((254 - max(eb, 1)) << 23);
        if (!pad) {
          const float hx = __fmul_rn(rintf(__fmul_rn(ox.h, inv)), grid);
          const float hy = __fmul_rn(rintf(__fmul_rn(oy.h, inv)), grid);
          g = make_float4(hx, hy, __fadd_rn(__fsub_rn(ox.h, hx), ox.l), __fadd_rn(__fsub_rn(oy.h, hy), oy.l));
        }
      }
      geo[lane] = g;
      F::df cv{0.0f, 0.0f};
      if (!pad) {
        const F::df gx = F::norm(g.x, g.z), gy = F::norm(g.y, g.w);
        cv = nngp_bfr::cov_df<COV>(F::sumsq(gx.h, gx.l, gy.h, gy.l), ck, tab, cpp);
      }
      __syncwarp();
      constexpr int NIT = M / 2;
#pragma unroll 1
      for (int t = 0; t < NIT; t++) {
        // rows t and M - 1 - t fill lanes 0 .. M - 2: lane c < t takes (t, c), lane c >= t (M - 1 - t, c - t)
        const int r = lane < t ? t : M - 1 - t;
        const int c = lane < t ? lane : min(lane - t, M - 1);
        const float4 gr = geo[r], gc = geo[c];
        F::df ex, ey;
        F::fast_two_sum(__fsub_rn(gr.x, gc.x), __fsub_rn(gr.z, gc.z), ex.h, ex.l);
        F::fast_two_sum(__fsub_rn(gr.y, gc.y), __fsub_rn(gr.w, gc.w), ey.h, ey.l);
        const F::df v = nngp_bfr::cov_df<COV>(F::sumsq(ex.h, ex.l, ey.h, ey.l), ck, tab, cpp);
        if (lane < M - 1) {
          const bool live = r < mi;  // rows past m_i are the identity's
          const float vh = live ? v.h : 0.0f, vl = live ? v.l : 0.0f;
          const int a = LD * r + c, at = LD * c + r;
          chs[a] = vh;
          chs[at] = vh;
          cls[a] = vl;
          cls[at] = vl;
        }
      }
      chs[rb + lane] = pad ? 1.0f : Sd.h;  // the diagonal (identity past m_i)
      cls[rb + lane] = pad ? 0.0f : Sd.l;
      __syncwarp();

      // ---- 2. right-looking Cholesky in double-float: lane r holds row r
      float rh[M], rl[M];  // row r of C, then of L (hi and lo parts)
#pragma unroll
      for (int c = 0; c < M; c++) {
        rh[c] = chs[rb + c];
        rl[c] = cls[rb + c];
      }
      bool ok = true;
      float pmin = 3.4e38f, pmax = 0.0f;
      F::df ivmine{1.0f, 0.0f};
      chol_step<M, 0>(rh, rl, lane, ok, pmin, pmax, ivmine);
      // z = L^-1 c: lane k's numerator times its 1 / L_kk, broadcast at step k (L's diagonal and
      // upper part are zero in the row, so every step is a plain update)
      F::df t = cv;
#pragma unroll
      for (int k = 0; k < M; k++) t = F::sub(t, F::mul(F::df{rh[k], rl[k]}, shfl_df(F::mul(t, ivmine), k)));
      const F::df zmine = F::mul(t, ivmine);
      const F::df Fd = F::sub(Sd, warp_sum_df(F::mul(zmine, zmine)));
      // L to shared memory (zero on and above the diagonal) for the column reads of L' B = z
#pragma unroll
      for (int c = 0; c < M; c++) {
        chs[rb + c] = rh[c];
        cls[rb + c] = rl[c];
      }
      __syncwarp();
      t = zmine;
#pragma unroll 4
      for (int k = M - 1; k >= 0; k--)
        t = F::sub(t, F::mul(F::df{chs[LD * k + lane], cls[LD * k + lane]}, shfl_df(F::mul(t, ivmine), k)));
      const F::df bmine = F::mul(t, ivmine);
      const float ratio = pmax / pmin;
      if (!__all_sync(kFull, ok && Fd.h > nngp_bfr::kMinFRel * Sd.h && ratio * ratio <= kMaxPivotRatio2)) {
        tile_ok = false;
        break;  // the tile goes to the FP64 kernel
      }

      // ---- 3. FP64 epilogue
      const double Fi = F::to_double(Fd);
      const double bd = pad ? 0.0 : F::to_double(bmine);
      const double logF = log(Fi);
      if constexpr (MODE == 0) {
        if (!pad) dp->B[off + lane] = bd;
        if (lane == 0) {
          dp->F[i] = Fi;
          acc0 += logF;
        }
      } else {
        double rv[NNGP_MAX_NV];
#pragma unroll
        for (int v = 0; v < NNGP_MAX_NV; v++) {
          rv[v] = 0.0;
          if (v < nv) {
            const double s = warp_sum_d(pad ? 0.0 : bd * dp->V[(size_t)nbk * nv + v]);
            rv[v] = dp->V[(size_t)i * nv + v] - s;
          }
        }
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
              const int c = a + rem;
              double ra = 0.0, rc = 0.0;
#pragma unroll
              for (int v = 0; v < NNGP_MAX_NV; v++) {
                if (v == a) ra = rv[v];
                if (v == c) rc = rv[v];
              }
              val = ra * rc * invF;
            }
            if (s == 0) acc0 += val;
            else acc1 += val;
          }
        }
      }
      __syncwarp();  // the warp's buffers are rewritten by the next location
    }
    if (!tile_ok) {
      if (lane == 0) {
        int cnt = 0;
        for (int i = tj * kTile; i < i_end; i++) cnt += jp->flags[i] != 0;
        list64[atomicAdd(count64, 1)] = tile;
        atomicAdd(locs64, (unsigned long long)cnt);
      }
      __syncwarp();
      continue;
    }
    (void)nflag;
    double *partial = jp->partial + (size_t)tj * ng;
    if (lane < ng) partial[lane] = acc0;
    if (lane + 32 < ng) partial[lane + 32] = acc1;
  }
}

// Walks the plan's flagged-tile list with four-warp blocks, a warp per tile, as many blocks as the
// SMs hold at once (at most one per tile); tiles it cannot certify go to the plan's FP64 list.
template <int M, int MODE, int COV>
int launch_wdf(nngp_ctx *ctx, const BFPlan *pl) {
  static bool configured[64] = {};  // the attribute is per device
  static int occ[64] = {};
  const int dev = ctx->device & 63;
  if (!configured[dev]) {
    NNGP_CUDA_TRY(ctx, cudaFuncSetAttribute(bfwdf_kernel<M, MODE, COV>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)kSmemBytes));
    int b = 0;
    NNGP_CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, bfwdf_kernel<M, MODE, COV>,
                                                                     32 * kWarpsPerBlock, kSmemBytes));
    occ[dev] = b > 0 ? b : 1;
    configured[dev] = true;
  }
  if (pl->tiles_fb <= 0) return NNGP_OK;
  const int cap = occ[dev] * (ctx->sm_count > 0 ? ctx->sm_count : 1);
  const int need = (pl->tiles_fb + kWarpsPerBlock - 1) / kWarpsPerBlock;
  const int grid = need < cap ? need : cap;
  bfwdf_kernel<M, MODE, COV><<<grid, 32 * kWarpsPerBlock, kSmemBytes, ctx->stream>>>(
      pl->d_datas, pl->d_thetas, pl->d_jobs_fb, pl->njobs, pl->nv, pl->d_fb_list, (const int *)pl->d_fb_words,
      pl->d_fb64_list, pl->d_fb64_count, pl->d_fb64_locs);
  NNGP_LAUNCH_CHECK(ctx);
  return NNGP_OK;
}

}  // namespace nngp_bfwdf
