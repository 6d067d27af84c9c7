// FP32R B/F kernel for neighbor bounds 16 < m <= 32 (M = 20, 24, 32): one warp per location
// (reference updateBF, src/rNNGP.cpp:46-101; updateConjBF, src/cNNGP.cpp:24-69; the
// likelihood sums of src/rNNGP.cpp:306-317 and Q, src/util.cpp:261-280).
//
// A 32-neighbor factor (528 entries) does not fit one thread's registers, so lane r of a warp
// owns row r of the neighborhood system.  A warp walks a tile of 32 consecutive locations of
// one job (job = one dataset at one parameter set), one location at a time:
//   1. geometry: lane k differences neighbor k from the location (float hi/lo coordinate
//      splits, as normalised double-float pairs); the largest offset of the location fixes a
//      common grid 2^e for the hi parts, so two hi parts subtract exactly; the quantised
//      offsets go to the warp's shared memory, one float4 per neighbor;
//   2. covariance in double-float (the arithmetic of the m <= 16 kernel, nngp_cov_df.cuh):
//      lane k evaluates c_k; the pairs of the strict lower triangle are spread over the lanes
//      by row pairs (rows t and M - 1 - t fill M - 1 lanes) and stored, hi and lo parts, at
//      (r, c) and (c, r) of the warp's padded matrices, so lane r then reads row r at
//      immediate offsets;
//   3. right-looking Cholesky of the hi parts with lane r holding row r in registers: step k
//      broadcasts the pivot and column k by shuffles (a broadcast through shared memory
//      would take fewer instructions, but the compiler then schedules its loads into more
//      than 255 live registers); L then goes to shared memory so that the back
//      substitution can read its columns;
//   4. forward and back substitution in float, one shuffle per step (lane k sends its
//      numerator times its own 1 / L_kk; L's zeroed diagonal and upper part make every step
//      one fma on every lane, with no lane tests);
//   5. one refinement step: lane r forms res_r = c_r - sum_c C[r][c] b_c over the
//      double-float entries (a compensated Dot2 sum), and the correction delta is solved with
//      the float factor; B = b + delta as an unevaluated float pair;
//   6. F = sigma^2 + tau^2 - B'c (a double-float warp sum), the error estimate of the m <= 16
//      kernel -- a location is flagged and left to the FP64 kernel when its float pivot fails,
//      when q^2 (sigma^2 + tau^2) > 1e-8 F (q = |delta|_inf / |b|_inf) or when
//      F < 1e-6 (sigma^2 + tau^2) --, log F, and in the fused pass r = (I - B) V and
//      r_a r_b / F.  Lane t adds value t of each location to its running double-float sum in
//      location order, so a tile's sums have a fixed order whatever the launch shape.
// Rows m_i <= r < 32 are the identity (c_r = 0, B_r = 0), so every step runs on all lanes.
#pragma once
#include <cuda_runtime.h>
#include "nngp_cov_df.cuh"

namespace nngp_bfw {

using nngp_bfr::CorDF;

constexpr unsigned kFull = 0xffffffffu;

// Per-warp shared memory (floats): the geometry (32 float4); the hi and lo parts of C and the
// float factor L as full 32 x 32 matrices with rows padded to 33 floats, (r, c) at 33 r + c,
// so lane r reads row r and lane c reads column c at immediate offsets from its own base
// without bank conflicts (bank (r + c) mod 32); the exp and Matern table (nngp_cov_df.cuh), the
// float solution b and the fused pass's residuals r_v (hi, lo).  Entries outside the M x M block are
// zero (set once per kernel), L's strict upper triangle and diagonal are stored as zero.
template <int M>
struct WShape {
  static constexpr int NL = M * (M - 1) / 2;  // strict lower triangle
  static constexpr int LD = 33;
  static constexpr int MAT = 32 * LD;
  static constexpr int GEO = 0;
  static constexpr int CH = GEO + 4 * 32;
  static constexpr int CL = CH + MAT;
  static constexpr int LT = CL + MAT;
  static constexpr int TAB = LT + MAT;
  static constexpr int BV = TAB + nngp_bfr::kTabFloats;
  static constexpr int RV = BV + 32;
  static constexpr int WARP_FLOATS = (RV + 2 * NNGP_MAX_NV + 3) & ~3;
};


// Sum over the warp of a double-float value (butterfly; the double-float add is commutative,
// so every lane ends with the same sum)
__device__ __forceinline__ nngp_df::df warp_sum_df(nngp_df::df p) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const nngp_df::df q{__shfl_xor_sync(kFull, p.h, o), __shfl_xor_sync(kFull, p.l, o)};
    p = nngp_df::add(p, q);
  }
  return p;
}

// (b + delta)(x + xl) as a double-float (the delta * xl term is below the pair's precision)
__device__ __forceinline__ nngp_df::df prod_df(float b, float delta, float x, float xl) {
  const float ph = __fmul_rn(b, x);
  const float pe = __fmaf_rn(b, x, -ph);
  return nngp_df::norm(ph, __fmaf_rn(delta, x, __fmaf_rn(b, xl, pe)));
}

template <int M, int MODE, int COV>
__global__ void __launch_bounds__(128, 4) bfw_kernel(const BFData *__restrict__ datas,
                                                  const CovParams *__restrict__ thetas,
                                                  const BFJob *__restrict__ jobs, int njobs, int tile_begin,
                                                  int tile_end, int nv) {
  namespace F = nngp_df;
  namespace G = nngp_df2;
  using S = WShape<M>;
  extern __shared__ __align__(16) float smem_w[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  float *ws = smem_w + (size_t)warp * S::WARP_FLOATS;
  float4 *geo = reinterpret_cast<float4 *>(ws + S::GEO);
  float *chs = ws + S::CH, *cls = ws + S::CL, *lts = ws + S::LT, *tab = ws + S::TAB;
  float *bvs = ws + S::BV, *rvs = ws + S::RV;
  const int ng = MODE == 0 ? 1 : 1 + nv * (nv + 1) / 2;
  const int rb = S::LD * lane;  // this lane's row in the padded matrices
  for (int k = lane; k < 3 * S::MAT; k += 32) chs[k] = 0.0f;  // CH, CL, LT are contiguous
  __syncwarp();

  for (int kt = blockIdx.x * wpb + warp; kt < tile_end - tile_begin; kt += gridDim.x * wpb) {
    const int tile = tile_begin + kt;
    // the job's and dataset's fields are read where they are used (pointers rather than copies
    // keep the location loop's live registers down)
    const BFJob *jp = jobs + nngp_find_job(jobs, njobs, tile);
    const BFData *dp = datas + jp->data;
    const CovParams *cpp = thetas + jp->theta;
    const int tj = tile - jp->tile0;
    if constexpr (COV == NNGP_COV_GAU || COV == NNGP_COV_ANY) {
      if (nngp_route_double_float(*cpp)) {  // the job's parameter set: warp-uniform
        // every location to the double-float re-solve, nothing from the float factor here
        if (tj * 32 + lane < dp->n) nngp_flag_for_fp64(*jp, tj * 32 + lane);
        double *partial = jp->partial + (size_t)tj * ng;
        if (lane < ng) partial[lane] = 0.0;
        if (lane + 32 < ng) partial[lane + 32] = 0.0;
        continue;
      }
    }
    const CorDF ck = nngp_bfr::cor_prepare<COV>(cpp);
    const F::df Sd{cpp->dfDiag[0], cpp->dfDiag[1]};  // the diagonal sigma^2 + tau^2
    nngp_bfr::fill_tab<COV>(tab, ck, cpp, lane);  // the warp's exp table and Matern coefficients
    __syncwarp();
    F::df acc0{0.0f, 0.0f}, acc1{0.0f, 0.0f};
    const int n = dp->n;
    const int i_end = min(n, (tj + 1) * 32);
    const float4 *xyf = reinterpret_cast<const float4 *>(dp->xyf);
    const int *nnLU = dp->nnLU;

#pragma unroll 1
    for (int i = tj * 32; i < i_end; i++) {
      const int off = nnLU[i];
      const int mi = min(nnLU[n + i], M);
      const bool pad = lane >= mi;  // identity row

      // ---- 1. geometry
      const float4 pi4 = xyf[i];
      F::df ox{0.0f, 0.0f}, oy{0.0f, 0.0f};
      int nbk = 0;
      if (!pad) {
        nbk = dp->nnIndx[off + lane];
        const float4 q = xyf[nbk];
        ox = F::diff(q.x, q.z, pi4.x, pi4.z);
        oy = F::diff(q.y, q.w, pi4.y, pi4.w);
      }
      // largest |offset| hi part (non-negative floats order as their bit patterns)
      const float omax = fmaxf(1e-30f, __int_as_float((int)__reduce_max_sync(
                                           kFull, (unsigned)__float_as_int(fmaxf(fabsf(ox.h), fabsf(oy.h))))));
      float4 g = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      {
        const int eb = ((__float_as_int(omax) >> 23) & 0xff) - 22;  // biased exponent of 2^e
        const float grid = __int_as_float(max(eb, 1) << 23), inv = __int_as_float((254 - max(eb, 1)) << 23);
        if (!pad) {
          const float hx = __fmul_rn(rintf(__fmul_rn(ox.h, inv)), grid);
          const float hy = __fmul_rn(rintf(__fmul_rn(oy.h, inv)), grid);
          g = make_float4(hx, hy, __fadd_rn(__fsub_rn(ox.h, hx), ox.l), __fadd_rn(__fsub_rn(oy.h, hy), oy.l));
        }
      }
      geo[lane] = g;

      // ---- 2. covariance: c_k on lane k, then the strict lower triangle spread over the lanes
      F::df cv{0.0f, 0.0f};
      if (!pad) {
        const F::df gx = F::norm(g.x, g.z), gy = F::norm(g.y, g.w);
        cv = nngp_bfr::cov_df<COV>(F::sumsq(gx.h, gx.l, gy.h, gy.l), ck, tab, cpp);
      }
      __syncwarp();
      // the strict lower triangle by row pairs: iteration t covers rows t and M - 1 - t, whose
      // t + (M - 1 - t) = M - 1 pairs fill lanes 0 .. M - 2 (lane c < t: (t, c); lane c >= t:
      // (M - 1 - t, c - t)); two iterations per packed evaluation
      constexpr int NIT = M / 2;
#pragma unroll 1
      for (int t = 0; t < NIT; t += 2) {
        int r[2], c[2];
        float4 gr[2], gc[2];
#pragma unroll
        for (int u = 0; u < 2; u++) {
          const int tt = min(t + u, NIT - 1);
          r[u] = lane < tt ? tt : M - 1 - tt;
          c[u] = lane < tt ? lane : min(lane - tt, M - 1);
          gr[u] = geo[r[u]];
          gc[u] = geo[c[u]];
        }
        F::df v[2];
        if constexpr (nngp_bfr::kPacked<COV>) {
          // hi parts on the common grid: their difference is exact
          G::df2 ex, ey;
          G::fast_two_sum(G::sub(G::pack(gr[0].x, gr[1].x), G::pack(gc[0].x, gc[1].x)),
                          G::sub(G::pack(gr[0].z, gr[1].z), G::pack(gc[0].z, gc[1].z)), ex.h, ex.l);
          G::fast_two_sum(G::sub(G::pack(gr[0].y, gr[1].y), G::pack(gc[0].y, gc[1].y)),
                          G::sub(G::pack(gr[0].w, gr[1].w), G::pack(gc[0].w, gc[1].w)), ey.h, ey.l);
          const G::df2 rr = nngp_bfr::cov_df2<COV>(G::sumsq(ex, ey), ck, tab);
          v[0] = F::df{G::first(rr.h), G::first(rr.l)};
          v[1] = F::df{G::second(rr.h), G::second(rr.l)};
        } else {
#pragma unroll
          for (int u = 0; u < 2; u++) {
            F::df ex, ey;
            F::fast_two_sum(__fsub_rn(gr[u].x, gc[u].x), __fsub_rn(gr[u].z, gc[u].z), ex.h, ex.l);
            F::fast_two_sum(__fsub_rn(gr[u].y, gc[u].y), __fsub_rn(gr[u].w, gc[u].w), ey.h, ey.l);
            v[u] = nngp_bfr::cov_df<COV>(F::sumsq(ex.h, ex.l, ey.h, ey.l), ck, tab, cpp);
          }
        }
#pragma unroll
        for (int u = 0; u < 2; u++) {
          if (t + u < NIT && lane < M - 1) {
            const bool live = r[u] < mi;  // rows past m_i are the identity's
            const float vh = live ? v[u].h : 0.0f, vl = live ? v[u].l : 0.0f;
            const int a = S::LD * r[u] + c[u], at = S::LD * c[u] + r[u];
            chs[a] = vh;
            chs[at] = vh;
            cls[a] = vl;
            cls[at] = vl;
          }
        }
      }
      chs[rb + lane] = pad ? 1.0f : Sd.h;  // the diagonal (identity past m_i)
      cls[rb + lane] = pad ? 0.0f : Sd.l;
      __syncwarp();

      // ---- 3. Cholesky of the hi parts: lane r holds row r (entries c <= r are meaningful)
      float row[M];
#pragma unroll
      for (int c = 0; c < M; c++) row[c] = chs[rb + c];
      bool ok = true;
      float ivmine = 1.0f;  // 1 / L_rr on lane r
#pragma unroll
      for (int k = 0; k < M; k++) {
        const float dk = __shfl_sync(kFull, row[k], k);
        ok = ok && (dk > 0.0f);
        const float ik = rsqrtf(dk);
        if (lane == k) ivmine = ik;
        const float lk = __fmul_rn(row[k], ik);  // L[r][k] on lane r > k
        row[k] = lk;
        if (k + 1 < M) {
#pragma unroll
          for (int j = k + 1; j < M; j++) row[j] = fmaf(-lk, __shfl_sync(kFull, lk, j), row[j]);
        }
      }
      // the strictly lower part of row r is L's; the diagonal and the upper part (scratch) are
      // zeroed, so the substitutions below need no per-step lane tests; the row goes to shared
      // memory for the column reads of the back substitution
#pragma unroll
      for (int c = 0; c < M; c++) {
        row[c] = c < lane ? row[c] : 0.0f;
        lts[rb + c] = row[c];
      }
      __syncwarp();

      // ---- 4. L z = c, L' b = z: lane r holds component r.  Step k broadcasts lane k's
      // numerator times its 1 / L_kk; lane r's numerator is final once step r - 1 is done (the
      // later steps subtract zero from it), so the solution is numerator x 1 / L_rr at the end.
      float t = cv.h;
#pragma unroll
      for (int k = 0; k < M; k++) t = fmaf(-row[k], __shfl_sync(kFull, __fmul_rn(t, ivmine), k), t);
      t = __fmul_rn(t, ivmine);
#pragma unroll 8
      for (int k = M - 1; k >= 0; k--)
        t = fmaf(-lts[S::LD * k + lane], __shfl_sync(kFull, __fmul_rn(t, ivmine), k), t);
      const float bmine = __fmul_rn(t, ivmine);
      bvs[lane] = bmine;
      const float bmax = __int_as_float((int)__reduce_max_sync(kFull, (unsigned)__float_as_int(fabsf(bmine))));
      __syncwarp();

      // ---- 5. refinement: res_r = c_r - sum_c C[r][c] b_c (Dot2 over the double-float entries)
      float sh = 0.0f, sl = 0.0f;
#pragma unroll 8
      for (int c = 0; c < M; c++) {
        const float bc = bvs[c];
        F::dot2_acc(sh, sl, chs[rb + c], bc);
        sl = fmaf(cls[rb + c], bc, sl);
      }
      t = __fadd_rn(__fsub_rn(__fsub_rn(cv.h, sh), sl), cv.l);
#pragma unroll
      for (int k = 0; k < M; k++) t = fmaf(-row[k], __shfl_sync(kFull, __fmul_rn(t, ivmine), k), t);
      t = __fmul_rn(t, ivmine);
#pragma unroll 8
      for (int k = M - 1; k >= 0; k--)
        t = fmaf(-lts[S::LD * k + lane], __shfl_sync(kFull, __fmul_rn(t, ivmine), k), t);
      const float dmine = __fmul_rn(t, ivmine);
      const float dmax = __int_as_float((int)__reduce_max_sync(kFull, (unsigned)__float_as_int(fabsf(dmine))));

      // ---- 6. F, error estimate, log F, likelihood terms
      const F::df bc = warp_sum_df(prod_df(bmine, dmine, cv.h, cv.l));
      const F::df Fd = F::sub(Sd, bc);
      const float q = dmax / fmaxf(bmax, 1e-30f);
      const bool bad = !ok || !(Fd.h > nngp_bfr::kMinFRel * Sd.h) || !(q * q * Sd.h <= nngp_bfr::kTolF * Fd.h);
      if (bad && lane == 0) nngp_flag_for_fp64(*jp, i);
      const F::df lf = bad ? F::df{0.0f, 0.0f} : F::log(Fd);
      if constexpr (MODE == 0) {
        if (!bad) {
          if (!pad) dp->B[off + lane] = (double)bmine + (double)dmine;
          if (lane == 0) dp->F[i] = F::to_double(Fd);
        }
        if (lane == 0) acc0 = F::add(acc0, lf);
      } else {
        // r_v = V_iv - sum_k B_k V_nb(k)v, four columns per round of gathers
        const float2 *Vf = dp->Vf;
#pragma unroll 1
        for (int v0 = 0; v0 < nv; v0 += 4) {
          float2 qv[4], vi[4];
#pragma unroll
          for (int j = 0; j < 4; j++) {
            const bool col = v0 + j < nv;
            qv[j] = (!pad && col) ? Vf[(size_t)nbk * nv + v0 + j] : make_float2(0.0f, 0.0f);
            vi[j] = col ? Vf[(size_t)i * nv + v0 + j] : make_float2(0.0f, 0.0f);
          }
#pragma unroll
          for (int j = 0; j < 4; j++) {
            if (v0 + j < nv) {
              const F::df s = warp_sum_df(prod_df(bmine, dmine, qv[j].x, qv[j].y));
              const F::df rv = F::sub(F::df{vi[j].x, vi[j].y}, s);
              if (lane == 0) {
                rvs[2 * (v0 + j)] = rv.h;
                rvs[2 * (v0 + j) + 1] = rv.l;
              }
            }
          }
        }
        __syncwarp();
        const F::df invF = bad ? F::df{0.0f, 0.0f} : F::recip(Fd);
        // lane t: value t of the location (0: log F; then r_a r_b / F over a <= b, row-major)
#pragma unroll
        for (int s = 0; s < 2; s++) {
          const int tt = lane + 32 * s;
          if (tt < ng) {
            F::df val = lf;
            if (tt > 0) {
              int rem = tt - 1, a = 0;
              while (rem >= nv - a) {
                rem -= nv - a;
                a++;
              }
              const int c = a + rem;
              const F::df ta = F::mul(F::df{rvs[2 * a], rvs[2 * a + 1]}, invF);
              val = bad ? F::df{0.0f, 0.0f} : F::mul(ta, F::df{rvs[2 * c], rvs[2 * c + 1]});
            }
            if (s == 0) acc0 = F::add(acc0, val);
            else acc1 = F::add(acc1, val);
          }
        }
      }
      __syncwarp();  // the warp's buffers are rewritten by the next location
    }
    double *partial = jp->partial + (size_t)tj * ng;
    if (lane < ng) partial[lane] = F::to_double(acc0);
    if (lane + 32 < ng) partial[lane + 32] = F::to_double(acc1);
  }
}

constexpr int kWarpsPerBlock = 4;  // the largest block (the kernel's launch bounds)

template <int M>
constexpr size_t warp_smem(int wpb) {
  return sizeof(float) * WShape<M>::WARP_FLOATS * (size_t)wpb;
}

// Raises the kernel's dynamic shared-memory limit to the largest block's (once per device).
template <int M, int MODE, int COV>
cudaError_t configure_warp(int device) {
  static bool configured[64] = {};  // the attribute is per device
  const int dev = device & 63;
  if (configured[dev]) return cudaSuccess;
  const cudaError_t e = cudaFuncSetAttribute(bfw_kernel<M, MODE, COV>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)warp_smem<M>(kWarpsPerBlock));
  if (e == cudaSuccess) configured[dev] = true;
  return e;
}

// Launches the kernel on the plan's primary tiles [t0, t1) (tile = 32 locations of one job):
// blocks of wpb (1 - 4) warps (54.5 KB of shared memory per four warps at M = 32), `grid`
// blocks (0: one tile per warp; fewer: each warp loops over tiles).  Each warp reduces its own
// tiles, so the shape never changes a result.
template <int M, int MODE, int COV>
int launch_warp(nngp_ctx *ctx, const BFPlan *pl, int t0, int t1, int wpb, int grid) {
  NNGP_CUDA_TRY(ctx, (configure_warp<M, MODE, COV>(ctx->device)));
  if (t1 <= t0) return NNGP_OK;
  if (wpb < 1 || wpb > kWarpsPerBlock) wpb = kWarpsPerBlock;
  const int full = (t1 - t0 + wpb - 1) / wpb;
  if (grid <= 0 || grid > full) grid = full;
  bfw_kernel<M, MODE, COV><<<grid, 32 * wpb, warp_smem<M>(wpb), ctx->stream>>>(pl->d_datas, pl->d_thetas,
                                                                            pl->d_jobs, pl->njobs, t0, t1, pl->nv);
  NNGP_LAUNCH_CHECK(ctx);
  return NNGP_OK;
}

// Blocks of wpb warps one SM holds at once (current device).
template <int M, int MODE, int COV>
int occupancy_warp(int wpb) {
  int dev = 0, blocks = 0;
  cudaGetDevice(&dev);
  if (wpb < 1 || wpb > kWarpsPerBlock || configure_warp<M, MODE, COV>(dev) != cudaSuccess) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, bfw_kernel<M, MODE, COV>, 32 * wpb,
                                                    warp_smem<M>(wpb)) != cudaSuccess)
    return 0;
  return blocks;
}

}  // namespace nngp_bfw
