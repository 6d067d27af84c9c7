// Double-float re-solve of the locations the FP32R register kernel (m <= 16,
// nngp_bfr_kernel.cuh) flags -- a float pivot failed or the float solve's error estimate was
// too large, typically a gaussian covariance with a small nugget (condition numbers ~1e7).
// Instead of handing them all to the FP64 kernel, whose pipe runs at 1/64 of the FP32 rate on
// GB300, this kernel solves them in double-float arithmetic (about 48-bit significands) on
// the FP32 pipe (reference updateBF, src/rNNGP.cpp:46-101, and the likelihood sums of
// src/rNNGP.cpp:306-317; the double-float arithmetic of nngp_df.cuh, the covariance of
// nngp_cov_df.cuh):
//   1. neighbor offsets from the split coordinates as double-float pairs on a common grid
//      (as the register kernel), the covariance c and the lower triangle of C in double-float;
//   2. the row-oriented (Banachiewicz) Cholesky factor L in double-float with the forward
//      solve z = L^-1 c fused in, then F = sigma^2 + tau^2 - z'z (the squared norm of the
//      forward solve, accurate where F is a small difference) and B = L^-T z;
//   3. log F and, in the fused pass, r = (I - B) V and r_a r_b / F in FP64 (a few dozen FP64
//      operations per location), summed over the tile in a fixed order.
// Every dot product runs as two independent sums (even and odd terms) and the covariance
// entries are evaluated two at a time, so consecutive double-float operations seldom wait on
// each other: the kernel holds only about four warps per SM (its triangles fill the shared
// memory), and latency, not arithmetic, bounds it.
// The kernel walks the FP32R pass's list of flagged FP64 tiles (64 locations each, the FP64
// kernel's tile) and solves every flagged location of a tile.  A location it cannot certify --
// a non-positive double-float pivot, F < 1e-6 (sigma^2 + tau^2), or a squared pivot ratio (a
// lower bound of the condition number) above 1e10 -- sends its whole tile on to the FP64
// kernel (a second list), so every tile's partial sums come from one kernel and keep their
// fixed order.  Each thread keeps its triangle in shared memory, element e of thread t at
// e * TPB + t (hi and lo parts in separate arrays), so every access is bank-conflict free.
#pragma once
#include <cuda_runtime.h>
#include "nngp_cov_df.cuh"

namespace nngp_bfdf {

constexpr int M = 16;    // the register kernel's largest neighbor bound
constexpr int TPB = 64;  // the FP64 tile of m <= 16 (the unit of the flagged-tile list)
constexpr int NT = M * (M + 1) / 2;
constexpr int kNGMax = 1 + NNGP_MAX_NV * (NNGP_MAX_NV + 1) / 2;
// floats per thread: L hi and lo (NT each), z / c hi and lo (M each), geometry (4 M)
constexpr int kThreadFloats = 2 * NT + 2 * M + 4 * M;
constexpr size_t kSmemBytes = sizeof(float) * ((size_t)kThreadFloats * TPB + (TPB / 32) * nngp_bfr::kTabFloats) +
                              sizeof(double) * (TPB / 32) * kNGMax;
constexpr float kMaxPivotRatio2 = 1e10f;  // squared pivot ratio above which FP64 takes over

__host__ __device__ constexpr int tri(int r, int c) { return r * (r + 1) / 2 + c; }  // c <= r

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <int MODE, int COV>
__global__ void __launch_bounds__(TPB) bfdf_kernel(const BFData *__restrict__ datas,
                                                 const CovParams *__restrict__ thetas,
                                                 const BFJob *__restrict__ jobs_fb, int njobs, int nv,
                                                 const int *__restrict__ tile_list, const int *__restrict__ tile_count,
                                                 int *__restrict__ list64, int *__restrict__ count64,
                                                 unsigned long long *__restrict__ locs64) {
  namespace F = nngp_df;
  extern __shared__ __align__(16) float smem_d[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  float *Lh = smem_d, *Ll = Lh + NT * TPB;
  float *zh = Ll + NT * TPB, *zl = zh + M * TPB;
  float4 *geo = reinterpret_cast<float4 *>(zl + M * TPB);
  float *tab = smem_d + (size_t)kThreadFloats * TPB + warp * nngp_bfr::kTabFloats;
  double *wbuf = reinterpret_cast<double *>(smem_d + (size_t)kThreadFloats * TPB + (TPB / 32) * nngp_bfr::kTabFloats);
#define LH(r, c) Lh[tri(r, c) * TPB + tid]
#define LL(r, c) Ll[tri(r, c) * TPB + tid]
#define ZH(k) zh[(k) * TPB + tid]
#define ZL(k) zl[(k) * TPB + tid]
#define GEO(k) geo[(k) * TPB + tid]

  const int ntodo = *tile_count;
  for (int kt = blockIdx.x; kt < ntodo; kt += gridDim.x) {
    const int tile = tile_list[kt];
    const BFJob job = jobs_fb[nngp_find_job(jobs_fb, njobs, tile)];
    const BFData d = datas[job.data];
    const CovParams *cpp = thetas + job.theta;
    const int tj = tile - job.tile0;
    const int i = tj * TPB + tid;
    const bool active = i < d.n && job.flags[i] != 0;
    const nngp_bfr::CorDF ck = nngp_bfr::cor_prepare<COV>(cpp);
    const F::df Sd{cpp->dfDiag[0], cpp->dfDiag[1]};
    nngp_bfr::fill_tab<COV>(tab, ck, cpp, lane);
    __syncwarp();
    int mi = 0, off = 0;
    if (active) {
      off = d.nnLU[i];
      mi = min(d.nnLU[d.n + i], M);
    }
    bool ok = true;
    F::df Fd{1.0f, 0.0f};
    if (active) {
      // ---- 1. geometry and covariance (double-float)
      const float4 *xyf = reinterpret_cast<const float4 *>(d.xyf);
      const float4 pi4 = xyf[i];
      float omax = 1e-30f;
      for (int k = 0; k < mi; k++) {
        const float4 q = xyf[d.nnIndx[off + k]];
        const F::df ox = F::diff(q.x, q.z, pi4.x, pi4.z), oy = F::diff(q.y, q.w, pi4.y, pi4.w);
        GEO(k) = make_float4(ox.h, oy.h, ox.l, oy.l);
        omax = fmaxf(omax, fmaxf(fabsf(ox.h), fabsf(oy.h)));
      }
      // hi parts on a common grid 2^e >= 2^-22 max |offset|: two hi parts subtract exactly
      const int eb = ((__float_as_int(omax) >> 23) & 0xff) - 22;
      const float grid = __int_as_float(max(eb, 1) << 23), inv = __int_as_float((254 - max(eb, 1)) << 23);
      for (int k = 0; k < mi; k++) {
        const float4 g = GEO(k);
        const float hx = __fmul_rn(rintf(__fmul_rn(g.x, inv)), grid);
        const float hy = __fmul_rn(rintf(__fmul_rn(g.y, inv)), grid);
        const float4 q = make_float4(hx, hy, __fadd_rn(__fsub_rn(g.x, hx), g.z), __fadd_rn(__fsub_rn(g.y, hy), g.w));
        GEO(k) = q;
        const F::df gx = F::norm(q.x, q.z), gy = F::norm(q.y, q.w);
        const F::df c = nngp_bfr::cov_df<COV>(F::sumsq(gx.h, gx.l, gy.h, gy.l), ck, tab, cpp);
        ZH(k) = c.h;
        ZL(k) = c.l;
      }
      // the strict lower triangle two entries at a time (independent evaluations interleave)
      for (int r = 0; r < mi; r++) {
        const float4 gr = GEO(r);
        for (int c = 0; c < r; c += 2) {
          const int c1 = c + 1 < r ? c + 1 : c;
          const float4 ga = GEO(c), gb = GEO(c1);
          F::df ax, ay, bx, by;
          F::fast_two_sum(__fsub_rn(gr.x, ga.x), __fsub_rn(gr.z, ga.z), ax.h, ax.l);
          F::fast_two_sum(__fsub_rn(gr.y, ga.y), __fsub_rn(gr.w, ga.w), ay.h, ay.l);
          F::fast_two_sum(__fsub_rn(gr.x, gb.x), __fsub_rn(gr.z, gb.z), bx.h, bx.l);
          F::fast_two_sum(__fsub_rn(gr.y, gb.y), __fsub_rn(gr.w, gb.w), by.h, by.l);
          const F::df va = nngp_bfr::cov_df<COV>(F::sumsq(ax.h, ax.l, ay.h, ay.l), ck, tab, cpp);
          const F::df vb = nngp_bfr::cov_df<COV>(F::sumsq(bx.h, bx.l, by.h, by.l), ck, tab, cpp);
          LH(r, c) = va.h;
          LL(r, c) = va.l;
          LH(r, c1) = vb.h;  // c1 == c on an odd row end: the same value again
          LL(r, c1) = vb.l;
        }
        LH(r, r) = Sd.h;
        LL(r, r) = Sd.l;
      }
      // ---- 2. Cholesky (row by row) with z = L^-1 c; the diagonal slots end holding 1 / L_rr
      float pmin = 3.4e38f, pmax = 0.0f;
      F::df zz{0.0f, 0.0f};
      for (int r = 0; r < mi && ok; r++) {
        for (int c = 0; c < r; c++) {
          F::df s0{0.0f, 0.0f}, s1{0.0f, 0.0f};
          int k = 0;
          for (; k + 1 < c; k += 2) {
            s0 = F::add(s0, F::mul(F::df{LH(r, k), LL(r, k)}, F::df{LH(c, k), LL(c, k)}));
            s1 = F::add(s1, F::mul(F::df{LH(r, k + 1), LL(r, k + 1)}, F::df{LH(c, k + 1), LL(c, k + 1)}));
          }
          if (k < c) s0 = F::add(s0, F::mul(F::df{LH(r, k), LL(r, k)}, F::df{LH(c, k), LL(c, k)}));
          const F::df s = F::sub(F::df{LH(r, c), LL(r, c)}, F::add(s0, s1));
          const F::df l = F::mul(s, F::df{LH(c, c), LL(c, c)});  // times 1 / L_cc
          LH(r, c) = l.h;
          LL(r, c) = l.l;
        }
        F::df d0{0.0f, 0.0f}, d1{0.0f, 0.0f}, z0{0.0f, 0.0f}, z1{0.0f, 0.0f};
        int k = 0;
        for (; k + 1 < r; k += 2) {
          const F::df la{LH(r, k), LL(r, k)}, lb{LH(r, k + 1), LL(r, k + 1)};
          d0 = F::add(d0, F::mul(la, la));
          d1 = F::add(d1, F::mul(lb, lb));
          z0 = F::add(z0, F::mul(la, F::df{ZH(k), ZL(k)}));
          z1 = F::add(z1, F::mul(lb, F::df{ZH(k + 1), ZL(k + 1)}));
        }
        if (k < r) {
          const F::df la{LH(r, k), LL(r, k)};
          d0 = F::add(d0, F::mul(la, la));
          z0 = F::add(z0, F::mul(la, F::df{ZH(k), ZL(k)}));
        }
        const F::df dg = F::sub(F::df{LH(r, r), LL(r, r)}, F::add(d0, d1));
        F::df zr = F::sub(F::df{ZH(r), ZL(r)}, F::add(z0, z1));
        ok = dg.h > 0.0f;
        if (!ok) break;
        const F::df lrr = F::sqrt(dg);
        pmin = fminf(pmin, lrr.h);
        pmax = fmaxf(pmax, lrr.h);
        const F::df ir = F::recip(lrr);
        LH(r, r) = ir.h;
        LL(r, r) = ir.l;
        zr = F::mul(zr, ir);
        ZH(r) = zr.h;
        ZL(r) = zr.l;
        zz = F::add(zz, F::mul(zr, zr));
      }
      if (ok) {
        Fd = F::sub(Sd, zz);
        const float ratio = pmax / pmin;
        ok = Fd.h > nngp_bfr::kMinFRel * Sd.h && ratio * ratio <= kMaxPivotRatio2;
      }
      if (ok) {
        // ---- B = L^-T z (in place of z)
        for (int k = mi - 1; k >= 0; k--) {
          F::df b0{0.0f, 0.0f}, b1{0.0f, 0.0f};
          int r = k + 1;
          for (; r + 1 < mi; r += 2) {
            b0 = F::add(b0, F::mul(F::df{LH(r, k), LL(r, k)}, F::df{ZH(r), ZL(r)}));
            b1 = F::add(b1, F::mul(F::df{LH(r + 1, k), LL(r + 1, k)}, F::df{ZH(r + 1), ZL(r + 1)}));
          }
          if (r < mi) b0 = F::add(b0, F::mul(F::df{LH(r, k), LL(r, k)}, F::df{ZH(r), ZL(r)}));
          const F::df b = F::mul(F::sub(F::df{ZH(k), ZL(k)}, F::add(b0, b1)), F::df{LH(k, k), LL(k, k)});
          ZH(k) = b.h;
          ZL(k) = b.l;
        }
      }
    }
    // a tile with a location this kernel cannot certify goes to the FP64 kernel whole
    const int nfail = __syncthreads_count(active && !ok);
    if (nfail) {
      const int nflag = __syncthreads_count(active);
      if (tid == 0) {
        list64[atomicAdd(count64, 1)] = tile;
        atomicAdd(locs64, (unsigned long long)nflag);
      }
      continue;
    }
    // ---- 3. log F and the likelihood terms in FP64, tile sums in a fixed order
    const double Fi = F::to_double(Fd);
    double logF = 0.0;
    double rv[NNGP_MAX_NV] = {};
    if (active) {
      logF = log(Fi);
      if (MODE == 0) {
        for (int k = 0; k < mi; k++) d.B[off + k] = (double)ZH(k) + (double)ZL(k);
        d.F[i] = Fi;
      } else {
        for (int v = 0; v < nv; v++) rv[v] = d.V[(size_t)i * nv + v];
        for (int k = 0; k < mi; k++) {
          const double bk = (double)ZH(k) + (double)ZL(k);
          const double *vrow = d.V + (size_t)d.nnIndx[off + k] * nv;
          for (int v = 0; v < nv; v++) rv[v] = fma(-bk, vrow[v], rv[v]);
        }
      }
    }
    const double invF = active ? 1.0 / Fi : 0.0;
    const int ng = MODE == 0 ? 1 : 1 + nv * (nv + 1) / 2;
    for (int k = 0; k < ng; k++) {
      double val = logF;
      if (k > 0) {
        int t = k - 1, a = 0;
        while (t >= nv - a) {
          t -= nv - a;
          a++;
        }
        double ra = 0.0, rb = 0.0;
#pragma unroll
        for (int v = 0; v < NNGP_MAX_NV; v++) {
          if (v == a) ra = rv[v];
          if (v == a + t) rb = rv[v];
        }
        val = ra * rb * invF;
      }
      val = warp_sum_d(val);
      if (lane == 0) wbuf[warp * kNGMax + k] = val;
    }
    __syncthreads();
    for (int k = tid; k < ng; k += TPB) {
      double acc = 0.0;
#pragma unroll
      for (int w = 0; w < TPB / 32; w++) acc += wbuf[w * kNGMax + k];
      job.partial[(size_t)tj * ng + k] = acc;
    }
    __syncthreads();
  }
#undef LH
#undef LL
#undef ZH
#undef ZL
#undef GEO
}

// Walks the plan's flagged-tile list with about two blocks per SM; tiles it cannot certify are
// appended to the plan's FP64 list.
template <int MODE, int COV>
int launch_df(nngp_ctx *ctx, const BFPlan *pl) {
  static bool configured[64] = {};  // the attribute is per device
  const int dev = ctx->device & 63;
  if (!configured[dev]) {
    NNGP_CUDA_TRY(ctx, cudaFuncSetAttribute(bfdf_kernel<MODE, COV>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)kSmemBytes));
    configured[dev] = true;
  }
  if (pl->tiles_fb <= 0) return NNGP_OK;
  const int cap = 2 * (ctx->sm_count > 0 ? ctx->sm_count : 1);
  const int grid = pl->tiles_fb < cap ? pl->tiles_fb : cap;
  bfdf_kernel<MODE, COV><<<grid, TPB, kSmemBytes, ctx->stream>>>(
      pl->d_datas, pl->d_thetas, pl->d_jobs_fb, pl->njobs, pl->nv, pl->d_fb_list, (const int *)pl->d_fb_words,
      pl->d_fb64_list, pl->d_fb64_count, pl->d_fb64_locs);
  NNGP_LAUNCH_CHECK(ctx);
  return NNGP_OK;
}

}  // namespace nngp_bfdf
