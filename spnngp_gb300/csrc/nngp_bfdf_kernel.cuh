// Double-float re-solve of the locations the FP32R kernels flag for m <= 24 (the register
// kernel, nngp_bfr_kernel.cuh, and the warp kernel's 20- and 24-row forms,
// nngp_bfw_kernel.cuh) -- a float pivot failed or the float solve's error estimate was too
// large, typically a gaussian covariance with a small nugget (condition numbers ~1e7).
// Instead of handing them all to the FP64 kernel, whose pipe runs at 1/64 of the FP32 rate on
// GB300, this kernel solves them in double-float arithmetic (about 48-bit significands) on
// the FP32 pipe (reference updateBF, src/rNNGP.cpp:46-101, and the likelihood sums of
// src/rNNGP.cpp:306-317; the double-float arithmetic of nngp_df.cuh, the covariance of
// nngp_cov_df.cuh):
//   1. neighbor offsets from the split coordinates as double-float pairs on a common grid
//      (as the FP32R kernels), the covariance c and the lower triangle of C in double-float;
//   2. the Cholesky factor of the augmented matrix [C c; c' S] (S = sigma^2 + tau^2) in
//      double-float, right-looking (outer-product form): its last row is z = L^-1 c and its
//      last pivot is F = S - z'z, the quantity NNGP needs (accurate where F is a small
//      difference); then B = L^-T z by the same outer-product form run backwards;
//   3. log F and, in the fused pass, r = (I - B) V and r_a r_b / F in FP64 (a few dozen FP64
//      operations per location), summed over the tile in a fixed order.
// The right-looking form leaves every update of a step independent of the others.  With its
// triangles filling the shared memory the kernel holds only four warps per SM, so the
// independence has to show within a thread: every loop issues a batch of loads (four updates,
// four rows, two covariance pairs), then the arithmetic, then the stores -- a store to shared
// memory holds back the next iteration's loads otherwise, since the compiler cannot tell the
// indices apart.  Rows are stored as float pairs (k, k + 1), each row of the lower triangle
// with its diagonal padded to an even length, so one 64-bit shared load brings two entries and
// one packed f32x2 instruction updates both (a - l b with the hi product carried exactly by
// an fma, the cross terms rounded below 2^-23 of the product); the covariance entries are
// evaluated two at a time.  (A row-by-row factorization with compensated dot products issued
// about one instruction at a time; fully unrolling the factorization per neighbor bound cut
// the instruction count by 40 % but overflowed the instruction cache.)
// The kernel walks the FP32R pass's list of flagged FP64 tiles (the FP64 kernel's tile: 64
// locations up to 16 neighbors, 32 beyond; one tile per block) and solves every flagged
// location of a tile.  A location it cannot certify --
// a non-positive double-float pivot, F < 1e-6 (sigma^2 + tau^2), or a squared pivot ratio (a
// lower bound of the condition number) above 1e10 -- sends its whole tile on to the FP64
// kernel (a second list), so every tile's partial sums come from one kernel and keep their
// fixed order.  Each thread keeps its matrix in shared memory, pair p of thread t at
// p * TPB + t (hi and lo parts in separate arrays), so every access is bank-conflict free.
#pragma once
#include <cuda_runtime.h>
#include "nngp_cov_df.cuh"

namespace nngp_bfdf {

constexpr int kNGMax = 1 + NNGP_MAX_NV * (NNGP_MAX_NV + 1) / 2;
// Row r (entries 0 .. r, padded to an even count) starts at pair (r + 1)^2 / 4.
__host__ __device__ constexpr int row_pair0(int r) { return (r + 1) * (r + 1) / 4; }
// The kernel for neighbor bound M (16 or 24): a block is one FP64 tile (the unit of the
// flagged-tile list: 64 locations for m <= 16, 32 beyond), a thread one location; the
// augmented matrix has M + 1 rows.  Shared memory per thread: the triangle's hi and lo pairs,
// the column buffer's hi and lo pairs (entries 0 .. M + 1), the geometry (a float4 per row).
template <int M>
struct Shape {
  static constexpr int TPB = M <= 16 ? 64 : 32;
  static constexpr int MA = M + 1;
  static constexpr int NP = row_pair0(MA);
  static constexpr int NCP = (MA + 1) / 2;
  static constexpr int kThreadBytes = 8 * (2 * NP + 2 * NCP) + 16 * MA;
  static constexpr size_t kSmemBytes = (size_t)kThreadBytes * TPB +
                                       sizeof(float) * (TPB / 32) * nngp_bfr::kTabFloats +
                                       sizeof(double) * (TPB / 32) * kNGMax;
  static constexpr int kBlocksPerSM = (int)((228 * 1024) / (kSmemBytes + 1024));  // 2 at M = 16 and 24
  static_assert(kSmemBytes <= 227 * 1024 && kBlocksPerSM >= 1, "one block per SM at least");
};
constexpr float kMaxPivotRatio2 = 1e10f;  // squared pivot ratio above which FP64 takes over

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

using nngp_df2::p2;

// a - l b on both halves for double-float a, l, b, given nl = -l (normalised result): the hi
// parts' sum exact (two_sum), the product of the hi parts exact (fma), the cross terms rounded
// (below 2^-23 of the product)
__device__ __forceinline__ void fms(p2 &ah, p2 &al, p2 lh, p2 nlh, p2 nll, p2 bh, p2 bl) {
  namespace G = nngp_df2;
  const p2 pn = G::mul(nlh, bh);     // -(lh bh) rounded
  const p2 pe = G::fma(lh, bh, pn);  // its rounding error, exactly
  const p2 t = G::fma(nlh, bl, G::fma(nll, bh, G::sub(al, pe)));
  p2 s, e;
  G::two_sum(ah, pn, s, e);
  G::fast_two_sum(s, G::add(e, t), ah, al);
}

// sigma^2 rho for two squared distances (double-float), packed where the model allows
template <int COV>
__device__ __forceinline__ nngp_df2::df2 cov_two(nngp_df2::df2 d2, const nngp_bfr::CorDF &ck, const float *tab,
                                                 const CovParams *cp) {
  namespace G = nngp_df2;
  if constexpr (nngp_bfr::kPacked<COV>) {
    return nngp_bfr::cov_df2<COV>(d2, ck, tab);
  } else {
    const nngp_df::df a = nngp_bfr::cov_df<COV>(nngp_df::df{G::first(d2.h), G::first(d2.l)}, ck, tab, cp);
    const nngp_df::df b = nngp_bfr::cov_df<COV>(nngp_df::df{G::second(d2.h), G::second(d2.l)}, ck, tab, cp);
    return G::df2{G::pack(a.h, b.h), G::pack(a.l, b.l)};
  }
}

template <int M, int MODE, int COV>
__global__ void __launch_bounds__(Shape<M>::TPB) bfdf_kernel(const BFData *__restrict__ datas,
                                                 const CovParams *__restrict__ thetas,
                                                 const BFJob *__restrict__ jobs_fb, int njobs, int nv,
                                                 const int *__restrict__ tile_list, const int *__restrict__ tile_count,
                                                 int *__restrict__ list64, int *__restrict__ count64,
                                                 unsigned long long *__restrict__ locs64) {
  namespace F = nngp_df;
  namespace G = nngp_df2;
  using S = Shape<M>;
  constexpr int TPB = S::TPB, MA = S::MA, NP = S::NP, NCP = S::NCP;
  extern __shared__ __align__(16) float smem_d[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  p2 *Ah = reinterpret_cast<p2 *>(smem_d), *Al = Ah + NP * TPB;
  p2 *Ch = Al + NP * TPB, *Cl = Ch + NCP * TPB;
  float4 *geo = reinterpret_cast<float4 *>(Cl + NCP * TPB);
  float *tab = reinterpret_cast<float *>(geo + MA * TPB) + warp * nngp_bfr::kTabFloats;
  double *wbuf = reinterpret_cast<double *>(reinterpret_cast<float *>(geo + MA * TPB) + (TPB / 32) * nngp_bfr::kTabFloats);
  // pair q of a pair array, and element k (of the pairs starting at q0) as a float
#define PR(a, q) a[(q) * TPB + tid]
#define EL(a, q0, k) reinterpret_cast<float *>(&a[((q0) + ((k) >> 1)) * TPB + tid])[(k) & 1]
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
      // ---- 1. geometry (the location itself last, at the origin) and the augmented matrix.
      // Every loop below issues a batch of independent loads, then the arithmetic, then the
      // stores: a store to shared memory would otherwise hold back the next iteration's loads
      // (the compiler cannot tell the indices apart) and leave one instruction in flight.
      const float4 *xyf = reinterpret_cast<const float4 *>(d.xyf);
      const float4 pi4 = xyf[i];
      float omax = 1e-30f;
      for (int k0 = 0; k0 < mi; k0 += 8) {  // eight gathers in flight
        int nb[8];
#pragma unroll
        for (int u = 0; u < 8; u++) nb[u] = k0 + u < mi ? d.nnIndx[off + k0 + u] : i;
        float4 q[8];
#pragma unroll
        for (int u = 0; u < 8; u++) q[u] = xyf[nb[u]];
#pragma unroll
        for (int u = 0; u < 8; u++) {
          const F::df ox = F::diff(q[u].x, q[u].z, pi4.x, pi4.z), oy = F::diff(q[u].y, q[u].w, pi4.y, pi4.w);
          omax = fmaxf(omax, fmaxf(fabsf(ox.h), fabsf(oy.h)));  // zero past m_i (nb = i)
          if (k0 + u < mi) GEO(k0 + u) = make_float4(ox.h, oy.h, ox.l, oy.l);
        }
      }
      // hi parts on a common grid 2^e >= 2^-22 max |offset|: two hi parts subtract exactly
      const int eb = ((__float_as_int(omax) >> 23) & 0xff) - 22;
      const float grid = __int_as_float(max(eb, 1) << 23), inv = __int_as_float((254 - max(eb, 1)) << 23);
      for (int k0 = 0; k0 < mi; k0 += 4) {
        float4 g[4];
#pragma unroll
        for (int u = 0; u < 4; u++) g[u] = GEO(min(k0 + u, mi - 1));
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const float hx = __fmul_rn(rintf(__fmul_rn(g[u].x, inv)), grid);
          const float hy = __fmul_rn(rintf(__fmul_rn(g[u].y, inv)), grid);
          g[u] = make_float4(hx, hy, __fadd_rn(__fsub_rn(g[u].x, hx), g[u].z), __fadd_rn(__fsub_rn(g[u].y, hy), g[u].w));
        }
#pragma unroll
        for (int u = 0; u < 4; u++)
          if (k0 + u < mi) GEO(k0 + u) = g[u];
      }
      GEO(mi) = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      // row r: C_r0 .. C_r,r-1 and S (row mi: c' and S), four entries per step; an even row
      // ends in the pair (S, 0)
      PR(Ah, 0) = G::pack(Sd.h, 0.0f);
      PR(Al, 0) = G::pack(Sd.l, 0.0f);
      for (int r = 1; r <= mi; r++) {
        const int fr = row_pair0(r);
        const float4 gr = GEO(r);
        const p2 grx = G::splat(gr.x), gry = G::splat(gr.y), grz = G::splat(gr.z), grw = G::splat(gr.w);
        for (int c = 0; c < r; c += 4) {
          const float4 a0 = GEO(c), a1 = GEO(min(c + 1, r - 1)), b0 = GEO(min(c + 2, r - 1)), b1 = GEO(min(c + 3, r - 1));
          G::df2 ex, ey, fx, fy;
          G::fast_two_sum(G::sub(grx, G::pack(a0.x, a1.x)), G::sub(grz, G::pack(a0.z, a1.z)), ex.h, ex.l);
          G::fast_two_sum(G::sub(gry, G::pack(a0.y, a1.y)), G::sub(grw, G::pack(a0.w, a1.w)), ey.h, ey.l);
          G::fast_two_sum(G::sub(grx, G::pack(b0.x, b1.x)), G::sub(grz, G::pack(b0.z, b1.z)), fx.h, fx.l);
          G::fast_two_sum(G::sub(gry, G::pack(b0.y, b1.y)), G::sub(grw, G::pack(b0.w, b1.w)), fy.h, fy.l);
          const G::df2 va = cov_two<COV>(G::sumsq(ex, ey), ck, tab, cpp);
          const G::df2 vb = cov_two<COV>(G::sumsq(fx, fy), ck, tab, cpp);
          const int q = fr + (c >> 1);
          PR(Ah, q) = c + 1 < r ? va.h : G::pack(G::first(va.h), Sd.h);
          PR(Al, q) = c + 1 < r ? va.l : G::pack(G::first(va.l), Sd.l);
          if (c + 2 < r) {
            PR(Ah, q + 1) = c + 3 < r ? vb.h : G::pack(G::first(vb.h), Sd.h);
            PR(Al, q + 1) = c + 3 < r ? vb.l : G::pack(G::first(vb.l), Sd.l);
          }
        }
        if (!(r & 1)) {
          PR(Ah, fr + (r >> 1)) = G::pack(Sd.h, 0.0f);
          PR(Al, fr + (r >> 1)) = G::pack(Sd.l, 0.0f);
        }
      }
#pragma unroll
      for (int q = 0; q < NCP; q++) PR(Ch, q) = PR(Cl, q) = 0;
      // ---- 2. right-looking Cholesky of the augmented matrix; the diagonal slots end holding
      // 1 / L_KK, row mi ends holding z and, on its diagonal, F
      float pmin = 3.4e38f, pmax = 0.0f;
      for (int K = 0; K < mi; K++) {
        const int fk = row_pair0(K);
        const F::df dK = F::norm(EL(Ah, fk, K), EL(Al, fk, K));
        ok = dK.h > 0.0f;
        if (!ok) break;
        const F::df lkk = F::sqrt(dK);
        pmin = fminf(pmin, lkk.h);
        pmax = fmaxf(pmax, lkk.h);
        const F::df ik = F::recip(lkk);
        EL(Ah, fk, K) = ik.h;
        EL(Al, fk, K) = ik.l;
        EL(Ch, 0, K) = 0.0f;  // the update below leaves column K itself alone
        EL(Cl, 0, K) = 0.0f;
        // column K of L, also into the column buffer, four rows per step
        for (int r0 = K + 1; r0 <= mi; r0 += 4) {
          float xh[4], xl[4];
#pragma unroll
          for (int u = 0; u < 4; u++) {
            const int fr = row_pair0(min(r0 + u, mi));
            xh[u] = EL(Ah, fr, K);
            xl[u] = EL(Al, fr, K);
          }
          F::df l[4];
#pragma unroll
          for (int u = 0; u < 4; u++) l[u] = F::mul(F::df{xh[u], xl[u]}, ik);
#pragma unroll
          for (int u = 0; u < 4; u++) {
            const int r = r0 + u;
            if (r <= mi) {
              const int fr = row_pair0(r);
              EL(Ah, fr, K) = l[u].h;
              EL(Al, fr, K) = l[u].l;
              EL(Ch, 0, r) = l[u].h;
              EL(Cl, 0, r) = l[u].l;
            }
          }
        }
        // A_rj -= L_rK L_jK for K < j <= r <= mi: pairs (r, q), q from the one holding K + 1
        // to the one holding r, walked four at a time in row order
        const int q0 = (K + 1) >> 1;
        int r = K + 1, q = q0;
        while (r <= mi) {
          int at[4], cq[4], cr[4];
          bool on[4];
#pragma unroll
          for (int u = 0; u < 4; u++) {
            on[u] = r <= mi;
            cr[u] = min(r, mi);
            cq[u] = min(q, cr[u] >> 1);
            at[u] = row_pair0(cr[u]) + cq[u];
            if (++q > (r >> 1)) {
              r++;
              q = q0;
            }
          }
          p2 ah[4], al[4], bh[4], bl[4], lh[4], nlh[4], nll[4];
#pragma unroll
          for (int u = 0; u < 4; u++) {
            ah[u] = PR(Ah, at[u]);
            al[u] = PR(Al, at[u]);
            bh[u] = PR(Ch, cq[u]);
            bl[u] = PR(Cl, cq[u]);
            const float xh = EL(Ch, 0, cr[u]), xl = EL(Cl, 0, cr[u]);
            lh[u] = G::splat(xh);
            nlh[u] = G::splat(-xh);
            nll[u] = G::splat(-xl);
          }
#pragma unroll
          for (int u = 0; u < 4; u++) fms(ah[u], al[u], lh[u], nlh[u], nll[u], bh[u], bl[u]);
#pragma unroll
          for (int u = 0; u < 4; u++)
            if (on[u]) {
              PR(Ah, at[u]) = ah[u];
              PR(Al, at[u]) = al[u];
            }
        }
      }
      const int fz = row_pair0(mi);
      if (ok) {
        Fd = F::norm(EL(Ah, fz, mi), EL(Al, fz, mi));
        const float ratio = pmax / pmin;
        ok = Fd.h > nngp_bfr::kMinFRel * Sd.h && ratio * ratio <= kMaxPivotRatio2;
      }
      if (ok) {
        // ---- B = L^-T z in place of z: b_r = z_r / L_rr, then z_k -= L_rk b_r for k < r
        for (int r = mi - 1; r >= 0; r--) {
          const int fr = row_pair0(r);
          const F::df b = F::mul(F::df{EL(Ah, fz, r), EL(Al, fz, r)}, F::df{EL(Ah, fr, r), EL(Al, fr, r)});
          EL(Ah, fz, r) = b.h;
          EL(Al, fz, r) = b.l;
          const p2 bh = G::splat(b.h), nbh = G::splat(-b.h), nbl = G::splat(-b.l);
          const int nq = r >> 1;
          for (int q0 = 0; q0 < nq; q0 += 4) {
            p2 zh[4], zl[4], xh[4], xl[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
              const int q = min(q0 + u, nq - 1);
              zh[u] = PR(Ah, fz + q);
              zl[u] = PR(Al, fz + q);
              xh[u] = PR(Ah, fr + q);
              xl[u] = PR(Al, fr + q);
            }
#pragma unroll
            for (int u = 0; u < 4; u++) fms(zh[u], zl[u], bh, nbh, nbl, xh[u], xl[u]);
#pragma unroll
            for (int u = 0; u < 4; u++)
              if (q0 + u < nq) {
                PR(Ah, fz + q0 + u) = zh[u];
                PR(Al, fz + q0 + u) = zl[u];
              }
          }
          if (r & 1) {  // entry r - 1 opens the pair that ends on the diagonal
            const F::df z = F::sub(F::df{EL(Ah, fz, r - 1), EL(Al, fz, r - 1)},
                                   F::mul(b, F::df{EL(Ah, fr, r - 1), EL(Al, fr, r - 1)}));
            EL(Ah, fz, r - 1) = z.h;
            EL(Al, fz, r - 1) = z.l;
          }
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
    const int fz = row_pair0(mi);
    const double Fi = F::to_double(Fd);
    double logF = 0.0;
    double rv[NNGP_MAX_NV] = {};
    if (active) {
      logF = log(Fi);
      if (MODE == 0) {
        for (int k = 0; k < mi; k++) d.B[off + k] = (double)EL(Ah, fz, k) + (double)EL(Al, fz, k);
        d.F[i] = Fi;
      } else {
        for (int v = 0; v < nv; v++) rv[v] = d.V[(size_t)i * nv + v];
        for (int k = 0; k < mi; k++) {
          const double bk = (double)EL(Ah, fz, k) + (double)EL(Al, fz, k);
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
#undef PR
#undef EL
#undef GEO
}

// Walks the plan's flagged-tile list with as many blocks as the SMs hold at once (one tile per
// block); tiles it cannot certify are appended to the plan's FP64 list.
template <int M, int MODE, int COV>
int launch_df(nngp_ctx *ctx, const BFPlan *pl) {
  using S = Shape<M>;
  static bool configured[64] = {};  // the attribute is per device
  const int dev = ctx->device & 63;
  if (!configured[dev]) {
    NNGP_CUDA_TRY(ctx, cudaFuncSetAttribute(bfdf_kernel<M, MODE, COV>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)S::kSmemBytes));
    configured[dev] = true;
  }
  if (pl->tiles_fb <= 0) return NNGP_OK;
  const int cap = S::kBlocksPerSM * (ctx->sm_count > 0 ? ctx->sm_count : 1);
  const int grid = pl->tiles_fb < cap ? pl->tiles_fb : cap;
  bfdf_kernel<M, MODE, COV><<<grid, S::TPB, S::kSmemBytes, ctx->stream>>>(
      pl->d_datas, pl->d_thetas, pl->d_jobs_fb, pl->njobs, pl->nv, pl->d_fb_list, (const int *)pl->d_fb_words,
      pl->d_fb64_list, pl->d_fb64_count, pl->d_fb64_locs);
  NNGP_LAUNCH_CHECK(ctx);
  return NNGP_OK;
}

}  // namespace nngp_bfdf
