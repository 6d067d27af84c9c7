// FP32R B/F kernel for neighbor counts m <= 16 with the Cholesky factor held in
// registers (reference updateBF, src/rNNGP.cpp:46-101; updateConjBF,
// src/cNNGP.cpp:24-69; the likelihood sums of src/rNNGP.cpp:306-317 and Q,
// src/util.cpp:261-280).
//
// One thread solves one location's M x M neighborhood system; one warp owns a
// tile of 32 consecutive locations of one job (job = one dataset at one
// parameter set), and each warp reduces its own tile, so blocks are only a
// launch-shape choice: the warps of a block may serve different jobs, and the
// results do not depend on the number of warps per block or on the grid size
// (the autotuner in nngp_bf.cu picks both).
//
// Per thread:
//   1. geometry: neighbor offsets from the location, differenced from the float
//      (hi, lo) split of the coordinates, as normalised double-float pairs
//      (exact to about 2^-48); one float4 per neighbor in shared memory;
//   2. covariance build in a rolled loop: the c vector and the strict lower
//      triangle of C in double-float (distance, sqrt and exp carried in float
//      pairs on the FP32 pipe: about 1e-13 relative, where GB300's FP64 pipe
//      would cost 64 float instructions per double one); hi parts and lo parts
//      in shared memory;
//   3. the hi parts into registers: right-looking Cholesky, forward and back
//      substitution in float, all on registers;
//   4. one refinement step with the residual of the accurate system: c - C b
//      row by row as a compensated (Dot2) dot product over the double-float
//      entries, fused with the forward substitution of the correction; B = b +
//      delta is kept as an unevaluated float pair.  The refinement converges to
//      the FP64 solution at rate ~ kappa * 2^-24 per step;
//   5. F = sigma^2 + tau^2 - B'c, log F, the residuals r = (I - B) V and the
//      Gram terms r_a r_b / F in double-float; per-warp sums of those, in a
//      fixed order, go to the job's partial array as doubles.
// Rows m_i <= r < M are padded with the identity (c_r = 0), which solves to
// B_r = 0 exactly, so every loop in step 3-5 runs without predicates.
//
// Error control: after the one step the error left in B is about q^2 |b| with
// q = |delta|_inf / |b|_inf (the float solve's relative error), which moves F by
// about q^2 (sigma^2 + tau^2).  A location is flagged -- it contributes nothing
// here and the FP64 kernel re-solves it -- when its float pivot fails, or when
// that estimate exceeds 1e-8 F, or when F < 1e-6 (sigma^2 + tau^2).
#pragma once
#include <cuda_runtime.h>
#include "nngp_df.cuh"
#include "nngp_internal.h"
#include "nngp_math.cuh"

namespace nngp_bfr {

constexpr int kNGMax = 1 + NNGP_MAX_NV * (NNGP_MAX_NV + 1) / 2;
constexpr float kTolF = 1e-8f;    // accepted F error estimate, relative to F
constexpr float kMinFRel = 1e-6f;  // smaller F (relative to sigma^2 + tau^2) goes to FP64

template <int M>
struct Shape {
  static constexpr int NL = M * (M - 1) / 2;  // strict lower triangle of C
  static constexpr int NC = NL + M;           // ... followed by the c vector
  static constexpr int LANE = nngp_bfr_lane_floats(M);  // hi parts, lo parts, geometry (or staging)
  static constexpr int TAB = 64;              // per-warp exp table (32 hi, 32 lo)
  static constexpr size_t WARP_BYTES = nngp_bfr_warp_bytes(M);
  static constexpr int MAX_WPB = nngp_bfr_max_wpb(M);
};
__host__ __device__ constexpr int lidx(int r, int c) { return r * (r - 1) / 2 + c; }  // r > c

// Per-tile constants of the correlation function in double-float.
struct CorDF {
  nngp_df::df K;   // exp argument scale in units of ln2/32: -phi 32/ln2 (times d), gaussian -phi^2 32/ln2 (times d^2)
  nngp_df::df P;   // phi
  nngp_df::df S2;  // sigma^2
  float pfh[9], pfl[9];  // matern nu = k + 1/2: polynomial coefficients
  int halfk;
  int model;
};

template <int COV>
__device__ __forceinline__ CorDF cor_prepare(const CovParams *cp) {
  namespace F = nngp_df;
  CorDF k{};
  const int model = COV == NNGP_COV_ANY ? cp->model : COV;
  k.model = model;
  k.halfk = cp->halfk;
  k.P = F::from_double(cp->phi);
  k.S2 = F::from_double(cp->sigmaSq);
  const double c32 = 46.166241308446828;  // 32 / ln 2
  k.K = F::from_double(model == 3 ? -(cp->phi * cp->phi) * c32 : -cp->phi * c32);
  if (model == 2 && cp->halfk >= 0) {
#pragma unroll
    for (int j = 0; j < 9; j++) {
      const F::df c = F::from_double(cp->poly[j]);
      k.pfh[j] = c.h;
      k.pfl[j] = c.l;
    }
  }
  return k;
}

// sigma^2 rho(d) in double-float from d^2 (double-float).  The exp-based models read
// sigma^2 2^(j/32) from the warp's table; the general-nu Matern evaluates K_nu in FP64.
template <int COV>
__device__ __forceinline__ nngp_df::df cov_df(nngp_df::df d2, const CorDF &k, const float *tab,
                                              const CovParams *cp) {
  namespace F = nngp_df;
  const int model = COV == NNGP_COV_ANY ? k.model : COV;
  if (model == 3) {  // gaussian: exp(-(phi d)^2)
    const F::df u = F::mul(k.K, d2);
    return F::exp_u(u.h, u.l, tab);
  }
  const F::df d = F::sqrt(d2);
  if (model == 0) {  // exponential
    const F::df u = F::mul(k.K, d);
    return F::exp_u(u.h, u.l, tab);
  }
  if (model == 1) {  // spherical: 1 - 1.5 t + 0.5 t^3 for t = phi d < 1
    const F::df t = F::mul(k.P, d);
    if (!(t.h < 1.0f)) return F::df{0.0f, 0.0f};
    const F::df t3 = F::mul(F::mul(t, t), t);
    const F::df rho = F::sub(F::add(F::df{1.0f, 0.0f}, F::df{0.5f * t3.h, 0.5f * t3.l}),
                             F::mul(t, F::df{1.5f, 0.0f}));
    return F::mul(k.S2, rho);
  }
  // matern
  if (COV == NNGP_COV_ANY && k.halfk < 0) {
    const double dd = (double)d.h + (double)d.l;
    return F::mul(k.S2, F::from_double(nngp_cor_d<NNGP_COV_ANY>(dd, *cp)));
  }
  const F::df u = F::mul(k.K, d);
  const F::df E = F::exp_u(u.h, u.l, tab);
  if (k.halfk <= 0) return E;
  const F::df x = F::mul(k.P, d);
  F::df s{k.pfh[8], k.pfl[8]};
#pragma unroll
  for (int j = 7; j >= 0; j--)
    if (j < k.halfk) s = F::add(F::mul(s, x), F::df{k.pfh[j], k.pfl[j]});
    else if (j == k.halfk) s = F::df{k.pfh[j], k.pfl[j]};
  return F::mul(E, s);
}

__device__ __forceinline__ int find_job(const BFJob *jobs, int njobs, int tile) {
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].tile0 <= tile) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

template <int M, int MODE, int COV>
__global__ void __launch_bounds__(256, 1) bfr_kernel(const BFData *__restrict__ datas,
                                                     const CovParams *__restrict__ thetas,
                                                     const BFJob *__restrict__ jobs, int njobs,
                                                     int tile_begin, int tile_end, int nv) {
  using S = Shape<M>;
  namespace F = nngp_df;
  extern __shared__ __align__(16) float smem_f[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  float *ws = smem_f + (size_t)warp * (32 * S::LANE + S::TAB);
  float *tab = ws + 32 * S::LANE;
  float4 *geo = reinterpret_cast<float4 *>(ws + 32 * 2 * S::NC);
#define CS(e) ws[(e) * 32 + lane]
#define CL(e) ws[(S::NC + (e)) * 32 + lane]
#define GEO(k) geo[(k) * 32 + lane]
  // C and c are read again after the factorization: volatile reads stop the compiler from
  // keeping the first reads alive in registers beside the factor (which spills)
  volatile float *wv = ws;
#define CSV(e) wv[(e) * 32 + lane]
#define CLV(e) wv[(S::NC + (e)) * 32 + lane]
  constexpr int kStage = 2 * NNGP_MAX_NV;  // first staging slot of the per-warp sums

  for (int tile = tile_begin + blockIdx.x * wpb + warp; tile < tile_end; tile += gridDim.x * wpb) {
    const BFJob job = jobs[find_job(jobs, njobs, tile)];
    const BFData d = datas[job.data];
    const CovParams *cpp = thetas + job.theta;
    const int tj = tile - job.tile0;
    const int i = tj * 32 + lane;
    const bool active = i < d.n;
    int mi = 0, off = 0;
    if (active) {
      off = d.nnLU[i];
      mi = min(d.nnLU[d.n + i], M);
    }
    const double sigmaSq = cpp->sigmaSq, tauSq = cpp->tauSq;
    const CorDF ck = cor_prepare<COV>(cpp);
    const F::df Sd = F::from_double(sigmaSq + tauSq);  // the diagonal sigma^2 + tau^2
    {  // the warp's exp table: sigma^2 2^(j/32)
      const float2 t2 = F::kExp2Tab[lane];
      const F::df e = F::mul(ck.S2, F::df{t2.x, t2.y});
      tab[lane] = e.h;
      tab[32 + lane] = e.l;
    }
    __syncwarp();

    // ---- 1. geometry
    const float4 *xyf = reinterpret_cast<const float4 *>(d.xyf);
    const float4 pi4 = active ? xyf[i] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int k = 0; k < M; k++) {
      if (k < mi) {
        const float4 q = xyf[d.nnIndx[off + k]];
        const F::df ox = F::diff(q.x, q.z, pi4.x, pi4.z), oy = F::diff(q.y, q.w, pi4.y, pi4.w);
        GEO(k) = make_float4(ox.h, oy.h, ox.l, oy.l);
      }
    }
    // ---- 2. covariance build (rolled), double-float: the c vector, then the strict lower
    // triangle as one loop over its pairs in storage order (four independent pairs in flight)
#pragma unroll 4
    for (int r = 0; r < mi; r++) {
      const float4 g = GEO(r);
      const F::df cr = cov_df<COV>(F::sumsq(g.x, g.z, g.y, g.w), ck, tab, cpp);
      CS(S::NL + r) = cr.h;
      CL(S::NL + r) = cr.l;
    }
    {
      const int npairs = mi * (mi - 1) / 2;
      int r = 1, c = 0;
#pragma unroll 4
      for (int e = 0; e < npairs; e++) {
        const float4 g = GEO(r), h = GEO(c);
        const F::df ex = F::diff(g.x, g.z, h.x, h.z), ey = F::diff(g.y, g.w, h.y, h.w);
        const F::df v = cov_df<COV>(F::sumsq(ex.h, ex.l, ey.h, ey.l), ck, tab, cpp);
        CS(e) = v.h;  // e == lidx(r, c)
        CL(e) = v.l;
        if (++c == r) {
          r++;
          c = 0;
        }
      }
    }
#pragma unroll 1
    for (int r = mi; r < M; r++) {  // identity padding
      CS(S::NL + r) = 0.0f;
      CL(S::NL + r) = 0.0f;
      float *rowh = &CS(lidx(r, 0));
      float *rowl = &CL(lidx(r, 0));
#pragma unroll 1
      for (int c = 0; c < r; c++) rowh[c * 32] = rowl[c * 32] = 0.0f;
    }

    // ---- 3. Cholesky and solves on registers (hi parts)
    float L[S::NL > 0 ? S::NL : 1];
#pragma unroll
    for (int e = 0; e < S::NL; e++) L[e] = CS(e);
    float D[M];
#pragma unroll
    for (int k = 0; k < M; k++) D[k] = (k < mi) ? Sd.h : 1.0f;
    bool ok = true;
#pragma unroll
    for (int k = 0; k < M; k++) {
      ok = ok && (D[k] > 0.0f);
      const float inv = rsqrtf(D[k]);
      D[k] = inv;  // D now holds 1 / L_kk
#pragma unroll
      for (int r = k + 1; r < M; r++) L[lidx(r, k)] *= inv;
#pragma unroll
      for (int j = k + 1; j < M; j++) {
        const float ljk = L[lidx(j, k)];
        D[j] = fmaf(-ljk, ljk, D[j]);
#pragma unroll
        for (int r = j + 1; r < M; r++) L[lidx(r, j)] = fmaf(-L[lidx(r, k)], ljk, L[lidx(r, j)]);
      }
    }
    float b[M];
#pragma unroll
    for (int r = 0; r < M; r++) b[r] = CS(S::NL + r);
#pragma unroll
    for (int k = 0; k < M; k++) {  // L z = c
      b[k] *= D[k];
#pragma unroll
      for (int r = k + 1; r < M; r++) b[r] = fmaf(-L[lidx(r, k)], b[k], b[r]);
    }
#pragma unroll
    for (int k = M - 1; k >= 0; k--) {  // L' b = z
      b[k] *= D[k];
#pragma unroll
      for (int r = 0; r < k; r++) b[r] = fmaf(-L[lidx(k, r)], b[k], b[r]);
    }

    // ---- 4. refinement: res = c - C b over the double-float entries (Dot2), L L' w = res
    float w[M];
#pragma unroll
    for (int r = 0; r < M; r++) w[r] = 0.0f;
#pragma unroll
    for (int r = 0; r < M; r++) {
      float sh = 0.0f, sl = 0.0f;
#pragma unroll
      for (int c = 0; c < M; c++) {
        float eh, el;
        if (c == r) {
          eh = (r < mi) ? Sd.h : 1.0f;
          el = (r < mi) ? Sd.l : 0.0f;
        } else {
          eh = c < r ? CSV(lidx(r, c)) : CSV(lidx(c, r));
          el = c < r ? CLV(lidx(r, c)) : CLV(lidx(c, r));
        }
        F::dot2_acc(sh, sl, eh, b[c]);
        sl = fmaf(el, b[c], sl);
      }
      const float res = __fadd_rn(__fsub_rn(__fsub_rn(CSV(S::NL + r), sh), sl), CLV(S::NL + r));
      w[r] = (res - w[r]) * D[r];
#pragma unroll
      for (int j = r + 1; j < M; j++) w[j] = fmaf(L[lidx(j, r)], w[r], w[j]);
    }
#pragma unroll
    for (int k = M - 1; k >= 0; k--) {
      w[k] *= D[k];
#pragma unroll
      for (int r = 0; r < k; r++) w[r] = fmaf(-L[lidx(k, r)], w[k], w[r]);
    }
    // B = b + w (unevaluated float pair)

    // ---- 5. F, error estimate, log F, likelihood terms
    float dh = 0.0f, dl = 0.0f, bmax = 0.0f, wmax = 0.0f;
#pragma unroll
    for (int k = 0; k < M; k++) {
      const float ch = CSV(S::NL + k), cl = CLV(S::NL + k);
      F::dot2_acc(dh, dl, b[k], ch);
      dl = fmaf(w[k], ch, fmaf(b[k], cl, dl));
      bmax = fmaxf(bmax, fabsf(b[k]));
      wmax = fmaxf(wmax, fabsf(w[k]));
    }
    const F::df Fd = F::sub(Sd, F::norm(dh, dl));
    const float q = wmax / fmaxf(bmax, 1e-30f);
    const bool bad = !ok || !(Fd.h > kMinFRel * Sd.h) || !(q * q * Sd.h <= kTolF * Fd.h);
    if (active && bad) nngp_flag_for_fp64(job, i);
    const bool use = active && !bad;
    const F::df lf = use ? F::log(Fd) : F::df{0.0f, 0.0f};
    if constexpr (MODE == 0) {
      if (use) {
#pragma unroll
        for (int k = 0; k < M; k++)
          if (k < mi) d.B[off + k] = (double)b[k] + (double)w[k];
        d.F[i] = F::to_double(Fd);
      }
      CS(kStage) = lf.h;
      CS(kStage + 1) = lf.l;
    } else {
      int nb[M];
#pragma unroll
      for (int k = 0; k < M; k++) nb[k] = (k < mi) ? d.nnIndx[off + k] : 0;
      const float2 *Vf = d.Vf;
      // r_v = V_iv - sum_k B_k V_nb(k)v, staged at slots 2v, 2v + 1
#pragma unroll 1
      for (int v = 0; v < nv; v++) {
        float ah = 0.0f, al = 0.0f;
#pragma unroll
        for (int k = 0; k < M; k++) {
          if (k < mi) {
            const float2 q = Vf[(size_t)nb[k] * nv + v];
            F::dot2_acc(ah, al, b[k], q.x);
            al = fmaf(b[k], q.y, fmaf(w[k], q.x, al));
          }
        }
        const float2 vi = active ? Vf[(size_t)i * nv + v] : make_float2(0.f, 0.f);
        const F::df rv = F::sub(F::df{vi.x, vi.y}, F::norm(ah, al));
        CS(2 * v) = rv.h;
        CS(2 * v + 1) = rv.l;
      }
      const F::df invF = use ? F::recip(Fd) : F::df{0.0f, 0.0f};
      CS(kStage) = lf.h;
      CS(kStage + 1) = lf.l;
      int t = 1;
#pragma unroll 1
      for (int a = 0; a < nv; a++) {
        const F::df ta = F::mul(F::df{CS(2 * a), CS(2 * a + 1)}, invF);
#pragma unroll 1
        for (int c = a; c < nv; c++, t++) {
          const F::df g = F::mul(ta, F::df{CS(2 * c), CS(2 * c + 1)});
          CS(kStage + 2 * t) = g.h;
          CS(kStage + 2 * t + 1) = g.l;
        }
      }
    }

    // ---- per-warp sums: lane t adds value t over the 32 lanes, starting at lane t
    // (a fixed order; the rotation keeps the shared-memory reads conflict-free)
    __syncwarp();
    const int ng = MODE == 0 ? 1 : 1 + nv * (nv + 1) / 2;
    for (int t = lane; t < ng; t += 32) {
      const float *vh = ws + (size_t)(kStage + 2 * t) * 32;
      const float *vl = vh + 32;
      F::df acc{0.0f, 0.0f};
#pragma unroll 4
      for (int s = 0; s < 32; s++) {
        const int src = (s + t) & 31;
        acc = F::add(acc, F::df{vh[src], vl[src]});
      }
      job.partial[(size_t)tj * ng + t] = F::to_double(acc);
    }
    __syncwarp();
  }
#undef CS
#undef CSV
#undef CL
#undef CLV
#undef GEO
}

template <int M>
constexpr size_t smem_bytes(int wpb) {
  return Shape<M>::WARP_BYTES * (size_t)wpb;
}

// Raises the kernel's dynamic shared-memory limit to what the largest block (MAX_WPB warps)
// needs (once per device; the attribute is per device).
template <int M, int MODE, int COV>
cudaError_t configure(int device) {
  static bool configured[64] = {};
  const int dev = device & 63;
  if (configured[dev]) return cudaSuccess;
  const cudaError_t e = cudaFuncSetAttribute(bfr_kernel<M, MODE, COV>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem_bytes<M>(Shape<M>::MAX_WPB));
  if (e == cudaSuccess) configured[dev] = true;
  return e;
}

// Launches the kernel on the plan's primary tiles [t0, t1) with wpb warps per block and `grid`
// blocks.
template <int M, int MODE, int COV>
int launch_reg(nngp_ctx *ctx, const BFPlan *pl, int wpb, int grid, int t0, int t1) {
  NNGP_CUDA_TRY(ctx, (configure<M, MODE, COV>(ctx->device)));
  if (t1 <= t0) return NNGP_OK;
  bfr_kernel<M, MODE, COV><<<grid, 32 * wpb, smem_bytes<M>(wpb), ctx->stream>>>(
      pl->d_datas, pl->d_thetas, pl->d_jobs, pl->njobs, t0, t1, pl->nv);
  NNGP_LAUNCH_CHECK(ctx);
  return NNGP_OK;
}

// Blocks of wpb warps one SM holds at once (on the current device).
template <int M, int MODE, int COV>
int occupancy(int wpb) {
  if (wpb > Shape<M>::MAX_WPB) return 0;
  int dev = 0, blocks = 0;
  cudaGetDevice(&dev);
  if (configure<M, MODE, COV>(dev) != cudaSuccess) return 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, bfr_kernel<M, MODE, COV>, 32 * wpb,
                                                    smem_bytes<M>(wpb)) != cudaSuccess)
    return 1;
  return blocks > 0 ? blocks : 1;
}

}  // namespace nngp_bfr
