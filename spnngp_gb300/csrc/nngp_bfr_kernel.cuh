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
#include "nngp_cov_df.cuh"

namespace nngp_bfr {

constexpr int kNGMax = 1 + NNGP_MAX_NV * (NNGP_MAX_NV + 1) / 2;

// Per-lane layout (floats, each interleaved over the warp's 32 lanes): [0, NL) hi parts of
// the strict lower triangle, [NL, NC) hi parts of c, [NC, NC + M) lo parts of c, then (without
// tensor memory) the NL lo parts of the strict lower triangle, then the geometry.  With TM the
// strict lower triangle's lo parts live in tensor memory instead, as full symmetric rows of 16
// columns (row r at columns 16 r .. 16 r + 15 of the warp's range), so the residual reads a
// row with one load.
template <int M, bool TM = false>
struct Shape {
  static constexpr int NL = M * (M - 1) / 2;  // strict lower triangle of C
  static constexpr int NC = NL + M;           // ... followed by the c vector
  static constexpr int CLO = NC;              // lo parts of c
  static constexpr int LLO = NC + M;          // lo parts of the strict lower triangle (!TM)
  static constexpr int GEO = NC + M + (TM ? 0 : NL);
  static constexpr int LANE = nngp_bfr_lane_floats(M, TM);
  static constexpr int TAB = kTabFloats;      // per-warp table (exp, Matern polynomial)
  static constexpr size_t WARP_BYTES = nngp_bfr_warp_bytes(M, TM);
  static constexpr int MAX_WPB = nngp_bfr_max_wpb(M, TM);
  static_assert(GEO + 4 * M <= LANE, "layout exceeds the lane's share");
  static_assert(WARP_BYTES == sizeof(float) * (32 * (size_t)LANE + TAB), "warp size disagrees with the layout");
};

// Tensor-memory access (tcgen05): one 32-bit value per lane and column.  A warp reaches the
// lanes of its quarter (32 (warp % 4) ..) only; the caller adds that lane base.
__device__ __forceinline__ void tm_st(unsigned addr, float v) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x1.b32 [%0], {%1};" ::"r"(addr), "f"(v));
}
__device__ __forceinline__ void tm_ld16(unsigned addr, float (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=f"(r[0]), "=f"(r[1]), "=f"(r[2]), "=f"(r[3]), "=f"(r[4]), "=f"(r[5]), "=f"(r[6]), "=f"(r[7]), "=f"(r[8]),
        "=f"(r[9]), "=f"(r[10]), "=f"(r[11]), "=f"(r[12]), "=f"(r[13]), "=f"(r[14]), "=f"(r[15])
      : "r"(addr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tm_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
__host__ __device__ constexpr int lidx(int r, int c) { return r * (r - 1) / 2 + c; }  // r > c

// (r, c) of strict-lower-triangle entry e in storage order, packed r << 8 | c (M <= 16); read
// warp-uniformly, so the build loop's iterations carry no dependency through the indices
struct PairTable {
  unsigned short rc[120];
  constexpr PairTable() : rc() {
    int e = 0;
    for (int r = 1; r < 16; r++)
      for (int c = 0; c < r; c++) rc[e++] = (unsigned short)(r << 8 | c);
  }
};
static __constant__ PairTable kPairs = PairTable();

template <int M, int MODE, int COV, bool TM>
__global__ void __launch_bounds__(256, 1) bfr_kernel(const BFData *__restrict__ datas,
                                                     const CovParams *__restrict__ thetas,
                                                     const BFJob *__restrict__ jobs, int njobs,
                                                     int tile_begin, int tile_end, int nv) {
  using S = Shape<M, TM>;
  namespace F = nngp_df;
  extern __shared__ __align__(16) float smem_f[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  float *ws = smem_f + (size_t)warp * (32 * S::LANE + S::TAB);
  float *tab = ws + 32 * S::LANE;
  float4 *geo = reinterpret_cast<float4 *>(ws + 32 * S::GEO);
#define CS(e) ws[(e) * 32 + lane]
#define CLC(r) ws[(S::CLO + (r)) * 32 + lane]
#define CLL(e) ws[(S::LLO + (e)) * 32 + lane]
#define GEO(k) geo[(k) * 32 + lane]
  // C and c are read again after the factorization: volatile reads stop the compiler from
  // keeping the first reads alive in registers beside the factor (which spills)
  volatile float *wv = ws;
#define CSV(e) wv[(e) * 32 + lane]
#define CLCV(r) wv[(S::CLO + (r)) * 32 + lane]
#define CLLV(e) wv[(S::LLO + (e)) * 32 + lane]
  // tensor memory (TM): the CTA's warp 0 allocates 256 columns per four warps; warp w owns lane
  // quarter w % 4 and columns 256 (w / 4) .. + 255 of the allocation
  __shared__ unsigned tm_alloc_base;
  unsigned tm0 = 0;
  const unsigned tm_cols = wpb > 4 ? 512u : 256u;
  if constexpr (TM) {
    if (warp == 0) {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                       (unsigned)__cvta_generic_to_shared(&tm_alloc_base)),
                   "r"(tm_cols));
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    tm0 = tm_alloc_base + ((32u * (unsigned)(warp & 3)) << 16) + 256u * (unsigned)(warp >> 2);
  }
  constexpr int kStage = 2 * NNGP_MAX_NV;  // first staging slot of the per-warp sums

  for (int tile = tile_begin + blockIdx.x * wpb + warp; tile < tile_end; tile += gridDim.x * wpb) {
    const BFJob job = jobs[nngp_find_job(jobs, njobs, tile)];
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
    if constexpr (COV == NNGP_COV_GAU || COV == NNGP_COV_ANY) {
      if (nngp_route_double_float(*cpp)) {  // the job's parameter set: warp-uniform
        // every location to the double-float re-solve, nothing from the float factor here
        if (active) nngp_flag_for_fp64(job, i);
        const int ngz = MODE == 0 ? 1 : 1 + nv * (nv + 1) / 2;
        for (int t = lane; t < ngz; t += 32) job.partial[(size_t)tj * ngz + t] = 0.0;
        continue;
      }
    }
    const CorDF ck = cor_prepare<COV>(cpp);
    const F::df Sd{cpp->dfDiag[0], cpp->dfDiag[1]};  // the diagonal sigma^2 + tau^2
    fill_tab<COV>(tab, ck, cpp, lane);  // the warp's exp table and Matern coefficients
    __syncwarp();

    // ---- 1. geometry: offsets from the location as double-float pairs whose hi parts lie on a
    // common grid 2^e with 2^e >= 2^-22 max|offset|, so the hi parts of two offsets subtract
    // exactly (at most 24 bits) and a pair difference needs no error-free transformation
    const float4 *xyf = reinterpret_cast<const float4 *>(d.xyf);
    const float4 pi4 = active ? xyf[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    F::df ox[M], oy[M];
    float omax = 1e-30f;
#pragma unroll
    for (int k = 0; k < M; k++) {
      ox[k] = oy[k] = F::df{0.0f, 0.0f};
      if (k < mi) {
        const float4 q = xyf[d.nnIndx[off + k]];
        ox[k] = F::diff(q.x, q.z, pi4.x, pi4.z);
        oy[k] = F::diff(q.y, q.w, pi4.y, pi4.w);
        omax = fmaxf(omax, fmaxf(fabsf(ox[k].h), fabsf(oy[k].h)));
      }
    }
    {
      const int eb = ((__float_as_int(omax) >> 23) & 0xff) - 22;  // biased exponent of 2^e
      const float grid = __int_as_float(max(eb, 1) << 23), inv = __int_as_float((254 - max(eb, 1)) << 23);
#pragma unroll
      for (int k = 0; k < M; k++) {
        if (k < mi) {
          const float hx = __fmul_rn(rintf(__fmul_rn(ox[k].h, inv)), grid);
          const float hy = __fmul_rn(rintf(__fmul_rn(oy[k].h, inv)), grid);
          GEO(k) = make_float4(hx, hy, __fadd_rn(__fsub_rn(ox[k].h, hx), ox[k].l),
                               __fadd_rn(__fsub_rn(oy[k].h, hy), oy[k].l));
        }
      }
    }
    // ---- 2. covariance build (rolled), double-float: the c vector, then the strict lower
    // triangle as one loop over its pairs in storage order.  Each step handles four pairs with
    // all loads first, then the four (independent) evaluations, then the stores: shared-memory
    // stores and loads through one base pointer may alias as far as the compiler knows, so a
    // plain unrolled loop would run its iterations one after another.
#pragma unroll 1
    for (int r0 = 0; r0 < mi; r0 += 4) {
      float4 g[4];
#pragma unroll
      for (int j = 0; j < 4; j++) g[j] = GEO(min(r0 + j, mi - 1));
      F::df v[4];
      if constexpr (kPacked<COV>) {
        namespace G = nngp_df2;
#pragma unroll
        for (int t = 0; t < 2; t++) {
          G::df2 gx, gy;
          G::two_sum(G::pack(g[2 * t].x, g[2 * t + 1].x), G::pack(g[2 * t].z, g[2 * t + 1].z), gx.h, gx.l);
          G::two_sum(G::pack(g[2 * t].y, g[2 * t + 1].y), G::pack(g[2 * t].w, g[2 * t + 1].w), gy.h, gy.l);
          const G::df2 r = cov_df2<COV>(G::sumsq(gx, gy), ck, tab);
          v[2 * t] = F::df{G::first(r.h), G::first(r.l)};
          v[2 * t + 1] = F::df{G::second(r.h), G::second(r.l)};
        }
      } else {
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const F::df gx = F::norm(g[j].x, g[j].z), gy = F::norm(g[j].y, g[j].w);
          v[j] = cov_df<COV>(F::sumsq(gx.h, gx.l, gy.h, gy.l), ck, tab, cpp);
        }
      }
#pragma unroll
      for (int j = 0; j < 4; j++)
        if (r0 + j < mi) {
          CS(S::NL + r0 + j) = v[j].h;
          CLC(r0 + j) = v[j].l;
        }
    }
    {
      // every lane covers all NL pairs of the bound (a warp-uniform trip count: the tensor-memory
      // stores are warp-collective); a pair in a padded row (r >= m_i) is stored as 0
#pragma unroll 1
      for (int e0 = 0; e0 < S::NL; e0 += 4) {
        float4 g[4], h[4];
        int rr[4], cc[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const int rc = kPairs.rc[min(e0 + j, S::NL - 1)];
          rr[j] = rc >> 8;
          cc[j] = rc & 255;
          g[j] = GEO(min(rr[j], M - 1));
          h[j] = GEO(cc[j]);
        }
        F::df v[4];
        if constexpr (kPacked<COV>) {
          namespace G = nngp_df2;
#pragma unroll
          for (int t = 0; t < 2; t++) {
            const int a = 2 * t, b2 = 2 * t + 1;
            // hi parts on the common grid: their difference is exact
            G::df2 ex, ey;
            G::fast_two_sum(G::sub(G::pack(g[a].x, g[b2].x), G::pack(h[a].x, h[b2].x)),
                            G::sub(G::pack(g[a].z, g[b2].z), G::pack(h[a].z, h[b2].z)), ex.h, ex.l);
            G::fast_two_sum(G::sub(G::pack(g[a].y, g[b2].y), G::pack(h[a].y, h[b2].y)),
                            G::sub(G::pack(g[a].w, g[b2].w), G::pack(h[a].w, h[b2].w)), ey.h, ey.l);
            const G::df2 r = cov_df2<COV>(G::sumsq(ex, ey), ck, tab);
            v[a] = F::df{G::first(r.h), G::first(r.l)};
            v[b2] = F::df{G::second(r.h), G::second(r.l)};
          }
        } else {
#pragma unroll
          for (int j = 0; j < 4; j++) {
            // hi parts on the common grid: their difference is exact
            F::df ex, ey;
            F::fast_two_sum(__fsub_rn(g[j].x, h[j].x), __fsub_rn(g[j].z, h[j].z), ex.h, ex.l);
            F::fast_two_sum(__fsub_rn(g[j].y, h[j].y), __fsub_rn(g[j].w, h[j].w), ey.h, ey.l);
            v[j] = cov_df<COV>(F::sumsq(ex.h, ex.l, ey.h, ey.l), ck, tab, cpp);
          }
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
          if (e0 + j < S::NL) {
            const bool live = rr[j] < mi;
            const float vh = live ? v[j].h : 0.0f, vl = live ? v[j].l : 0.0f;
            CS(e0 + j) = vh;  // e == lidx(r, c)
            if constexpr (TM) {
              tm_st(tm0 + 16u * rr[j] + cc[j], vl);
              tm_st(tm0 + 16u * cc[j] + rr[j], vl);
            } else {
              CLL(e0 + j) = vl;
            }
          }
        }
      }
    }
#pragma unroll 1
    for (int r = mi; r < M; r++) {  // identity padding of c
      CS(S::NL + r) = 0.0f;
      CLC(r) = 0.0f;
    }
    if constexpr (TM) tm_wait_st();

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
      // C[r][c] b[c] over c, even and odd c in the two halves of a packed compensated sum (the
      // 16-neighbor bound keeps the scalar sum: its registers are full)
      namespace G = nngp_df2;
      float lo_row[16];
      if constexpr (TM) tm_ld16(tm0 + 16u * r, lo_row);
      if constexpr (M >= 16) {
        float shs = 0.0f, sls = 0.0f;
#pragma unroll
        for (int c = 0; c < M; c++) {
          float eh, el;
          if (c == r) {
            eh = (r < mi) ? Sd.h : 1.0f;
            el = (r < mi) ? Sd.l : 0.0f;
          } else {
            eh = c < r ? CSV(lidx(r, c)) : CSV(lidx(c, r));
            if constexpr (TM) el = lo_row[c];
            else el = c < r ? CLLV(lidx(r, c)) : CLLV(lidx(c, r));
          }
          F::dot2_acc(shs, sls, eh, b[c]);
          sls = fmaf(el, b[c], sls);
        }
        const float res = __fadd_rn(__fsub_rn(__fsub_rn(CSV(S::NL + r), shs), sls), CLCV(r));
        w[r] = (res - w[r]) * D[r];
#pragma unroll
        for (int j = r + 1; j < M; j++) w[j] = fmaf(L[lidx(j, r)], w[r], w[j]);
        continue;
      }
      G::p2 sh = 0ull, sl = 0ull;
#pragma unroll
      for (int c0 = 0; c0 < M; c0 += 2) {
        float eh[2], el[2], bc[2];
#pragma unroll
        for (int u = 0; u < 2; u++) {
          const int c = c0 + u;
          eh[u] = el[u] = bc[u] = 0.0f;
          if (c < M) {
            bc[u] = b[c];
            if (c == r) {
              eh[u] = (r < mi) ? Sd.h : 1.0f;
              el[u] = (r < mi) ? Sd.l : 0.0f;
            } else {
              eh[u] = c < r ? CSV(lidx(r, c)) : CSV(lidx(c, r));
              if constexpr (TM) el[u] = lo_row[c];
              else el[u] = c < r ? CLLV(lidx(r, c)) : CLLV(lidx(c, r));
            }
          }
        }
        const G::p2 b2 = G::pack(bc[0], bc[1]);
        G::dot2_acc(sh, sl, G::pack(eh[0], eh[1]), b2);
        sl = G::fma(G::pack(el[0], el[1]), b2, sl);
      }
      const F::df cb = G::fold(sh, sl);
      const float res = __fadd_rn(__fsub_rn(__fsub_rn(CSV(S::NL + r), cb.h), cb.l), CLCV(r));
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
    float bmax = 0.0f, wmax = 0.0f;
    F::df bc;
    {
      namespace G = nngp_df2;
      G::p2 dh = 0ull, dl = 0ull;
#pragma unroll
      for (int k0 = 0; k0 < M; k0 += 2) {
        const int k1 = k0 + 1 < M ? k0 + 1 : k0;
        const float z1 = k0 + 1 < M ? 1.0f : 0.0f;  // the odd half of the last step is empty
        const G::p2 ch = G::pack(CSV(S::NL + k0), z1 * CSV(S::NL + k1));
        const G::p2 cl = G::pack(CLCV(k0), z1 * CLCV(k1));
        const G::p2 bb = G::pack(b[k0], z1 * b[k1]), ww = G::pack(w[k0], z1 * w[k1]);
        G::dot2_acc(dh, dl, bb, ch);
        dl = G::fma(ww, ch, G::fma(bb, cl, dl));
      }
      bc = G::fold(dh, dl);
#pragma unroll
      for (int k = 0; k < M; k++) {
        bmax = fmaxf(bmax, fabsf(b[k]));
        wmax = fmaxf(wmax, fabsf(w[k]));
      }
    }
    const F::df Fd = F::sub(Sd, F::norm(bc.h, bc.l));
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
      // r_v = V_iv - sum_k B_k V_nb(k)v, staged at slots 2v, 2v + 1.  Four columns at a time:
      // all of a group's gathers are issued before their first use (one memory round trip
      // per group instead of one per column; the factor's registers are free by now)
#pragma unroll 1
      for (int v0 = 0; v0 < nv; v0 += 4) {
        float2 q[4][M], vi[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
#pragma unroll
          for (int k = 0; k < M; k++)
            q[j][k] = (k < mi && v0 + j < nv) ? Vf[(size_t)nb[k] * nv + v0 + j] : make_float2(0.f, 0.f);
          vi[j] = (active && v0 + j < nv) ? Vf[(size_t)i * nv + v0 + j] : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
          if (v0 + j < nv) {
            namespace G = nngp_df2;
            G::p2 ah = 0ull, al = 0ull;
#pragma unroll
            for (int k0 = 0; k0 < M; k0 += 2) {
              const int k1 = k0 + 1 < M ? k0 + 1 : k0;
              const float z1 = k0 + 1 < M ? 1.0f : 0.0f;
              const G::p2 bb = G::pack(b[k0], z1 * b[k1]), ww = G::pack(w[k0], z1 * w[k1]);
              const G::p2 qh = G::pack(q[j][k0].x, q[j][k1].x), ql = G::pack(q[j][k0].y, q[j][k1].y);
              G::dot2_acc(ah, al, bb, qh);
              al = G::fma(bb, ql, G::fma(ww, qh, al));
            }
            const F::df s2 = G::fold(ah, al);
            const F::df rv = F::sub(F::df{vi[j].x, vi[j].y}, F::norm(s2.h, s2.l));
            CS(2 * (v0 + j)) = rv.h;
            CS(2 * (v0 + j) + 1) = rv.l;
          }
        }
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
  if constexpr (TM) {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0)
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tm_alloc_base), "r"(tm_cols));
  }
#undef CS
#undef CSV
#undef CLC
#undef CLCV
#undef CLL
#undef CLLV
#undef GEO
}

template <int M, bool TM>
constexpr size_t smem_bytes(int wpb) {
  return Shape<M, TM>::WARP_BYTES * (size_t)wpb;
}

// Raises the kernel's dynamic shared-memory limit to what the largest block (MAX_WPB warps)
// needs (once per device; the attribute is per device).
template <int M, int MODE, int COV, bool TM>
cudaError_t configure(int device) {
  static bool configured[64] = {};
  const int dev = device & 63;
  if (configured[dev]) return cudaSuccess;
  const cudaError_t e = cudaFuncSetAttribute(bfr_kernel<M, MODE, COV, TM>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem_bytes<M, TM>(Shape<M, TM>::MAX_WPB));
  if (e == cudaSuccess) configured[dev] = true;
  return e;
}

template <int M, int MODE, int COV, bool TM>
int launch_tm(nngp_ctx *ctx, const BFPlan *pl, int wpb, int grid, int t0, int t1) {
  NNGP_CUDA_TRY(ctx, (configure<M, MODE, COV, TM>(ctx->device)));
  if (t1 <= t0) return NNGP_OK;
  bfr_kernel<M, MODE, COV, TM><<<grid, 32 * wpb, smem_bytes<M, TM>(wpb), ctx->stream>>>(
      pl->d_datas, pl->d_thetas, pl->d_jobs, pl->njobs, t0, t1, pl->nv);
  NNGP_LAUNCH_CHECK(ctx);
  return NNGP_OK;
}

// Launches the kernel on the plan's primary tiles [t0, t1) with wpb warps per block and `grid`
// blocks; tm selects the variant with the covariance's lo parts in tensor memory (wpb 4 or 8).
template <int M, int MODE, int COV>
int launch_reg(nngp_ctx *ctx, const BFPlan *pl, int wpb, int grid, int t0, int t1, int tm) {
  if constexpr (nngp_bfr_has_tm(M)) {
    if (tm) {
      if (wpb != 4 && wpb != 8)
        return nngp_fail(ctx, NNGP_ERR_ARG, "the tensor-memory B/F kernel runs 4 or 8 warps per block");
      return launch_tm<M, MODE, COV, true>(ctx, pl, wpb, grid, t0, t1);
    }
  }
  return launch_tm<M, MODE, COV, false>(ctx, pl, wpb, grid, t0, t1);
}

// Blocks of wpb warps one SM holds at once (on the current device); 0 when the shape is not
// available for this variant.
template <int M, int MODE, int COV>
int occupancy(int wpb, int tm) {
  int dev = 0, blocks = 0;
  cudaGetDevice(&dev);
  if constexpr (nngp_bfr_has_tm(M)) {
    if (tm) {
      if (wpb != 4 && wpb != 8) return 0;
      if (configure<M, MODE, COV, true>(dev) != cudaSuccess) return 0;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, bfr_kernel<M, MODE, COV, true>, 32 * wpb,
                                                        smem_bytes<M, true>(wpb)) != cudaSuccess)
        return 0;
      // at most 512 tensor-memory columns per SM: 256 per four warps
      const int tm_cap = wpb == 8 ? 1 : 2;
      return blocks < tm_cap ? blocks : tm_cap;
    }
  }
  if (tm || wpb > Shape<M, false>::MAX_WPB) return 0;
  if (configure<M, MODE, COV, false>(dev) != cudaSuccess) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, bfr_kernel<M, MODE, COV, false>, 32 * wpb,
                                                    smem_bytes<M, false>(wpb)) != cudaSuccess)
    return 0;
  return blocks;
}

}  // namespace nngp_bfr
