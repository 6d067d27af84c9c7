// Double-float covariance evaluation shared by the FP32R B/F kernels (nngp_bfr_kernel.cuh,
// thread per location for m <= 16; nngp_bfw_kernel.cuh, warp per location for 16 < m <= 32):
// the correlation functions of the reference's spCor (src/util.cpp:208-245) in float pairs on the
// FP32 pipe, and the error-control thresholds both kernels apply.
#pragma once
#include <cuda_runtime.h>
#include "nngp_df.cuh"
#include "nngp_internal.h"
#include "nngp_math.cuh"

namespace nngp_bfr {

// Error control after the one refinement step (the error left in B is about q^2 |b|, q the
// float solve's relative correction |delta| / |b|): a location is re-solved in FP64 when
// q^2 (sigma^2 + tau^2) exceeds kTolF F, or when F < kMinFRel (sigma^2 + tau^2).
constexpr float kTolF = 1e-8f;    // accepted F error estimate, relative to F
constexpr float kMinFRel = 1e-6f;  // smaller F (relative to sigma^2 + tau^2) goes to FP64

// Per-tile constants of the correlation function in double-float.
struct CorDF {
  nngp_df::df K;   // exp argument scale in units of ln2/32: -phi 32/ln2 (times d), gaussian -phi^2 32/ln2 (times d^2)
  nngp_df::df P;   // phi
  nngp_df::df S2;  // sigma^2
  int halfk;
  int model;
};

// The warp's table (floats, in shared memory): sigma^2 2^(j/32) for j < 32 (hi at j, lo at
// 32 + j), then the Matern nu = k + 1/2 polynomial coefficients (hi at 64 + j, lo at 80 + j,
// j <= 8).  Shared rather than in registers: the coefficients would hold 18 registers for the
// whole pass (the compiler puts them on the stack instead).
constexpr int kTabFloats = 96;
constexpr int kTabPolyHi = 64;
constexpr int kTabPolyLo = 80;

// Reads the parameter set's prepared double-float constants (cov_prepare): no FP64 here.
template <int COV>
__device__ __forceinline__ CorDF cor_prepare(const CovParams *cp) {
  CorDF k{};
  k.model = COV == NNGP_COV_ANY ? cp->model : COV;
  k.halfk = cp->halfk;
  k.K = nngp_df::df{cp->dfK[0], cp->dfK[1]};
  k.P = nngp_df::df{cp->dfPhi[0], cp->dfPhi[1]};
  k.S2 = nngp_df::df{cp->dfS2[0], cp->dfS2[1]};
  return k;
}

// Writes the warp's table (kTabFloats floats at tab) for parameter set cp; every lane of the
// warp takes part, the caller synchronises the warp before the first read.
template <int COV>
__device__ __forceinline__ void fill_tab(float *tab, const CorDF &k, const CovParams *cp, int lane) {
  const float2 t2 = nngp_df::kExp2Tab[lane];
  const nngp_df::df e = nngp_df::mul(k.S2, nngp_df::df{t2.x, t2.y});
  tab[lane] = e.h;
  tab[32 + lane] = e.l;
  if (COV == NNGP_COV_MAT_HALF || COV == NNGP_COV_ANY) {
    if (lane < 9) {
      tab[kTabPolyHi + lane] = cp->dfPoly[lane][0];
      tab[kTabPolyLo + lane] = cp->dfPoly[lane][1];
    }
  }
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
  F::df s{tab[kTabPolyHi + k.halfk], tab[kTabPolyLo + k.halfk]};
  for (int j = k.halfk - 1; j >= 0; j--) s = F::add(F::mul(s, x), F::df{tab[kTabPolyHi + j], tab[kTabPolyLo + j]});
  return F::mul(E, s);
}

// Models whose correlation is one exp of a scaled distance (times a polynomial for the
// half-integer Matern) take the packed path: two pairs per instruction stream (Blackwell
// f32x2), the same arithmetic as cov_df on each half.
template <int COV>
constexpr bool kPacked = COV == NNGP_COV_EXP || COV == NNGP_COV_GAU || COV == NNGP_COV_MAT_HALF;

template <int COV>
__device__ __forceinline__ nngp_df2::df2 cov_df2(nngp_df2::df2 d2, const CorDF &k, const float *tab) {
  namespace G = nngp_df2;
  const G::df2 K{G::splat(k.K.h), G::splat(k.K.l)};
  if constexpr (COV == NNGP_COV_GAU) return G::exp_u(G::mul(K, d2), tab);
  const G::df2 d = G::sqrt(d2);
  const G::df2 E = G::exp_u(G::mul(K, d), tab);
  if constexpr (COV == NNGP_COV_MAT_HALF) {
    if (k.halfk <= 0) return E;
    const G::df2 x = G::mul(G::df2{G::splat(k.P.h), G::splat(k.P.l)}, d);
    G::df2 s{G::splat(tab[kTabPolyHi + k.halfk]), G::splat(tab[kTabPolyLo + k.halfk])};
    for (int j = k.halfk - 1; j >= 0; j--)
      s = G::add(G::mul(s, x), G::df2{G::splat(tab[kTabPolyHi + j]), G::splat(tab[kTabPolyLo + j])});
    return G::mul(E, s);
  }
  return E;
}

}  // namespace nngp_bfr
