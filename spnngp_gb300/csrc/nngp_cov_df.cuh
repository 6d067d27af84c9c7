// Double-float covariance evaluation shared by the FP32R B/F kernels (nngp_bfr_kernel.cuh,
// thread per location for m <= 16; nngp_bfw_kernel.cuh, warp per location for 16 < m <= 32):
// the correlation functions of the reference's spCor (src/util.cpp:208-245) in float pairs on the
// FP32 pipe, the error-control thresholds both kernels apply, and the tile -> job lookup.
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
  float pfh[9], pfl[9];  // matern nu = k + 1/2: polynomial coefficients
  int halfk;
  int model;
};

// Reads the parameter set's prepared double-float constants (cov_prepare): no FP64 here.
template <int COV>
__device__ __forceinline__ CorDF cor_prepare(const CovParams *cp) {
  CorDF k{};
  k.model = COV == NNGP_COV_ANY ? cp->model : COV;
  k.halfk = cp->halfk;
  k.K = nngp_df::df{cp->dfK[0], cp->dfK[1]};
  k.P = nngp_df::df{cp->dfPhi[0], cp->dfPhi[1]};
  k.S2 = nngp_df::df{cp->dfS2[0], cp->dfS2[1]};
  if (COV == NNGP_COV_MAT_HALF || (COV == NNGP_COV_ANY && k.model == 2 && k.halfk >= 0)) {
#pragma unroll
    for (int j = 0; j < 9; j++) {
      k.pfh[j] = cp->dfPoly[j][0];
      k.pfl[j] = cp->dfPoly[j][1];
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

// Models whose correlation is one exp of a scaled distance take the packed path: two pairs per
// instruction stream (Blackwell f32x2), same arithmetic as cov_df.
template <int COV>
constexpr bool kPacked = COV == NNGP_COV_EXP || COV == NNGP_COV_GAU;

template <int COV>
__device__ __forceinline__ nngp_df2::df2 cov_df2(nngp_df2::df2 d2, const CorDF &k, const float *tab) {
  namespace G = nngp_df2;
  const G::df2 K{G::splat(k.K.h), G::splat(k.K.l)};
  if constexpr (COV == NNGP_COV_GAU) return G::exp_u(G::mul(K, d2), tab);
  else return G::exp_u(G::mul(K, G::sqrt(d2)), tab);
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

}  // namespace nngp_bfr
