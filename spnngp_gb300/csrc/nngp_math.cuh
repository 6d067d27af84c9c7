// Device math of the NNGP correlation models (reference src/util.cpp:208-245).
//
//   model 0 exponential  exp(-phi d)
//   model 1 spherical    1 - 1.5 phi d + 0.5 (phi d)^3 for 0 < d <= 1/phi, 0 beyond, 1 at 0
//   model 2 matern       (phi d)^nu / (2^(nu-1) Gamma(nu)) K_nu(phi d), 1 at 0
//   model 3 gaussian     exp(-(phi d)^2)
//
// K_nu (FP64) uses Temme's series for x <= 2 and Steed's continued fraction
// CF2 for x > 2 on mu = nu - round(nu), then forward recurrence, the published
// method R's own bessel_k_ex also builds on.  Matern with nu = k + 1/2
// (k <= 8) uses the exact closed form exp(-x) * poly(x) prepared in CovParams.
#pragma once
#include <cuda_runtime.h>
#include "nngp_internal.h"

// 1/Gamma(z) = sum_{k=1}^{26} c_k z^k (Abramowitz & Stegun 6.1.34)
__device__ __constant__ double NNGP_RGAMMA[26] = {
    1.0000000000000000,  0.5772156649015329,  -0.6558780715202538, -0.0420026350340952,
    0.1665386113822915,  -0.0421977345555443, -0.0096219715278770, 0.0072189432466630,
    -0.0011651675918591, -0.0002152416741149, 0.0001280502823882,  -0.0000201348547807,
    -0.0000012504934821, 0.0000011330272320,  -0.0000002056338417, 0.0000000061160950,
    0.0000000050020075,  -0.0000000011812746, 0.0000000001043427,  0.0000000000077823,
    -0.0000000000036968, 0.0000000000005100,  -0.0000000000000206, -0.0000000000000054,
    0.0000000000000014,  0.0000000000000001};

__device__ inline double nngp_bessel_k(double x, double nu) {
  if (!(x > 0.0)) return (x == 0.0) ? __longlong_as_double(0x7ff0000000000000ll) : nan("");
  if (nu < 0.0) nu = -nu;
  const int nl = (int)(nu + 0.5);
  const double mu = nu - nl;
  const double mu2 = mu * mu;
  const double xi = 1.0 / x, xi2 = 2.0 * xi;
  const double eps = 1e-16;
  double kmu, kmu1;
  if (x <= 2.0) {
    double even = 0.0, odd = 0.0;
#pragma unroll
    for (int k = 26; k >= 1; k--) {
      if (k % 2 == 0) even = even * mu2 + NNGP_RGAMMA[k - 1];
      else odd = odd * mu2 + NNGP_RGAMMA[k - 1];
    }
    const double g1 = -even, g2 = odd;
    const double rg_plus = g2 - mu * g1, rg_minus = g2 + mu * g1;
    const double pimu = 3.141592653589793 * mu;
    const double fact = (fabs(pimu) < eps) ? 1.0 : pimu / sin(pimu);
    const double d = -log(0.5 * x);
    const double sigma = mu * d;
    const double fact2 = (fabs(sigma) < eps) ? 1.0 : sinh(sigma) / sigma;
    double f = fact * (g1 * cosh(sigma) + g2 * fact2 * d);
    const double es = exp(sigma);
    double p = 0.5 * es / rg_plus;
    double q = 0.5 / (es * rg_minus);
    double c = 1.0;
    const double x2q = 0.25 * x * x;
    double sum = f, sum1 = p;
#pragma unroll 1
    for (int k = 1; k < 200; k++) {
      f = (k * f + p + q) / (k * k - mu2);
      c *= x2q / k;
      p /= (k - mu);
      q /= (k + mu);
      const double del = c * f;
      sum += del;
      sum1 += c * (p - k * f);
      if (fabs(del) < fabs(sum) * eps) break;
    }
    kmu = sum;
    kmu1 = sum1 * xi2;
  } else {
    double b = 2.0 * (1.0 + x);
    double d = 1.0 / b;
    double h = d, delh = d;
    double q1 = 0.0, q2 = 1.0;
    const double a1 = 0.25 - mu2;
    double q = a1, c = a1, a = -a1;
    double s = 1.0 + q * delh;
#pragma unroll 1
    for (int k = 2; k < 2000; k++) {
      a -= 2.0 * (k - 1);
      c = -a * c / k;
      const double qn = (q1 - b * q2) / a;
      q1 = q2;
      q2 = qn;
      q += c * qn;
      b += 2.0;
      d = 1.0 / (b + a * d);
      delh = (b * d - 1.0) * delh;
      h += delh;
      const double dels = q * delh;
      s += dels;
      if (fabs(dels / s) < eps) break;
    }
    h = a1 * h;
    kmu = sqrt(3.141592653589793 / (2.0 * x)) * exp(-x) / s;
    kmu1 = kmu * (mu + x + 0.5 - h) * xi;
  }
#pragma unroll 1
  for (int k = 1; k <= nl; k++) {
    const double t = (mu + k) * xi2 * kmu1 + kmu;
    kmu = kmu1;
    kmu1 = t;
  }
  return kmu;
}

// Matern correlation at x = phi * d > 0.
__device__ inline double nngp_matern_d(double x, const CovParams &cp) {
  if (cp.halfk >= 0) {
    double s = cp.poly[cp.halfk];
    for (int j = cp.halfk - 1; j >= 0; j--) s = s * x + cp.poly[j];
    return exp(-x) * s;
  }
  return cp.mconst * pow(x, cp.nu) * nngp_bessel_k(x, cp.nu);
}

// COV (NNGP_COV_* of nngp_internal.h) selects the formula at compile time: a kernel compiled
// for one model carries no switch and no dead branches in its unrolled covariance build.

// Matern with nu = k + 1/2: exp(-x) * poly(x), x = phi d.
template <typename R>
__device__ inline R nngp_matern_half(R x, const CovParams &cp) {
  R s = (R)cp.poly[cp.halfk];
#pragma unroll 1
  for (int j = cp.halfk - 1; j >= 0; j--) s = s * x + (R)cp.poly[j];
  if constexpr (sizeof(R) == 4) return expf(-x) * s;
  else return exp(-x) * s;
}

// Correlation (no sigma^2) at distance d, FP64.
template <int COV = NNGP_COV_ANY>
__device__ inline double nngp_cor_d(double d, const CovParams &cp) {
  const int model = COV == NNGP_COV_ANY ? cp.model : COV;
  switch (model) {
    case 0:
      return exp(-cp.phi * d);
    case 1: {
      const double inv = 1.0 / cp.phi;
      if (d > 0 && d <= inv) {
        const double t = cp.phi * d;
        return 1.0 - 1.5 * t + 0.5 * (t * t * t);
      }
      return (d >= inv) ? 0.0 : 1.0;
    }
    case 2: {
      const double x = d * cp.phi;
      if (!(x > 0.0)) return 1.0;
      if constexpr (COV == NNGP_COV_ANY) return nngp_matern_d(x, cp);
      return nngp_matern_half(x, cp);
    }
    default: {
      const double t = cp.phi * d;
      return exp(-(t * t));
    }
  }
}

// Correlation in FP32 from a squared distance d2 (the refined path).  Matern at a
// general nu goes through the FP64 Bessel evaluation (NNGP_COV_ANY only).
template <int COV = NNGP_COV_ANY>
__device__ inline float nngp_cor_f(float d2, const CovParams &cp, float phif) {
  const int model = COV == NNGP_COV_ANY ? cp.model : COV;
  switch (model) {
    case 0:
      return expf(-phif * sqrtf(d2));
    case 1: {
      const float d = sqrtf(d2);
      const float t = phif * d;
      if (d > 0.0f && t <= 1.0f) return 1.0f - 1.5f * t + 0.5f * (t * t * t);
      return (t >= 1.0f) ? 0.0f : 1.0f;
    }
    case 2: {
      const float x = phif * sqrtf(d2);
      if (!(x > 0.0f)) return 1.0f;
      if constexpr (COV == NNGP_COV_ANY) {
        if (cp.halfk < 0) return (float)nngp_matern_d((double)x, cp);
      }
      return nngp_matern_half(x, cp);
    }
    default:
      return expf(-(phif * phif) * d2);
  }
}
