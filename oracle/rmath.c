/*
 * TEST ORACLE ONLY -- never linked into the product library.
 *
 * The pieces of R's Rmath / sort library that the spNNGP hot path calls and
 * that are not part of the reference tree (R >= 3.5.0, DESCRIPTION:11; exact
 * version unpinned), restated here from their published algorithms:
 *
 *  or_bessel_k       K_nu(x), unscaled -- R's bessel_k_ex(x, nu, 1.0, bk) as
 *                    called at src/util.cpp:234. Temme's (1975) series for
 *                    x <= 2 and Steed's continued fraction CF2 (Thompson &
 *                    Barnett 1986) for x > 2 on mu = nu - round(nu), then the
 *                    forward recurrence K_{mu+k+1} = 2(mu+k)/x K_{mu+k} + K_{mu+k-1}.
 *                    Gamma1/Gamma2 of Temme's series come from the power series
 *                    of 1/Gamma(z) (Abramowitz & Stegun 6.1.34).
 *  or_gammafn        Gamma(x) (src/util.cpp:234), via the C library tgamma.
 *  or_rsort_with_index
 *                    R's rsort_with_index (src/nn.cpp:104,176,197,243): Shell
 *                    sort with Knuth's 3h+1 gaps, first gap the smallest one
 *                    above n/9, NaN last, moving an element only past strictly
 *                    greater keys.  The tie order of the neighbor lists depends
 *                    on exactly this gap sequence and comparison, so the GPU
 *                    kernels use the same sequence.
 *  streams           R's rnorm / runif (src/rNNGP.cpp:327-333,349,
 *                    src/util.cpp:36) read host-fed streams: rnorm(mu, sd) is
 *                    mu + sd*z with z the next normal; it consumes nothing when
 *                    sd == 0 or mu is not finite, and runif(a, b) consumes
 *                    nothing when a == b (R's argument rules).
 */
#include <math.h>
#include <stddef.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* 1/Gamma(z) = sum_{k=1}^{26} c_k z^k  (Abramowitz & Stegun 6.1.34) */
static const double RGAMMA_SERIES[26] = {
    1.0000000000000000,  0.5772156649015329,  -0.6558780715202538, -0.0420026350340952,
    0.1665386113822915,  -0.0421977345555443, -0.0096219715278770, 0.0072189432466630,
    -0.0011651675918591, -0.0002152416741149, 0.0001280502823882,  -0.0000201348547807,
    -0.0000012504934821, 0.0000011330272320,  -0.0000002056338417, 0.0000000061160950,
    0.0000000050020075,  -0.0000000011812746, 0.0000000001043427,  0.0000000000077823,
    -0.0000000000036968, 0.0000000000005100,  -0.0000000000000206, -0.0000000000000054,
    0.0000000000000014,  0.0000000000000001};

/* Temme's Gamma1(mu) = (1/G(1-mu) - 1/G(1+mu)) / (2 mu) and Gamma2(mu) = (1/G(1-mu) + 1/G(1+mu)) / 2
 * for |mu| <= 1/2, from the odd/even parts of the 1/Gamma series. */
static void temme_gamma12(double mu, double *g1, double *g2) {
  const double mu2 = mu * mu;
  double even = 0.0, odd = 0.0;
  /* even k (c_2, c_4, ...) give -Gamma1; odd k (c_1, c_3, ...) give Gamma2; Horner from the top */
  for (int k = 26; k >= 1; k--) {
    if (k % 2 == 0) even = even * mu2 + RGAMMA_SERIES[k - 1];
    else odd = odd * mu2 + RGAMMA_SERIES[k - 1];
  }
  *g1 = -even;
  *g2 = odd;
}

double or_bessel_k(double x, double nu) {
  if (isnan(x) || isnan(nu)) return x + nu;
  if (x < 0.0) return NAN;
  if (x == 0.0) return INFINITY;
  if (nu < 0.0) nu = -nu;
  const int nl = (int)(nu + 0.5);
  const double mu = nu - nl; /* |mu| <= 1/2 */
  const double mu2 = mu * mu;
  const double xi = 1.0 / x, xi2 = 2.0 * xi;
  const double eps = 1e-16;
  double kmu, kmu1;
  if (x <= 2.0) {
    double g1, g2;
    temme_gamma12(mu, &g1, &g2);
    const double rg_plus = g2 - mu * g1;  /* 1/Gamma(1+mu) */
    const double rg_minus = g2 + mu * g1; /* 1/Gamma(1-mu) */
    const double pimu = M_PI * mu;
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
    for (int k = 1; k < 10000; k++) {
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
    for (int k = 2; k < 100000; k++) {
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
    kmu = sqrt(M_PI / (2.0 * x)) * exp(-x) / s;
    kmu1 = kmu * (mu + x + 0.5 - h) * xi;
  }
  for (int k = 1; k <= nl; k++) {
    const double t = (mu + k) * xi2 * kmu1 + kmu;
    kmu = kmu1;
    kmu1 = t;
  }
  return kmu;
}

double or_gammafn(double x) { return tgamma(x); }

static int cmp_nan_last(double a, double b) {
  const int na = isnan(a), nb = isnan(b);
  if (na && nb) return 0;
  if (na) return 1;
  if (nb) return -1;
  return (a < b) ? -1 : ((a > b) ? 1 : 0);
}

void or_rsort_with_index(double *x, int *idx, int n) {
  int gap = 1;
  while (gap <= n / 9) gap = 3 * gap + 1;
  for (; gap > 0; gap /= 3) {
    for (int i = gap; i < n; i++) {
      const double key = x[i];
      const int tag = idx[i];
      int j = i;
      while (j >= gap && cmp_nan_last(x[j - gap], key) > 0) {
        x[j] = x[j - gap];
        idx[j] = idx[j - gap];
        j -= gap;
      }
      x[j] = key;
      idx[j] = tag;
    }
  }
}

/* ---- host-fed random streams ---- */
static const double *g_norm = NULL, *g_unif = NULL;
static long g_norm_len = 0, g_unif_len = 0, g_norm_pos = 0, g_unif_pos = 0;
static int g_stream_overrun = 0;

void or_stream_set(const double *normals, long n_norm, const double *unifs, long n_unif) {
  g_norm = normals; g_norm_len = n_norm; g_norm_pos = 0;
  g_unif = unifs; g_unif_len = n_unif; g_unif_pos = 0;
  g_stream_overrun = 0;
}
void or_stream_used(long *n_norm, long *n_unif, int *overrun) {
  *n_norm = g_norm_pos; *n_unif = g_unif_pos; *overrun = g_stream_overrun;
}
double or_next_normal(void) {
  if (g_norm_pos >= g_norm_len) { g_stream_overrun = 1; return 0.0; }
  return g_norm[g_norm_pos++];
}
double or_next_unif(void) {
  if (g_unif_pos >= g_unif_len) { g_stream_overrun = 1; return 0.5; }
  return g_unif[g_unif_pos++];
}
double or_rnorm(double mu, double sd) {
  if (isnan(mu) || !isfinite(sd) || sd < 0.0) return NAN;
  if (sd == 0.0 || !isfinite(mu)) return mu;
  return mu + sd * or_next_normal();
}
double or_runif(double a, double b) {
  if (!isfinite(a) || !isfinite(b) || b < a) return NAN;
  if (a == b) return a;
  return a + (b - a) * or_next_unif();
}
