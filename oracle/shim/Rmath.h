/* Minimal stand-in for R's <Rmath.h> (test oracle only). rnorm/runif read
 * host-fed streams; gammafn and bessel_k_ex are this project's own code. */
#ifndef NNGP_SHIM_RMATH_H
#define NNGP_SHIM_RMATH_H
#include <math.h>
#ifndef M_PI
#define M_PI 3.141592653589793238462643383280
#endif
#ifdef __cplusplus
extern "C" {
#endif
double rnorm(double mu, double sigma);
double runif(double a, double b);
double norm_rand(void);
double unif_rand(void);
double gammafn(double x);
double bessel_k_ex(double x, double alpha, double expo, double *bk);
#ifdef __cplusplus
}
#endif
#endif
