// Small dense FP64 routines for the p x p algebra of the beta / conjugate steps
// (reference src/rNNGP.cpp:288-291, src/cNNGP.cpp:235-239, src/util.cpp:28-41),
// one thread per problem, column-major with leading dimension p, lower
// triangle as LAPACK's uplo = 'L'.
#pragma once
#include <cuda_runtime.h>

// Lower Cholesky in place; returns false on a non-positive pivot.
__device__ inline bool small_potrf(double *a, int p) {
  for (int j = 0; j < p; j++) {
    double d = a[j * p + j];
    for (int k = 0; k < j; k++) d -= a[k * p + j] * a[k * p + j];
    if (!(d > 0.0)) return false;
    d = sqrt(d);
    a[j * p + j] = d;
    const double r = 1.0 / d;
    for (int i = j + 1; i < p; i++) {
      double s = a[j * p + i];
      for (int k = 0; k < j; k++) s -= a[k * p + i] * a[k * p + j];
      a[j * p + i] = s * r;
    }
  }
  return true;
}

// Inverse from the lower factor (lower triangle of inv(A) overwrites the factor).
__device__ inline void small_potri(double *a, int p) {
  for (int j = p - 1; j >= 0; j--) {
    a[j * p + j] = 1.0 / a[j * p + j];
    const double ajj = -a[j * p + j];
    for (int c = p - 1; c > j; c--) {
      const double t = a[j * p + c];
      if (t != 0.0) {
        for (int r = p - 1; r > c; r--) a[j * p + r] += t * a[c * p + r];
        a[j * p + c] = t * a[c * p + c];
      }
    }
    for (int r = j + 1; r < p; r++) a[j * p + r] *= ajj;
  }
  for (int j = 0; j < p; j++)
    for (int i = j; i < p; i++) {
      double s = 0.0;
      for (int k = i; k < p; k++) s += a[i * p + k] * a[j * p + k];
      a[j * p + i] = s;
    }
}

// y = A x from the lower triangle.
__device__ inline void small_symv(const double *a, int p, const double *x, double *y) {
  for (int i = 0; i < p; i++) {
    double s = 0.0;
    for (int k = 0; k < p; k++) s += ((k <= i) ? a[k * p + i] : a[i * p + k]) * x[k];
    y[i] = s;
  }
}
