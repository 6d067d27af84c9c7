/*
 * TEST ORACLE ONLY -- never linked into the product library.
 *
 * The dense BLAS/LAPACK subset that the spNNGP hot path calls (reference
 * src/rNNGP.cpp:86-89, src/cNNGP.cpp:59-62,235-239,273-298,
 * src/rNNGPPredict.cpp:166-181, src/util.cpp:39-40), written here from the
 * textbook (unblocked, column-major, reference-BLAS argument conventions) so
 * that both the oracle restatement and the shim build of the reference's own
 * sources have the same small-matrix arithmetic without an external LAPACK.
 *
 *   dpotrf  lower Cholesky, Cholesky-Banachiewicz column sweep (LAPACK dpotf2)
 *   dpotri  inverse from the factor: inv(L) (dtrti2) then inv(L)' inv(L) (dlauu2)
 *   dsymv   y = alpha*A*x + beta*y from the lower triangle
 *   dgemv   'N' and 'T'
 *   dtrmv   lower / no-transpose / non-unit
 *   ddot, dcopy, daxpy
 *
 * Only uplo = 'L' is implemented, which is the only form the hot path uses.
 */
#include <math.h>
#include <stddef.h>

#define A_(i, j) a[(size_t)(j) * (size_t)ld + (size_t)(i)]

double ddot_(const int *n, const double *x, const int *incx, const double *y, const int *incy) {
  double s = 0.0;
  int ix = *incx >= 0 ? 0 : (1 - *n) * *incx;
  int iy = *incy >= 0 ? 0 : (1 - *n) * *incy;
  for (int k = 0; k < *n; k++, ix += *incx, iy += *incy) s += x[ix] * y[iy];
  return s;
}

void dcopy_(const int *n, const double *x, const int *incx, double *y, const int *incy) {
  int ix = *incx >= 0 ? 0 : (1 - *n) * *incx;
  int iy = *incy >= 0 ? 0 : (1 - *n) * *incy;
  for (int k = 0; k < *n; k++, ix += *incx, iy += *incy) y[iy] = x[ix];
}

void daxpy_(const int *n, const double *alpha, const double *x, const int *incx, double *y,
            const int *incy) {
  if (*alpha == 0.0) return;
  int ix = *incx >= 0 ? 0 : (1 - *n) * *incx;
  int iy = *incy >= 0 ? 0 : (1 - *n) * *incy;
  for (int k = 0; k < *n; k++, ix += *incx, iy += *incy) y[iy] += *alpha * x[ix];
}

void dgemv_(const char *trans, const int *m, const int *n, const double *alpha, const double *a,
            const int *lda, const double *x, const int *incx, const double *beta, double *y,
            const int *incy) {
  const int ld = *lda;
  const int notrans = (trans[0] == 'N' || trans[0] == 'n');
  const int leny = notrans ? *m : *n;
  const int lenx = notrans ? *n : *m;
  int ky = *incy >= 0 ? 0 : (1 - leny) * *incy;
  int kx = *incx >= 0 ? 0 : (1 - lenx) * *incx;
  /* y = beta*y */
  for (int k = 0, iy = ky; k < leny; k++, iy += *incy) y[iy] = (*beta == 0.0) ? 0.0 : *beta * y[iy];
  if (*alpha == 0.0) return;
  if (notrans) {
    for (int j = 0, jx = kx; j < *n; j++, jx += *incx) {
      const double t = *alpha * x[jx];
      for (int i = 0, iy = ky; i < *m; i++, iy += *incy) y[iy] += t * A_(i, j);
    }
  } else {
    for (int j = 0, jy = ky; j < *n; j++, jy += *incy) {
      double t = 0.0;
      for (int i = 0, ix = kx; i < *m; i++, ix += *incx) t += A_(i, j) * x[ix];
      y[jy] += *alpha * t;
    }
  }
}

void dsymv_(const char *uplo, const int *n, const double *alpha, const double *a, const int *lda,
            const double *x, const int *incx, const double *beta, double *y, const int *incy) {
  (void)uplo; /* lower triangle only */
  const int ld = *lda;
  int kx = *incx >= 0 ? 0 : (1 - *n) * *incx;
  int ky = *incy >= 0 ? 0 : (1 - *n) * *incy;
  for (int k = 0, iy = ky; k < *n; k++, iy += *incy) y[iy] = (*beta == 0.0) ? 0.0 : *beta * y[iy];
  if (*alpha == 0.0) return;
  for (int j = 0, jx = kx, jy = ky; j < *n; j++, jx += *incx, jy += *incy) {
    const double t1 = *alpha * x[jx];
    double t2 = 0.0;
    y[jy] += t1 * A_(j, j);
    for (int i = j + 1, ix = jx + *incx, iy = jy + *incy; i < *n; i++, ix += *incx, iy += *incy) {
      y[iy] += t1 * A_(i, j);
      t2 += A_(i, j) * x[ix];
    }
    y[jy] += *alpha * t2;
  }
}

void dtrmv_(const char *uplo, const char *trans, const char *diag, const int *n, const double *a,
            const int *lda, double *x, const int *incx) {
  (void)uplo; (void)trans; (void)diag; /* 'L','N','N' only */
  const int ld = *lda;
  const int inc = *incx;
  int kx = inc >= 0 ? 0 : (1 - *n) * inc;
  /* x := L x, swept from the last column so that x[j] is read before it is overwritten */
  for (int j = *n - 1; j >= 0; j--) {
    const int jx = kx + j * inc;
    const double t = x[jx];
    if (t != 0.0) {
      for (int i = *n - 1; i > j; i--) x[kx + i * inc] += t * A_(i, j);
      x[jx] = t * A_(j, j);
    }
  }
}

/* Lower Cholesky, one column at a time: a(j,j) <- sqrt(a(j,j) - sum_k a(j,k)^2), then the column
 * below it.  info = j+1 on the first non-positive (or NaN) pivot. */
void dpotrf_(const char *uplo, const int *n, double *a, const int *lda, int *info) {
  (void)uplo;
  const int ld = *lda;
  *info = 0;
  for (int j = 0; j < *n; j++) {
    double d = A_(j, j);
    for (int k = 0; k < j; k++) d -= A_(j, k) * A_(j, k);
    if (!(d > 0.0)) { A_(j, j) = d; *info = j + 1; return; }
    d = sqrt(d);
    A_(j, j) = d;
    const double r = 1.0 / d;
    for (int i = j + 1; i < *n; i++) {
      double s = A_(i, j);
      for (int k = 0; k < j; k++) s -= A_(i, k) * A_(j, k);
      A_(i, j) = s * r;
    }
  }
}

/* Inverse of an SPD matrix from its lower Cholesky factor (overwrites the lower triangle). */
void dpotri_(const char *uplo, const int *n, double *a, const int *lda, int *info) {
  (void)uplo;
  const int ld = *lda;
  const int nn = *n;
  *info = 0;
  for (int j = 0; j < nn; j++)
    if (A_(j, j) == 0.0) { *info = j + 1; return; }
  /* inv(L) in place, last column first: column j of inv(L) below the diagonal is
   * -inv(L)(j+1:,j+1:) * L(j+1:,j) / L(j,j). */
  for (int j = nn - 1; j >= 0; j--) {
    A_(j, j) = 1.0 / A_(j, j);
    const double ajj = -A_(j, j);
    /* x = T * x with T = inv(L)(j+1:, j+1:) lower triangular, x = column j below the diagonal */
    for (int c = nn - 1; c > j; c--) {
      const double t = A_(c, j);
      if (t != 0.0) {
        for (int r = nn - 1; r > c; r--) A_(r, j) += t * A_(r, c);
        A_(c, j) = t * A_(c, c);
      }
    }
    for (int r = j + 1; r < nn; r++) A_(r, j) *= ajj;
  }
  /* inv(A) = inv(L)' * inv(L); lower triangle: out(i,j) = sum_{k>=i} Linv(k,i) Linv(k,j), i>=j.
   * Column j only reads columns >= j of inv(L), and rows are visited from the top so each entry is
   * read before it is overwritten. */
  for (int j = 0; j < nn; j++) {
    for (int i = j; i < nn; i++) {
      double s = 0.0;
      for (int k = i; k < nn; k++) s += A_(k, i) * A_(k, j);
      A_(i, j) = s;
    }
  }
}
