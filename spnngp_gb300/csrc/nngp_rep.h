// Replicate solve (nngp_rep.cu): the batched draw y_rep = X beta + (I - B)^-1 F^(1/2) z for
// many parameter sets, by a dataflow triangular solve over the neighbor DAG.
#pragma once

#include <vector>
#include "nngp_internal.h"

// nRep replicates of one dataset (all pointers device memory).  Replicate r uses parameter set
// d_theta[r], coefficients beta[r bs_r + j bs_j] (j < p), normals z[d_zoff[r] + i] (i < n), and
// writes yRep[r n + i].  xb_first = 0 sums v + beta_0 X_0 + beta_1 X_1 + ... (rNNGPReplicated's
// dgemv); xb_first = 1 sums (beta_0 X_0 + beta_1 X_1 + ...) + v (the response MCMC's dgemv
// then daxpy).  cov is the correlation code covering every d_theta (NNGP_COV_*).
struct RepSpec {
  int n, m, p, nRep, precision, cov, xb_first;
  const double *xy;
  const float *xyf;
  const int *nnIndx, *nnLU;
  const double *X;
  const CovParams *d_theta;
  const double *beta;
  int64_t bs_r, bs_j;
  const double *z;
  const long long *d_zoff;
  double *yRep;
  unsigned long long *d_status;
};
int nngp_replicate_solve(nngp_ctx *ctx, const RepSpec &s);
