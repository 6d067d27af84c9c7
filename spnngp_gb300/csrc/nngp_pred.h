// Arguments of the prediction-point neighborhood solves (kernel in
// nngp_pred_kernel.cuh, drivers in nngp_conj.cu).
#pragma once
#include "nngp_internal.h"

namespace nngp_pred {

enum { KIND_CONJ = 0, KIND_RESP = 1 };

struct PredArgs {
  int n, m, p, n0, npar;  // npar = parameter sets (g grid points or nSamples)
  const double *xy;       // training coords, interleaved
  const double *V;        // training [X y], n x (p+1) row-major
  const double *c0;       // prediction coords, n0 x 2 column-major
  const double *X0;       // n0 x p column-major
  const int *nn0;         // n0 x m column-major
  const CovParams *par;   // npar parameter sets
  // conjugate: betaHat (p x g), Vinv (p*p x g, lower), ab (2 x g); response: beta (p x nS), z (n0*nS)
  const double *beta;
  const double *Vinv;
  const double *ab;
  const double *z;
  double *out0;           // conj: y0Hat (n0 x g); resp: y0 (n0 x nS)
  double *out1;           // conj: y0HatVar
  unsigned long long *status;
};

template <int M, bool R32, int KIND>
int launch_pred(nngp_ctx *ctx, const PredArgs &a);

}  // namespace nngp_pred
