// Measurement utility (no counterpart in the reference): sustained FMA throughput
// of the FP64 and FP32 CUDA-core pipes, used as the denominator of the B/F
// pass's roofline fraction.  Eight independent FMA chains per thread keep the
// pipes busy; the result is 2 * FMAs / elapsed seconds.
#include <cuda_runtime.h>
#include "nngp_internal.h"

namespace {
template <typename T>
__global__ void fma_chains_kernel(T *out, int iters, T a, T b) {
  T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
#pragma unroll 1
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int u = 0; u < 8; u++) {
      x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
      x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
  }
  const T s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (s == (T)-1.2345) out[0] = s;  // keeps the chains live
}
}  // namespace

extern "C" int nngp_measure_peak(nngp_ctx *ctx, int fp64, double *flops_per_s) {
  if (!ctx || !flops_per_s) return NNGP_ERR_ARG;
  cudaSetDevice(ctx->device);
  double *out;
  NNGP_ALLOC(ctx, out, double, S_MISC, 1);
  const int threads = 256, blocks = ctx->sm_count * 8;
  const int iters = fp64 ? 64 : 4096;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 4; rep++) {
    cudaEventRecord(e0, ctx->stream);
    if (fp64)
      fma_chains_kernel<double><<<blocks, threads, 0, ctx->stream>>>(out, iters, 0.999999, 1e-7);
    else
      fma_chains_kernel<float><<<blocks, threads, 0, ctx->stream>>>((float *)out, iters, 0.999999f, 1e-7f);
    cudaEventRecord(e1, ctx->stream);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;  // first launch is warm-up
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return nngp_fail(ctx, NNGP_ERR_CUDA, cudaGetErrorString(e));
  const double fmas = 64.0 * iters * (double)threads * blocks;
  *flops_per_s = 2.0 * fmas / (best * 1e-3);
  return NNGP_OK;
}
