// A fused likelihood pass that allocates no memory.
//
// nngp_loglik_gram_dev builds its working buffers (interleaved coordinates,
// row-major [X y], per-tile partial sums, job tables) with cudaMalloc /
// cudaMallocAsync.  Some callers cannot allocate device memory at the moment
// they need the likelihood: an R session whose memory is policed by a host
// allocator it does not control, a serving process that reserves all HBM up
// front and forbids allocations on its request path, or a host that must not
// trigger the allocator's implicit device synchronisation in the middle of a
// latency-critical loop.  For them, nngp_loglik_gram_noalloc runs the same FP64
// fused pass with its working memory in one statically sized __device__ array
// that lives in this library's module: every GPU that loads the library holds
// kScratchBytes (about 5.3 MB) for the life of the process.
//
// Limits and rules (also stated in include/spnngp_gb300.h):
//   - n <= kMaxN (65,536) locations, m <= 32, nv <= 8;
//     larger requests are rejected with NNGP_ERR_ARG and a message;
//   - the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (and sets the kernel's shared-memory attribute);
//   - no call may be made while its stream is being captured into a CUDA graph:
//     each call copies host stack values to the device and waits for its stream
//     before it returns, neither of which a graph can hold; such a call returns
//     NNGP_ERR_ARG;
//   - all calls share the one array and it keeps the previous call's contents:
//     the status word is reset by every call, everything else is overwritten
//     before it is read; calls whose work overlaps on the GPU (two streams, or
//     two host threads) race on the array and must be serialised by the caller.
#include <cuda_runtime.h>
#include <cstdio>
#include <string>
#include "nngp_internal.h"

namespace {

constexpr int kMaxN = 65536;
constexpr int kMaxNV = NNGP_MAX_NV;
constexpr int kNGMax = 1 + kMaxNV * (kMaxNV + 1) / 2;
constexpr int kMaxTiles = (kMaxN + 31) / 32;  // bounds every FP64 tile size (64 or 32)

// byte layout of the static scratch (each piece 256-byte aligned)
constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kOffXY = 0;
constexpr size_t kOffV = kOffXY + align256(sizeof(double) * 2 * kMaxN);
constexpr size_t kOffPartial = kOffV + align256(sizeof(double) * (size_t)kMaxN * kMaxNV);
// the allocating pass's two-level reduction: chunks of 1024 tiles, then the chunk sums in order
constexpr int kMaxChunks = (kMaxTiles + 1023) / 1024;
constexpr size_t kOffPartial2 = kOffPartial + align256(sizeof(double) * (size_t)kMaxTiles * kNGMax);
constexpr size_t kOffOut = kOffPartial2 + align256(sizeof(double) * 2 * kNGMax * (size_t)kMaxChunks);
constexpr size_t kOffTheta = kOffOut + align256(sizeof(double) * 2 * kNGMax);
constexpr size_t kOffData = kOffTheta + align256(sizeof(CovParams));
constexpr size_t kOffJob = kOffData + align256(sizeof(BFData));
constexpr size_t kOffStatus = kOffJob + align256(sizeof(BFJob));
constexpr size_t kScratchBytes = kOffStatus + align256(sizeof(unsigned long long));

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
static unsigned char *g_scratch_addr[kMaxDevices] = {};

__global__ void na_interleave_kernel(const double *__restrict__ cm, int n, double *__restrict__ xy) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    xy[2 * i] = cm[i];
    xy[2 * i + 1] = cm[n + i];
  }
}

__global__ void na_row_major_kernel(const double *__restrict__ cm, int n, int nv, double *__restrict__ rm) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < (long)n * nv) {
    const int i = (int)(t / nv), v = (int)(t % nv);
    rm[t] = cm[(size_t)v * n + i];
  }
}

// Writes the pass's sums (log F first, then the Gram entries a <= b, row-major) as logDet and
// the full nv x nv Gram into the caller's device buffers.
__global__ void na_unpack_kernel(const double *__restrict__ sums, int nv, double *__restrict__ logDet,
                                 double *__restrict__ gram) {
  if (threadIdx.x != 0) return;
  *logDet = sums[0];
  int k = 1;
  for (int a = 0; a < nv; a++)
    for (int b = a; b < nv; b++, k++) {
      gram[(size_t)b * nv + a] = sums[k];
      gram[(size_t)a * nv + b] = sums[k];
    }
}

int fail(nngp_ctx *ctx, int status, const char *msg) {
  nngp_fail(ctx, status, msg);
  return status;
}

}  // namespace

// Same contract as nngp_loglik_gram_dev in FP64 (device pointers in and out;
// theta on the host), with no allocation; see the header comment above.
extern "C" int nngp_loglik_gram_noalloc(void *stream, int n, int m, int nv, const double *coords,
                                        const int *nnIndx, const int *nnIndxLU, const double *V,
                                        int covModel, const double *theta, double *logDet, double *gram,
                                        char *errbuf, int errlen) {
  nngp_ctx ctx;  // stack-only context: carries the stream and the error text, owns no device memory
  ctx.stream = (cudaStream_t)stream;
  int st = NNGP_OK;
  auto report = [&](int s) {
    if (s != NNGP_OK && errbuf && errlen > 0) snprintf(errbuf, (size_t)errlen, "%s", ctx.err.c_str());
    return s;
  };
  if (n < 1 || m < 1 || m > NNGP_MAX_M || n < m)
    return report(fail(&ctx, NNGP_ERR_ARG, "nngp_loglik_gram_noalloc: n >= m and 1 <= m <= 32 required"));
  if (n > kMaxN)
    return report(fail(&ctx, NNGP_ERR_ARG,
                       "nngp_loglik_gram_noalloc: n exceeds the static scratch limit of 65536 locations; "
                       "use nngp_loglik_gram_dev"));
  if (nv < 1 || nv > kMaxNV) return report(fail(&ctx, NNGP_ERR_ARG, "nngp_loglik_gram_noalloc: 1 <= nv <= 8 required"));
  if (covModel < 0 || covModel > 3)
    return report(fail(&ctx, NNGP_ERR_ARG, "nngp_loglik_gram_noalloc: cov.model is not correctly specified"));
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(ctx.stream, &cap) != cudaSuccess) {
    cudaGetLastError();
    return report(fail(&ctx, NNGP_ERR_CUDA, "nngp_loglik_gram_noalloc: invalid stream"));
  }
  if (cap != cudaStreamCaptureStatusNone)
    return report(fail(&ctx, NNGP_ERR_ARG,
                       "nngp_loglik_gram_noalloc: must not be called while its stream is being captured"));
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return report(fail(&ctx, NNGP_ERR_CUDA, "nngp_loglik_gram_noalloc: no usable CUDA device"));
  ctx.device = dev;
  // one-time set-up on this device: the array's device address (host code cannot use the symbol itself)
  if (!g_scratch_addr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return report(fail(&ctx, NNGP_ERR_CUDA,
                         (std::string("nngp_loglik_gram_noalloc: cudaGetSymbolAddress failed: ") +
                          cudaGetErrorString(e)).c_str()));
    }
    g_scratch_addr[dev] = (unsigned char *)p;
  }
  unsigned char *base = g_scratch_addr[dev];
  double *xy = (double *)(base + kOffXY);
  double *Vrm = (double *)(base + kOffV);
  double *partial = (double *)(base + kOffPartial);
  double *partial2 = (double *)(base + kOffPartial2);
  double *sums = (double *)(base + kOffOut);
  CovParams *d_theta = (CovParams *)(base + kOffTheta);
  BFData *d_data = (BFData *)(base + kOffData);
  BFJob *d_job = (BFJob *)(base + kOffJob);
  unsigned long long *d_status = (unsigned long long *)(base + kOffStatus);

  CovParams cp{};
  cp.model = covModel;
  cp.sigmaSq = theta[0];
  cp.tauSq = theta[1];
  cp.phi = theta[2];
  cp.nu = covModel == 2 ? theta[3] : 0.0;
  cov_prepare(cp);
  BFData d{};
  d.n = n;
  d.m = m;
  d.nv = nv;
  d.xy = xy;
  d.nnIndx = nnIndx;
  d.nnLU = nnIndxLU;
  d.V = Vrm;
  const int tpb = m <= 16 ? 64 : 32;  // FP64 tile of the B/F kernel
  BFJob job{};
  job.data = 0;
  job.theta = 0;
  job.tile0 = 0;
  job.ntiles = (n + tpb - 1) / tpb;
  job.partial = partial;
  job.flags = nullptr;
  BFPlan plan;  // host description only; every pointer refers to the static array
  plan.precision = NNGP_FP64;
  plan.mode = 1;
  plan.mmax = m;
  plan.nv = nv;
  plan.ng = 1 + nv * (nv + 1) / 2;
  plan.njobs = 1;
  plan.tiles = job.ntiles;
  plan.d_datas = d_data;
  plan.d_thetas = d_theta;
  plan.d_jobs = d_job;
  plan.d_partial = partial;
  plan.d_status = d_status;
  plan.red_chunks = (job.ntiles + 1023) / 1024;
  plan.d_partial2 = partial2;

  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_theta, &cp, sizeof cp, cudaMemcpyHostToDevice, ctx.stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_data, &d, sizeof d, cudaMemcpyHostToDevice, ctx.stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_job, &job, sizeof job, cudaMemcpyHostToDevice, ctx.stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_status, 0xFF, sizeof(unsigned long long), ctx.stream);
  if (e != cudaSuccess)
    return report(fail(&ctx, NNGP_ERR_CUDA, (std::string("nngp_loglik_gram_noalloc: ") + cudaGetErrorString(e)).c_str()));
  na_interleave_kernel<<<(n + 255) / 256, 256, 0, ctx.stream>>>(coords, n, xy);
  na_row_major_kernel<<<(unsigned)(((long)n * nv + 255) / 256), 256, 0, ctx.stream>>>(V, n, nv, Vrm);
  plan.cov = nngp_plan_cov(&cp, 1);
  st = nngp_bf_launch(&ctx, &plan, false, false);
  if (!st) st = nngp_bf_finish(&ctx, &plan, sums);  // the allocating pass's reduction, same order
  if (st) return report(st);
  na_unpack_kernel<<<1, 32, 0, ctx.stream>>>(sums, nv, logDet, gram);
  e = cudaGetLastError();
  if (e != cudaSuccess)
    return report(fail(&ctx, NNGP_ERR_CUDA, (std::string("nngp_loglik_gram_noalloc: ") + cudaGetErrorString(e)).c_str()));
  // the status word is read back into host stack memory
  unsigned long long h = NNGP_STATUS_OK;
  e = cudaMemcpyAsync(&h, d_status, sizeof h, cudaMemcpyDeviceToHost, ctx.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx.stream);
  if (e != cudaSuccess)
    return report(fail(&ctx, NNGP_ERR_CUDA, (std::string("nngp_loglik_gram_noalloc: ") + cudaGetErrorString(e)).c_str()));
  if (h != NNGP_STATUS_OK) {
    char buf[160];
    snprintf(buf, sizeof buf,
             "nngp_loglik_gram_noalloc: neighborhood covariance not positive definite at location %lld",
             (long long)(h & 0xFFFFFFFFFFFFull));
    return report(fail(&ctx, NNGP_ERR_NOT_SPD, buf));
  }
  return NNGP_OK;
}
