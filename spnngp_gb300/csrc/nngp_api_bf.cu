// C-ABI entry points of the B/F pass: updateBF / updateConjBF (src/rNNGP.cpp:46-101,
// src/cNNGP.cpp:24-69), Q (src/util.cpp:261-280) and the fused likelihood/Gram pass.
#include <cuda_runtime.h>
#include <cmath>
#include <cstring>
#include "nngp_internal.h"

namespace {

// col-major n x nv -> row-major n x nv, and (when rmf is given) its float (hi, lo) split, for
// locations [i0, i1)
__global__ void to_row_major_kernel(const double *__restrict__ cm, int n, int nv, int i0, int i1,
                                    double *__restrict__ rm, float2 *__restrict__ rmf) {
  const long t = (long)i0 * nv + (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < (long)i1 * nv) {
    const int i = (int)(t / nv), v = (int)(t % nv);
    const double x = cm[(size_t)v * n + i];
    rm[t] = x;
    if (rmf) {
      const float h = (float)x;
      rmf[t] = make_float2(h, (float)(x - (double)h));
    }
  }
}

// Q: per-tile sums of (u_i - B_i u_N)(v_i - B_i v_N) / F_i.
__global__ void q_kernel(const double *__restrict__ B, const double *__restrict__ F,
                         const double *__restrict__ u, const double *__restrict__ v, int n,
                         const int *__restrict__ nnIndx, const int *__restrict__ nnLU,
                         double *__restrict__ partial) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double q = 0.0;
  if (i < n) {
    double a = 0.0, b = 0.0;
    const int off = nnLU[i], cnt = nnLU[n + i];
    for (int j = 0; j < cnt; j++) {
      const double w = B[off + j];
      const int k = nnIndx[off + j];
      a += w * u[k];
      b += w * v[k];
    }
    q = (u[i] - a) * (v[i] - b) / F[i];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) q += __shfl_xor_sync(0xffffffffu, q, o);
  __shared__ double wb[8];
  if ((threadIdx.x & 31) == 0) wb[threadIdx.x >> 5] = q;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += wb[w];
    partial[blockIdx.x] = s;
  }
}

__global__ void sum_kernel(const double *__restrict__ x, int cnt, double *__restrict__ out) {
  __shared__ double s[256];
  double a = 0.0;
  for (int t = threadIdx.x; t < cnt; t += 256) a += x[t];
  s[threadIdx.x] = a;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = s[0];
}

int check_common(nngp_ctx *ctx, int n, int m, int covModel) {
  if (!ctx) return NNGP_ERR_ARG;
  if (n < 1 || m < 1 || m > NNGP_MAX_M) return nngp_fail(ctx, NNGP_ERR_ARG, "n >= 1 and 1 <= m <= 32 required");
  if (n < m) return nngp_fail(ctx, NNGP_ERR_ARG, "n must be at least m (the packed neighbor layout needs n >= m)");
  if (covModel < 0 || covModel > 3) return nngp_fail(ctx, NNGP_ERR_ARG, "cov.model is not correctly specified");
  return NNGP_OK;
}

CovParams make_params(int covModel, double sigmaSq, double tauSq, double phi, double nu) {
  CovParams c{};
  c.model = covModel;
  c.sigmaSq = sigmaSq;
  c.tauSq = tauSq;
  c.phi = phi;
  c.nu = nu;
  cov_prepare(c);
  return c;
}

// Host arrays a host-pointer entry point streams in (each null when already on the device).
struct HostIn {
  const double *coords = nullptr;  // n x 2 column-major
  const int *nnIndx = nullptr;
  const int *nnLU = nullptr;       // [offsets | counts]
  const double *V = nullptr;       // n x nv column-major
};

// Location chunks of the streamed form: 64 K locations first, each next chunk twice the last
// (a chunk's B/F work then takes about as long as the next chunk's copies, and the first
// wait is short), boundaries on multiples of 128 so they fall on tile boundaries of every
// kernel.  Inputs below 192 K locations go in one piece.
std::vector<int> chunk_bounds(int n) {
  std::vector<int> b{0};
  if (n >= 196608) {
    for (long step = 65536, a = 0; a + step < n;) {
      a += step;
      if (n - a < step / 2) break;  // fold a short tail into the last chunk
      b.push_back((int)a);
      step *= 2;
    }
  }
  b.push_back(n);
  return b;
}

// Single-evaluation pass.  coords are n x 2 column-major (device).  With `hin`, the device
// arrays d_coords_cm, d_nnIndx, d_nnLU and d_V_cm are filled from host memory here, one
// location chunk at a time on the copy stream, and each chunk's conversions and B/F tiles run
// as soon as its copies land (the neighbors of a location precede it in the ordering, so they
// are in the same or an earlier chunk).  The pass is the same either way: one job over all
// locations whose tiles are launched in pieces, so results do not depend on the chunking.
// log det and (gram != nullptr) the nv x nv Gram from the packed sums (log F, then the upper
// triangle a <= b row-major)
__global__ void unpack_out_kernel(const double *__restrict__ packed, int nv, double *__restrict__ ld,
                                  double *__restrict__ gram) {
  const int t = threadIdx.x;
  if (t == 0) *ld = packed[0];
  if (!gram) return;
  for (int k = t; k < nv * (nv + 1) / 2; k += blockDim.x) {
    int rem = k, a = 0;
    while (rem >= nv - a) {
      rem -= nv - a;
      a++;
    }
    const int b = a + rem;
    gram[(size_t)b * nv + a] = packed[1 + k];
    gram[(size_t)a * nv + b] = packed[1 + k];
  }
}

int run_single(nngp_ctx *ctx, int mode, int n, int m, int nv, const double *d_coords_cm,
               const int *d_nnIndx, const int *d_nnLU, const double *d_V_cm, const CovParams &cp,
               int precision, double *d_B, double *d_F, double *h_out, const HostIn *hin = nullptr,
               double *d_ld = nullptr, double *d_gram = nullptr) {
  if (precision != NNGP_FP64 && precision != NNGP_FP32R)
    return nngp_fail(ctx, NNGP_ERR_ARG, "precision must be 0 (FP64) or 1 (FP32R)");
  double *xy, *Vrm = nullptr;
  float *xyf = nullptr;
  float2 *Vf = nullptr;
  NNGP_ALLOC(ctx, xy, double, S_COORDS, 2 * (size_t)n);
  if (precision == NNGP_FP32R) NNGP_ALLOC(ctx, xyf, float, S_XYF, 4 * (size_t)n);
  if (mode == 1) {
    NNGP_ALLOC(ctx, Vrm, double, S_V, (size_t)n * nv);
    // V changes from call to call under a cached plan: the FP32R kernels' float split is
    // refreshed here rather than by the plan
    if (precision == NNGP_FP32R) NNGP_ALLOC(ctx, Vf, float2, S_VF, (size_t)n * nv);
  }
  CovParams *d_theta;
  unsigned long long *d_status;
  double *d_out;
  NNGP_ALLOC(ctx, d_theta, CovParams, S_THETA, 1);
  NNGP_ALLOC(ctx, d_status, unsigned long long, S_STATUS, 1);
  const int ng = mode == 1 ? 1 + nv * (nv + 1) / 2 : 1;
  NNGP_ALLOC(ctx, d_out, double, S_RED, 2 * (size_t)ng);
  BFData d{};
  d.n = n;
  d.m = m;
  d.nv = nv;
  d.xy = xy;
  d.xyf = xyf;
  d.nnIndx = d_nnIndx;
  d.nnLU = d_nnLU;
  d.V = Vrm;
  d.Vf = Vf;
  d.B = d_B;
  d.F = d_F;
  char key[512];
  snprintf(key, sizeof key, "%d/%d/%d/%d/%d/%d/%p/%p/%p/%p/%p/%p/%p/%p/%p/%p", nngp_plan_cov(&cp, 1), mode, precision, n, m, nv, (const void *)xy,
           (const void *)xyf, (const void *)Vf,
           (const void *)d_nnIndx, (const void *)d_nnLU, (const void *)Vrm, (void *)d_B, (void *)d_F,
           (void *)d_theta, (void *)d_status);
  int st = NNGP_OK;
  if (!ctx->cache_plan || ctx->cache_key != key) {
    nngp_bf_cache_release(ctx);
    BFPlan *plan = new BFPlan();
    st = nngp_bf_plan(ctx, plan, precision, mode, nv, {d}, d_theta, {PassEval{0, 0}}, d_status,
                      nngp_plan_cov(&cp, 1));
    if (st) {
      nngp_bf_plan_free(ctx, plan);
      delete plan;
      return st;
    }
    ctx->cache_plan = plan;
    ctx->cache_key = key;
  }
  const BFPlan *pl = ctx->cache_plan;
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(d_theta, &cp, sizeof cp, cudaMemcpyHostToDevice, ctx->stream));
  if ((st = nngp_reset_status(ctx, d_status))) return st;
  if ((st = nngp_bf_begin(ctx, pl))) return st;
  const int tile = nngp_bf_tile(precision, m);
  const std::vector<int> bounds = hin ? chunk_bounds(n) : std::vector<int>{0, n};
  const int nchunks = (int)bounds.size() - 1;
  cudaStream_t cs = ctx->stream;
  if (hin) {
    if (!ctx->copy_stream) NNGP_CUDA_TRY(ctx, cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
    cs = ctx->copy_stream;
    while ((int)ctx->chunk_events.size() < nchunks + 1) {
      cudaEvent_t e;
      NNGP_CUDA_TRY(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      ctx->chunk_events.push_back(e);
    }
    // the copies overwrite buffers the previous call's kernels read: start after them
    NNGP_CUDA_TRY(ctx, cudaEventRecord(ctx->chunk_events[nchunks], ctx->stream));
    NNGP_CUDA_TRY(ctx, cudaStreamWaitEvent(cs, ctx->chunk_events[nchunks], 0));
  }
  for (int k = 0; k < nchunks; k++) {
    const int a = bounds[k], b = bounds[k + 1];
    if (hin) {
      auto h2d = [&](void *dst, const void *src, size_t bytes) {
        return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, cs) : cudaSuccess;
      };
      double *dc = const_cast<double *>(d_coords_cm);
      int *dlu = const_cast<int *>(d_nnLU), *dnn = const_cast<int *>(d_nnIndx);
      const int64_t o0 = hin->nnLU[a], o1 = (int64_t)hin->nnLU[b - 1] + hin->nnLU[n + b - 1];
      NNGP_CUDA_TRY(ctx, h2d(dc + a, hin->coords + a, sizeof(double) * (b - a)));
      NNGP_CUDA_TRY(ctx, h2d(dc + n + a, hin->coords + n + a, sizeof(double) * (b - a)));
      NNGP_CUDA_TRY(ctx, h2d(dlu + a, hin->nnLU + a, sizeof(int) * (b - a)));
      NNGP_CUDA_TRY(ctx, h2d(dlu + n + a, hin->nnLU + n + a, sizeof(int) * (b - a)));
      NNGP_CUDA_TRY(ctx, h2d(dnn + o0, hin->nnIndx + o0, sizeof(int) * (size_t)(o1 - o0)));
      if (mode == 1)
        for (int v = 0; v < nv; v++)
          NNGP_CUDA_TRY(ctx, h2d(const_cast<double *>(d_V_cm) + (size_t)v * n + a, hin->V + (size_t)v * n + a,
                                 sizeof(double) * (b - a)));
      NNGP_CUDA_TRY(ctx, cudaEventRecord(ctx->chunk_events[k], cs));
      NNGP_CUDA_TRY(ctx, cudaStreamWaitEvent(ctx->stream, ctx->chunk_events[k], 0));
    }
    if ((st = nngp_prepare_coords(ctx, d_coords_cm, n, xy, xyf, a, b))) return st;
    if (mode == 1) {
      const long cnt = (long)(b - a) * nv;
      to_row_major_kernel<<<(unsigned)((cnt + 255) / 256), 256, 0, ctx->stream>>>(d_V_cm, n, nv, a, b, Vrm, Vf);
      NNGP_LAUNCH_CHECK(ctx);
    }
    if ((st = nngp_bf_primary(ctx, pl, a / tile, (b + tile - 1) / tile))) return st;
  }
  if ((st = nngp_bf_finish(ctx, pl, d_out))) return st;
  if (d_ld) {
    // device outputs: unpacked on the device, no host round trip
    unpack_out_kernel<<<1, 64, 0, ctx->stream>>>(d_out, nv, d_ld, d_gram);
    NNGP_LAUNCH_CHECK(ctx);
  } else {
    NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(h_out, d_out, sizeof(double) * ng, cudaMemcpyDeviceToHost, ctx->stream));
  }
  return nngp_check_status(ctx, d_status, mode == 0 ? "updateBF" : "loglik_gram");
}

// Unpacks the upper-triangle (a <= b, row-major) sums into a full nv x nv matrix.
void unpack_gram(const double *packed, int nv, double *gram) {
  int k = 0;
  for (int a = 0; a < nv; a++)
    for (int b = a; b < nv; b++) {
      gram[(size_t)b * nv + a] = packed[k];
      gram[(size_t)a * nv + b] = packed[k];
      k++;
    }
}

}  // namespace

extern "C" {

int nngp_updateBF_dev(nngp_ctx *ctx, int n, int m, const double *coords, const int *nnIndx,
                      const int *nnIndxLU, int covModel, const double *theta, int precision,
                      double *B, double *F, double *logDet) {
  int st = check_common(ctx, n, m, covModel);
  if (st) return st;
  cudaSetDevice(ctx->device);
  const CovParams cp = make_params(covModel, theta[0], theta[1], theta[2], covModel == 2 ? theta[3] : 0.0);
  return run_single(ctx, 0, n, m, 0, coords, nnIndx, nnIndxLU, nullptr, cp, precision, B, F, nullptr, nullptr,
                    logDet, nullptr);
}

int nngp_loglik_gram_dev(nngp_ctx *ctx, int n, int m, int nv, const double *coords,
                         const int *nnIndx, const int *nnIndxLU, const double *V, int covModel,
                         const double *theta, int precision, double *logDet, double *gram) {
  int st = check_common(ctx, n, m, covModel);
  if (st) return st;
  if (nv < 1 || nv > NNGP_MAX_NV) return nngp_fail(ctx, NNGP_ERR_ARG, "1 <= nv <= 8 required");
  cudaSetDevice(ctx->device);
  const CovParams cp = make_params(covModel, theta[0], theta[1], theta[2], covModel == 2 ? theta[3] : 0.0);
  return run_single(ctx, 1, n, m, nv, coords, nnIndx, nnIndxLU, V, cp, precision, nullptr, nullptr, nullptr,
                    nullptr, logDet, gram);
}

int nngp_updateBF(nngp_ctx *ctx, int n, int m, const double *coords, const int *nnIndx,
                  const int *nnIndxLU, int covModel, const double *theta, int precision,
                  double *B, double *F, double *logDet) {
  int st = check_common(ctx, n, m, covModel);
  if (st) return st;
  cudaSetDevice(ctx->device);
  const int64_t nI = nngp_nindx(n, m);
  double *dc, *dB, *dF;
  int *dnn, *dlu;
  NNGP_ALLOC(ctx, dc, double, S_COORDS0, 2 * (size_t)n);
  NNGP_ALLOC(ctx, dnn, int, S_NNINDX, (size_t)(nI > 0 ? nI : 1));
  NNGP_ALLOC(ctx, dlu, int, S_NNLU, 2 * (size_t)n);
  NNGP_ALLOC(ctx, dB, double, S_B, (size_t)(nI > 0 ? nI : 1));
  NNGP_ALLOC(ctx, dF, double, S_F, (size_t)n);
  const CovParams cp = make_params(covModel, theta[0], theta[1], theta[2], covModel == 2 ? theta[3] : 0.0);
  HostIn hin;
  hin.coords = coords;
  hin.nnIndx = nnIndx;
  hin.nnLU = nnIndxLU;
  st = run_single(ctx, 0, n, m, 0, dc, dnn, dlu, nullptr, cp, precision, dB, dF, logDet, &hin);
  if (st) return st;
  if (nI > 0) NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(B, dB, sizeof(double) * nI, cudaMemcpyDeviceToHost, ctx->stream));
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(F, dF, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
  NNGP_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  // location 0 has no neighbors; the reference stores B[0] = 0 before location 1
  // overwrites that slot, so nothing further is needed here.
  return NNGP_OK;
}

int nngp_updateConjBF(nngp_ctx *ctx, int n, int m, const double *coords, const int *nnIndx,
                      const int *nnIndxLU, int covModel, double phi, double alpha, double nu,
                      int precision, double *B, double *F) {
  const double theta[4] = {1.0, alpha, phi, nu};
  double ld = 0.0;
  return nngp_updateBF(ctx, n, m, coords, nnIndx, nnIndxLU, covModel, theta, precision, B, F, &ld);
}

int nngp_loglik_gram(nngp_ctx *ctx, int n, int m, int nv, const double *coords,
                     const int *nnIndx, const int *nnIndxLU, const double *V, int covModel,
                     const double *theta, int precision, double *logDet, double *gram) {
  int st = check_common(ctx, n, m, covModel);
  if (st) return st;
  if (nv < 1 || nv > NNGP_MAX_NV) return nngp_fail(ctx, NNGP_ERR_ARG, "1 <= nv <= 8 required");
  cudaSetDevice(ctx->device);
  const int64_t nI = nngp_nindx(n, m);
  double *dc, *dV;
  int *dnn, *dlu;
  NNGP_ALLOC(ctx, dc, double, S_COORDS0, 2 * (size_t)n);
  NNGP_ALLOC(ctx, dnn, int, S_NNINDX, (size_t)(nI > 0 ? nI : 1));
  NNGP_ALLOC(ctx, dlu, int, S_NNLU, 2 * (size_t)n);
  NNGP_ALLOC(ctx, dV, double, S_V2, (size_t)n * nv);
  const CovParams cp = make_params(covModel, theta[0], theta[1], theta[2], covModel == 2 ? theta[3] : 0.0);
  HostIn hin;
  hin.coords = coords;
  hin.nnIndx = nnIndx;
  hin.nnLU = nnIndxLU;
  hin.V = V;
  double packed[1 + NNGP_MAX_NV * (NNGP_MAX_NV + 1) / 2];
  st = run_single(ctx, 1, n, m, nv, dc, dnn, dlu, dV, cp, precision, nullptr, nullptr, packed, &hin);
  if (st) return st;
  *logDet = packed[0];
  unpack_gram(packed + 1, nv, gram);
  return NNGP_OK;
}

int nngp_Q(nngp_ctx *ctx, const double *B, const double *F, const double *u, const double *v,
           int n, const int *nnIndx, const int *nnIndxLU, double *q) {
  if (!ctx || n < 1) return nngp_fail(ctx, NNGP_ERR_ARG, "n >= 1 required");
  cudaSetDevice(ctx->device);
  // the packed length is the sum of the counts
  int64_t nI = 0;
  {
    // counts are the second half of nnIndxLU; offsets of the last location + its count
    nI = (int64_t)nnIndxLU[n - 1] + nnIndxLU[2 * n - 1];
  }
  double *dB, *dF, *du, *dv, *dpart, *dq;
  int *dI, *dLU;
  NNGP_ALLOC(ctx, dB, double, S_B, (size_t)(nI > 0 ? nI : 1));
  NNGP_ALLOC(ctx, dF, double, S_F, (size_t)n);
  NNGP_ALLOC(ctx, du, double, S_U, (size_t)n);
  NNGP_ALLOC(ctx, dv, double, S_V2, (size_t)n);
  NNGP_ALLOC(ctx, dI, int, S_NNINDX, (size_t)(nI > 0 ? nI : 1));
  NNGP_ALLOC(ctx, dLU, int, S_NNLU, 2 * (size_t)n);
  const int nb = (n + 255) / 256;
  NNGP_ALLOC(ctx, dpart, double, S_PARTIAL, (size_t)nb);
  NNGP_ALLOC(ctx, dq, double, S_RED, 1);
  if (nI > 0) {
    NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(dB, B, sizeof(double) * nI, cudaMemcpyHostToDevice, ctx->stream));
    NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(dI, nnIndx, sizeof(int) * nI, cudaMemcpyHostToDevice, ctx->stream));
  }
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(dF, F, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(du, u, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(dv, v, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(dLU, nnIndxLU, sizeof(int) * 2 * n, cudaMemcpyHostToDevice, ctx->stream));
  q_kernel<<<nb, 256, 0, ctx->stream>>>(dB, dF, du, dv, n, dI, dLU, dpart);
  NNGP_LAUNCH_CHECK(ctx);
  sum_kernel<<<1, 256, 0, ctx->stream>>>(dpart, nb, dq);
  NNGP_LAUNCH_CHECK(ctx);
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(q, dq, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  NNGP_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return NNGP_OK;
}

}  // extern "C"
