#include <cuda_runtime.h>
#include <type_traits>
#include "nngp_internal.h"

// Host side of the B/F pass: plans (job tables), dispatch to the kernel
// instantiations of nngp_bf_inst.cu (one object per neighbor bound, precision and
// correlation code), and the fixed-order reductions.  The kernel itself is
// documented in nngp_bf_kernel.cuh.
namespace nngp_bf {
template <int M, bool R32, int MODE, int COV>
int launch_one(nngp_ctx *ctx, const BFPlan *pl, bool fallback_pass);
template <int M, bool R32>
constexpr int bf_tpb() {
  return R32 ? (M <= 16 ? 128 : 64) : (M <= 16 ? 64 : 32);
}
}  // namespace nngp_bf
using namespace nngp_bf;

namespace {
// Fixed-order reduction of per-tile partials: block `job`, value v.
__global__ void reduce_partials_kernel(const BFJob *__restrict__ jobs, int ng,
                                       double *__restrict__ out) {
  const BFJob job = jobs[blockIdx.x];
  __shared__ double sbuf[256];
  for (int v = 0; v < ng; v++) {
    double s = 0.0;
    for (int t = threadIdx.x; t < job.ntiles; t += 256) s += job.partial[(size_t)t * ng + v];
    sbuf[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
      if (threadIdx.x < w) sbuf[threadIdx.x] += sbuf[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[(size_t)blockIdx.x * ng + v] = sbuf[0];
    __syncthreads();
  }
}

}  // namespace

namespace {
template <int MODE, int COV>
int launch_mode_c(nngp_ctx *ctx, const BFPlan *pl, bool fp32r, bool fallback_pass) {
  if (pl->mmax <= 16)
    return fp32r ? launch_one<16, true, MODE, COV>(ctx, pl, fallback_pass)
                 : launch_one<16, false, MODE, COV>(ctx, pl, fallback_pass);
  return fp32r ? launch_one<32, true, MODE, COV>(ctx, pl, fallback_pass)
               : launch_one<32, false, MODE, COV>(ctx, pl, fallback_pass);
}

template <int MODE>
int launch_mode(nngp_ctx *ctx, const BFPlan *pl, bool fp32r, bool fallback_pass) {
  switch (pl->cov) {
    case NNGP_COV_EXP: return launch_mode_c<MODE, NNGP_COV_EXP>(ctx, pl, fp32r, fallback_pass);
    case NNGP_COV_SPH: return launch_mode_c<MODE, NNGP_COV_SPH>(ctx, pl, fp32r, fallback_pass);
    case NNGP_COV_MAT_HALF: return launch_mode_c<MODE, NNGP_COV_MAT_HALF>(ctx, pl, fp32r, fallback_pass);
    case NNGP_COV_GAU: return launch_mode_c<MODE, NNGP_COV_GAU>(ctx, pl, fp32r, fallback_pass);
    default: return launch_mode_c<MODE, NNGP_COV_ANY>(ctx, pl, fp32r, fallback_pass);
  }
}

int launch_pass(nngp_ctx *ctx, const BFPlan *pl, bool fp32r, bool fallback_pass) {
  return pl->mode == 0 ? launch_mode<0>(ctx, pl, fp32r, fallback_pass)
                       : launch_mode<1>(ctx, pl, fp32r, fallback_pass);
}

__global__ void add_into_kernel(double *__restrict__ dst, const double *__restrict__ src, int count) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < count) dst[t] += src[t];
}

}  // namespace

int nngp_bf_tile(int precision, int mmax) {
  if (precision == NNGP_FP32R) return mmax <= 16 ? bf_tpb<16, true>() : bf_tpb<32, true>();
  return mmax <= 16 ? bf_tpb<16, false>() : bf_tpb<32, false>();
}

void *nngp_malloc_async(nngp_ctx *ctx, size_t bytes) {
  void *p = nullptr;
  if (cudaMallocAsync(&p, bytes ? bytes : 16, ctx->stream) != cudaSuccess) return nullptr;
  return p;
}
void nngp_free_async(nngp_ctx *ctx, void *p) {
  if (p) cudaFreeAsync(p, ctx->stream);
}

static int build_jobs(int tpb, const std::vector<BFData> &datas, const std::vector<PassEval> &evals,
                      int ng, std::vector<BFJob> &jobs, size_t &partial_elems, int &tiles) {
  jobs.clear();
  tiles = 0;
  partial_elems = 0;
  for (const PassEval &e : evals) {
    BFJob j{};
    j.data = e.data;
    j.theta = e.theta;
    j.tile0 = tiles;
    j.ntiles = (datas[e.data].n + tpb - 1) / tpb;
    tiles += j.ntiles;
    j.partial = reinterpret_cast<double *>(partial_elems);  // offset, fixed up later
    partial_elems += (size_t)j.ntiles * ng;
    jobs.push_back(j);
  }
  return NNGP_OK;
}

int nngp_bf_plan(nngp_ctx *ctx, BFPlan *pl, int precision, int mode, int nv,
                 const std::vector<BFData> &datas, const CovParams *d_thetas,
                 const std::vector<PassEval> &evals, unsigned long long *d_status, int cov) {
  *pl = BFPlan();
  pl->cov = cov;
  pl->precision = precision;
  pl->mode = mode;
  pl->nv = mode == 1 ? nv : 0;
  pl->ng = mode == 1 ? 1 + nv * (nv + 1) / 2 : 1;
  pl->njobs = (int)evals.size();
  pl->d_thetas = d_thetas;
  pl->d_status = d_status;
  int mmax = 0;
  for (const BFData &d : datas) mmax = d.m > mmax ? d.m : mmax;
  pl->mmax = mmax;
  if (mmax > NNGP_MAX_M) return nngp_fail(ctx, NNGP_ERR_ARG, "m exceeds the supported maximum (32)");
  if (pl->nv > NNGP_MAX_NV) return nngp_fail(ctx, NNGP_ERR_ARG, "too many columns in the fused pass (max 8)");
  auto own = [&](size_t bytes) -> void * {
    void *p = nngp_malloc_async(ctx, bytes);
    if (p) pl->owned.push_back(p);
    return p;
  };
  // primary jobs
  std::vector<BFJob> jobs, jobs_fb;
  size_t pe = 0, pe_fb = 0;
  build_jobs(nngp_bf_tile(precision, mmax), datas, evals, pl->ng, jobs, pe, pl->tiles);
  pl->d_partial = (double *)own(sizeof(double) * pe);
  if (!pl->d_partial) return nngp_fail(ctx, NNGP_ERR_NO_MEMORY, "device allocation failed");
  if (precision == NNGP_FP32R) {
    build_jobs(nngp_bf_tile(NNGP_FP64, mmax), datas, evals, pl->ng, jobs_fb, pe_fb, pl->tiles_fb);
    pl->d_partial_fb = (double *)own(sizeof(double) * pe_fb);
    size_t fb = 0;
    for (const PassEval &e : evals) fb += (size_t)datas[e.data].n;
    pl->flags_bytes = fb;
    pl->d_flags = (unsigned char *)own(fb);
    if (!pl->d_partial_fb || !pl->d_flags) return nngp_fail(ctx, NNGP_ERR_NO_MEMORY, "device allocation failed");
  }
  size_t foff = 0;
  for (size_t k = 0; k < jobs.size(); k++) {
    jobs[k].partial = pl->d_partial + reinterpret_cast<size_t>(jobs[k].partial);
    if (precision == NNGP_FP32R) {
      jobs_fb[k].partial = pl->d_partial_fb + reinterpret_cast<size_t>(jobs_fb[k].partial);
      jobs[k].flags = jobs_fb[k].flags = pl->d_flags + foff;
      foff += (size_t)datas[evals[k].data].n;
    }
  }
  pl->d_datas = (BFData *)own(sizeof(BFData) * datas.size());
  pl->d_jobs = (BFJob *)own(sizeof(BFJob) * jobs.size());
  if (!pl->d_datas || !pl->d_jobs) return nngp_fail(ctx, NNGP_ERR_NO_MEMORY, "device allocation failed");
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(pl->d_datas, datas.data(), sizeof(BFData) * datas.size(),
                                     cudaMemcpyHostToDevice, ctx->stream));
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(pl->d_jobs, jobs.data(), sizeof(BFJob) * jobs.size(),
                                     cudaMemcpyHostToDevice, ctx->stream));
  if (precision == NNGP_FP32R) {
    pl->d_jobs_fb = (BFJob *)own(sizeof(BFJob) * jobs_fb.size());
    if (!pl->d_jobs_fb) return nngp_fail(ctx, NNGP_ERR_NO_MEMORY, "device allocation failed");
    NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(pl->d_jobs_fb, jobs_fb.data(), sizeof(BFJob) * jobs_fb.size(),
                                       cudaMemcpyHostToDevice, ctx->stream));
  }
  // the host vectors die at return: make the copies complete first
  NNGP_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return NNGP_OK;
}

int nngp_bf_run(nngp_ctx *ctx, const BFPlan *pl, double *d_out) {
  int st;
  const bool fp32r = pl->precision == NNGP_FP32R;
  if (fp32r) NNGP_CUDA_TRY(ctx, cudaMemsetAsync(pl->d_flags, 0, pl->flags_bytes, ctx->stream));
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  if (ctx->timing) {
    for (cudaEvent_t *e : {&t0, &t1}) {
      if (!ctx->event_pool.empty()) {
        *e = ctx->event_pool.back();
        ctx->event_pool.pop_back();
      } else {
        cudaEventCreate(e);
      }
    }
    cudaEventRecord(t0, ctx->stream);
  }
  if ((st = launch_pass(ctx, pl, fp32r, false))) return st;
  if (ctx->timing) {
    cudaEventRecord(t1, ctx->stream);
    ctx->timed.emplace_back(t0, t1);
  }
  reduce_partials_kernel<<<pl->njobs, 256, 0, ctx->stream>>>(pl->d_jobs, pl->ng, d_out);
  NNGP_LAUNCH_CHECK(ctx);
  if (fp32r) {
    // FP64 re-solve of the flagged locations, then fold its sums in
    if ((st = launch_pass(ctx, pl, false, true))) return st;
    double *tmp = d_out + (size_t)pl->njobs * pl->ng;  // caller provides 2 x njobs x ng
    reduce_partials_kernel<<<pl->njobs, 256, 0, ctx->stream>>>(pl->d_jobs_fb, pl->ng, tmp);
    NNGP_LAUNCH_CHECK(ctx);
    const int cnt = pl->njobs * pl->ng;
    add_into_kernel<<<(cnt + 255) / 256, 256, 0, ctx->stream>>>(d_out, tmp, cnt);
    NNGP_LAUNCH_CHECK(ctx);
  }
  return NNGP_OK;
}

int nngp_bf_launch(nngp_ctx *ctx, const BFPlan *pl, bool fp32r, bool fallback_pass) {
  return launch_pass(ctx, pl, fp32r, fallback_pass);
}

void nngp_bf_plan_free(nngp_ctx *ctx, BFPlan *pl) {
  for (void *p : pl->owned) nngp_free_async(ctx, p);
  pl->owned.clear();
}

void nngp_bf_cache_release(nngp_ctx *ctx) {
  if (ctx->cache_plan) {
    nngp_bf_plan_free(ctx, ctx->cache_plan);
    delete ctx->cache_plan;
    ctx->cache_plan = nullptr;
    ctx->cache_key.clear();
  }
}

extern "C" {
int nngp_set_kernel_timing(nngp_ctx *ctx, int on) {
  ctx->timing = on != 0;
  return NNGP_OK;
}
int nngp_kernel_time(nngp_ctx *ctx, double *ms, int64_t *launches) {
  NNGP_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  double total = 0.0;
  for (auto &pr : ctx->timed) {
    float t = 0.f;
    cudaEventElapsedTime(&t, pr.first, pr.second);
    total += t;
    ctx->event_pool.push_back(pr.first);
    ctx->event_pool.push_back(pr.second);
  }
  if (launches) *launches = (int64_t)ctx->timed.size();
  ctx->timed.clear();
  if (ms) *ms = total;
  return NNGP_OK;
}
}

namespace {
__global__ void prepare_coords_kernel(const double *__restrict__ cm, int n, double *__restrict__ xy,
                                      float *__restrict__ xyf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double x = cm[i], y = cm[n + i];
  if (xy) {
    xy[2 * i] = x;
    xy[2 * i + 1] = y;
  }
  if (xyf) {
    const float hx = (float)x, hy = (float)y;
    reinterpret_cast<float4 *>(xyf)[i] = make_float4(hx, hy, (float)(x - (double)hx), (float)(y - (double)hy));
  }
}
}  // namespace

int nngp_prepare_coords(nngp_ctx *ctx, const double *cm, int n, double *xy, float *xyf) {
  if (n <= 0) return NNGP_OK;
  prepare_coords_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(cm, n, xy, xyf);
  NNGP_LAUNCH_CHECK(ctx);
  return NNGP_OK;
}
