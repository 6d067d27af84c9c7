// Context management, error reporting, scratch buffers and device status words.
#include <cuda_runtime.h>
#include <cstring>
#include "nngp_internal.h"

int nngp_fail(nngp_ctx *ctx, int status, const std::string &msg, int64_t loc) {
  if (ctx) {
    ctx->err = msg;
    ctx->err_loc = loc;
  }
  return status;
}

void *nngp_scratch(nngp_ctx *ctx, int slot, size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (ctx->scratch_cap[slot] >= bytes) return ctx->scratch[slot];
  if (ctx->scratch[slot]) {
    cudaStreamSynchronize(ctx->stream);
    cudaFree(ctx->scratch[slot]);
    ctx->scratch[slot] = nullptr;
    ctx->scratch_cap[slot] = 0;
  }
  const size_t cap = bytes + bytes / 4;  // headroom for slowly growing requests
  void *p = nullptr;
  if (cudaMalloc(&p, cap) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  ctx->scratch[slot] = p;
  ctx->scratch_cap[slot] = cap;
  return p;
}

void *nngp_pinned(nngp_ctx *ctx, size_t bytes) {
  if (ctx->pinned_cap >= bytes) return ctx->pinned;
  if (ctx->pinned) {
    cudaStreamSynchronize(ctx->stream);
    cudaFreeHost(ctx->pinned);
  }
  ctx->pinned = nullptr;
  ctx->pinned_cap = 0;
  if (cudaMallocHost(&ctx->pinned, bytes) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  ctx->pinned_cap = bytes;
  return ctx->pinned;
}

int nngp_reset_status(nngp_ctx *ctx, unsigned long long *d_status) {
  NNGP_CUDA_TRY(ctx, cudaMemsetAsync(d_status, 0xFF, sizeof(unsigned long long), ctx->stream));
  return NNGP_OK;
}

// Reads the status word (synchronizes the stream) and maps it to an error.
int nngp_check_status(nngp_ctx *ctx, unsigned long long *d_status, const char *what) {
  unsigned long long h = 0;
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(&h, d_status, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
  NNGP_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  if (h == NNGP_STATUS_OK) return NNGP_OK;
  const unsigned code = (unsigned)(h >> 48);
  const int64_t loc = (int64_t)(h & 0xFFFFFFFFFFFFull);
  char buf[256];
  if (code == 1) {
    snprintf(buf, sizeof buf, "%s: neighborhood covariance not positive definite at location %lld (dpotrf failed)",
             what, (long long)loc);
    return nngp_fail(ctx, NNGP_ERR_NOT_SPD, buf, loc);
  }
  if (code == 2) {
    snprintf(buf, sizeof buf, "%s: beta Gram matrix not positive definite (dpotrf failed)", what);
    return nngp_fail(ctx, NNGP_ERR_NOT_SPD, buf, loc);
  }
  if (code == 3) {
    snprintf(buf, sizeof buf, "%s: a host-fed random stream ran out", what);
    return nngp_fail(ctx, NNGP_ERR_STREAM, buf, loc);
  }
  snprintf(buf, sizeof buf, "%s: device status %u at %lld", what, code, (long long)loc);
  return nngp_fail(ctx, NNGP_ERR_CUDA, buf, loc);
}

extern "C" {

int nngp_create(int device, nngp_ctx **out) {
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= device || device < 0) {
    cudaGetLastError();
    return NNGP_ERR_CUDA;
  }
  if (cudaSetDevice(device) != cudaSuccess) return NNGP_ERR_CUDA;
  nngp_ctx *ctx = new nngp_ctx();
  ctx->device = device;
  cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
  if (cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete ctx;
    return NNGP_ERR_CUDA;
  }
  ctx->stream = ctx->own_stream;
  // keep freed stream-ordered allocations in the pool between calls
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t thr = ~0ull;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  *out = ctx;
  return NNGP_OK;
}

void nngp_destroy(nngp_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  nngp_bf_cache_release(ctx);
  cudaStreamSynchronize(ctx->stream);
  for (int s = 0; s < S_NUM_SLOTS; s++)
    if (ctx->scratch[s]) cudaFree(ctx->scratch[s]);
  if (ctx->pinned) cudaFreeHost(ctx->pinned);
  for (auto &pr : ctx->timed) {
    cudaEventDestroy(pr.first);
    cudaEventDestroy(pr.second);
  }
  for (cudaEvent_t e : ctx->event_pool) cudaEventDestroy(e);
  for (cudaEvent_t e : ctx->chunk_events) cudaEventDestroy(e);
  if (ctx->copy_stream) {
    cudaStreamSynchronize(ctx->copy_stream);
    cudaStreamDestroy(ctx->copy_stream);
  }
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
}

const char *nngp_error_message(const nngp_ctx *ctx) { return ctx ? ctx->err.c_str() : "no context"; }
int64_t nngp_error_location(const nngp_ctx *ctx) { return ctx ? ctx->err_loc : -1; }

int nngp_set_stream(nngp_ctx *ctx, void *stream) {
  ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
  return NNGP_OK;
}
void *nngp_get_stream(const nngp_ctx *ctx) { return (void *)ctx->stream; }

int nngp_synchronize(nngp_ctx *ctx) {
  NNGP_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return NNGP_OK;
}

int64_t nngp_launch_count(const nngp_ctx *ctx) { return ctx->launches; }
void nngp_reset_launch_count(nngp_ctx *ctx) { ctx->launches = 0; }
int nngp_max_neighbors(void) { return NNGP_MAX_M; }
int64_t nngp_n_indx(int n, int m) { return nngp_nindx(n, m); }

}  // extern "C"
