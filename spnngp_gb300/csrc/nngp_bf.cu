#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>
#include "nngp_internal.h"

// Host side of the B/F pass: plans (job tables), dispatch to the kernel
// instantiations (nngp_bf_inst.cu: the FP64 shared-memory kernel for m <= 24, one
// object per neighbor bound and correlation code; nngp_bfwd_inst.cu: the FP64
// warp-per-location kernel for 24 < m <= 32; nngp_bfr_inst.cu: the register FP32R kernel for
// m <= 16; nngp_bfw_inst.cu: the warp-per-location FP32R kernel for
// 16 < m <= 32), the autotuner of the register kernel's launch shape, and the
// fixed-order reductions.  The kernels are documented in nngp_bf_kernel.cuh,
// nngp_bfwd_kernel.cuh, nngp_bfr_kernel.cuh and nngp_bfw_kernel.cuh.
namespace nngp_bf {
template <int M, int MODE, int COV>
int launch_one(nngp_ctx *ctx, const BFPlan *pl, bool fallback_pass, int t0, int t1);
template <int M>
constexpr int bf_tpb() {
  return M <= 16 ? 64 : 32;
}
}  // namespace nngp_bf
namespace nngp_bfr {
template <int M, int MODE, int COV>
int launch_reg(nngp_ctx *ctx, const BFPlan *pl, int wpb, int grid, int t0, int t1, int tm);
template <int M, int MODE, int COV>
int occupancy(int wpb, int tm);
}  // namespace nngp_bfr
namespace nngp_bfw {
template <int M, int MODE, int COV>
int launch_warp(nngp_ctx *ctx, const BFPlan *pl, int t0, int t1, int wpb, int grid);
template <int M, int MODE, int COV>
int occupancy_warp(int wpb);
}  // namespace nngp_bfw
namespace nngp_bfwd {
template <int M, int MODE, int COV>
int launch_warp_d(nngp_ctx *ctx, const BFPlan *pl, bool fallback_pass, int t0, int t1, int wpb, int grid);
}  // namespace nngp_bfwd
namespace nngp_bfdf {
template <int M, int MODE, int COV>
int launch_df(nngp_ctx *ctx, const BFPlan *pl);
}  // namespace nngp_bfdf
namespace nngp_bfwdf {
template <int M, int MODE, int COV>
int launch_wdf(nngp_ctx *ctx, const BFPlan *pl);
}  // namespace nngp_bfwdf
using namespace nngp_bf;

namespace {
// Number of non-zero flag bytes (grid-stride; one atomic per thread).
__global__ void count_flags_kernel(const unsigned char *__restrict__ flags, size_t n,
                                   unsigned long long *__restrict__ out) {
  unsigned long long c = 0;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    c += flags[k] != 0;
  if (c) atomicAdd(out, c);
}

// Fixed-order reduction of per-tile partials in two levels.  Level 1: block (job, b) sums
// tiles [b C, (b + 1) C) of the job (C = kReduceChunk); thread t sums tiles t, t + 256, ... of
// the chunk, value by value in order, then a fixed binary tree over the 256 threads (pairs
// t, t + w for w = 128, 64, ..., 1), every value's tree in the same barriers.  Values are taken
// eight at a time so each thread reads whole rows of the tile-major partial array
// (contiguous across the warp).  With jobs_fb, the FP64 re-solve's partials of the tiles marked
// in fb_marks are summed the same way into a second slot (skipped when no tile was recorded:
// fb_count == 0).  Level 2: the chunk sums in chunk order, the re-solve's sums added last.  A
// job of at most C tiles gets the single-block order (x + 0.0 == x).
constexpr int kReduceChunk = 1024;

__global__ void reduce_chunks_kernel(const BFJob *__restrict__ jobs, const BFJob *__restrict__ jobs_fb,
                                     const unsigned *__restrict__ fb_marks, const int *__restrict__ fb_count,
                                     int ng, int nchunks, double *__restrict__ out2) {
  const int jid = blockIdx.x / nchunks, b = blockIdx.x % nchunks;
  const BFJob job = jobs[jid];
  __shared__ double sbuf16[16][256];
  const bool any_fb = jobs_fb && *fb_count > 0;
  double *o = out2 + (size_t)blockIdx.x * 2 * ng;
  const int t0 = b * kReduceChunk;
  const int t1 = min(job.ntiles, t0 + kReduceChunk);
  for (int v0 = 0; v0 < ng; v0 += 8) {
    double acc[8], accf[8];
#pragma unroll
    for (int j = 0; j < 8; j++) acc[j] = accf[j] = 0.0;
    for (int t = t0 + threadIdx.x; t < t1; t += 256) {
      const double *row = job.partial + (size_t)t * ng + v0;
#pragma unroll
      for (int j = 0; j < 8; j++)
        if (v0 + j < ng) acc[j] += row[j];
    }
    if (any_fb) {
      const BFJob jf = jobs_fb[jid];
      const int f1 = min(jf.ntiles, t0 + kReduceChunk);
      for (int t = t0 + threadIdx.x; t < f1; t += 256) {
        if (!fb_marks[jf.tile0 + t]) continue;
        const double *row = jf.partial + (size_t)t * ng + v0;
#pragma unroll
        for (int j = 0; j < 8; j++)
          if (v0 + j < ng) accf[j] += row[j];
      }
    }
    // the sixteen trees (eight values, main and re-solve sums) side by side: per value the
    // order of block_sum256, one barrier per level for all of them
#pragma unroll
    for (int j = 0; j < 8; j++) {
      sbuf16[j][threadIdx.x] = acc[j];
      sbuf16[8 + j][threadIdx.x] = accf[j];
    }
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
      if (threadIdx.x < w) {
#pragma unroll
        for (int j = 0; j < 16; j++) sbuf16[j][threadIdx.x] += sbuf16[j][threadIdx.x + w];
      }
      __syncthreads();
    }
    if (threadIdx.x < 8 && v0 + (int)threadIdx.x < ng) {
      const int j = threadIdx.x;
      o[v0 + j] = sbuf16[j][0];
      o[ng + v0 + j] = jobs_fb ? sbuf16[8 + j][0] : 0.0;
    }
    __syncthreads();
  }
}

__global__ void reduce_final_kernel(const double *__restrict__ out2, int ng, int nchunks, bool with_fb,
                                    double *__restrict__ out) {
  const int jid = blockIdx.x;
  for (int v = threadIdx.x; v < ng; v += blockDim.x) {
    double s = 0.0, sf = 0.0;
    const double *o = out2 + (size_t)jid * nchunks * 2 * ng + v;
    int b = 0;
    for (; b + 8 <= nchunks; b += 8) {  // eight chunks' loads in flight, added in chunk order
      double x[8], xf[8];
#pragma unroll
      for (int u = 0; u < 8; u++) {
        x[u] = o[(size_t)(b + u) * 2 * ng];
        xf[u] = o[(size_t)(b + u) * 2 * ng + ng];
      }
#pragma unroll
      for (int u = 0; u < 8; u++) {
        s += x[u];
        sf += xf[u];
      }
    }
    for (; b < nchunks; b++) {
      s += o[(size_t)b * 2 * ng];
      sf += o[(size_t)b * 2 * ng + ng];
    }
    out[(size_t)jid * ng + v] = with_fb ? s + sf : s;
  }
}

}  // namespace

namespace {
// The FP64 kernel: the FP64 form's primary pass, or the re-solve of the locations an FP32R
// pass flagged (fallback_pass)
template <int MODE, int COV>
int launch_mode_c(nngp_ctx *ctx, const BFPlan *pl, bool fallback_pass, int t0, int t1) {
  if (pl->mmax <= 16) return launch_one<16, MODE, COV>(ctx, pl, fallback_pass, t0, t1);
  // 24-neighbor bound: the thread-per-location kernel still holds two blocks per SM and beats the
  // warp form (38 against 67 ms at n = 1e6); at 32 the warp form wins (97 against 206 ms)
  if (pl->mmax <= 24) return launch_one<24, MODE, COV>(ctx, pl, fallback_pass, t0, t1);
  return nngp_bfwd::launch_warp_d<32, MODE, COV>(ctx, pl, fallback_pass, t0, t1, 4, 0);
}

template <int MODE>
int launch_mode(nngp_ctx *ctx, const BFPlan *pl, bool fallback_pass, int t0, int t1) {
  switch (pl->cov) {
    case NNGP_COV_EXP: return launch_mode_c<MODE, NNGP_COV_EXP>(ctx, pl, fallback_pass, t0, t1);
    case NNGP_COV_SPH: return launch_mode_c<MODE, NNGP_COV_SPH>(ctx, pl, fallback_pass, t0, t1);
    case NNGP_COV_MAT_HALF: return launch_mode_c<MODE, NNGP_COV_MAT_HALF>(ctx, pl, fallback_pass, t0, t1);
    case NNGP_COV_GAU: return launch_mode_c<MODE, NNGP_COV_GAU>(ctx, pl, fallback_pass, t0, t1);
    default: return launch_mode_c<MODE, NNGP_COV_ANY>(ctx, pl, fallback_pass, t0, t1);
  }
}

// The warp-per-location FP32R kernel (16 < m <= 32) on tiles [t0, t1) with wpb warps per block
// and `grid` blocks (0: one tile per warp), or (query_occ) its blocks per SM at wpb.
template <int M, int MODE, int COV>
int warp_call_c(nngp_ctx *ctx, const BFPlan *pl, int t0, int t1, int wpb, int grid, bool query_occ) {
  return query_occ ? nngp_bfw::occupancy_warp<M, MODE, COV>(wpb)
                   : nngp_bfw::launch_warp<M, MODE, COV>(ctx, pl, t0, t1, wpb, grid);
}
template <int M, int MODE>
int warp_call_m(nngp_ctx *ctx, const BFPlan *pl, int t0, int t1, int wpb, int grid, bool query_occ) {
  switch (pl->cov) {
    case NNGP_COV_EXP: return warp_call_c<M, MODE, NNGP_COV_EXP>(ctx, pl, t0, t1, wpb, grid, query_occ);
    case NNGP_COV_SPH: return warp_call_c<M, MODE, NNGP_COV_SPH>(ctx, pl, t0, t1, wpb, grid, query_occ);
    case NNGP_COV_MAT_HALF: return warp_call_c<M, MODE, NNGP_COV_MAT_HALF>(ctx, pl, t0, t1, wpb, grid, query_occ);
    case NNGP_COV_GAU: return warp_call_c<M, MODE, NNGP_COV_GAU>(ctx, pl, t0, t1, wpb, grid, query_occ);
    default: return warp_call_c<M, MODE, NNGP_COV_ANY>(ctx, pl, t0, t1, wpb, grid, query_occ);
  }
}
int warp_call(nngp_ctx *ctx, const BFPlan *pl, int t0, int t1, int wpb = 4, int grid = 0, bool query_occ = false) {
  const bool m1 = pl->mode == 1;
  if (pl->mmax <= 20)
    return m1 ? warp_call_m<20, 1>(ctx, pl, t0, t1, wpb, grid, query_occ)
              : warp_call_m<20, 0>(ctx, pl, t0, t1, wpb, grid, query_occ);
  if (pl->mmax <= 24)
    return m1 ? warp_call_m<24, 1>(ctx, pl, t0, t1, wpb, grid, query_occ)
              : warp_call_m<24, 0>(ctx, pl, t0, t1, wpb, grid, query_occ);
  return m1 ? warp_call_m<32, 1>(ctx, pl, t0, t1, wpb, grid, query_occ)
            : warp_call_m<32, 0>(ctx, pl, t0, t1, wpb, grid, query_occ);
}

// ---------------------------------------------------------------- register kernel
// Calls launch_reg (query_occ false) or occupancy (true) of the plan's instantiation.
template <int M, int MODE>
int reg_call_m(nngp_ctx *ctx, const BFPlan *pl, int wpb, int grid, bool query_occ, int t0, int t1, int tm) {
  using namespace nngp_bfr;
  switch (pl->cov) {
    case NNGP_COV_EXP:
      return query_occ ? occupancy<M, MODE, NNGP_COV_EXP>(wpb, tm) : launch_reg<M, MODE, NNGP_COV_EXP>(ctx, pl, wpb, grid, t0, t1, tm);
    case NNGP_COV_SPH:
      return query_occ ? occupancy<M, MODE, NNGP_COV_SPH>(wpb, tm) : launch_reg<M, MODE, NNGP_COV_SPH>(ctx, pl, wpb, grid, t0, t1, tm);
    case NNGP_COV_MAT_HALF:
      return query_occ ? occupancy<M, MODE, NNGP_COV_MAT_HALF>(wpb, tm)
                       : launch_reg<M, MODE, NNGP_COV_MAT_HALF>(ctx, pl, wpb, grid, t0, t1, tm);
    case NNGP_COV_GAU:
      return query_occ ? occupancy<M, MODE, NNGP_COV_GAU>(wpb, tm) : launch_reg<M, MODE, NNGP_COV_GAU>(ctx, pl, wpb, grid, t0, t1, tm);
    default:
      return query_occ ? occupancy<M, MODE, NNGP_COV_ANY>(wpb, tm) : launch_reg<M, MODE, NNGP_COV_ANY>(ctx, pl, wpb, grid, t0, t1, tm);
  }
}
int reg_call(nngp_ctx *ctx, const BFPlan *pl, int wpb, int grid, bool query_occ, int t0, int t1, int tm) {
  const bool m1 = pl->mode == 1;
  switch (pl->reg_m) {
    case 10:
      return m1 ? reg_call_m<10, 1>(ctx, pl, wpb, grid, query_occ, t0, t1, tm)
                : reg_call_m<10, 0>(ctx, pl, wpb, grid, query_occ, t0, t1, tm);
    case 15:
      return m1 ? reg_call_m<15, 1>(ctx, pl, wpb, grid, query_occ, t0, t1, tm)
                : reg_call_m<15, 0>(ctx, pl, wpb, grid, query_occ, t0, t1, tm);
    default:
      return m1 ? reg_call_m<16, 1>(ctx, pl, wpb, grid, query_occ, t0, t1, tm)
                : reg_call_m<16, 0>(ctx, pl, wpb, grid, query_occ, t0, t1, tm);
  }
}

// Blocks of the launch shape (wpb, grid_mode) for this plan: grid_mode 0 gives every warp one
// tile; k > 0 caps the grid at k x (resident blocks per SM) x SMs, each warp looping over tiles.
int reg_grid(nngp_ctx *ctx, const BFPlan *pl, int wpb, int grid_mode, int ntiles, int tm) {
  const int full = (ntiles + wpb - 1) / wpb;
  if (grid_mode <= 0) return full > 0 ? full : 1;
  const int occ = reg_call(ctx, pl, wpb, 0, true, 0, 0, tm);
  const long cap = (long)grid_mode * occ * (ctx->sm_count > 0 ? ctx->sm_count : 1);
  return (int)(cap < full ? cap : full);
}

// Tuning class: kernel variant and size class.  Sizes from the sample cap up share one class
// (the sample, and so the choice, is the same for them).
std::string tune_key(const BFPlan *pl, int ntiles) {
  int bucket = 0;
  while ((1 << (bucket + 1)) <= ntiles && (1 << (bucket + 1)) <= 65536) bucket++;
  char k[96];
  snprintf(k, sizeof k, "M=%d mode=%d cov=%d tiles~2^%d", pl->reg_m, pl->mode, pl->cov, bucket);
  return k;
}

// Times every candidate shape on the plan itself (each run rewrites the same outputs with
// the same values: the results do not depend on the shape) and keeps the fastest.
int tune_reg(nngp_ctx *ctx, const BFPlan *pl, TuneEntry &best, int t0, int t1) {
  // shared-memory layouts: 1-6 (8) warps per block; tensor-memory layout: 4 or 8 warps
  struct Cand {
    int wpb, tm;
  };
  static const Cand kCand[] = {{1, 0}, {2, 0}, {3, 0}, {4, 0}, {5, 0}, {6, 0}, {8, 0}, {4, 1}, {8, 1}};
  static const int kGrid[] = {0, 1, 2};
  cudaEvent_t e0, e1;
  NNGP_CUDA_TRY(ctx, cudaEventCreate(&e0));
  NNGP_CUDA_TRY(ctx, cudaEventCreate(&e1));
  best = TuneEntry();
  best.ms = 1e30;
  std::string detail;
  int st = NNGP_OK;
  for (const Cand &cd : kCand) {
    const int wpb = cd.wpb, tm = cd.tm;
    if (tm ? !nngp_bfr_has_tm(pl->reg_m) || wpb > nngp_bfr_max_wpb(pl->reg_m, true)
           : wpb > nngp_bfr_max_wpb(pl->reg_m, false))
      continue;
    if (reg_call(ctx, pl, wpb, 0, true, 0, 0, tm) <= 0) continue;  // no block of this shape fits
    const int full = reg_grid(ctx, pl, wpb, 0, t1 - t0, tm);
    for (int gm : kGrid) {
      const int grid = reg_grid(ctx, pl, wpb, gm, t1 - t0, tm);
      if (gm > 0 && grid >= full) continue;  // same as the one-tile-per-warp grid
      if ((st = reg_call(ctx, pl, wpb, grid, false, t0, t1, tm))) break;  // warm-up
      cudaEventRecord(e0, ctx->stream);
      if ((st = reg_call(ctx, pl, wpb, grid, false, t0, t1, tm))) break;
      cudaEventRecord(e1, ctx->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess) {
        st = nngp_fail(ctx, NNGP_ERR_CUDA, "autotune: event synchronisation failed");
        break;
      }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      char buf[64];
      snprintf(buf, sizeof buf, "%s%dx%d%s:%.4f", detail.empty() ? "" : " ", wpb, grid, tm ? "t" : "", ms);
      detail += buf;
      if (ms < best.ms) {
        best.ms = ms;
        best.wpb = wpb;
        best.grid_mode = gm;
        best.tm = tm;
      }
    }
    if (st) break;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  best.detail = detail;
  return st;
}

// Passes smaller than kTuneMinTiles (64 K locations) run the default shape: their time is
// launch overhead more than shape.  Tuning times candidates on at most kTuneSampleTiles.
constexpr int kTuneMinTiles = 2048;
constexpr int kTuneSampleTiles = 65536;

int run_reg(nngp_ctx *ctx, const BFPlan *pl, int t0, int t1) {
  int wpb = 4, gm = 0, tm = 0;
  if (ctx->force_wpb > 0) {
    wpb = ctx->force_wpb;
    gm = ctx->force_grid_mode;
    tm = ctx->force_tm && nngp_bfr_has_tm(pl->reg_m) ? 1 : 0;
  } else {
    const std::string key = tune_key(pl, t1 - t0);
    auto it = ctx->tuned.find(key);
    if (it != ctx->tuned.end()) {
      wpb = it->second.wpb;
      gm = it->second.grid_mode;
      tm = it->second.tm;
    } else if (ctx->autotune && t1 - t0 >= kTuneMinTiles) {
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      cudaStreamIsCapturing(ctx->stream, &cs);
      if (cs == cudaStreamCaptureStatusNone) {
        // candidates are timed on a bounded sample of the plan's tiles (a large plan -- a
        // 5000-job conjugate sweep -- would otherwise spend seconds per candidate)
        TuneEntry e;
        const int st = tune_reg(ctx, pl, e, t0, t1 - t0 > kTuneSampleTiles ? t0 + kTuneSampleTiles : t1);
        if (st) return st;
        ctx->tuned[key] = e;
        wpb = e.wpb;
        gm = e.grid_mode;
        tm = e.tm;
      }
    }
  }
  if (tm) {
    wpb = wpb > 4 ? 8 : 4;  // the tensor-memory layout runs 4 or 8 warps per block
  } else {
    const int wmax = nngp_bfr_max_wpb(pl->reg_m);
    if (wpb > wmax) wpb = wmax;  // a forced shape larger than the block limit of this bound
  }
  return reg_call(ctx, pl, wpb, reg_grid(ctx, pl, wpb, gm, t1 - t0, tm), false, t0, t1, tm);
}

// Launch shape of a warp-per-location kernel, tuned like the register kernel's: warps per
// block 1, 2 or 4, each with one tile per warp or a persistent grid of 1 or 2 x resident
// blocks x SMs, timed on the plan's own tiles (at most kTuneSampleTiles) on its first pass of
// a size class; passes under stream capture or of fewer than kTuneMinTiles tiles use the tuned
// or the default shape (4 warps, one tile per warp).  call(t0, t1, wpb, grid) launches the
// kernel, occ(wpb) returns its blocks per SM (0: that block size cannot run).
template <class Call, class Occ>
int run_tuned_warps(nngp_ctx *ctx, const std::string &key, int t0, int t1, Call call, Occ occ) {
  auto grid_of = [&](int wpb, int gm, int ntiles) {
    const int full = (ntiles + wpb - 1) / wpb;
    if (gm <= 0) return full;
    const long cap = (long)gm * occ(wpb) * (ctx->sm_count > 0 ? ctx->sm_count : 1);
    return (int)(cap < full ? (cap > 0 ? cap : 1) : full);
  };
  auto it = ctx->tuned.find(key);
  if (it == ctx->tuned.end() && ctx->autotune && t1 - t0 >= kTuneMinTiles) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(ctx->stream, &cs);
    if (cs == cudaStreamCaptureStatusNone) {
      const int s1 = t1 - t0 > kTuneSampleTiles ? t0 + kTuneSampleTiles : t1;
      TuneEntry best;
      best.ms = 1e30;
      cudaEvent_t e0, e1;
      NNGP_CUDA_TRY(ctx, cudaEventCreate(&e0));
      NNGP_CUDA_TRY(ctx, cudaEventCreate(&e1));
      int st = NNGP_OK;
      for (int wpb : {1, 2, 4}) {
        if (occ(wpb) <= 0) continue;
        const int full = grid_of(wpb, 0, s1 - t0);
        for (int gm : {0, 1, 2}) {
          const int grid = grid_of(wpb, gm, s1 - t0);
          if (gm > 0 && grid >= full) continue;
          if ((st = call(t0, s1, wpb, grid))) break;  // warm-up
          cudaEventRecord(e0, ctx->stream);
          if ((st = call(t0, s1, wpb, grid))) break;
          cudaEventRecord(e1, ctx->stream);
          if (cudaEventSynchronize(e1) != cudaSuccess) {
            st = nngp_fail(ctx, NNGP_ERR_CUDA, "autotune: event synchronisation failed");
            break;
          }
          float ms = 0.f;
          cudaEventElapsedTime(&ms, e0, e1);
          char buf[48];
          snprintf(buf, sizeof buf, "%s%dx%d:%.4f", best.detail.empty() ? "" : " ", wpb, grid, ms);
          best.detail += buf;
          if (ms < best.ms) {
            best.ms = ms;
            best.wpb = wpb;
            best.grid_mode = gm;
          }
        }
        if (st) break;
      }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      if (st) return st;
      it = ctx->tuned.emplace(key, best).first;
    }
  }
  const int wpb = it != ctx->tuned.end() ? it->second.wpb : 4;
  const int gm = it != ctx->tuned.end() ? it->second.grid_mode : 0;
  return call(t0, t1, wpb, grid_of(wpb, gm, t1 - t0));
}

// The FP32R warp kernel (16 < m <= 32), tuning classes "warp M=20|24|32 ...".
int run_warp(nngp_ctx *ctx, const BFPlan *pl, int t0, int t1) {
  std::string key = tune_key(pl, t1 - t0);  // "M=<reg_m> ...": the warp kernel's bound instead
  key = "warp M=" + std::to_string(pl->mmax <= 20 ? 20 : pl->mmax <= 24 ? 24 : 32) + key.substr(key.find(' '));
  return run_tuned_warps(
      ctx, key, t0, t1, [&](int a, int b, int wpb, int grid) { return warp_call(ctx, pl, a, b, wpb, grid); },
      [&](int wpb) { return warp_call(ctx, pl, 0, 0, wpb, 0, true); });
}

template <int M>
int launch_df_m(nngp_ctx *ctx, const BFPlan *pl) {
  using nngp_bfdf::launch_df;
  const bool fused = pl->mode == 1;
  switch (pl->cov) {
    case NNGP_COV_EXP: return fused ? launch_df<M, 1, NNGP_COV_EXP>(ctx, pl) : launch_df<M, 0, NNGP_COV_EXP>(ctx, pl);
    case NNGP_COV_SPH: return fused ? launch_df<M, 1, NNGP_COV_SPH>(ctx, pl) : launch_df<M, 0, NNGP_COV_SPH>(ctx, pl);
    case NNGP_COV_MAT_HALF:
      return fused ? launch_df<M, 1, NNGP_COV_MAT_HALF>(ctx, pl) : launch_df<M, 0, NNGP_COV_MAT_HALF>(ctx, pl);
    case NNGP_COV_GAU: return fused ? launch_df<M, 1, NNGP_COV_GAU>(ctx, pl) : launch_df<M, 0, NNGP_COV_GAU>(ctx, pl);
    default: return fused ? launch_df<M, 1, NNGP_COV_ANY>(ctx, pl) : launch_df<M, 0, NNGP_COV_ANY>(ctx, pl);
  }
}
int launch_wdf_32(nngp_ctx *ctx, const BFPlan *pl) {
  using nngp_bfwdf::launch_wdf;
  const bool fused = pl->mode == 1;
  switch (pl->cov) {
    case NNGP_COV_EXP: return fused ? launch_wdf<32, 1, NNGP_COV_EXP>(ctx, pl) : launch_wdf<32, 0, NNGP_COV_EXP>(ctx, pl);
    case NNGP_COV_SPH: return fused ? launch_wdf<32, 1, NNGP_COV_SPH>(ctx, pl) : launch_wdf<32, 0, NNGP_COV_SPH>(ctx, pl);
    case NNGP_COV_MAT_HALF:
      return fused ? launch_wdf<32, 1, NNGP_COV_MAT_HALF>(ctx, pl) : launch_wdf<32, 0, NNGP_COV_MAT_HALF>(ctx, pl);
    case NNGP_COV_GAU: return fused ? launch_wdf<32, 1, NNGP_COV_GAU>(ctx, pl) : launch_wdf<32, 0, NNGP_COV_GAU>(ctx, pl);
    default: return fused ? launch_wdf<32, 1, NNGP_COV_ANY>(ctx, pl) : launch_wdf<32, 0, NNGP_COV_ANY>(ctx, pl);
  }
}

// The double-float re-solve of an FP32R plan's flagged tiles: thread per location for bounds
// 16 and 24 (nngp_bfdf_kernel.cuh; the flagged-tile list's tile is the FP64 kernel's, 64
// locations up to 16 neighbors and 32 beyond), warp per location for 32 (nngp_bfwdf_kernel.cuh:
// a thread-per-location triangle of that size leaves one 32-thread block per SM).
int launch_df_any(nngp_ctx *ctx, const BFPlan *pl) {
  if (pl->mmax <= 16) return launch_df_m<16>(ctx, pl);
  return pl->mmax <= 24 ? launch_df_m<24>(ctx, pl) : launch_wdf_32(ctx, pl);
}

// Primary pass over tiles [t0, t1), or (fallback_pass) the FP64 re-solve of the recorded tiles.
int launch_pass(nngp_ctx *ctx, const BFPlan *pl, bool fp32r, bool fallback_pass, int t0, int t1) {
  if (fp32r && !fallback_pass) return pl->reg_m > 0 ? run_reg(ctx, pl, t0, t1) : run_warp(ctx, pl, t0, t1);
  return pl->mode == 0 ? launch_mode<0>(ctx, pl, fallback_pass, t0, t1)
                       : launch_mode<1>(ctx, pl, fallback_pass, t0, t1);
}

}  // namespace

int nngp_bf_tile(int precision, int mmax) {
  if (precision == NNGP_FP32R) return 32;  // both FP32R kernels' tiles are one warp's
  return mmax <= 16 ? bf_tpb<16>() : bf_tpb<32>();
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
  pl->reg_m = nngp_reg_m(precision, mmax);
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
    pl->d_fb_words = (unsigned *)own(sizeof(unsigned) * (1 + (size_t)pl->tiles_fb));
    pl->d_fb_list = (int *)own(sizeof(int) * (size_t)(pl->tiles_fb > 0 ? pl->tiles_fb : 1));
    if (!pl->d_fb_words || !pl->d_fb_list) return nngp_fail(ctx, NNGP_ERR_NO_MEMORY, "device allocation failed");
    // flagged tiles: double-float kernel first, then FP64 for the tiles it cannot certify
    pl->d_fb64_list = (int *)own(sizeof(int) * (size_t)(pl->tiles_fb > 0 ? pl->tiles_fb : 1));
    pl->d_fb64_locs = (unsigned long long *)own(2 * sizeof(unsigned long long));
    if (!pl->d_fb64_list || !pl->d_fb64_locs) return nngp_fail(ctx, NNGP_ERR_NO_MEMORY, "device allocation failed");
    pl->d_fb64_count = reinterpret_cast<int *>(pl->d_fb64_locs + 1);
    size_t fb = 0;
    for (const PassEval &e : evals) fb += (size_t)datas[e.data].n;
    pl->flags_bytes = fb;
    pl->d_flags = (unsigned char *)own(fb);
    if (!pl->d_partial_fb || !pl->d_flags) return nngp_fail(ctx, NNGP_ERR_NO_MEMORY, "device allocation failed");
  }
  {
    int most = 1;
    for (const BFJob &j : jobs) most = std::max(most, (j.ntiles + kReduceChunk - 1) / kReduceChunk);
    for (const BFJob &j : jobs_fb) most = std::max(most, (j.ntiles + kReduceChunk - 1) / kReduceChunk);
    pl->red_chunks = most;
    pl->d_partial2 = (double *)own(sizeof(double) * 2 * (size_t)pl->ng * pl->njobs * most);
    if (!pl->d_partial2) return nngp_fail(ctx, NNGP_ERR_NO_MEMORY, "device allocation failed");
  }
  size_t foff = 0;
  for (size_t k = 0; k < jobs.size(); k++) {
    jobs[k].partial = pl->d_partial + reinterpret_cast<size_t>(jobs[k].partial);
    if (precision == NNGP_FP32R) {
      jobs_fb[k].partial = pl->d_partial_fb + reinterpret_cast<size_t>(jobs_fb[k].partial);
      jobs[k].flags = jobs_fb[k].flags = pl->d_flags + foff;
      foff += (size_t)datas[evals[k].data].n;
      jobs[k].fb_tile0 = jobs_fb[k].tile0;
      jobs[k].fb_tpb = nngp_bf_tile(NNGP_FP64, mmax);
      jobs[k].fb_count = (int *)pl->d_fb_words;
      jobs[k].fb_marks = pl->d_fb_words + 1;
      jobs[k].fb_list = pl->d_fb_list;
    }
  }
  // the FP32R kernels read V as float (hi, lo) pairs: split it once for callers that did not
  // provide them (their V stays fixed for the plan's lifetime)
  std::vector<BFData> dv(datas);
  if (precision == NNGP_FP32R && mode == 1) {
    for (BFData &d : dv) {
      if (d.Vf || !d.V) continue;
      float2 *vf = (float2 *)own(sizeof(float2) * (size_t)d.n * nv);
      if (!vf) return nngp_fail(ctx, NNGP_ERR_NO_MEMORY, "device allocation failed");
      int st = nngp_split_v(ctx, d.V, (int64_t)d.n * nv, vf);
      if (st) return st;
      d.Vf = vf;
    }
  }
  pl->d_datas = (BFData *)own(sizeof(BFData) * datas.size());
  pl->d_jobs = (BFJob *)own(sizeof(BFJob) * jobs.size());
  if (!pl->d_datas || !pl->d_jobs) return nngp_fail(ctx, NNGP_ERR_NO_MEMORY, "device allocation failed");
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(pl->d_datas, dv.data(), sizeof(BFData) * dv.size(),
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

int nngp_bf_begin(nngp_ctx *ctx, const BFPlan *pl) {
  if (pl->precision == NNGP_FP32R) {
    NNGP_CUDA_TRY(ctx, cudaMemsetAsync(pl->d_flags, 0, pl->flags_bytes, ctx->stream));
    NNGP_CUDA_TRY(ctx, cudaMemsetAsync(pl->d_fb_words, 0, sizeof(unsigned) * (1 + (size_t)pl->tiles_fb), ctx->stream));
    if (pl->d_fb64_locs)
      NNGP_CUDA_TRY(ctx, cudaMemsetAsync(pl->d_fb64_locs, 0, 2 * sizeof(unsigned long long), ctx->stream));
  }
  return NNGP_OK;
}

int nngp_bf_primary(nngp_ctx *ctx, const BFPlan *pl, int t0, int t1) {
  if (t1 > pl->tiles) t1 = pl->tiles;
  if (t0 < 0) t0 = 0;
  if (t1 <= t0) return NNGP_OK;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (ctx->timing) {
    for (cudaEvent_t *e : {&e0, &e1}) {
      if (!ctx->event_pool.empty()) {
        *e = ctx->event_pool.back();
        ctx->event_pool.pop_back();
      } else {
        cudaEventCreate(e);
      }
    }
    cudaEventRecord(e0, ctx->stream);
  }
  const int st = launch_pass(ctx, pl, pl->precision == NNGP_FP32R, false, t0, t1);
  if (ctx->timing) {
    cudaEventRecord(e1, ctx->stream);
    ctx->timed.emplace_back(e0, e1);
  }
  return st;
}

int nngp_bf_finish(nngp_ctx *ctx, const BFPlan *pl, double *d_out) {
  int st;
  const bool fp32r = pl->precision == NNGP_FP32R;
  // FP32R: the re-solve of the recorded tiles (double-float first, FP64 for the tiles it
  // cannot certify), folded into the same fixed-order sums
  if (fp32r && (st = launch_df_any(ctx, pl))) return st;
  if (fp32r && (st = launch_pass(ctx, pl, false, true, 0, 0))) return st;
  reduce_chunks_kernel<<<pl->njobs * pl->red_chunks, 256, 0, ctx->stream>>>(
      pl->d_jobs, fp32r ? pl->d_jobs_fb : nullptr, fp32r ? pl->d_fb_words + 1 : nullptr,
      fp32r ? (const int *)pl->d_fb_words : nullptr, pl->ng, pl->red_chunks, pl->d_partial2);
  NNGP_LAUNCH_CHECK(ctx);
  reduce_final_kernel<<<pl->njobs, 64, 0, ctx->stream>>>(pl->d_partial2, pl->ng, pl->red_chunks, fp32r, d_out);
  NNGP_LAUNCH_CHECK(ctx);
  return NNGP_OK;
}

int nngp_bf_run(nngp_ctx *ctx, const BFPlan *pl, double *d_out) {
  int st;
  if ((st = nngp_bf_begin(ctx, pl))) return st;
  if ((st = nngp_bf_primary(ctx, pl, 0, pl->tiles))) return st;
  return nngp_bf_finish(ctx, pl, d_out);
}

int nngp_bf_launch(nngp_ctx *ctx, const BFPlan *pl, bool fp32r, bool fallback_pass) {
  return launch_pass(ctx, pl, fp32r, fallback_pass, 0, pl->tiles);
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
int nngp_set_autotune(nngp_ctx *ctx, int on) {
  if (!ctx) return NNGP_ERR_ARG;
  ctx->autotune = on != 0;
  return NNGP_OK;
}
int nngp_set_launch_shape(nngp_ctx *ctx, int warps_per_block, int grid_mode, int use_tmem) {
  if (!ctx) return NNGP_ERR_ARG;
  if (warps_per_block < 0 || warps_per_block > 8 || grid_mode < 0 || grid_mode > 64)
    return nngp_fail(ctx, NNGP_ERR_ARG, "launch shape: 0 <= warps_per_block <= 8, 0 <= grid_mode <= 64");
  ctx->force_wpb = warps_per_block;
  ctx->force_grid_mode = grid_mode;
  ctx->force_tm = use_tmem != 0;
  return NNGP_OK;
}
int nngp_autotune_report(nngp_ctx *ctx, char *buf, int len) {
  if (!ctx) return NNGP_ERR_ARG;
  std::string out;
  for (const auto &kv : ctx->tuned) {
    char line[160];
    snprintf(line, sizeof line, "%s: wpb=%d grid_mode=%d tmem=%d ms=%.4f | ", kv.first.c_str(), kv.second.wpb,
             kv.second.grid_mode, kv.second.tm, kv.second.ms);
    out += line;
    out += kv.second.detail;
    out += "\n";
  }
  if (buf && len > 0) {
    const size_t k = out.size() < (size_t)(len - 1) ? out.size() : (size_t)(len - 1);
    memcpy(buf, out.data(), k);
    buf[k] = 0;
  }
  return (int)ctx->tuned.size();
}
int nngp_fp32r_tiers(nngp_ctx *ctx, int64_t *double_float, int64_t *fp64) {
  if (!ctx || !double_float || !fp64) return NNGP_ERR_ARG;
  int64_t total = 0, locations = 0;
  const int st = nngp_fp32r_resolved(ctx, &total, &locations);
  if (st) return st;
  *double_float = 0;
  *fp64 = total;
  const BFPlan *pl = ctx->cache_plan;
  if (pl && pl->precision == NNGP_FP32R && pl->d_fb64_locs) {
    unsigned long long h = 0;
    NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(&h, pl->d_fb64_locs, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
    NNGP_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    *fp64 = (int64_t)h;
    *double_float = total - (int64_t)h;
  }
  return NNGP_OK;
}
int nngp_fp32r_resolved(nngp_ctx *ctx, int64_t *resolved, int64_t *locations) {
  if (!ctx || !resolved || !locations) return NNGP_ERR_ARG;
  *resolved = *locations = 0;
  const BFPlan *pl = ctx->cache_plan;
  if (!pl || pl->precision != NNGP_FP32R || pl->flags_bytes == 0) return NNGP_OK;
  unsigned long long *d_cnt = (unsigned long long *)nngp_malloc_async(ctx, sizeof(unsigned long long));
  if (!d_cnt) return nngp_fail(ctx, NNGP_ERR_NO_MEMORY, "device allocation failed");
  unsigned long long h = 0;
  NNGP_CUDA_TRY(ctx, cudaMemsetAsync(d_cnt, 0, sizeof h, ctx->stream));
  count_flags_kernel<<<256, 256, 0, ctx->stream>>>(pl->d_flags, pl->flags_bytes, d_cnt);
  NNGP_LAUNCH_CHECK(ctx);
  NNGP_CUDA_TRY(ctx, cudaMemcpyAsync(&h, d_cnt, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
  nngp_free_async(ctx, d_cnt);
  NNGP_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  *resolved = (int64_t)h;
  *locations = (int64_t)pl->flags_bytes;
  return NNGP_OK;
}
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
__global__ void split_v_kernel(const double *__restrict__ V, int64_t count, float2 *__restrict__ Vf) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < count) {
    const double v = V[t];
    const float h = (float)v;
    Vf[t] = make_float2(h, (float)(v - (double)h));
  }
}

__global__ void prepare_coords_kernel(const double *__restrict__ cm, int n, int i0, int i1,
                                      double *__restrict__ xy, float *__restrict__ xyf) {
  const int i = i0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= i1) return;
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

int nngp_split_v(nngp_ctx *ctx, const double *V, int64_t count, float2 *Vf) {
  if (count <= 0) return NNGP_OK;
  split_v_kernel<<<(unsigned)((count + 255) / 256), 256, 0, ctx->stream>>>(V, count, Vf);
  NNGP_LAUNCH_CHECK(ctx);
  return NNGP_OK;
}

int nngp_prepare_coords(nngp_ctx *ctx, const double *cm, int n, double *xy, float *xyf, int i0, int i1) {
  if (i1 < 0 || i1 > n) i1 = n;
  if (i1 <= i0) return NNGP_OK;
  prepare_coords_kernel<<<(i1 - i0 + 255) / 256, 256, 0, ctx->stream>>>(cm, n, i0, i1, xy, xyf);
  NNGP_LAUNCH_CHECK(ctx);
  return NNGP_OK;
}
