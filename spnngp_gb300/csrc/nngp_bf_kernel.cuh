// Kernel template of the B/F neighborhood-solve pass (instantiated in
// nngp_bf_inst_*.cu, dispatched from nngp_bf.cu): one thread solves one location's m x m
// neighborhood system (reference updateBF, src/rNNGP.cpp:46-101, and
// updateConjBF, src/cNNGP.cpp:24-69).
//
// Layout: a block owns a tile of TPB consecutive locations of one job (job =
// one dataset at one parameter set).  Each thread keeps the packed lower
// triangle of its covariance in shared memory, interleaved across threads
// (element e of thread t at tri[e*TPB + t], so every access is bank-conflict
// free), and the row being factored plus 1/diag in registers.  The Cholesky is
// the row-oriented (Banachiewicz) form: row r of L needs only rows < r, one
// shared load per FMA.  The forward solve for c is fused into the factor loop;
// B is the back substitution.
//
// This is the FP64 form (everything in double) for neighbor bounds m <= 24 (the
// 32-neighbor bound runs the warp-per-location kernel of nngp_bfwd_kernel.cuh),
// and the FP64 re-solve of the locations the FP32R kernels flag (nngp_bfr_kernel.cuh for m <= 16,
// nngp_bfw_kernel.cuh for 16 < m <= 32): that pass walks the list of flagged
// tiles and solves only the flagged locations.
//
// Modes: 0 writes B (packed, nIndx) and F and per-tile sums of log F;
//        1 (fused likelihood) writes no B/F but per-tile sums of log F and of
//        r_a r_b / F for r = (I - B) V at the location, V = [X y].
// Per-tile sums are reduced in a fixed order, so results do not depend on the
// launch shape or on block scheduling.
#pragma once
#include <cuda_runtime.h>
#include "nngp_internal.h"
#include "nngp_math.cuh"

namespace nngp_bf {

constexpr int kNGMax = 1 + NNGP_MAX_NV * (NNGP_MAX_NV + 1) / 2;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <int M>
__host__ __device__ constexpr int tri_size() { return M * (M + 1) / 2; }
__host__ __device__ constexpr int tri_at(int r, int c) { return r * (r + 1) / 2 + c; }

// v[k] for a runtime k < NNGP_MAX_NV without indexing a local array
__device__ __forceinline__ double pick_nv(const double (&v)[NNGP_MAX_NV], int k) {
  double r = 0.0;
#pragma unroll
  for (int t = 0; t < NNGP_MAX_NV; t++)
    if (t == k) r = v[t];
  return r;
}

// --------------------------------------------------------------------- kernel
template <int M, int MODE, int TPB, int COV>
__global__ void __launch_bounds__(TPB, 2) bf_kernel(const BFData *__restrict__ datas,
                                                 const CovParams *__restrict__ thetas,
                                                 const BFJob *__restrict__ jobs, int njobs,
                                                 int tile_begin, int tile_end, int nv,
                                                 unsigned long long *__restrict__ status,
                                                 int only_flagged, const int *__restrict__ tile_list,
                                                 const int *__restrict__ tile_count) {
  constexpr int TRI = tri_size<M>();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double *tri = reinterpret_cast<double *>(smem_raw);
  double *geo = tri + (size_t)TRI * TPB;  // per-neighbor absolute (x, y)
  double *wbuf = geo + (size_t)2 * M * TPB;
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
#define TRI_(r, c) tri[(size_t)tri_at((r), (c)) * TPB + tid]
#define GEO_(k, q) geo[(size_t)((k) * 2 + (q)) * TPB + tid]

  // the FP64 re-solve walks the list of tiles the FP32R pass recorded; the other passes walk
  // tiles [tile_begin, tile_end)
  const int ntodo = tile_list ? *tile_count : tile_end - tile_begin;
  for (int kt = blockIdx.x; kt < ntodo; kt += gridDim.x) {
    const int tile = tile_list ? tile_list[kt] : tile_begin + kt;
    const int jid = nngp_find_job(jobs, njobs, tile);
    const BFJob job = jobs[jid];
    const BFData d = datas[job.data];
    const CovParams *cpp = thetas + job.theta;
    const double sigmaSq = cpp->sigmaSq, tauSq = cpp->tauSq;
    const int tj = tile - job.tile0;
    const int i = tj * TPB + tid;
    bool active = i < d.n;
    if (active && only_flagged) active = job.flags[i] != 0;
    // the flagged-only pass skips tiles with nothing to re-solve (block-uniform), leaving
    // zero partial sums for them
    if (only_flagged && !__syncthreads_or(active)) {
      const int ngz = MODE == 0 ? 1 : 1 + nv * (nv + 1) / 2;
      for (int k = tid; k < ngz; k += TPB) job.partial[(size_t)tj * ngz + k] = 0.0;
      continue;
    }

    int mi = 0, off = 0;
    int nb[M];
    if (active) {
      off = d.nnLU[i];
      mi = d.nnLU[d.n + i];
    }
#pragma unroll
    for (int k = 0; k < M; k++) {
      nb[k] = 0;
      if (k < mi) {
        nb[k] = d.nnIndx[off + k];
        const double2 q = reinterpret_cast<const double2 *>(d.xy)[nb[k]];
        GEO_(k, 0) = q.x;
        GEO_(k, 1) = q.y;
      }
    }

    // ---- covariance build: c (registers) and the lower triangle of C (shared)
    double cv[M];
    double xi = 0.0, yi = 0.0;
    if (active) {
      const double2 p = reinterpret_cast<const double2 *>(d.xy)[i];
      xi = p.x;
      yi = p.y;
    }
#pragma unroll
    for (int r = 0; r < M; r++) {
      cv[r] = 0.0;
      if (r < mi) {
        const double xr = GEO_(r, 0), yr = GEO_(r, 1);
        const double ax = xi - xr, ay = yi - yr;
        cv[r] = sigmaSq * nngp_cor_d<COV>(sqrt(ax * ax + ay * ay), *cpp);
#pragma unroll
        for (int c = 0; c <= r; c++) {
          const double bx = xr - GEO_(c, 0), by = yr - GEO_(c, 1);
          double e = sigmaSq * nngp_cor_d<COV>(sqrt(bx * bx + by * by), *cpp);
          if (c == r) e += tauSq;
          TRI_(r, c) = e;
        }
      }
    }

    // ---- Cholesky (row-oriented) fused with the forward solve L z = c; two partial sums per
    // inner product shorten the dependency chains
    double invd[M], z[M];
    bool ok = true;
#pragma unroll
    for (int r = 0; r < M; r++) {
      invd[r] = 0.0;
      z[r] = 0.0;
      if (r < mi) {
        double row[M];
#pragma unroll
        for (int c = 0; c <= r; c++) {
          double s0 = TRI_(r, c), s1 = 0.0;
#pragma unroll
          for (int k = 0; k < c; k++) {
            const double l = (c == r) ? row[k] : TRI_(c, k);
            if (k & 1) s1 -= row[k] * l;
            else s0 -= row[k] * l;
          }
          const double s = s0 + s1;
          if (c < r) {
            row[c] = s * invd[c];
          } else {
            ok = ok && (s > 0.0);
            const double dg = sqrt(s);
            row[r] = dg;
            invd[r] = 1.0 / dg;
          }
        }
        double zs0 = cv[r], zs1 = 0.0;
#pragma unroll
        for (int k = 0; k < r; k++) {
          if (k & 1) zs1 -= row[k] * z[k];
          else zs0 -= row[k] * z[k];
        }
        z[r] = (zs0 + zs1) * invd[r];
#pragma unroll
        for (int c = 0; c <= r; c++) TRI_(r, c) = row[c];
      }
    }

    // ---- back substitution L' B = z
    double Bd[M];
#pragma unroll
    for (int k = M - 1; k >= 0; k--) {
      Bd[k] = 0.0;
      if (k < mi) {
        Bd[k] = z[k] * invd[k];
#pragma unroll
        for (int r = 0; r < k; r++) z[r] -= TRI_(k, r) * Bd[k];
      }
    }
    if (!ok && active) nngp_record_status(status, 1, i);

    // ---- F = sigma^2 + tau^2 - B'c
    double Fi;
    {
      double dot = 0.0;
#pragma unroll
      for (int k = 0; k < M; k++)
        if (k < mi) dot = fma(Bd[k], cv[k], dot);
      Fi = sigmaSq - dot + tauSq;
    }
    const double logF = active ? log(Fi) : 0.0;

    if (MODE == 0) {
      if (active) {
#pragma unroll
        for (int k = 0; k < M; k++)
          if (k < mi) d.B[off + k] = Bd[k];
        d.F[i] = Fi;
      }
      const double s = warp_sum(logF);
      if (lane == 0) wbuf[warp * kNGMax] = s;
      __syncthreads();
      if (tid == 0) {
        double acc = 0.0;
#pragma unroll
        for (int t = 0; t < TPB / 32; t++) acc += wbuf[t * kNGMax];
        job.partial[tj] = acc;
      }
    } else {
      // r_v = V_i,v - sum_k B_k V_N(k),v for the nv columns, then r_a r_b / F
      double rv[NNGP_MAX_NV];
#pragma unroll
      for (int v = 0; v < NNGP_MAX_NV; v++) {
        rv[v] = 0.0;
        if (active && v < nv) {
          double s = d.V[(size_t)i * nv + v];
#pragma unroll
          for (int k = 0; k < M; k++)
            if (k < mi) s = fma(-Bd[k], d.V[(size_t)nb[k] * nv + v], s);
          rv[v] = s;
        }
      }
      const double invF = active ? 1.0 / Fi : 0.0;
      const int ng = 1 + nv * (nv + 1) / 2;
      for (int k = 0; k < ng; k++) {
        double val;
        if (k == 0) {
          val = logF;
        } else {
          int t = k - 1, a = 0;
          while (t >= nv - a) {
            t -= nv - a;
            a++;
          }
          val = pick_nv(rv, a) * pick_nv(rv, a + t) * invF;
        }
        val = warp_sum(val);
        if (lane == 0) wbuf[warp * kNGMax + k] = val;
      }
      __syncthreads();
      for (int k = tid; k < ng; k += TPB) {
        double acc = 0.0;
#pragma unroll
        for (int t = 0; t < TPB / 32; t++) acc += wbuf[t * kNGMax + k];
        job.partial[(size_t)tj * ng + k] = acc;
      }
    }
    __syncthreads();
  }
#undef TRI_
#undef GEO_
}

template <int M>
constexpr int bf_tpb() {
  return M <= 16 ? 64 : 32;
}

template <int M, int MODE, int COV>
int launch_one(nngp_ctx *ctx, const BFPlan *pl, bool fallback_pass, int t0, int t1) {
  constexpr int TPB = bf_tpb<M>();
  const size_t smem = sizeof(double) * ((size_t)tri_size<M>() + (size_t)2 * M) * TPB +
                      sizeof(double) * (TPB / 32) * kNGMax;
  auto kern = bf_kernel<M, MODE, TPB, COV>;
  static bool configured[64] = {};  // the attribute is per device
  const int dev = ctx->device & 63;
  if (!configured[dev]) {
    NNGP_CUDA_TRY(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    configured[dev] = true;
  }
  const int tiles = fallback_pass ? pl->tiles_fb : t1 - t0;
  const BFJob *jobs = fallback_pass ? pl->d_jobs_fb : pl->d_jobs;
  if (tiles <= 0) return NNGP_OK;
  // the re-solve pass: a grid of about two blocks per SM walks the recorded tiles (none
  // recorded: every block returns at once)
  int grid = tiles;
  if (fallback_pass) {
    const int cap = 2 * (ctx->sm_count > 0 ? ctx->sm_count : 1);
    grid = tiles < cap ? tiles : cap;
  }
  kern<<<grid, TPB, smem, ctx->stream>>>(pl->d_datas, pl->d_thetas, jobs, pl->njobs,
                                         fallback_pass ? 0 : t0, fallback_pass ? pl->tiles_fb : t1, pl->nv,
                                         pl->d_status, fallback_pass ? 1 : 0,
                                         fallback_pass ? pl->d_fb64_list : nullptr,
                                         fallback_pass ? (const int *)pl->d_fb64_count : nullptr);
  NNGP_LAUNCH_CHECK(ctx);
  return NNGP_OK;
}

}  // namespace nngp_bf
