// Internal host-side structures of the spnngp_gb300 library: the context
// (device, stream, error state, launch counter) and grow-only device scratch
// buffers.  Included by every translation unit of the library.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "../../include/spnngp_gb300.h"

// Largest neighbor count the dense kernels handle (registers / shared memory are
// sized from it at compile time).
constexpr int NNGP_MAX_M = 32;
// Largest neighbor count of the neighbor-search kernels (lists live in local memory).
constexpr int NNGP_MAX_M_SEARCH = 64;
// Largest number of columns of V = [X y] in the fused likelihood pass.
constexpr int NNGP_MAX_NV = 8;

// Named scratch slots; each is a grow-only device allocation owned by the context.
enum ScratchSlot {
  S_COORDS = 0, S_NNINDX, S_NNLU, S_B, S_F, S_V, S_PARTIAL, S_RED, S_THETA, S_STATUS,
  S_U, S_V2, S_IDX, S_IDX2, S_SORT_TMP, S_XS, S_YS, S_OS, S_NNDIST, S_COORDS0,
  S_NNINDX0, S_OUT0, S_OUT1, S_OUT2, S_OUT3, S_OUT4, S_OUT5, S_STREAM_N, S_STREAM_U,
  S_X, S_Y, S_MISC, S_JOBS, S_DATAS, S_MISC2, S_MISC3, S_XYF, S_VF, S_GKEY, S_GKEY2, S_GJ, S_GJ2,
  S_GXY, S_GSTART, S_GREDO, S_NUM_SLOTS
};

struct BFPlan;

// Launch shape of the register B/F kernel chosen by the autotuner for one kernel variant
// and size class: warps per block, and the grid (0: one block per wpb warp tiles; k > 0: a
// persistent grid of k x occupancy x SMs blocks).  `ms` is the timed pass, `detail` lists
// every candidate's time.
struct TuneEntry {
  int wpb = 4;
  int grid_mode = 0;
  int tm = 0;  // 1: the kernel variant keeping the covariance's lo parts in tensor memory
  double ms = 0.0;
  std::string detail;
};

struct nngp_ctx {
  int device = 0;
  int sm_count = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  std::string err;
  int64_t err_loc = -1;
  int64_t launches = 0;
  void *scratch[S_NUM_SLOTS] = {};
  size_t scratch_cap[S_NUM_SLOTS] = {};
  // pinned host staging for small results
  void *pinned = nullptr;
  size_t pinned_cap = 0;
  // optional timing of the B/F kernels: events recorded around each primary launch
  bool timing = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> timed;
  std::vector<cudaEvent_t> event_pool;
  // last single-evaluation plan, reused while its key (pointers, sizes, mode) is unchanged
  BFPlan *cache_plan = nullptr;
  std::string cache_key;
  // register B/F kernel launch shapes: autotuned on first use (outside stream capture), or
  // forced by nngp_set_launch_shape (force_wpb > 0)
  bool autotune = true;
  int force_wpb = 0, force_grid_mode = 0, force_tm = 0;
  std::map<std::string, TuneEntry> tuned;
  // host-pointer entry points stream their inputs in on this stream, chunk by chunk, while
  // the context stream computes (created on first use)
  cudaStream_t copy_stream = nullptr;
  std::vector<cudaEvent_t> chunk_events;
};
void nngp_bf_cache_release(nngp_ctx *ctx);

// Records an error on the context and returns the status.
int nngp_fail(nngp_ctx *ctx, int status, const std::string &msg, int64_t loc = -1);

// Returns a device buffer of at least `bytes` for `slot` (grows, never shrinks).
void *nngp_scratch(nngp_ctx *ctx, int slot, size_t bytes);
void *nngp_pinned(nngp_ctx *ctx, size_t bytes);

#define NNGP_CUDA_TRY(ctx, expr)                                                        \
  do {                                                                                  \
    cudaError_t e_ = (expr);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return nngp_fail((ctx), NNGP_ERR_CUDA, std::string(#expr ": ") + cudaGetErrorString(e_)); \
  } while (0)

#define NNGP_LAUNCH_CHECK(ctx)                                                          \
  do {                                                                                  \
    (ctx)->launches++;                                                                  \
    cudaError_t e_ = cudaGetLastError();                                                \
    if (e_ != cudaSuccess)                                                              \
      return nngp_fail((ctx), NNGP_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e_)); \
  } while (0)

#define NNGP_ALLOC(ctx, ptr, type, slot, count)                                          \
  do {                                                                                  \
    (ptr) = (type *)nngp_scratch((ctx), (slot), sizeof(type) * (size_t)(count));        \
    if (!(ptr)) return nngp_fail((ctx), NNGP_ERR_NO_MEMORY, "device allocation failed"); \
  } while (0)

inline int64_t nngp_nindx(int n, int m) {
  // (1+m)/2*m + (n-m-1)*m, evaluated as the reference does (src/rNNGP.cpp:218)
  return (int64_t)((double)(1 + m) / 2 * m + (double)((int64_t)(n - m - 1) * m));
}

// ------------------------------------------------------------ covariance params
// One parameter set of the correlation model, prepared on the host (or on the
// device by the MCMC kernels): model 0 exponential, 1 spherical, 2 matern,
// 3 gaussian.  For matern, mconst = 1 / (2^(nu-1) Gamma(nu)); when nu = k + 1/2
// with k <= 8 the closed form exp(-x) * sum_j poly[j] x^j is used (halfk = k),
// otherwise halfk = -1 and K_nu is evaluated by series / continued fraction.
struct CovParams {
  double sigmaSq, tauSq, phi, nu, mconst;
  double poly[9];
  int model;
  int halfk;
  // the FP32R register kernel's constants as double-float (hi, lo) pairs: the exp argument
  // scale in units of ln2/32 (-phi 32/ln2, gaussian -phi^2 32/ln2), phi, sigma^2,
  // sigma^2 + tau^2, and the Matern polynomial
  float dfK[2], dfPhi[2], dfS2[2], dfDiag[2];
  float dfPoly[9][2];
};

// Parameter sets whose FP32R pass hands every location to the double-float re-solve without
// trying the float factor: a gaussian covariance (model code 3) with a nugget at most 1e-4 of
// sigma^2.  Its neighborhood systems have condition numbers of 1e4 and more, so the float
// factor's error estimate flags essentially every location; the rule depends on the
// parameters alone, so a location's result never depends on the batch or on earlier calls.
__host__ __device__ inline bool nngp_route_double_float(const CovParams &c) {
  return c.model == 3 && c.tauSq <= 1e-4 * c.sigmaSq;
}

__host__ __device__ inline void cov_split(double v, float (&out)[2]) {
  out[0] = (float)v;
  out[1] = (float)(v - (double)out[0]);
}

// Fills mconst / halfk / poly from model and nu, and the double-float constants.  Callable on
// host and device.
__host__ __device__ inline void cov_prepare(CovParams &c) {
  c.halfk = -1;
  c.mconst = 0.0;
  for (int j = 0; j < 9; j++) c.poly[j] = 0.0;
  const double c32 = 46.166241308446828;  // 32 / ln 2
  cov_split(c.model == 3 ? -(c.phi * c.phi) * c32 : -c.phi * c32, c.dfK);
  cov_split(c.phi, c.dfPhi);
  cov_split(c.sigmaSq, c.dfS2);
  cov_split(c.sigmaSq + c.tauSq, c.dfDiag);
  for (int j = 0; j < 9; j++) c.dfPoly[j][0] = c.dfPoly[j][1] = 0.0f;
  if (c.model != 2) return;
  c.mconst = 1.0 / (pow(2.0, c.nu - 1.0) * tgamma(c.nu));
  const double k = c.nu - 0.5;
  if (k >= 0.0 && k <= 8.0 && k == floor(k)) {
    const int K = (int)k;
    c.halfk = K;
    // rho(x) = exp(-x) * K!/(2K)! * sum_{j=0}^{K} (K+j)!/(j!(K-j)!) (2x)^(K-j)
    double fact[18];
    fact[0] = 1.0;
    for (int t = 1; t < 18; t++) fact[t] = fact[t - 1] * t;
    const double lead = fact[K] / fact[2 * K];
    for (int j = 0; j <= K; j++) {
      const int pw = K - j;
      c.poly[pw] = lead * fact[K + j] / (fact[j] * fact[K - j]) * ldexp(1.0, pw);
    }
    for (int j = 0; j < 9; j++) cov_split(c.poly[j], c.dfPoly[j]);
  }
}

// ------------------------------------------------------------- fused-pass jobs
// One dataset as the dense kernels see it (all device pointers).
struct BFData {
  int n, m, nv;
  const double *xy;      // n x 2 interleaved (x, y)
  const float *xyf;      // n x 4 (x hi, y hi, x lo, y lo): the FP32R kernels' coordinates
  const int *nnIndx;     // packed neighbor lists
  const int *nnLU;       // [offsets | counts], 2n
  const double *V;       // n x nv row-major, fused pass only
  const float2 *Vf;      // V as float (hi, lo) pairs, n x nv row-major: the FP32R fused pass
                         // (filled by the plan when the caller leaves it null)
  double *B;             // nIndx, standalone pass only
  double *F;             // n, standalone pass only
};
// One (dataset, parameter set) evaluation, covering tiles [tile0, tile0 + ntiles).
struct BFJob {
  int data;
  int theta;
  int tile0;
  int ntiles;
  double *partial;       // ntiles x NG per-tile partial sums
  unsigned char *flags;  // n bytes: locations the FP32R kernel hands to the FP64 kernel
  // FP32R primary jobs: where a flagged location's FP64 re-solve tile is recorded (the plan's
  // [count | marks] words and tile list); fb_tile0 / fb_tpb place location i in FP64 tile
  // fb_tile0 + i / fb_tpb
  int fb_tile0;
  int fb_tpb;
  unsigned *fb_marks;
  int *fb_count;
  int *fb_list;
};

// Records that FP32R location i of `job` goes to the FP64 kernel: its flag, and its FP64 tile
// once in the tile list (the list's order varies from run to run; each listed tile writes its
// own partial slot, so the sums do not).
__device__ __forceinline__ void nngp_flag_for_fp64(const BFJob &job, int i) {
  job.flags[i] = 1;
  const int ft = job.fb_tile0 + i / job.fb_tpb;
  if (atomicExch(job.fb_marks + ft, 1u) == 0u) job.fb_list[atomicAdd(job.fb_count, 1)] = ft;
}

// The job owning `tile` (jobs sorted by tile0): a binary search over the job table.
__device__ __forceinline__ int nngp_find_job(const BFJob *jobs, int njobs, int tile) {
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].tile0 <= tile) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Records a failed location in the pass's status word: the smallest (code, location) wins.
__device__ __forceinline__ void nngp_record_status(unsigned long long *st, unsigned long long code, long long loc) {
  atomicMin(st, (code << 48) | (unsigned long long)(loc & 0xFFFFFFFFFFFFll));
}

// A prepared B/F pass over a set of (dataset, parameter set) evaluations.  The
// job tables live on the device, so nngp_bf_run only launches kernels (it can be
// captured into a CUDA graph).  Parameter sets are read from device memory at
// run time, so callers may rewrite them between runs.
struct BFPlan {
  int precision = 0, mode = 0, mmax = 0, nv = 0, ng = 0;
  int reg_m = 0;  // > 0: the primary pass runs the register kernel instantiated for this M
  int cov = 4;  // NNGP_COV_* code of the kernels the plan runs (NNGP_COV_ANY: any parameter set)
  int njobs = 0, tiles = 0, tiles_fb = 0;
  BFData *d_datas = nullptr;
  const CovParams *d_thetas = nullptr;
  BFJob *d_jobs = nullptr, *d_jobs_fb = nullptr;
  double *d_partial = nullptr, *d_partial_fb = nullptr;
  unsigned char *d_flags = nullptr;
  size_t flags_bytes = 0;
  // FP32R: [count | marks (tiles_fb)] words and the list of FP64 tiles to re-solve
  unsigned *d_fb_words = nullptr;
  int *d_fb_list = nullptr;
  // the tiles the FP64 kernel re-solves: those the double-float kernel (which walks the list
  // above first) could not certify, with the number of flagged locations in them
  int *d_fb64_list = nullptr;
  int *d_fb64_count = nullptr;
  unsigned long long *d_fb64_locs = nullptr;
  // fixed-order reduction: the tiles of a job are summed in chunks of 1024 tiles (one block
  // each; red_chunks is the most any job has), then the chunk sums in order
  int red_chunks = 0;
  double *d_partial2 = nullptr;
  unsigned long long *d_status = nullptr;
  std::vector<void *> owned;
};
struct PassEval {
  int data;
  int theta;
};
// Correlation-function codes the B/F kernels are compiled for: a kernel compiled for one
// model evaluates only that formula; NNGP_COV_ANY switches on each parameter set's model and
// is the only one that carries the general-nu Matern evaluation.
enum : int { NNGP_COV_EXP = 0, NNGP_COV_SPH = 1, NNGP_COV_MAT_HALF = 2, NNGP_COV_GAU = 3, NNGP_COV_ANY = 4 };
// Builds a plan (device allocations owned by the plan, stream-ordered).  cov must cover every
// parameter set the plan will ever run with (see nngp_plan_cov).
int nngp_bf_plan(nngp_ctx *ctx, BFPlan *plan, int precision, int mode, int nv,
                 const std::vector<BFData> &datas, const CovParams *d_thetas,
                 const std::vector<PassEval> &evals, unsigned long long *d_status, int cov = NNGP_COV_ANY);
// The narrowest kernel code covering these (fixed) parameter sets: their common model, with
// Matern only when every nu is k + 1/2 (k <= 8); NNGP_COV_ANY otherwise.
inline int nngp_plan_cov(const CovParams *cps, int count) {
  if (count < 1) return NNGP_COV_ANY;
  const int model = cps[0].model;
  for (int k = 0; k < count; k++) {
    if (cps[k].model != model) return NNGP_COV_ANY;
    if (model == 2 && cps[k].halfk < 0) return NNGP_COV_ANY;
  }
  return model;
}
// Launches the kernel instantiation the plan needs (primary pass, or the FP64 re-solve of the
// flagged locations when fallback_pass).
int nngp_bf_launch(nngp_ctx *ctx, const BFPlan *plan, bool fp32r, bool fallback_pass);
// Launches the pass; d_out receives njobs x ng sums (log F first, then the Gram
// entries r_a r_b / F over a <= b, row-major).
int nngp_bf_run(nngp_ctx *ctx, const BFPlan *plan, double *d_out);
// The same pass in pieces, for callers that stream their inputs in: begin (clears the FP32R
// flags), the primary kernel over tiles [t0, t1) as often as needed to cover every tile
// (tile = location / nngp_bf_tile(precision, m) of a single-job plan), then finish (FP64
// re-solve of flagged locations and the fixed-order sums).  Results are identical to
// nngp_bf_run's.
int nngp_bf_begin(nngp_ctx *ctx, const BFPlan *plan);
int nngp_bf_primary(nngp_ctx *ctx, const BFPlan *plan, int t0, int t1);
int nngp_bf_finish(nngp_ctx *ctx, const BFPlan *plan, double *d_out);
// Locations per primary tile of a plan with this precision and largest m.
int nngp_bf_tile(int precision, int mmax);
void nngp_bf_plan_free(nngp_ctx *ctx, BFPlan *plan);
// Stream-ordered device allocation (pooled), freed with nngp_free_async.
void *nngp_malloc_async(nngp_ctx *ctx, size_t bytes);
void nngp_free_async(nngp_ctx *ctx, void *p);

// Neighbor bounds the register FP32R kernel is instantiated for (m <= 16), ascending.
constexpr int NNGP_REG_MS[] = {10, 15, 16};
// The smallest instantiated bound >= m, or 0 when the register kernel does not apply.
inline int nngp_reg_m(int precision, int mmax) {
  if (precision != NNGP_FP32R) return 0;
  for (int M : NNGP_REG_MS)
    if (mmax <= M) return M;
  return 0;
}
// Shared memory of the register kernel, per lane: the hi parts of the strict lower triangle
// and of the c vector, the lo parts of the c vector, the lo parts of the strict lower triangle
// (only when they are not kept in tensor memory, tm = false), one float4 of geometry per
// neighbor (the epilogue's staging of 2 NNGP_MAX_NV + 2 (1 + NV(NV+1)/2) floats reuses the
// front); per warp a 96-float table (exp table, Matern polynomial coefficients).  Blocks hold
// at most 8 warps and 227 KB; with tm the
// warps per block are 4 or 8 (every lane quarter of the tensor memory in use).
constexpr int nngp_bfr_lane_floats(int M, bool tm = false) {
  const int nl = M * (M - 1) / 2;
  const int raw = nl + 2 * M + (tm ? 0 : nl) + 4 * M;
  const int red = 2 * NNGP_MAX_NV + 2 * (1 + NNGP_MAX_NV * (NNGP_MAX_NV + 1) / 2);
  return ((raw > red ? raw : red) + 3) & ~3;
}
constexpr size_t nngp_bfr_warp_bytes(int M, bool tm = false) {
  return sizeof(float) * (32 * (size_t)nngp_bfr_lane_floats(M, tm) + 96);
}
constexpr int nngp_bfr_max_wpb(int M, bool tm = false) {
  const int w = (int)((size_t)227 * 1024 / nngp_bfr_warp_bytes(M, tm));
  return tm ? (w >= 8 ? 8 : (w >= 4 ? 4 : 0)) : (w < 8 ? w : 8);
}
// Neighbor bounds whose register kernel also comes with the lo parts in tensor memory.
constexpr bool nngp_bfr_has_tm(int M) { return M >= 15; }
// Writes V (n x nv row-major doubles) as float (hi, lo) pairs.
int nngp_split_v(nngp_ctx *ctx, const double *V, int64_t count, float2 *Vf);

// Writes the interleaved double coordinates (xy, may be null) and their float hi/lo
// split (xyf, may be null) from the n x 2 column-major coordinates, for locations
// [i0, i1) (default: all).
int nngp_prepare_coords(nngp_ctx *ctx, const double *cm, int n, double *xy, float *xyf, int i0 = 0,
                        int i1 = -1);

// Device status word: 0xFFFF..FF = ok, otherwise (code << 48) | location.
constexpr unsigned long long NNGP_STATUS_OK = ~0ull;
int nngp_check_status(nngp_ctx *ctx, unsigned long long *d_status, const char *what);
int nngp_reset_status(nngp_ctx *ctx, unsigned long long *d_status);
