/*
 * spnngp_gb300 -- C ABI of the GB300 (sm_103a) NNGP hot path.
 *
 * Every entry point below replaces one native routine of the R package spNNGP
 * (v1.0.1) that its R front-ends reach through .Call; the comment on each
 * names the routine and its file:line in the spNNGP source tree.  The
 * conventions are the reference's own:
 *   - matrices are column-major double, indices 0-based int32;
 *   - the packed neighbor arrays use nnIndxLU = [offsets (n) | counts (n)] and
 *     hold nIndx = (1+m)/2*m + (n-m-1)*m entries (src/rNNGP.cpp:218);
 *   - covModel: 0 exponential, 1 spherical, 2 matern, 3 gaussian (R/spNNGP.R:172);
 *   - response theta = (sigma^2, tau^2, phi[, nu]) (src/rNNGP.cpp:182-190);
 *     conjugate thetaAlpha is nTheta x g with rows (phi, alpha[, nu])
 *     (src/cNNGP.cpp:147-151, R/spConjNNGP.R:207-210);
 *   - data arrive already permuted into the NNGP order.
 * The "host" entry points take host pointers (exactly what the reference's
 * .Call receives) and copy to and from the device inside the call; the
 * "_dev" entry points take device pointers for data kept resident in HBM.
 *
 * Errors: every call returns an nngp_status.  NNGP_ERR_NOT_SPD carries the
 * 0-based location (or prediction point) whose neighborhood covariance had a
 * non-positive pivot, retrievable with nngp_error_location(); the reference
 * raises Rf_error("c++ Rf_error: dpotrf failed") in that case
 * (src/rNNGP.cpp:86).  Nothing falls back to the CPU: without a usable GB300
 * every call returns NNGP_ERR_CUDA.
 *
 * Random numbers are never drawn inside the library.  The MCMC routines read
 * host-fed streams of standard normals and uniforms in the order the
 * reference consumes R's generator, so an R binding fills them with
 * norm_rand()/unif_rand() and reproduces the reference's chain draw for draw.
 */
#ifndef SPNNGP_GB300_H
#define SPNNGP_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct nngp_ctx nngp_ctx;

typedef enum {
  NNGP_OK = 0,
  NNGP_ERR_ARG = 1,         /* invalid argument (sizes, covModel, m out of range ...) */
  NNGP_ERR_CUDA = 2,        /* CUDA runtime error or no usable device */
  NNGP_ERR_NOT_SPD = 3,     /* a neighborhood covariance (or the p x p Gram) is not SPD */
  NNGP_ERR_NO_MEMORY = 4,   /* device allocation failed */
  NNGP_ERR_STREAM = 5       /* a host-fed random stream is too short */
} nngp_status;

typedef enum {
  NNGP_FP64 = 0,  /* plain FP64 throughout */
  NNGP_FP32R = 1  /* FP32 Cholesky + one refinement against the covariance in double-float;
                     locations it cannot certify re-solved in double-float, then FP64 */
} nngp_precision;

/* ---------------------------------------------------------------- context */
int nngp_create(int device, nngp_ctx **ctx);
void nngp_destroy(nngp_ctx *ctx);
const char *nngp_error_message(const nngp_ctx *ctx);
int64_t nngp_error_location(const nngp_ctx *ctx);
/* cudaStream_t to launch on (NULL = the context's own stream). */
int nngp_set_stream(nngp_ctx *ctx, void *stream);
void *nngp_get_stream(const nngp_ctx *ctx);
int nngp_synchronize(nngp_ctx *ctx);
/* Kernels this library launched since the counter was last reset. */
int64_t nngp_launch_count(const nngp_ctx *ctx);
void nngp_reset_launch_count(nngp_ctx *ctx);
/* Largest neighbor count the kernels accept (m <= this). */
int nngp_max_neighbors(void);
int64_t nngp_n_indx(int n, int m);

/* ---------------------------------------------------------- neighbor search */

/* Ordered kNN by the mean-distance code-book search: for every location the
 * m nearest predecessors, bit-exact with the reference including its tie
 * order.  Replaces mkNNIndxCB (src/nn.cpp:213-258, called from R/nn.R:71);
 * outputs are written in place as the reference does. */
int nngp_mkNNIndxCB(nngp_ctx *ctx, int n, int m, const double *coords, int *nnIndx,
                    double *nnDist, int *nnIndxLU);

/* Ordered kNN by exhaustive scan in index order; same result contract as the
 * reference's brute-force search.  Replaces mkNNIndx (src/nn.cpp:63-111,
 * called from R/nn.R:45). */
int nngp_mkNNIndx(nngp_ctx *ctx, int n, int m, const double *coords, int *nnIndx,
                  double *nnDist, int *nnIndxLU);

/* Reverse neighbor index: uIndx lists, for each location, the locations that
 * have it as a neighbor (increasing order for searchType 0 and 2, decreasing
 * for 1), uIndxLU = [offsets | counts], uiIndx the position inside each such
 * list.  Replaces mkUIndx (src/nn.cpp:25-56, src/util.cpp:72-185, called from
 * R/nn.R:19). */
int nngp_mkUIndx(nngp_ctx *ctx, int n, int m, const int *nnIndx, int *uIndx, int *uIndxLU,
                 int *uiIndx, const int *nnIndxLU, int searchType);

/* Unconstrained exact kNN of n0 prediction points among n training points,
 * nnIdx n0 x k column-major 0-based, nnDist the Euclidean distances (may be
 * NULL); ascending distance, ties by smaller training index.  Replaces the
 * RANN::nn2 calls at R/spConjNNGP.R:158,311 and R/generics.R:642. */
int nngp_nn2(nngp_ctx *ctx, int n, const double *coords, int n0, const double *coords0, int k,
             int *nnIdx, double *nnDist);

/* -------------------------------------------------------------- B, F and Q */

/* B_i = C_N(i)^-1 c_i and F_i = sigma^2 + tau^2 - B_i'c_i for every location,
 * and logDet = sum_i log F_i.  theta = (sigma^2, tau^2, phi[, nu]).
 * Replaces updateBF (src/rNNGP.cpp:46-101). */
int nngp_updateBF(nngp_ctx *ctx, int n, int m, const double *coords, const int *nnIndx,
                  const int *nnIndxLU, int covModel, const double *theta, int precision,
                  double *B, double *F, double *logDet);

/* Conjugate form: sigma^2 = 1, nugget alpha.  Replaces updateConjBF
 * (src/cNNGP.cpp:24-69). */
int nngp_updateConjBF(nngp_ctx *ctx, int n, int m, const double *coords, const int *nnIndx,
                      const int *nnIndxLU, int covModel, double phi, double alpha, double nu,
                      int precision, double *B, double *F);

/* q = u'(I-B)'F^-1(I-B)v.  Replaces Q (src/util.cpp:261-280). */
int nngp_Q(nngp_ctx *ctx, const double *B, const double *F, const double *u, const double *v,
           int n, const int *nnIndx, const int *nnIndxLU, double *q);

/* Fused likelihood pass: for the nv columns V = [X y] (n x nv, column-major),
 * logDet = sum log F_i and gram = V'(I-B)'F^-1(I-B)V (nv x nv, column-major,
 * symmetric) without writing B or F.  One call replaces one updateBF plus the
 * p(p+3)/2 + 1 Q calls of src/rNNGP.cpp:255-259,281-286 and src/cNNGP.cpp:224-245. */
int nngp_loglik_gram(nngp_ctx *ctx, int n, int m, int nv, const double *coords,
                     const int *nnIndx, const int *nnIndxLU, const double *V, int covModel,
                     const double *theta, int precision, double *logDet, double *gram);

/* ------------------------------------------------------------ model drivers */

/* Response-model Metropolis-within-Gibbs.  Argument meaning follows .Call
 * ("rNNGP", ...) (R/spNNGP.R:401-405, src/rNNGP.cpp:105-109): thetaStarting and
 * tuning are (sigma^2, tau^2, phi[, nu]).  normals/unifs are the host-fed
 * streams, consumed per iteration as: p normals for beta, n for the replicate
 * when repIndx[s] != 0, then one per proposal (phi, sigma^2, tau^2[, nu]) whose
 * tuning is non-zero, then one uniform.  Outputs betaSamples p x nSamples,
 * thetaSamples nTheta x nSamples, repSamples n x nRep (may be NULL when nRep
 * == 0), *nAccept.  Replaces rNNGP (src/rNNGP.cpp:103-421). */
int nngp_rNNGP(nngp_ctx *ctx, const double *y, const double *X, int p, int n, int m,
               const double *coords, int covModel, const int *nnIndx, const int *nnIndxLU,
               const double *sigmaSqIG, const double *tauSqIG, const double *phiUnif,
               const double *nuUnif, const double *betaStarting, const double *thetaStarting,
               const double *tuning, int nSamples, int nRep, const int *repIndx,
               const double *normals, int64_t nNormals, const double *unifs, int64_t nUnifs,
               int precision, double *betaSamples, double *thetaSamples, double *repSamples,
               int *nAccept);

/* One response-model chain of a batch (the arguments of nngp_rNNGP that may
 * differ between chains, without replicates).  nAccept is an output. */
typedef struct nngp_mcmc_problem {
  int n, m, covModel, nSamples;
  const double *y, *X, *coords;
  const int *nnIndx, *nnIndxLU;
  const double *sigmaSqIG, *tauSqIG, *phiUnif, *nuUnif;       /* host memory, 2 each */
  const double *betaStarting, *thetaStarting, *tuning;        /* host memory */
  const double *normals;
  int64_t nNormals;
  const double *unifs;
  int64_t nUnifs;
  double *betaSamples, *thetaSamples;
  int nAccept;
} nngp_mcmc_problem;

/* Independent response-model chains advanced together: each iteration runs
 * every chain's likelihood pass in one fused launch per neighbor-count class
 * (m <= 16, m <= 32), the whole iteration replayed as one CUDA graph.  Each
 * chain's draws are those nngp_rNNGP gives it alone on the same streams.
 * All chains share p.  resident != 0: y, X, coords, nnIndx, nnIndxLU,
 * normals, unifs, betaSamples and thetaSamples are device memory; resident ==
 * 0: host memory.  Replaces a loop of rNNGP calls (src/rNNGP.cpp:103-421) over
 * independent data sets, as a simulation study or a model-selection sweep runs it. */
int nngp_rNNGP_batch(nngp_ctx *ctx, int nprob, nngp_mcmc_problem *probs, int p, int precision,
                     int resident);

/* Conjugate NNGP over g parameter sets with prediction at n0 points.
 * Argument meaning follows .Call("cNNGP", ...) (R/spConjNNGP.R:336-338,
 * src/cNNGP.cpp:73-75).  Outputs betaHat p x g, ab 2 x g, bBInv p*p x g (lower
 * triangle, upper zero), bb p x g, y0Hat and y0HatVar n0 x g (may be NULL when
 * n0 == 0).  Replaces cNNGP (src/cNNGP.cpp:73-358). */
int nngp_cNNGP(nngp_ctx *ctx, const double *y, const double *X, int p, int n,
               const double *coords, const double *thetaAlpha, const int *nnIndx,
               const int *nnIndxLU, const double *X0, const double *coords0, int n0,
               const int *nnIndx0, int g, int m, const double *sigmaSqIG, int covModel,
               int precision, double *betaHat, double *ab, double *bBInv, double *bb,
               double *y0Hat, double *y0HatVar);

/* One dataset of a batched conjugate run (nngp_cNNGP_multi).  Inputs follow
 * nngp_cNNGP; thetaAlpha is nTheta x g for this dataset.  y0True (n0, may be
 * NULL) are held-out responses: when given, the run also scores every
 * parameter set by CRPS and RMSPE over the n0 points as R/util.R:247-255 does
 * (crps, rmspe: g each).  Outputs as nngp_cNNGP (y0Hat / y0HatVar may be NULL
 * when only the scores are wanted). */
typedef struct {
  int n, n0, g;
  const double *y, *X, *coords;
  const int *nnIndx, *nnIndxLU;
  const double *X0, *coords0;
  const int *nnIndx0;
  const double *thetaAlpha;
  const double *y0True;
  double *betaHat, *ab, *bBInv, *bb, *y0Hat, *y0HatVar, *crps, *rmspe;
} nngp_conj_problem;

/* Batched conjugate fits: every (dataset, parameter set) of every problem in
 * one fused likelihood launch, then the p x p algebra, the prediction solves
 * and the optional scores.  One call replaces the k-fold loop of
 * R/spConjNNGP.R:287-358 (k calls of src/cNNGP.cpp:73-358 plus crps/rmspe),
 * or a batch of independent fits.  All problems share p, m, sigmaSqIG and
 * covModel.  resident != 0: every array in probs except thetaAlpha is device
 * memory (nothing is copied); resident == 0: host memory.  thetaAlpha (nTheta x
 * g) is always host memory. */
int nngp_cNNGP_multi(nngp_ctx *ctx, int nprob, const nngp_conj_problem *probs, int p, int m,
                     const double *sigmaSqIG, int covModel, int precision, int resident);

/* Posterior predictive draws at q points for nSamples kept samples.  betaSamples
 * p x nSamples, thetaSamples nTheta x nSamples, z q*nSamples standard normals
 * with z[i*nSamples + s] used for (point i, sample s).  Output y0 q x nSamples.
 * Replaces rNNGPPredict (src/rNNGPPredict.cpp:25-223). */
int nngp_rNNGPPredict(nngp_ctx *ctx, const double *X, const double *y, const double *coords,
                      int n, int p, int m, const double *X0, const double *coords0, int q,
                      const int *nnIndx0, const double *betaSamples, const double *thetaSamples,
                      int nSamples, int covModel, const double *z, int precision, double *y0);

/* Replicated data y_rep = X beta_s + v_s, v_s drawn by the sequential NNGP
 * recurrence at every sample's theta; beta is nSamples x p, theta nTheta x
 * nSamples, normals n*nSamples consumed location by location, sample by sample.
 * Output yRep n x nSamples.  Replaces rNNGPReplicated
 * (src/rNNGPReplicated.cpp:74-244). */
int nngp_rNNGPReplicated(nngp_ctx *ctx, const double *X, int p, int n, int m,
                         const double *coords, int covModel, const int *nnIndx,
                         const int *nnIndxLU, const double *beta, const double *theta,
                         int nSamples, const double *normals, int precision, double *yRep);

/* Exact posterior draws of the conjugate model at its selected parameter set
 * (R/spConjNNGP.R:423-436, with rigamma and rmvn of R/util.R:1-11): for every
 * sample s, sigma^2 = b / gammas[s], beta = bBInv bb + sigma L z_s (L the lower
 * Cholesky factor of bBInv, z_s = normals[s p .. s p + p)), tau^2 = alpha
 * sigma^2.  gammas are host-fed Gamma(a, 1) variates (the draw behind R's
 * rgamma(1, shape = a, rate = b) = gammas[s] / b), bb and bBInv (p x p, lower
 * triangle read) as nngp_cNNGP returns them, a and b its ab.  Output samples
 * nSamples x (p + 2) column-major: beta, sigma.sq, tau.sq per row, the
 * layout of R's p.beta.theta.samples. */
int nngp_conj_posterior_samples(nngp_ctx *ctx, int p, const double *bb, const double *bBInv, double a, double b,
                                double alpha, int nSamples, const double *gammas, const double *normals,
                                double *samples);

/* ----------------------------------------------- device-resident variants
 * Same contracts as above; every pointer is device memory and the call is
 * asynchronous on the context stream (status and logDet/gram are available
 * after nngp_synchronize).  Coordinates are n x 2 column-major. */
int nngp_updateBF_dev(nngp_ctx *ctx, int n, int m, const double *coords, const int *nnIndx,
                      const int *nnIndxLU, int covModel, const double *theta, int precision,
                      double *B, double *F, double *logDet);
int nngp_loglik_gram_dev(nngp_ctx *ctx, int n, int m, int nv, const double *coords,
                         const int *nnIndx, const int *nnIndxLU, const double *V, int covModel,
                         const double *theta, int precision, double *logDet, double *gram);
int nngp_mkNNIndxCB_dev(nngp_ctx *ctx, int n, int m, const double *coords, int *nnIndx,
                        double *nnDist, int *nnIndxLU);
int nngp_nn2_dev(nngp_ctx *ctx, int n, const double *coords, int n0, const double *coords0, int k,
                 int *nnIdx, double *nnDist);

/* Measurement utility, no counterpart in the reference: sustained FMA
 * throughput (FLOP/s) of the FP64 (fp64 != 0) or FP32 CUDA-core pipe, the
 * denominator of the B/F pass's roofline fraction. */
int nngp_measure_peak(nngp_ctx *ctx, int fp64, double *flops_per_s);

/* Measurement utility, no counterpart in the reference: when on, CUDA events
 * are recorded on the launching stream around every primary launch of the B/F
 * pass kernel; nngp_kernel_time returns (and clears) their summed duration in
 * milliseconds and the number of launches timed. */
int nngp_set_kernel_timing(nngp_ctx *ctx, int on);
int nngp_kernel_time(nngp_ctx *ctx, double *ms, int64_t *launches);

/* Precision diagnostic, no counterpart in the reference: the number of
 * locations that the last FP32R pass of the single-dataset entry points
 * (updateBF, loglik_gram and their _dev forms) re-solved in higher precision
 * -- float pivot failed, error estimate above the bound, or F below 1e-6 of
 * sigma^2 + tau^2 -- and the number of locations that pass covered; 0 and 0
 * after an FP64 pass.  Synchronises the context's stream. */
int nngp_fp32r_resolved(nngp_ctx *ctx, int64_t *resolved, int64_t *locations);

/* Precision diagnostic, no counterpart in the reference: how the locations
 * counted by nngp_fp32r_resolved were re-solved -- in double-float arithmetic
 * on the FP32 pipe (every flagged location goes there first: a thread per
 * location for m <= 24, a warp per location beyond) or in FP64 (the tiles, 64
 * locations for m <= 16 and 32 beyond, holding a location the double-float
 * solve could not certify).  Synchronises the context's stream. */
int nngp_fp32r_tiers(nngp_ctx *ctx, int64_t *double_float, int64_t *fp64);

/* Launch-shape autotuner of the FP32R B/F kernels, no counterpart in the
 * reference (it stands in for the reference's n.omp.threads tuning).  For the
 * register kernel (m <= 16):
 * The first pass of a (neighbor bound, mode, correlation model, size class)
 * times every candidate shape -- warps per block 1-6 (8) with the covariance
 * kept in shared memory, or 4 / 8 with its low-order parts in the SM's tensor
 * memory, each as one tile per warp or a persistent grid of 1 or 2 x resident
 * blocks x SMs -- on the caller's own data (at most 64K tiles of it) and keeps
 * the fastest for the context; passes under stream capture, and passes of
 * fewer than 2048 tiles, use the tuned shape or the default (4 warps, shared
 * memory, one tile per warp).  Results are identical for every shape (each
 * warp reduces its own 32 locations and the sums are combined in a fixed
 * order), so tuning never changes a result.  nngp_set_autotune(ctx, 0) turns
 * tuning off (default shape); nngp_set_launch_shape forces a shape (wpb 0 =
 * back to tuning; use_tmem is honoured for m in 11..16); nngp_autotune_report
 * writes one line per tuned class ("key: wpb=W grid_mode=G tmem=T ms=X |
 * WxBLOCKS[t]:ms ...", one entry per candidate, t marking tensor memory) into
 * buf and returns the number of classes.  The warp-per-location FP32R kernel
 * (16 < m <= 32) is tuned the same way over 1, 2 or 4 warps per block, one tile
 * per warp or a persistent grid (classes "warp M=20|24|32 ..."). */
int nngp_set_autotune(nngp_ctx *ctx, int on);
int nngp_set_launch_shape(nngp_ctx *ctx, int warps_per_block, int grid_mode, int use_tmem);
int nngp_autotune_report(nngp_ctx *ctx, char *buf, int len);

/* No counterpart in the reference.  The FP64 fused likelihood pass of
 * nngp_loglik_gram_dev for callers that cannot allocate device memory when they
 * need it (a host whose allocator owns all device memory, a serving process that
 * reserves HBM up front and forbids allocation on its request path, a loop that
 * must not hit the allocator's implicit synchronisation).  It calls no
 * cudaMalloc / cudaFree or other allocating routine: its working memory is one
 * statically sized __device__ array in this library (about 5.3 MB, held by every
 * GPU that loads the library until the process exits).  Limits: n <= 65536,
 * m <= 32, nv <= 8; larger requests return NNGP_ERR_ARG with a message in errbuf.
 * stream is a cudaStream_t (NULL = legacy default stream); every array is a
 * device pointer except theta (host) and errbuf (host, may be NULL).  The first
 * call on a device looks up the array's address and configures the kernel.  No
 * call may be made while its stream is being captured into a CUDA graph (each
 * call copies host values and waits for its stream before returning): such a
 * call returns NNGP_ERR_ARG.  The sums are formed in the same order as
 * nngp_loglik_gram_dev's FP64 pass, so both give the same result.  All calls
 * share the array: calls whose work overlaps on the GPU race and must be
 * serialised by the caller. */
int nngp_loglik_gram_noalloc(void *stream, int n, int m, int nv, const double *coords,
                             const int *nnIndx, const int *nnIndxLU, const double *V, int covModel,
                             const double *theta, double *logDet, double *gram, char *errbuf,
                             int errlen);

#ifdef __cplusplus
}
#endif
#endif
