// Explicit instantiations of the FP64 warp-per-location B/F kernel (nngp_bfwd_kernel.cuh) for
// the neighbor bound BFWD_M (32) and correlation code BFWD_COV (NNGP_COV_*), both modes.
// The build compiles this file once per variant, in parallel.
#include "nngp_bfwd_kernel.cuh"
#if !defined(BFWD_M) || !defined(BFWD_COV)
#error "nngp_bfwd_inst.cu is compiled once per variant with -DBFWD_M and -DBFWD_COV"
#endif
namespace nngp_bfwd {
template int launch_warp_d<BFWD_M, 0, BFWD_COV>(nngp_ctx *, const BFPlan *, bool, int, int, int, int);
template int launch_warp_d<BFWD_M, 1, BFWD_COV>(nngp_ctx *, const BFPlan *, bool, int, int, int, int);
}  // namespace nngp_bfwd
