// Explicit instantiations of the warp-per-location FP32R B/F kernel (nngp_bfw_kernel.cuh) for
// one neighbor bound BFW_M (20, 24 or 32) and correlation code BFW_COV (NNGP_COV_*), both modes.
// The build compiles this file once per variant, in parallel.
#include "nngp_bfw_kernel.cuh"
#if !defined(BFW_M) || !defined(BFW_COV)
#error "nngp_bfw_inst.cu is compiled once per variant with -DBFW_M and -DBFW_COV"
#endif
namespace nngp_bfw {
template int launch_warp<BFW_M, 0, BFW_COV>(nngp_ctx *, const BFPlan *, int, int, int, int);
template int launch_warp<BFW_M, 1, BFW_COV>(nngp_ctx *, const BFPlan *, int, int, int, int);
template int occupancy_warp<BFW_M, 0, BFW_COV>(int);
template int occupancy_warp<BFW_M, 1, BFW_COV>(int);
}  // namespace nngp_bfw
