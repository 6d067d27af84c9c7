// Explicit instantiations of the warp-per-location double-float re-solve kernel
// (nngp_bfwdf_kernel.cuh) for one neighbor bound BFWDF_M (24 or 32) and correlation code
// BFWDF_COV (NNGP_COV_*), both modes.  The build compiles this file once per variant, in parallel.
#include "nngp_bfwdf_kernel.cuh"
#if !defined(BFWDF_M) || !defined(BFWDF_COV)
#error "nngp_bfwdf_inst.cu is compiled once per variant with -DBFWDF_M and -DBFWDF_COV"
#endif
namespace nngp_bfwdf {
template int launch_wdf<BFWDF_M, 0, BFWDF_COV>(nngp_ctx *, const BFPlan *);
template int launch_wdf<BFWDF_M, 1, BFWDF_COV>(nngp_ctx *, const BFPlan *);
}  // namespace nngp_bfwdf
