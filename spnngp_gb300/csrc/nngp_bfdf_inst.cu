// Explicit instantiations of the double-float re-solve kernel (nngp_bfdf_kernel.cuh) for one
// correlation code BFDF_COV (NNGP_COV_*), both modes.  The build compiles this file once per
// code, in parallel.
#include "nngp_bfdf_kernel.cuh"
#if !defined(BFDF_COV)
#error "nngp_bfdf_inst.cu is compiled once per variant with -DBFDF_COV"
#endif
namespace nngp_bfdf {
template int launch_df<0, BFDF_COV>(nngp_ctx *, const BFPlan *);
template int launch_df<1, BFDF_COV>(nngp_ctx *, const BFPlan *);
}  // namespace nngp_bfdf
