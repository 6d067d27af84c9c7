// Explicit instantiations of the double-float re-solve kernel (nngp_bfdf_kernel.cuh) for one
// neighbor bound BFDF_M (16, 24) and correlation code BFDF_COV (NNGP_COV_*), both modes.
// The build compiles this file once per (bound, code), in parallel.
#include "nngp_bfdf_kernel.cuh"
#if !defined(BFDF_M) || !defined(BFDF_COV)
#error "nngp_bfdf_inst.cu is compiled once per variant with -DBFDF_M and -DBFDF_COV"
#endif
namespace nngp_bfdf {
template int launch_df<BFDF_M, 0, BFDF_COV>(nngp_ctx *, const BFPlan *);
template int launch_df<BFDF_M, 1, BFDF_COV>(nngp_ctx *, const BFPlan *);
}  // namespace nngp_bfdf
