// Explicit instantiations of the FP64 B/F kernel launcher for one variant: neighbor bound
// BF_M (16 or 24) and correlation code BF_COV (NNGP_COV_*), both modes.  The build
// compiles this file once per variant, in parallel.
#include "nngp_bf_kernel.cuh"
#if !defined(BF_M) || !defined(BF_COV)
#error "nngp_bf_inst.cu is compiled once per variant with -DBF_M and -DBF_COV"
#endif
namespace nngp_bf {
template int launch_one<BF_M, 0, BF_COV>(nngp_ctx *, const BFPlan *, bool, int, int);
template int launch_one<BF_M, 1, BF_COV>(nngp_ctx *, const BFPlan *, bool, int, int);
}  // namespace nngp_bf
