// Explicit instantiations of the B/F kernel launcher for one variant: neighbor bound
// BF_M (16 or 32), precision BF_R32 (0 FP64, 1 FP32R) and correlation code BF_COV
// (NNGP_COV_*), both modes.  The build compiles this file once per variant, in parallel.
#include "nngp_bf_kernel.cuh"
#if !defined(BF_M) || !defined(BF_R32) || !defined(BF_COV)
#error "nngp_bf_inst.cu is compiled once per variant with -DBF_M, -DBF_R32 and -DBF_COV"
#endif
namespace nngp_bf {
template int launch_one<BF_M, (BF_R32 != 0), 0, BF_COV>(nngp_ctx *, const BFPlan *, bool, int, int);
template int launch_one<BF_M, (BF_R32 != 0), 1, BF_COV>(nngp_ctx *, const BFPlan *, bool, int, int);
}  // namespace nngp_bf
