// Instantiations of the B/F kernel for M = 16, FP32R (both modes).
#include "nngp_bf_kernel.cuh"
namespace nngp_bf {
template int launch_one<16, true, 0>(nngp_ctx *, const BFPlan *, bool);
template int launch_one<16, true, 1>(nngp_ctx *, const BFPlan *, bool);
}  // namespace nngp_bf
