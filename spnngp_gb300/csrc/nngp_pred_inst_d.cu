// Instantiations of the prediction kernel for FP64 (M = 16, 32; both kinds).
#include "nngp_pred_kernel.cuh"
namespace nngp_pred {
template int launch_pred<16, false, KIND_CONJ>(nngp_ctx *, const PredArgs &);
template int launch_pred<32, false, KIND_CONJ>(nngp_ctx *, const PredArgs &);
template int launch_pred<16, false, KIND_RESP>(nngp_ctx *, const PredArgs &);
template int launch_pred<32, false, KIND_RESP>(nngp_ctx *, const PredArgs &);
}  // namespace nngp_pred
