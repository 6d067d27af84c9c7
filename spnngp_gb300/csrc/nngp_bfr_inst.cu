// Explicit instantiations of the register FP32R B/F kernel (nngp_bfr_kernel.cuh) for one
// neighbor bound BFR_M and correlation code BFR_COV (NNGP_COV_*), both modes.  The build
// compiles this file once per variant, in parallel.
#include "nngp_bfr_kernel.cuh"
#if !defined(BFR_M) || !defined(BFR_COV)
#error "nngp_bfr_inst.cu is compiled once per variant with -DBFR_M and -DBFR_COV"
#endif
namespace nngp_bfr {
template int launch_reg<BFR_M, 0, BFR_COV>(nngp_ctx *, const BFPlan *, int, int, int, int, int);
template int launch_reg<BFR_M, 1, BFR_COV>(nngp_ctx *, const BFPlan *, int, int, int, int, int);
template int occupancy<BFR_M, 0, BFR_COV>(int, int);
template int occupancy<BFR_M, 1, BFR_COV>(int, int);
}  // namespace nngp_bfr
