// Batched threshold tuning kernel, FP64 data with double-float arithmetic (WC_F64_FAST).
#include "fit_kernel.cuh"

namespace wc {
int fit_launch_fast(const FitArgs& a, int grid, cudaStream_t s) { return fit_launch_p<PDD>(a, grid, s); }
int fit_blocks_per_sm_fast() { return fit_blocks_per_sm_p<PDD>(); }
}  // namespace wc
