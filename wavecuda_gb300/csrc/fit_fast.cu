// Batched threshold tuning kernel, FP64 data with double-float arithmetic (WC_F64_FAST).
// Block-level MODWT tiles: 104 KB of shared memory per CTA (batch_kernel.cuh).
#define WC_MOD_TILE_KB 104
#include "fit_kernel.cuh"

namespace wc {
int fit_launch_fast(const FitArgs& a, int grid, cudaStream_t s) { return fit_launch_p<PDD>(a, grid, s); }
int fit_blocks_per_sm_fast() { return fit_blocks_per_sm_p<PDD>(); }
}  // namespace wc
