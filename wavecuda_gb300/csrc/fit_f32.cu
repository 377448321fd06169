// Batched threshold tuning kernel, FP32 data and arithmetic (WC_F32).
// Block-level MODWT tiles: 104 KB of shared memory per CTA (batch_kernel.cuh).
#define WC_MOD_TILE_KB 104
#include "fit_kernel.cuh"

namespace wc {
int fit_launch_f32(const FitArgs& a, int grid, cudaStream_t s) { return fit_launch_p<PF32>(a, grid, s); }
int fit_blocks_per_sm_f32() { return fit_blocks_per_sm_p<PF32>(); }
}  // namespace wc
