// Batched smoothing kernel, FP32 data and arithmetic (WC_F32).
// Block-level MODWT tiles: 192 KB of shared memory per CTA (batch_kernel.cuh).
#define WC_MOD_TILE_KB 192
#include "batch_kernel.cuh"

namespace wc {
int batch_launch_f32(const BatchArgs& a, int grid, cudaStream_t s) {
  return batch_launch_p<PF32>(a, grid, s);
}
int batch_blocks_per_sm_f32() { return batch_blocks_per_sm_p<PF32>(); }
}  // namespace wc
