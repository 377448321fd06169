// Batched smoothing kernel, FP64 data with double-float arithmetic (WC_F64_FAST).
// Block-level MODWT tiles: 192 KB of shared memory per CTA (batch_kernel.cuh).
#define WC_MOD_TILE_KB 192
#include "batch_kernel.cuh"

namespace wc {
int batch_launch_fast(const BatchArgs& a, int grid, cudaStream_t s) {
  return batch_launch_p<PDD>(a, grid, s);
}
int batch_blocks_per_sm_fast() { return batch_blocks_per_sm_p<PDD>(); }
}  // namespace wc
