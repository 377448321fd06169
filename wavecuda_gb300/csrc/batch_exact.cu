// Batched smoothing kernel, FP64 data with the reference's roundings (WC_F64_EXACT).
#include "batch_kernel.cuh"

namespace wc {
int batch_launch_exact(const BatchArgs& a, int grid, cudaStream_t s) {
  return batch_launch_p<PExact>(a, grid, s);
}
int batch_blocks_per_sm_exact() { return batch_blocks_per_sm_p<PExact>(); }
}  // namespace wc
