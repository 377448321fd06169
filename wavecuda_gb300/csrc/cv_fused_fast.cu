// Fused cross-validation search kernel, FP64 data with double-float arithmetic (WC_F64_FAST).
#include "cv_fused_kernel.cuh"

namespace wc {
int cv_fused_launch_fast(const CvFusedArgs& a, int F, int ttype, int grid, size_t smem,
                          cudaStream_t s) {
  return cv_fused_launch_p<PDD>(a, F, ttype, grid, smem, s);
}
int cv_fused_occupancy_fast(int F, int ttype, size_t smem) {
  return cv_fused_occupancy_p<PDD>(F, ttype, smem);
}
}  // namespace wc
