// Fused cross-validation search kernel, FP64 data with the reference's roundings (WC_F64_EXACT).
#include "cv_fused_kernel.cuh"

namespace wc {
int cv_fused_launch_exact(const CvFusedArgs& a, int F, int ttype, int grid, size_t smem,
                          cudaStream_t s) {
  return cv_fused_launch_p<PExact>(a, F, ttype, grid, smem, s);
}
int cv_fused_occupancy_exact(int F, int ttype, size_t smem) {
  return cv_fused_occupancy_p<PExact>(F, ttype, smem);
}
}  // namespace wc
