// Fused cross-validation search kernel, FP32 data and arithmetic (WC_F32).
#include "cv_fused_kernel.cuh"

namespace wc {
int cv_fused_launch_f32(const CvFusedArgs& a, int F, int ttype, int grid, size_t smem,
                          cudaStream_t s) {
  return cv_fused_launch_p<PF32>(a, F, ttype, grid, smem, s);
}
int cv_fused_occupancy_f32(int F, int ttype, size_t smem) {
  return cv_fused_occupancy_p<PF32>(F, ttype, smem);
}
}  // namespace wc
