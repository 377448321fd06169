// Sequential FP64 sum of the CV loss terms, m = (((0 + v_0) + v_1) + ...) * 0.5,
// rounded exactly as the reference's loop (thresh.cpp:363-383) rounds it.
//
// First version: one thread walks the terms in order.  The loads are
// independent of the running sum and are issued ahead of it; the chain of
// dependent FP64 additions bounds the time.
#include "wc_common.cuh"

namespace wc {
namespace {

__global__ void seq_sum_kernel(const double* __restrict__ v, int64_t n, double* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double m = 0.0;
  int64_t i = 0;
  for (; i + 8 <= n; i += 8) {
    double a0 = v[i], a1 = v[i + 1], a2 = v[i + 2], a3 = v[i + 3];
    double a4 = v[i + 4], a5 = v[i + 5], a6 = v[i + 6], a7 = v[i + 7];
    m = __dadd_rn(m, a0); m = __dadd_rn(m, a1); m = __dadd_rn(m, a2); m = __dadd_rn(m, a3);
    m = __dadd_rn(m, a4); m = __dadd_rn(m, a5); m = __dadd_rn(m, a6); m = __dadd_rn(m, a7);
  }
  for (; i < n; i++) m = __dadd_rn(m, v[i]);
  *out = __dmul_rn(m, 0.5);
}

}  // namespace

int cv_sequential_sum(const double* terms, int64_t count, double* dev_out, cudaStream_t s) {
  seq_sum_kernel<<<1, 32, 0, s>>>(terms, count, dev_out);
  return after_launch("seq_sum_kernel");
}

}  // namespace wc
