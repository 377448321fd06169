// Batched smoothing: host-side sizing and precision dispatch of the
// persistent kernel in batch_kernel.cuh (one instantiation per precision, in
// batch_exact.cu, batch_fast.cu and batch_f32.cu).
#include <algorithm>

#include "wc_batch.h"
#include "wc_common.cuh"

namespace wc {

// Scratch bytes one CTA needs for a signal (see smooth_one's takes).
size_t batch_scratch_bytes(const BatchDesc& d, int prec) {
  const size_t ts = (prec == WC_F32) ? 4 : 8, vs = 8;
  const int64_t n = d.n, lenh = n / 2, J = d.J;
  const bool mod = d.ttype == 1;
  auto r = [](size_t b) { return ((b + 255) / 256) * 256; };
  size_t s = r(ts * n) + r(ts * (mod ? J * n : n)) + r(ts * (mod ? n : 1)) + 2 * r(vs * n) +
             r(8 * (mod ? J * n : n));
  if (d.threshtype == 2) {
    const int64_t lv1 = J - 1;
    s += 2 * (r(ts * (mod ? lv1 * lenh : lenh)) + r(ts * (mod ? lenh : 1))) + 4 * r(vs * lenh) +
         r(8 * lenh);
  }
  return s + 1024;
}

int batch_launch(const BatchArgs& a, int prec, int grid, cudaStream_t s) {
  switch (prec) {
    case WC_F64_EXACT: return batch_launch_exact(a, grid, s);
    case WC_F64_FAST: return batch_launch_fast(a, grid, s);
    case WC_F32: return batch_launch_f32(a, grid, s);
    default: return fail(WC_ERR_ARG, "unknown precision %d", prec);
  }
}

int batch_max_ctas(int prec) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int per = 1;
  switch (prec) {
    case WC_F64_EXACT: per = batch_blocks_per_sm_exact(); break;
    case WC_F64_FAST: per = batch_blocks_per_sm_fast(); break;
    default: per = batch_blocks_per_sm_f32(); break;
  }
  return sms * per;
}

}  // namespace wc
