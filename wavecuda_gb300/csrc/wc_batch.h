// Batched smoothing: descriptors shared by the persistent kernel (batch_kernel.cuh)
// and its host-side plan (batch_plan.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace wc {

struct BatchDesc {
  int64_t off, n;           // signal = data[off .. off+n)
  int J, ttype, F, threshtype, hardness, minl, maxl, pad;
  double thresh, tol;       // manual threshold; CV tolerance
  double sq_n, sq_nm1;      // sqrt(2 log n), sqrt(2 log(n-1)) from the host libm
  double rescale;           // sqrt(1 - log 2 / log n)
};

struct BatchResult {
  double thresh, thresh_univ, min_margin;
  int iterations, status;
  long long kept, zeroed;
};

struct BatchArgs {
  const BatchDesc* desc;
  BatchResult* res;
  const int* order;         // processing order (largest work first)
  int* counter;             // work-queue head
  int nsig;
  double* data;             // all signals, FP64, smoothed in place
  char* scratch;            // grid * scratch_per_cta bytes
  size_t scratch_per_cta;
};

size_t batch_scratch_bytes(const BatchDesc& d, int prec);
int batch_launch(const BatchArgs& a, int prec, int grid, cudaStream_t s);
int batch_max_ctas(int prec);

// Per-precision instantiations of the persistent kernel (batch_exact.cu,
// batch_fast.cu, batch_f32.cu): launch, and resident CTAs per SM.
int batch_launch_exact(const BatchArgs& a, int grid, cudaStream_t s);
int batch_launch_fast(const BatchArgs& a, int grid, cudaStream_t s);
int batch_launch_f32(const BatchArgs& a, int grid, cudaStream_t s);
int batch_blocks_per_sm_exact();
int batch_blocks_per_sm_fast();
int batch_blocks_per_sm_f32();

}  // namespace wc
