// Batched per-level threshold tuning: arguments shared by the persistent
// kernel (fit_kernel.cuh) and its host side (fit.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "wc_internal.h"

namespace wc {

constexpr int kFitLevels = WC_FIT_MAX_LEVELS;

// Per-signal results; the public record (wavecuda_gb300.h) is the same type.
using FitResult = wc_fit_result;

struct FitArgs {
  double* data;  // nsig signals of n FP64 values; smoothed in place when smooth
  int64_t n;
  int nsig, J, F, ttype, loss, minl, maxl, iters, smooth, has_lam0;
  double lr, eps_rel, sigma, sq2logn, rescale;
  double lam0[kFitLevels];
  FitResult* res;
  int* counter;
  char* scratch;
  size_t scratch_per_cta;
};

int fit_launch_f32(const FitArgs& a, int grid, cudaStream_t s);
int fit_launch_fast(const FitArgs& a, int grid, cudaStream_t s);
int fit_blocks_per_sm_f32();
int fit_blocks_per_sm_fast();

}  // namespace wc
