// Host side of batched per-level threshold tuning (fit_kernel.cuh):
// validation, per-CTA scratch sizing, the persistent grid, and the device-
// and host-buffer entry points.
#include <math.h>
#include <string.h>

#include <algorithm>

#include "wc_common.cuh"
#include "wc_fit.h"

namespace wc {
namespace {

size_t r256(size_t b) { return ((b + 255) / 256) * 256; }

// Scratch one CTA takes for one signal (mirrors fit_one's takes).
size_t fit_scratch_bytes(int64_t n, int J, int ttype, int loss, int prec) {
  const size_t tsz = (prec == WC_F32) ? 4 : 8;  // stored values (float or double)
  const size_t vs = (prec == WC_F32) ? 4 : 8;   // working values (float or float pair)
  const bool mod = ttype == 1;
  const int64_t h = n / 2;
  size_t s = r256(tsz * n) + r256(tsz * (mod ? (size_t)J * n : n)) + r256(tsz * (mod ? n : 1)) +
             3 * r256(vs * n) + r256(8 * (size_t)n);
  if (loss == WC_LOSS_CV) {
    const int Jl = J - 1;
    s += 2 * (r256(tsz * (mod ? (size_t)Jl * h : h)) + r256(tsz * (mod ? h : 1))) +
         4 * r256(vs * h);
  }
  return s + 1024;
}

int sm_count_dev() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 1;
}

int fit_run(double* x, int64_t n, int nsig, int nlevels, int F, int ttype, const wc_fit_opts* o,
            wc_fit_result* results, cudaStream_t s) {
  if (F < 1 || F > 4) return fail(WC_ERR_ARG, "unrecognised filter %d", F);
  if (ttype != 0 && ttype != 1) return fail(WC_ERR_ARG, "transform type %d", ttype);
  if (!x || !o || !results || nsig <= 0) return fail(WC_ERR_ARG, "bad tuning arguments");
  if (o->loss_type != WC_LOSS_SURE && o->loss_type != WC_LOSS_CV)
    return fail(WC_ERR_ARG, "unknown loss %d", o->loss_type);
  if (o->precision != WC_F32 && o->precision != WC_F64_FAST)
    return fail(WC_ERR_ARG, "threshold tuning runs in WC_F32 or WC_F64_FAST, not %d",
                o->precision);
  if (o->iterations < 0 || o->iterations > 100000) return fail(WC_ERR_ARG, "iterations %d", o->iterations);
  if (!(o->step >= 0.0) || !(o->eps >= 0.0)) return fail(WC_ERR_ARG, "step and eps must be >= 0");
  const int J = check_levels(n, nlevels, filter_len(F));
  if (J == 0) return fail(WC_ERR_LEVELS, "nlevels %d invalid for length %lld", nlevels, (long long)n);
  if (J > kFitLevels) return fail(WC_ERR_LEVELS, "at most %d levels", kFitLevels);
  const int maxl = o->maxlevel < 0 ? J - 1 : o->maxlevel;
  if (o->minlevel < 0 || maxl >= J || o->minlevel > maxl)
    return fail(WC_ERR_LEVELS, "level range [%d, %d] invalid for %d levels", o->minlevel, maxl, J);
  if (o->loss_type == WC_LOSS_CV) {
    if (J < 2 || check_levels(n / 2, J - 1, filter_len(F)) == 0)
      return fail(WC_ERR_LEVELS, "cross-validation needs the half-length signals to take %d levels",
                  J - 1);
    if (o->minlevel > std::min(maxl, J - 2))
      return fail(WC_ERR_LEVELS, "cross-validation thresholds no half level in [%d, %d]",
                  o->minlevel, maxl);
  }
  if ((int64_t)nsig > INT64_MAX / n) return fail(WC_ERR_ARG, "batch too large");

  FitArgs a{};
  a.data = x;
  a.n = n;
  a.nsig = nsig;
  a.J = J;
  a.F = F;
  a.ttype = ttype;
  a.loss = o->loss_type;
  a.minl = o->minlevel;
  a.maxl = maxl;
  a.iters = o->iterations;
  a.smooth = o->smooth ? 1 : 0;
  a.lr = o->step;
  a.eps_rel = o->eps;
  a.sigma = o->sigma;
  a.sq2logn = sqrt(2.0 * log((double)n));
  a.rescale = sqrt(1.0 - log(2.0) / log((double)n));
  a.has_lam0 = o->lambda0 ? 1 : 0;
  for (int l = 0; l < kFitLevels; l++) a.lam0[l] = (o->lambda0 && l < J) ? o->lambda0[l] : 0.0;

  const int per = (o->precision == WC_F32) ? fit_blocks_per_sm_f32() : fit_blocks_per_sm_fast();
  const int grid = (int)std::min<int64_t>(nsig, (int64_t)per * sm_count_dev());
  const size_t per_cta = r256(fit_scratch_bytes(n, J, ttype, o->loss_type, o->precision));
  const size_t res_bytes = r256(sizeof(FitResult) * (size_t)nsig);
  char* base = static_cast<char*>(workspace(kSlotTune, 256 + res_bytes + per_cta * grid));
  if (!base) return workspace_error();
  a.counter = reinterpret_cast<int*>(base);
  a.res = reinterpret_cast<FitResult*>(base + 256);
  a.scratch = base + 256 + res_bytes;
  a.scratch_per_cta = per_cta;
  WC_CUDA(cudaMemsetAsync(a.counter, 0, sizeof(int), s));
  {
    LaunchTimer lt("fit_batch", s);
    if (o->precision == WC_F32) WC_TRY(fit_launch_f32(a, grid, s));
    else WC_TRY(fit_launch_fast(a, grid, s));
  }
  WC_CUDA(cudaMemcpyAsync(results, a.res, sizeof(FitResult) * (size_t)nsig,
                          cudaMemcpyDeviceToHost, s));
  WC_CUDA(cudaStreamSynchronize(s));
  return WC_OK;
}

}  // namespace
}  // namespace wc

using namespace wc;

extern "C" {

int wc_fit_thresholds_device(double* x, int64_t len, int nsig, int nlevels, int filter, int ttype,
                             const wc_fit_opts* opts, wc_fit_result* results, void* stream) {
  clear_error();
  WC_TRY(ensure_device());
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : lib_stream();
  return fit_run(x, len, nsig, nlevels, filter, ttype, opts, results, s);
}

int wc_fit_thresholds(double* x, int64_t len, int nsig, int nlevels, int filter, int ttype,
                      const wc_fit_opts* opts, wc_fit_result* results) {
  clear_error();
  if (!x || len <= 0 || nsig <= 0) return fail(WC_ERR_ARG, "bad tuning arguments");
  if ((int64_t)nsig > INT64_MAX / 8 / len) return fail(WC_ERR_ARG, "batch too large");
  WC_TRY(ensure_device());
  cudaStream_t s = lib_stream();
  const size_t bytes = sizeof(double) * (size_t)len * (size_t)nsig;
  double* d = static_cast<double*>(workspace(kSlotStageA, bytes));
  if (!d) return workspace_error();
  WC_CUDA(cudaMemcpyAsync(d, x, bytes, cudaMemcpyHostToDevice, s));
  WC_TRY(fit_run(d, len, nsig, nlevels, filter, ttype, opts, results, s));
  WC_TRY(take_status(s));  // x stays untouched when a wait gave up
  if (opts->smooth) {
    WC_CUDA(cudaMemcpyAsync(x, d, bytes, cudaMemcpyDeviceToHost, s));
    WC_CUDA(cudaStreamSynchronize(s));
  }
  return WC_OK;
}

}  // extern "C"
