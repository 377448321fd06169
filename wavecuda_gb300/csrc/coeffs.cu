// Coefficient extraction and formatting: the level / translate / type
// labelling of WSTtoDT (R/rfunctions.R:925-1004) and the index sets of
// getCoeffLevel (R/rplotting.R:10-46), computed on the device for large n.
//
// WSTtoDT builds its table by first labelling every DWT coefficient level 1
// with translate 0.5 + floor(i/2) (0-based i) and then overwriting, for each
// level l >= 2, the details of that level with level l and the translates
// seq(2^(l-2), len/2, by = 2^(l-1)) in order, and the scaling slots with
// level J and level J's translates.  Every row therefore ends with the
// closed form used here: a coefficient at 0-based position i is the k-th of
// its level l, k = i >> l (details, l = ctz(i) + 1) or k = i >> J (scaling
// slots, i = 0 mod 2^J, l = J), with translate 2^(l-2) + k 2^(l-1) -- which
// is also 0.5 + floor(i/2) at l = 1, so the J = 1 case (no overwrite loop)
// agrees.  MODWT rows: block l (s_{l+1} then d_{l+1}, len values each) is
// level l + 1, translate t + 1, type s for the first half.  The table keeps
// the input order; without the scaling rows (scaling = FALSE) a DWT detail
// at position i is row i - ((i - 1) >> J) - 1 and a MODWT detail row
// l*len + t.  The plotting rows (forPlotting = TRUE: per-level min/max
// placeholders) are not produced: plotting is outside this library.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "wc_internal.h"

namespace wc {
namespace {

__global__ void wst_table_kernel(const double* __restrict__ w, int64_t len, int J, int ttype,
                                 int scaling, double* __restrict__ W, int32_t* __restrict__ level,
                                 double* __restrict__ translate, uint8_t* __restrict__ type) {
  const int64_t total = ttype == 0 ? len : 2 * (int64_t)J * len;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
    int lev;
    double tr;
    bool det;
    int64_t row;
    if (ttype == 0) {
      det = (i & (((int64_t)1 << J) - 1)) != 0;
      lev = det ? __ffsll(i) : J;
      const int64_t k = i >> lev;
      tr = ldexp(1.0, lev - 2) + (double)k * ldexp(1.0, lev - 1);
      row = scaling ? i : i - ((i - 1) >> J) - 1;
    } else {
      const int64_t blk = i / (2 * len), within = i - blk * 2 * len;
      det = within >= len;
      const int64_t t = det ? within - len : within;
      lev = (int)blk + 1;
      tr = (double)(t + 1);
      row = scaling ? i : blk * len + t;
    }
    if (!det && !scaling) continue;
    if (W) W[row] = w[i];
    if (level) level[row] = lev;
    if (translate) translate[row] = tr;
    if (type) type[row] = det ? 1 : 0;
  }
}

int check_table_args(int64_t len, int nlevels, int ttype) {
  if (len <= 1 || (len & (len - 1)) != 0)
    return fail(WC_ERR_ARG, "length %lld is not a power of 2 above 1", (long long)len);
  if (ttype == 2)
    return fail(WC_ERR_UNSUPPORTED,
                "packet-ordered MODWT coefficients have no WSTtoDT table (rfunctions.R:974)");
  if (ttype != 0 && ttype != 1) return fail(WC_ERR_ARG, "transform type %d not provided", ttype);
  int maxJ = 0;
  while (((int64_t)1 << (maxJ + 1)) <= len) maxJ++;
  if (nlevels < 1 || nlevels > maxJ)
    return fail(WC_ERR_LEVELS, "nlevels %d outside 1..%d for length %lld", nlevels, maxJ,
                (long long)len);
  return WC_OK;
}

int64_t table_rows(int64_t len, int J, int ttype, int scaling) {
  if (ttype == 0) return scaling ? len : len - (len >> J);
  return (scaling ? 2 : 1) * (int64_t)J * len;
}

int launch_table(const double* w, int64_t len, int J, int ttype, int scaling, double* W,
                 int32_t* level, double* translate, uint8_t* type, cudaStream_t s) {
  const int64_t total = ttype == 0 ? len : 2 * (int64_t)J * len;
  int sms = 0, dev = 0;
  WC_CUDA(cudaGetDevice(&dev));
  WC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int64_t blocks = std::min<int64_t>((total + 255) / 256, (int64_t)sms * 8);
  {
    LaunchTimer lt("wst_table", s);
    wst_table_kernel<<<(unsigned)blocks, 256, 0, s>>>(w, len, J, ttype, scaling, W, level,
                                                      translate, type);
  }
  return after_launch("wst_table_kernel");
}

}  // namespace
}  // namespace wc

using namespace wc;

extern "C" {

int wc_coeff_level_indices(int64_t len, int nlevels, int ttype, int level, int coeff_type,
                           int64_t* idx, int64_t capacity, int64_t* count) {
  clear_error();
  WC_TRY(check_table_args(len, nlevels, ttype));
  if (!count) return fail(WC_ERR_ARG, "null count");
  if (level < 1 || level > nlevels)
    return fail(WC_ERR_LEVELS, "integer level expected, between 1 and %d", nlevels);
  if (coeff_type != 0 && coeff_type != 1)
    return fail(WC_ERR_ARG, "coefficient type must be 0 (scaling) or 1 (detail)");
  int64_t start = 1, gap = 1;  // MODWT: 1..len whatever the level (rplotting.R:39-42)
  if (ttype == 0) {
    if (coeff_type == 0 && level != nlevels)
      return fail(WC_ERR_ARG, "DWT scaling coefficients exist at level %d only", nlevels);
    start = ((int64_t)1 << (level - 1)) * coeff_type + 1;
    gap = (int64_t)1 << level;
  }
  const int64_t n = (len - start) / gap + 1;
  *count = n;
  if (!idx) return WC_OK;
  if (capacity < n) return fail(WC_ERR_ARG, "index buffer holds %lld of %lld indices",
                                (long long)capacity, (long long)n);
  for (int64_t k = 0; k < n; k++) idx[k] = start + k * gap;
  return WC_OK;
}

int wc_wst_table_rows(int64_t len, int nlevels, int ttype, int scaling, int64_t* rows) {
  clear_error();
  WC_TRY(check_table_args(len, nlevels, ttype));
  if (!rows) return fail(WC_ERR_ARG, "null rows");
  *rows = table_rows(len, nlevels, ttype, scaling ? 1 : 0);
  return WC_OK;
}

int wc_wst_table_device(const double* w, int64_t len, int nlevels, int ttype, int scaling,
                        double* W, int32_t* level, double* translate, uint8_t* type,
                        void* stream) {
  clear_error();
  WC_TRY(check_table_args(len, nlevels, ttype));
  if (!w) return fail(WC_ERR_ARG, "null coefficient vector");
  WC_TRY(ensure_device());
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : lib_stream();
  return launch_table(w, len, nlevels, ttype, scaling ? 1 : 0, W, level, translate, type, s);
}

int wc_wst_table(const double* w, int64_t len, int nlevels, int ttype, int scaling, double* W,
                 int32_t* level, double* translate, uint8_t* type) {
  clear_error();
  WC_TRY(check_table_args(len, nlevels, ttype));
  if (!w) return fail(WC_ERR_ARG, "null coefficient vector");
  WC_TRY(ensure_device());
  const int sc = scaling ? 1 : 0;
  const int64_t total = ttype == 0 ? len : 2 * (int64_t)nlevels * len;
  const int64_t rows = table_rows(len, nlevels, ttype, sc);
  cudaStream_t s = lib_stream();
  double* dw = static_cast<double*>(workspace(kSlotStageA, sizeof(double) * (size_t)total));
  // Output columns packed in one buffer: W, translate (8 B), level (4 B), type (1 B).
  char* out = static_cast<char*>(workspace(kSlotStageB, (size_t)rows * 21 + 64));
  if (!dw || !out) return workspace_error();
  double* dW = reinterpret_cast<double*>(out);
  double* dT = dW + rows;
  int32_t* dL = reinterpret_cast<int32_t*>(dT + rows);
  uint8_t* dY = reinterpret_cast<uint8_t*>(dL + rows);
  WC_CUDA(cudaMemcpyAsync(dw, w, sizeof(double) * (size_t)total, cudaMemcpyHostToDevice, s));
  WC_TRY(launch_table(dw, len, nlevels, ttype, sc, W ? dW : nullptr, level ? dL : nullptr,
                      translate ? dT : nullptr, type ? dY : nullptr, s));
  WC_TRY(take_status(s));
  if (W) WC_CUDA(cudaMemcpyAsync(W, dW, sizeof(double) * (size_t)rows, cudaMemcpyDeviceToHost, s));
  if (translate)
    WC_CUDA(cudaMemcpyAsync(translate, dT, sizeof(double) * (size_t)rows, cudaMemcpyDeviceToHost, s));
  if (level)
    WC_CUDA(cudaMemcpyAsync(level, dL, sizeof(int32_t) * (size_t)rows, cudaMemcpyDeviceToHost, s));
  if (type) WC_CUDA(cudaMemcpyAsync(type, dY, (size_t)rows, cudaMemcpyDeviceToHost, s));
  WC_CUDA(cudaStreamSynchronize(s));
  return WC_OK;
}

}  // extern "C"
