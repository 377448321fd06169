// Thresholding (thresh.cpp:15-157), the universal threshold
// (thresh.cpp:170-201) and its exact median / MAD (utils.cpp:166-203).
//
// The reference sorts (qsort) to get medians.  Here the two middle order
// statistics are found by an exact radix select over the FP64 bit patterns:
// each double maps to a 64-bit key whose unsigned order is the numeric order
// (sign bit flipped for non-negative values, all bits inverted for negative
// ones), and 8 histogram passes of 8 bits fix the key of rank k, most
// significant digit first.  Both ranks (n-1)/2 and n/2 are tracked in the
// same passes.  The selected values are the same doubles qsort would put at
// those ranks, so 0.5*(a+b) and 1.4826*mad are bit-identical to the
// reference.
#include <math.h>

#include <algorithm>

#include "wc_common.cuh"

namespace wc {
namespace {

constexpr int kThreads = 256;

unsigned grid_for(int64_t n) {
  int64_t blocks = (n + kThreads - 1) / kThreads;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(blocks, 152 * 8));
}

// thresh_coef (thresh.cpp:142-157): |c| < t -> 0; soft moves c towards zero.
template <class T>
__device__ __forceinline__ T thresh_coef(T c, T t, int hardness) {
  if (fabs(c) < t) return T(0);
  if (hardness == 1) {
    if constexpr (sizeof(T) == 8) {
      return __dmul_rn((c < 0) ? -1.0 : 1.0, __dsub_rn(fabs(c), t));
    } else {
      return ((c < 0) ? -1.0f : 1.0f) * (fabsf(c) - t);
    }
  }
  return c;
}

// DWT, in place or in -> out (threshold_dwt, thresh.cpp:15-35).  Level of an
// index i > 0 is ctz(i); indices with ctz >= levels (and 0) are scaling
// coefficients: copied to out only at i == 0, or at every such slot when
// copy_scaling is set.
template <class T>
__global__ void thresh_dwt_kernel(const T* __restrict__ in, T* __restrict__ out, int64_t n,
                                  int levels, T t, int hardness, int minl, int maxl,
                                  int copy_scaling) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const bool inplace = (in == out);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    if (i == 0) {
      if (!inplace) out[0] = in[0];
      continue;
    }
    const int l = __ffsll((long long)i) - 1;
    if (l >= levels) {
      if (!inplace && copy_scaling) out[i] = in[i];
      continue;
    }
    if (l >= minl && l <= maxl) out[i] = thresh_coef(in[i], t, hardness);
    else if (!inplace) out[i] = in[i];
  }
}

// Time-ordered MODWT (threshold_modwt, thresh.cpp:41-83): d blocks of levels
// [minl, maxl] thresholded, everything else copied when out != in.
template <class T>
__global__ void thresh_modwt_kernel(const T* __restrict__ in, T* __restrict__ out, int64_t n,
                                    int levels, T t, int hardness, int minl, int maxl) {
  const int64_t total = 2 * n * (int64_t)levels;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const bool inplace = (in == out);
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += stride) {
    const int l = (int)(e / (2 * n));
    const bool det = (e - (int64_t)l * 2 * n) >= n;
    if (det && l >= minl && l <= maxl) out[e] = thresh_coef(in[e], t, hardness);
    else if (!inplace) out[e] = in[e];
  }
}

// ---------------------------------------------------------- radix select --

__device__ __forceinline__ uint64_t key_of(double v) {
  uint64_t u = (uint64_t)__double_as_longlong(v);
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
__host__ __device__ inline double value_of_key(uint64_t k) {
  uint64_t u = (k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double d;
  memcpy(&d, &u, 8);
  return d;
#endif
}

struct SelState {
  uint64_t prefix[2];
  uint64_t mask[2];
};

// Two histograms (ranks a and b) of digit (key >> shift) & 255 among the
// elements whose key matches the rank's current prefix.
__global__ void select_hist_kernel(SelectSource src, int64_t count, SelState st, int shift,
                                   unsigned long long* __restrict__ hist) {
  __shared__ unsigned int h[2][256];
  for (int i = threadIdx.x; i < 512; i += blockDim.x) (&h[0][0])[i] = 0;
  __syncthreads();
  const bool same = (st.prefix[0] == st.prefix[1]) && (st.mask[0] == st.mask[1]);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count; e += stride) {
    const int64_t seg = e / src.seg_len, off = e - seg * src.seg_len;
    const uint64_t k = key_of(src.base[seg * src.seg_stride + off]);
    const int digit = (int)((k >> shift) & 255);
    if ((k & st.mask[0]) == st.prefix[0]) atomicAdd(&h[0][digit], 1u);
    if (!same && (k & st.mask[1]) == st.prefix[1]) atomicAdd(&h[1][digit], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 512; i += blockDim.x) {
    const int r = i >> 8, d = i & 255;
    const unsigned int v = same ? h[0][d] : h[r][d];
    if (v) atomicAdd(&hist[i], (unsigned long long)v);
  }
}

// Absolute deviations |x - med| written compactly (utils.cpp:198).
__global__ void abs_dev_kernel(SelectSource src, int64_t count, double med,
                               double* __restrict__ dev) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count; e += stride) {
    const int64_t seg = e / src.seg_len, off = e - seg * src.seg_len;
    dev[e] = fabs(__dsub_rn(src.base[seg * src.seg_stride + off], med));
  }
}

// DWT details of levels [minl, maxl] (below `levels`) gathered level by
// level in index order (isolate_dlevels, wavutils.cpp:683-713).
__global__ void gather_dwt_kernel(const double* __restrict__ x, int64_t n, int levels,
                                  int minl, int maxl, double* __restrict__ dst) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = 1 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int l = __ffsll((long long)i) - 1;
    if (l >= levels || l < minl || l > maxl) continue;
    int64_t base = 0;
    for (int m = minl; m < l; m++) base += n >> (m + 1);
    dst[base + (i >> (l + 1))] = x[i];
  }
}

// Kept / zeroed counts over the details of levels [minl, maxl].
__global__ void count_kept_kernel(const double* __restrict__ data, int64_t n, int levels,
                                  int ttype, double t, int minl, int maxl,
                                  unsigned long long* __restrict__ out) {
  unsigned long long kept = 0, zeroed = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  if (ttype == 0) {
    for (int64_t i = 1 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
      const int l = __ffsll((long long)i) - 1;
      if (l >= levels || l < minl || l > maxl) continue;
      if (fabs(data[i]) < t) zeroed++; else kept++;
    }
  } else {
    const int64_t total = (int64_t)(maxl - minl + 1) * n;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += stride) {
      const int64_t l = minl + e / n, i = e - (l - minl) * n;
      if (fabs(data[(2 * l + 1) * n + i]) < t) zeroed++; else kept++;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    kept += __shfl_down_sync(0xffffffffu, kept, o);
    zeroed += __shfl_down_sync(0xffffffffu, zeroed, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (kept) atomicAdd(&out[0], kept);
    if (zeroed) atomicAdd(&out[1], zeroed);
  }
}

// Keys of ranks ka <= kb among `count` elements (8-bit digits, MSB first).
int select_two(const SelectSource& src, int64_t count, int64_t ka, int64_t kb, cudaStream_t s,
               double* va, double* vb) {
  auto* hist = static_cast<unsigned long long*>(workspace(kSlotSelect, 512 * sizeof(unsigned long long)));
  if (!hist) return workspace_error();
  unsigned long long h[512];
  SelState st{{0, 0}, {0, 0}};
  int64_t rank[2] = {ka, kb};
  const unsigned grid = grid_for(count);
  for (int shift = 56; shift >= 0; shift -= 8) {
    WC_CUDA(cudaMemsetAsync(hist, 0, 512 * sizeof(unsigned long long), s));
    select_hist_kernel<<<grid, kThreads, 0, s>>>(src, count, st, shift, hist);
    WC_TRY(after_launch("select_hist_kernel"));
    WC_CUDA(cudaMemcpyAsync(h, hist, sizeof(h), cudaMemcpyDeviceToHost, s));
    WC_CUDA(cudaStreamSynchronize(s));
    for (int r = 0; r < 2; r++) {
      const unsigned long long* hr = h + 256 * r;
      unsigned long long cum = 0;
      int d = 0;
      for (; d < 256; d++) {
        if ((unsigned long long)rank[r] < cum + hr[d]) break;
        cum += hr[d];
      }
      if (d == 256) return fail(WC_ERR_CUDA, "radix select lost rank %lld", (long long)rank[r]);
      rank[r] -= (int64_t)cum;
      st.prefix[r] |= (uint64_t)d << shift;
      st.mask[r] |= (uint64_t)255 << shift;
    }
  }
  *va = value_of_key(st.prefix[0]);
  *vb = value_of_key(st.prefix[1]);
  return WC_OK;
}

}  // namespace

int median_mad(const SelectSource& src, int64_t count, cudaStream_t s, double* median,
               double* mad) {
  if (count <= 0) {
    *median = 0.0;
    *mad = 0.0;
    return WC_OK;
  }
  double a, b;
  WC_TRY(select_two(src, count, (count - 1) / 2, count / 2, s, &a, &b));
  const double med = 0.5 * (a + b);
  *median = med;
  if (!mad) return WC_OK;
  auto* dev = static_cast<double*>(workspace(kSlotSelectData, sizeof(double) * (size_t)count));
  if (!dev) return workspace_error();
  abs_dev_kernel<<<grid_for(count), kThreads, 0, s>>>(src, count, med, dev);
  WC_TRY(after_launch("abs_dev_kernel"));
  SelectSource ds{dev, count, count, 1};
  WC_TRY(select_two(ds, count, (count - 1) / 2, count / 2, s, &a, &b));
  *mad = 1.4826 * (0.5 * (a + b));
  return WC_OK;
}

int univ_thresh(const double* data, int64_t n, int J, int ttype, int minl, int maxl,
                cudaStream_t s, double* out) {
  double med, mad;
  if (ttype == 0) {
    if (minl == 0 && maxl == J - 1) {
      // thresh.cpp:176-181: all of x[1..len-1], scaling slots included.
      SelectSource src{data + 1, n - 1, n - 1, 1};
      WC_TRY(median_mad(src, n - 1, s, &med, &mad));
      *out = mad * sqrt(2. * log((double)(n - 1)));
      return WC_OK;
    }
    int64_t cnt = 0;
    for (int l = minl; l <= maxl; l++) cnt += n >> (l + 1);
    auto* tmp = static_cast<double*>(workspace(kSlotReduce, sizeof(double) * (size_t)std::max<int64_t>(cnt, 1)));
    if (!tmp) return workspace_error();
    gather_dwt_kernel<<<grid_for(n), kThreads, 0, s>>>(data, n, J, minl, maxl, tmp);
    WC_TRY(after_launch("gather_dwt_kernel"));
    // Levels at or above J contribute no details (isolate_dlevels only walks
    // levels below J), so count what was gathered.
    int64_t got = 0;
    for (int l = minl; l <= maxl && l < J; l++) got += n >> (l + 1);
    SelectSource src{tmp, got, got, 1};
    WC_TRY(median_mad(src, got, s, &med, &mad));
    *out = mad * sqrt(2. * log((double)n));
    return WC_OK;
  }
  // MODWT: d blocks of levels 0 .. maxl-minl (isolate_dlevels starts at the
  // level-0 block whatever minl is, wavutils.cpp:716-722).
  const int64_t nb = maxl - minl + 1;
  SelectSource src{data + n, n, 2 * n, nb};
  WC_TRY(median_mad(src, nb * n, s, &med, &mad));
  *out = mad * sqrt(2. * log((double)n));
  return WC_OK;
}

int count_kept(const double* data, int64_t n, int J, int ttype, double t, int minl, int maxl,
               cudaStream_t s, int64_t* kept, int64_t* zeroed) {
  auto* c = static_cast<unsigned long long*>(workspace(kSlotSelect, 512 * sizeof(unsigned long long)));
  if (!c) return workspace_error();
  WC_CUDA(cudaMemsetAsync(c, 0, 2 * sizeof(unsigned long long), s));
  count_kept_kernel<<<grid_for(ttype == 0 ? n : n * (maxl - minl + 1)), kThreads, 0, s>>>(
      data, n, J, ttype, t, minl, maxl, c);
  WC_TRY(after_launch("count_kept_kernel"));
  unsigned long long h[2];
  WC_CUDA(cudaMemcpyAsync(h, c, sizeof(h), cudaMemcpyDeviceToHost, s));
  WC_CUDA(cudaStreamSynchronize(s));
  *kept = (int64_t)h[0];
  *zeroed = (int64_t)h[1];
  return WC_OK;
}

// In place (in == out) or in -> out threshold launches used by the ABI and
// the smoothing drivers.
template <class T>
int threshold_to(const T* in, T* out, int64_t n, int J, int ttype, double t, int hardness,
                 int minl, int maxl, int copy_scaling, cudaStream_t s) {
  if (ttype == 0) {
    thresh_dwt_kernel<T><<<grid_for(n), kThreads, 0, s>>>(in, out, n, J, (T)t, hardness, minl,
                                                          maxl, copy_scaling);
    return after_launch("thresh_dwt_kernel");
  }
  thresh_modwt_kernel<T><<<grid_for(2 * n * J), kThreads, 0, s>>>(in, out, n, J, (T)t, hardness,
                                                                  minl, maxl);
  return after_launch("thresh_modwt_kernel");
}
template int threshold_to<double>(const double*, double*, int64_t, int, int, double, int, int,
                                  int, int, cudaStream_t);
template int threshold_to<float>(const float*, float*, int64_t, int, int, double, int, int, int,
                                 int, cudaStream_t);

int threshold(void* data, int64_t n, int J, int ttype, double t, int hardness, int minl,
              int maxl, int prec, cudaStream_t s) {
  if (prec == WC_F32)
    return threshold_to<float>(static_cast<float*>(data), static_cast<float*>(data), n, J, ttype,
                               t, hardness, minl, maxl, 0, s);
  return threshold_to<double>(static_cast<double*>(data), static_cast<double*>(data), n, J, ttype,
                              t, hardness, minl, maxl, 0, s);
}

}  // namespace wc
