// Smoothing: forward transform, threshold, inverse (rfunctions.cu:71-137) with
// a manual, universal (thresh.cpp:170-201) or two-fold cross-validated
// threshold (CVT, thresh.cpp:203-342).
//
// CV follows the reference step by step: the noisy signal is split into even
// and odd halves (copyvecskip, thresh.cpp:244-245), both are transformed once
// with J-1 levels, and a golden-section search over t in [0, t_univ] keeps
// two candidates t1 < t2.  Each new candidate thresholds both halves (levels
// [minlevel, maxlevel-1]), inverts them and scores the interpolation error
// of thresh.cpp:344-385.  For the DWT and the time-ordered MODWT the whole
// search runs on the device in one persistent cooperative launch
// (cv_fused_kernel.cuh): no host round trip per step.  The packet-ordered
// MODWT keeps the step-by-step form, where only the scalar loss comes back
// to drive the reference's FP64 host logic.  Constants R = 0.61803399, at
// most 51 iterations, final rescale t / sqrt(1 - ln 2 / ln n).
//
// Bit-exact selection.  With soft thresholds the two losses compared in the
// last iterations differ by ~1e-16 relative, below rounding noise, so the
// search only reproduces the reference's choice if the losses are the
// reference's doubles.  In WC_F64_EXACT every term is computed with the
// reference's roundings and the sum is the reference's left-to-right
// sequential FP64 sum (cv_sum.cu), so the chosen threshold is bit-identical.
//
// Quirks kept on purpose (they change results):
//  * threshold_dwt into a separate vector never writes the coarse scaling
//    slots k*2^(J-1), k > 0 (thresh.cpp:15-35), so those slots keep the
//    previous inverse transform's output.  Each half-length work vector is
//    therefore a pair of buffers that trade roles (thresholded coefficients
//    are written over the previous reconstruction); both start zeroed, which
//    is what the reference sees from fresh zero-filled pages.
//  * when the half-length level range is invalid (maxlevel == 0 or
//    minlevel > maxlevel-1) the reference skips thresholding and its inverse
//    transform refuses to run (transform.cpp:5-8); the work vectors then stay
//    zero, and so they do here.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include <algorithm>

#include "wc_common.cuh"
#include "wc_cvfused.h"
#include "wc_grid.cuh"

namespace wc {

template <class T>
int threshold_to(const T* in, T* out, int64_t n, int J, int ttype, double t, int hardness,
                 int minl, int maxl, int copy_scaling, cudaStream_t s);
int cv_sequential_sum(const double* terms, int64_t count, double* dev_out, void* scratch,
                      cudaStream_t s);
size_t cv_sum_scratch_bytes(int64_t count);

namespace {

constexpr int kThreads = 256;

unsigned grid_for(int64_t n) {
  int64_t blocks = (n + kThreads - 1) / kThreads;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(blocks, 152 * 8));
}

template <class T>
__global__ void split_even_odd(const double* __restrict__ x, int64_t lenh, T* __restrict__ e,
                               T* __restrict__ o) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < lenh; j += stride) {
    e[j] = (T)x[2 * j];
    o[j] = (T)x[2 * j + 1];
  }
}

template <class A, class B>
__global__ void convert_kernel(const A* __restrict__ in, B* __restrict__ out, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    out[i] = (B)in[i];
}

// Loss terms of interp_mse (thresh.cpp:363-382), one per even/odd pair:
// v_j = (yie - xn[2j])^2 + (yio - xn[2j+1])^2, every operation rounded as in
// the reference.
template <class T>
__global__ void cv_terms_kernel(const T* __restrict__ ye, const T* __restrict__ yo,
                                const double* __restrict__ xn, int64_t lenh,
                                double* __restrict__ terms) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < lenh; j += stride) {
    double yie, yio;
    if (j == 0) {
      yie = (double)yo[0];
      yio = __dmul_rn(0.5, __dadd_rn((double)ye[0], (double)ye[1]));
    } else if (j == lenh - 1) {
      yio = (double)ye[lenh - 1];
      yie = __dmul_rn(0.5, __dadd_rn((double)yo[j], (double)yo[j - 1]));
    } else {
      yio = __dmul_rn(0.5, __dadd_rn((double)ye[j], (double)ye[j + 1]));
      yie = __dmul_rn(0.5, __dadd_rn((double)yo[j], (double)yo[j - 1]));
    }
    const double a = __dsub_rn(yie, xn[2 * j]);
    const double b = __dsub_rn(yio, xn[2 * j + 1]);
    terms[j] = __dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b));
  }
}

// check_len_levels with a level range (wavutils.cpp:66-77).
bool range_ok(int64_t n, int J, int minl, int maxl, int L) {
  int r = check_levels(n, J, L);
  if (r == 0 || minl < 0 || maxl < 0) return false;
  return minl <= maxl && maxl < r;
}

// One half-length work vector of the CV search (the reference's y1e etc.).
template <class T>
struct HalfVec {
  T* buf[2];     // DWT: the vector and its spare; MODWT: buf[0] = x
  T* mod;        // MODWT coefficients (2*lenh*(J-1))
  int cur;       // DWT: which buffer holds the vector
  int transformed;
  T* x() const { return buf[cur]; }
};

template <class T>
struct Ctx {
  int64_t n, lenh;
  int J, ttype, F, hardness, minl, maxl, prec, copy_scaling;
  cudaStream_t s;
  bool po;  // packet-ordered MODWT: time-ordered store, packet-ordered inverse
};

template <class T>
int transform_full(const Ctx<T>& c, void* x, void* coef, int64_t len, int J, int sense) {
  if (c.ttype == 0) {
    return sense == 1 ? dwt(x, coef, len, 1, J, c.F, c.prec, c.s)
                      : dwt(coef, x, len, 0, J, c.F, c.prec, c.s);
  }
  if (sense == 0 && c.po) return modwt_po_inverse_to(x, coef, len, J, c.F, c.prec, c.s);
  return modwt(x, coef, len, sense, J, c.F, c.prec, c.s);
}

// threshold(we, y, t, ...) then transform(y, BWD) (thresh.cpp:269-279).
template <class T>
int half_step(const Ctx<T>& c, const T* wcoef, HalfVec<T>& y, double t) {
  const int lv1 = c.J - 1;
  const int maxl1 = c.maxl - 1;
  if (range_ok(c.lenh, lv1, c.minl, maxl1, filter_len(c.F))) {
    T* dst = (c.ttype == 0) ? y.x() : y.mod;
    WC_TRY(threshold_to<T>(wcoef, dst, c.lenh, lv1, c.ttype, t, c.hardness, c.minl, maxl1,
                           c.copy_scaling, c.s));
    y.transformed = 1;
  }
  if (!y.transformed) return WC_OK;  // transform.cpp:5-8 refuses BWD
  if (c.ttype == 0) {
    WC_TRY(dwt(y.buf[y.cur], y.buf[1 - y.cur], c.lenh, 0, lv1, c.F, c.prec, c.s));
    y.cur = 1 - y.cur;
  } else {
    if (c.po) WC_TRY(modwt_po_inverse_to(y.buf[0], y.mod, c.lenh, lv1, c.F, c.prec, c.s));
    else WC_TRY(modwt(y.buf[0], y.mod, c.lenh, 0, lv1, c.F, c.prec, c.s));
  }
  y.transformed = 0;
  return WC_OK;
}

template <class T>
int loss(const Ctx<T>& c, const HalfVec<T>& ye, const HalfVec<T>& yo, const double* xn,
         double* terms, double* dsum, void* sum_scratch, double* m) {
  {
    LaunchTimer lt("cv_terms", c.s);
    cv_terms_kernel<T><<<grid_for(c.lenh), kThreads, 0, c.s>>>(ye.x(), yo.x(), xn, c.lenh, terms);
  }
  WC_TRY(after_launch("cv_terms_kernel"));
  WC_TRY(cv_sequential_sum(terms, c.lenh, dsum, sum_scratch, c.s));
  WC_CUDA(cudaMemcpyAsync(m, dsum, sizeof(double), cudaMemcpyDeviceToHost, c.s));
  WC_CUDA(cudaStreamSynchronize(c.s));
  return WC_OK;
}

// The golden-section search of CVT (thresh.cpp:249-320) in one cooperative
// launch: wec / woc are the transformed halves; returns the chosen threshold
// before the final rescale, the iteration count and the smallest relative
// loss margin.  Synchronous (the result comes back to the host).
template <class T>
int cv_search_fused(const Ctx<T>& c, const T* wec, const T* woc, const double* x, double t_univ,
                    double tol, double* t_out, int* iters, double* min_margin) {
  const int64_t lenh = c.lenh;
  const int J1 = c.J - 1;
  const int L = filter_len(c.F);
  const int64_t Cn = (lenh + 1023) / 1024;
  const int64_t ntop = lenh >> J1;
  auto al = [](size_t b) { return ((b + 255) / 256) * 256; };
  const size_t b_rec = al(sizeof(T) * (size_t)lenh), b_top = al(sizeof(T) * (size_t)ntop);
  const size_t b_bar = 16384;  // barrier words (grid_bar_words), the phase timer in the last 1 KB
  const size_t b_zero = al(sizeof(CvFusedState)) + b_bar + 4 * b_rec + 4 * b_top;
  const size_t need = b_zero + 4 * b_rec + al(sizeof(double) * (size_t)lenh) +
                      al(sizeof(double) * 2 * (size_t)Cn) + al(sizeof(int) * (size_t)Cn) +
                      al(sizeof(long long) * 3 * (size_t)Cn) +
                      al(sizeof(long long) * 48 * (size_t)Cn);
  char* base = static_cast<char*>(workspace(kSlotCvTerms, need));
  if (!base) return workspace_error();
  CvFusedArgs a{};
  size_t off = 0;
  a.st = reinterpret_cast<CvFusedState*>(base);
  off += al(sizeof(CvFusedState));
  a.bar = reinterpret_cast<unsigned int*>(base + off);
  off += b_bar;
  for (int k = 0; k < 4; k++, off += b_rec) a.rec[k] = base + off;
  for (int k = 0; k < 4; k++, off += b_top) a.top[k] = base + off;
  // off == b_zero: everything above starts at zero
  for (int h = 0; h < 2; h++)
    for (int k = 0; k < 2; k++, off += b_rec) a.tmp[h][k] = base + off;
  a.terms = reinterpret_cast<double*>(base + off);
  off += al(sizeof(double) * (size_t)lenh);
  a.chunk_s = reinterpret_cast<double*>(base + off);
  off += al(sizeof(double) * 2 * (size_t)Cn);
  a.chunk_e = reinterpret_cast<int*>(base + off);
  off += al(sizeof(int) * (size_t)Cn);
  a.chunk_q = reinterpret_cast<long long*>(base + off);
  off += al(sizeof(long long) * 3 * (size_t)Cn);
  a.sub_q = reinterpret_cast<long long*>(base + off);
  a.wcoef[0] = wec;
  a.wcoef[1] = woc;
  a.x = x;
  a.status = device_status_word();
  if (!a.status) return workspace_error();
  a.lenh = lenh;
  a.J1 = J1;
  a.minl = c.minl;
  a.maxl1 = c.maxl - 1;
  a.hardness = c.hardness;
  a.thr_on = range_ok(lenh, J1, c.minl, c.maxl - 1, L) ? 1 : 0;
  a.tol = tol;
  // Search start (thresh.cpp:249-260), in the reference's FP64 order.
  const double R = 0.61803399, C = 1. - R;
  const double ta = 0., tc = t_univ, tb = tc / 2.;
  CvFusedState st0{};
  st0.t0 = ta;
  st0.t2 = tb;
  st0.t1 = tb - C * (tb - ta);
  st0.t3 = tc;
  int dev = 0, sms = 1, coop = 0;
  WC_CUDA(cudaGetDevice(&dev));
  WC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  WC_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
  if (!coop) return fail(WC_ERR_UNSUPPORTED, "device without cooperative launch");
  // Dynamic shared memory: the exact replay's staging (1024 chunks'
  // candidate increments and binades; the first chunk's terms fit in it),
  // the MODWT tiles or the DWT coarse levels (two buffers of kCvCoarseMax).
  size_t smem = (c.prec == WC_F64_EXACT) ? (size_t)1024 * (3 * sizeof(long long) + sizeof(int)) : 0;
  const size_t vsize = (c.prec == WC_F32) ? 4 : 8;
  if (c.ttype == 1) {
    size_t gs = 0;
    WC_TRY(modwt_inv_groups(lenh, J1, c.F, c.prec, 0, a.grp, &a.ngroups, &gs));
    smem = std::max(smem, gs);
  } else {
    int lc = 0;
    while ((lenh >> lc) > kCvCoarseMax) lc++;
    a.dwt_lc = lc;
    if (lc <= J1 - 1) smem = std::max(smem, 2 * (size_t)kCvCoarseMax * vsize);
  }
  int per = 0;
  switch (c.prec) {
    case WC_F64_EXACT: per = cv_fused_occupancy_exact(c.F, c.ttype, smem); break;
    case WC_F64_FAST: per = cv_fused_occupancy_fast(c.F, c.ttype, smem); break;
    default: per = cv_fused_occupancy_f32(c.F, c.ttype, smem); break;
  }
  if (per < 1) return fail(WC_ERR_CUDA, "fused CV search: no resident CTA at %zu bytes", smem);
  const int grid = std::max(2, per * sms);
  if (sizeof(unsigned int) * grid_bar_words((unsigned)grid) > b_bar - 1024)
    return fail(WC_ERR_UNSUPPORTED, "fused CV search: grid of %d CTAs too large", grid);
  WC_CUDA(cudaMemsetAsync(base, 0, b_zero, c.s));
  // WAVECUDA_CV_TRACE=1: print the search's time per phase to stderr.
  static const bool trace_on = getenv("WAVECUDA_CV_TRACE") != nullptr;
  if (trace_on)
    a.trace = reinterpret_cast<unsigned long long*>(base + al(sizeof(CvFusedState)) + b_bar - 1024);
  WC_CUDA(cudaMemcpyAsync(a.st, &st0, sizeof(st0), cudaMemcpyHostToDevice, c.s));
  int r = WC_OK;
  switch (c.prec) {
    case WC_F64_EXACT: r = cv_fused_launch_exact(a, c.F, c.ttype, grid, smem, c.s); break;
    case WC_F64_FAST: r = cv_fused_launch_fast(a, c.F, c.ttype, grid, smem, c.s); break;
    default: r = cv_fused_launch_f32(a, c.F, c.ttype, grid, smem, c.s); break;
  }
  WC_TRY(r);
  CvFusedState st{};
  WC_CUDA(cudaMemcpyAsync(&st, a.st, sizeof(st), cudaMemcpyDeviceToHost, c.s));
  WC_CUDA(cudaStreamSynchronize(c.s));
  if (a.trace) {
    unsigned long long tr[kCvTraceSlots];
    WC_CUDA(cudaMemcpy(tr, a.trace, sizeof(tr), cudaMemcpyDeviceToHost));
    fprintf(stderr, "cv_fused_search phases (us, %d steps, grid %d, smem %zu):", st.iters + 2,
            grid, smem);
    for (int k = 0; k < kCvTraceSlots; k++)
      if (tr[k]) fprintf(stderr, " [%d] %.1f", k, tr[k] * 1e-3);
    fprintf(stderr, "\n");
  }
  *t_out = st.m1 < st.m2 ? st.t1 : st.t2;
  *iters = st.iters;
  *min_margin = st.min_margin;
  return WC_OK;
}

// Carves `count` buffers out of one workspace slot.
struct Carver {
  char* base;
  size_t off;
  template <class T>
  T* take(int64_t n) {
    T* p = reinterpret_cast<T*>(base + off);
    off += ((sizeof(T) * (size_t)n + 255) / 256) * 256;
    return p;
  }
};

template <class T>
int smooth_impl(double* x, int64_t n, int J, int ttype, int F, int threshtype, double* thresh,
                int hardness, int minl, int maxl, double tol, int prec, cudaStream_t s,
                wc_smooth_info* info) {
  const int L = filter_len(F);
  // Packet order (code 2) keeps its coefficients in time order here: the
  // thresholds, the universal threshold's MAD and the kept counts see the
  // same values; only the inverse differs (modwt_po_inverse_to).
  const bool po = (ttype == 2);
  if (po) ttype = 1;
  Ctx<T> c{n, n / 2, J, ttype, F, hardness, minl, maxl, prec, 0, s, po};
  const int64_t lenh = n / 2;
  const int64_t wlen = (ttype == 0) ? n : 2 * n * (int64_t)J;
  const int64_t hlen = (ttype == 0) ? lenh : 2 * lenh * (int64_t)std::max(J - 1, 1);

  // Workspace: full-length signal (T), full transform, and for CV the
  // half-length vectors.
  size_t need = 256 * 32 + sizeof(T) * (size_t)(n + wlen);
  if (threshtype == 2)
    need += sizeof(T) * (size_t)(2 * lenh + 2 * hlen + (po ? 4 * (2 * lenh + hlen) : 0));
  need += sizeof(double) * (size_t)wlen;  // FP64 copy of an FP32 transform (univ/counts)
  Carver cv{static_cast<char*>(workspace(kSlotCv, need)), 0};
  if (!cv.base) return workspace_error();
  T* xt = cv.take<T>(n);
  T* w = cv.take<T>(wlen);
  double* w64 = cv.take<double>(wlen);

  if constexpr (sizeof(T) == 8) {
    WC_CUDA(cudaMemcpyAsync(xt, x, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, s));
  } else {
    convert_kernel<double, T><<<grid_for(n), kThreads, 0, s>>>(x, xt, n);
    WC_TRY(after_launch("convert_kernel"));
  }
  auto as64 = [&](const T* v, int64_t cnt) -> const double* {
    if constexpr (sizeof(T) == 8) {
      return reinterpret_cast<const double*>(v);
    } else {
      convert_kernel<T, double><<<grid_for(cnt), kThreads, 0, s>>>(v, w64, cnt);
      return after_launch("convert_kernel") == WC_OK ? w64 : nullptr;
    }
  };

  double t = thresh ? *thresh : 0.0;
  double t_univ = 0.0, min_margin = INFINITY;
  int iters = 0;

  if (threshtype == 2) {
    if (!range_ok(n, J, minl, maxl, L) || J <= 1) {
      // thresh.cpp:223-231: CVT returns 0 and leaves x untouched.
      if (thresh) *thresh = 0.0;
      if (info) { *info = wc_smooth_info{}; info->levels = J; }
      return WC_OK;
    }
    const int lv1 = J - 1;
    T* we = cv.take<T>(lenh);
    T* wo = cv.take<T>(lenh);
    T* wec = cv.take<T>(hlen);
    T* woc = cv.take<T>(hlen);
    split_even_odd<T><<<grid_for(lenh), kThreads, 0, s>>>(x, lenh, we, wo);
    WC_TRY(after_launch("split_even_odd"));
    WC_TRY(transform_full(c, xt, w, n, J, 1));
    const double* wd = as64(w, wlen);
    if (!wd) return WC_ERR_CUDA;
    WC_TRY(univ_thresh(wd, n, J, ttype, minl, maxl, s, &t_univ));

    WC_TRY(transform_full(c, we, wec, lenh, lv1, 1));
    WC_TRY(transform_full(c, wo, woc, lenh, lv1, 1));
    if (!po) {
      WC_TRY(cv_search_fused<T>(c, wec, woc, x, t_univ, tol, &t, &iters, &min_margin));
    } else {
      HalfVec<T> y[4];
      for (int k = 0; k < 4; k++) {
        y[k].buf[0] = cv.take<T>(lenh);
        y[k].buf[1] = cv.take<T>(lenh);
        y[k].mod = cv.take<T>(hlen);
        y[k].cur = 0;
        y[k].transformed = 0;
      }
      // Zero the work vectors: the reference's are fresh zero-filled pages.
      WC_CUDA(cudaMemsetAsync(y[0].buf[0], 0,
                              (size_t)(reinterpret_cast<char*>(y[3].mod + hlen) -
                                       reinterpret_cast<char*>(y[0].buf[0])), s));
      const size_t tbytes = ((sizeof(double) * (size_t)(lenh + 64) + 255) / 256) * 256;
      char* tbase = static_cast<char*>(workspace(kSlotCvTerms, tbytes + cv_sum_scratch_bytes(lenh)));
      if (!tbase) return workspace_error();
      double* terms = reinterpret_cast<double*>(tbase);
      double* dsum = terms + lenh + 32;
      void* sscr = tbase + tbytes;
      const double R = 0.61803399, C = 1. - R;
      double ta = 0., tc = t_univ;
      double tb = tc / 2.;
      double t0 = ta, t2 = tb, t1 = tb - C * (tb - ta), t3 = tc;
      WC_TRY(half_step(c, wec, y[0], t1));
      WC_TRY(half_step(c, woc, y[1], t1));
      WC_TRY(half_step(c, wec, y[2], t2));
      WC_TRY(half_step(c, woc, y[3], t2));
      double m1, m2;
      WC_TRY(loss(c, y[0], y[1], x, terms, dsum, sscr, &m1));
      WC_TRY(loss(c, y[2], y[3], x, terms, dsum, sscr, &m2));
      while (fabs(t3 - t0) > tol * (t1 + t2)) {
        if (iters > 50) break;
        if (m1 != 0.0) min_margin = std::min(min_margin, fabs(m1 - m2) / fabs(m1));
        if (m2 < m1) {
          t0 = t1; t1 = t2; t2 = R * t2 + C * t3;
          m1 = m2;
          WC_TRY(half_step(c, wec, y[2], t2));
          WC_TRY(half_step(c, woc, y[3], t2));
          WC_TRY(loss(c, y[2], y[3], x, terms, dsum, sscr, &m2));
        } else {
          t3 = t2; t2 = t1; t1 = R * t1 + C * t0;
          m2 = m1;
          WC_TRY(half_step(c, wec, y[0], t1));
          WC_TRY(half_step(c, woc, y[1], t1));
          WC_TRY(loss(c, y[0], y[1], x, terms, dsum, sscr, &m1));
        }
        iters++;
      }
      t = m1 < m2 ? t1 : t2;
    }
    t = t / (sqrt(1. - log(2.) / log((double)n)));
  } else {
    WC_TRY(transform_full(c, xt, w, n, J, 1));
    if (threshtype == 1) {
      const double* wd = as64(w, wlen);
      if (!wd) return WC_ERR_CUDA;
      WC_TRY(univ_thresh(wd, n, J, ttype, 0, 0, s, &t_univ));
      t = t_univ;
    }
  }

  int64_t kept = 0, zeroed = 0;
  if (info && range_ok(n, J, minl, maxl, L)) {
    const double* wd = as64(w, wlen);
    if (!wd) return WC_ERR_CUDA;
    WC_TRY(count_kept(wd, n, J, ttype, t, minl, maxl, s, &kept, &zeroed));
  }
  // threshold(w, NULL, t, ...) silently does nothing on a bad level range
  // (thresh.cpp:114).
  if (range_ok(n, J, minl, maxl, L))
    WC_TRY(threshold_to<T>(w, w, n, J, ttype, t, hardness, minl, maxl, 0, s));
  WC_TRY(transform_full(c, xt, w, n, J, 0));
  if constexpr (sizeof(T) == 8) {
    WC_CUDA(cudaMemcpyAsync(x, xt, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, s));
  } else {
    convert_kernel<T, double><<<grid_for(n), kThreads, 0, s>>>(xt, x, n);
    WC_TRY(after_launch("convert_kernel"));
  }
  if (thresh && threshtype != 0) *thresh = t;
  if (info) {
    info->thresh = t;
    info->thresh_univ = t_univ;
    info->cv_iterations = iters;
    info->levels = J;
    info->kept = kept;
    info->zeroed = zeroed;
    info->min_margin = (threshtype == 2 && min_margin != INFINITY) ? min_margin : 0.0;
  }
  return WC_OK;
}

}  // namespace

int smooth(double* x, int64_t n, int J, int ttype, int F, int threshtype, double* thresh,
           int hardness, int minl, int maxl, double tol, int prec, cudaStream_t s,
           wc_smooth_info* info) {
  if (prec == WC_F32)
    return smooth_impl<float>(x, n, J, ttype, F, threshtype, thresh, hardness, minl, maxl, tol,
                              prec, s, info);
  return smooth_impl<double>(x, n, J, ttype, F, threshtype, thresh, hardness, minl, maxl, tol,
                             prec, s, info);
}

}  // namespace wc
