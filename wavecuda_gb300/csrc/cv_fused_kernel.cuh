// Fused two-fold cross-validation search (CVT, thresh.cpp:203-342) for one
// signal: the whole golden-section loop runs in one persistent cooperative
// launch, with no host round trip between steps.
//
// Before the launch the host splits the signal into its even and odd halves,
// transforms both (J1 = J - 1 levels) and computes the universal threshold
// that bounds the search.  Inside the kernel every CTA keeps its own copy of
// the search state (t0..t3, m1, m2), updated with the same FP64 operations
// in the same order from the same loss values, so all CTAs take the same
// branch without exchanging anything but the loss.  One golden step is:
//
//  1. threshold and inverse transform of both halves for the new candidate,
//     the threshold fused into the inverse (each coefficient is thresholded
//     once, as it is staged), level group by level group with a grid-wide
//     barrier between groups:
//       MODWT  row-view tiles of up to three levels (modwt_inv_tile);
//       DWT    the coarse levels (at most kCvCoarseMax outputs) in one CTA per
//              half, then one grid-wide pass per finer level;
//  2. the interpolation loss terms of interp_mse (thresh.cpp:344-385) and
//     their per-chunk FP64 sums; CTA 0 also replays the first chunk, which
//     depends on nothing else (exact FP64; the other precisions add the
//     chunk sums in a fixed order in every CTA and stop here);
//  3. per chunk, the binade of the running sum at its start (from the FP64
//     prefix of the chunk sums) and the integer increments of the chunk and
//     of its 64-term sub-chunks for the three candidate binades
//     (wc_seqsum.cuh);
//  4. one warp of CTA 0 replays the reference's left-to-right FP64 sum
//     exactly (walking the chunks, replaying only sub-chunks with a binade
//     crossing or a tie); every CTA reads the loss after the next barrier.
//
// Quirks kept (they change results): DWT work vectors keep the previous
// reconstruction in their coarse scaling slots k 2^J1, k > 0, because
// threshold_dwt into a separate vector never writes them (thresh.cpp:15-35);
// here the inverse reads those slots from a compact copy of the previous
// reconstruction (top[]), and slot 0 from the coefficients.  When the half
// level range is invalid nothing is thresholded or inverted and the
// reconstructions stay zero (transform.cpp:5-8).  At most 51 iterations.
#pragma once

#include <math.h>

#include "wc_cvfused.h"
#include "wc_dwt_math.cuh"
#include "wc_grid.cuh"
#include "wc_modwt_math.cuh"
#include "wc_seqsum.cuh"

namespace wc {
namespace {

constexpr int kCvThreads = 256;
constexpr int kCvSeg = 1024;  // chunks staged in shared memory by the replaying CTA

// Dynamic shared memory the replay and the loss phase need (bytes): a
// segment's candidate increments and binades, or the first chunk's terms.
constexpr size_t kCvSeqSmem = (size_t)kCvSeg * (3 * sizeof(long long) + sizeof(int));

// thresh_coef (thresh.cpp:142-157) on an FP64 value, bit-identical to
// `fabs(c) < t ? 0 : soft ? sign(c) * (fabs(c) - t) : c` with IEEE roundings:
// for t >= +0 and non-NaN c the comparison of magnitudes is the unsigned
// comparison of the bit patterns, and the product with -1 or 1 is a sign
// flip, so only the subtraction needs the FP64 unit.
__device__ __forceinline__ double cv_thresh(double c, double t, int hardness) {
  const unsigned long long cb = (unsigned long long)__double_as_longlong(c);
  const unsigned long long tb = (unsigned long long)__double_as_longlong(t);
  const unsigned long long mag = cb & 0x7FFFFFFFFFFFFFFFull;
  bool small;
  if ((long long)tb >= 0 && mag <= 0x7FF0000000000000ull) small = mag < tb;
  else small = fabs(c) < t;
  if (small) return 0.0;
  if (hardness != 1) return c;
  const double r = __dsub_rn(__longlong_as_double((long long)mag), t);
  const bool neg = (cb >> 63) && mag != 0;
  return neg ? __longlong_as_double(__double_as_longlong(r) ^ (long long)0x8000000000000000ull)
             : r;
}
__device__ __forceinline__ float cv_thresh(float c, float t, int hardness) {
  if (fabsf(c) < t) return 0.f;
  if (hardness == 1) return ((c < 0) ? -1.0f : 1.0f) * (fabsf(c) - t);
  return c;
}
// Double-float threshold (WC_F64_FAST): the same rule on (hi, lo) pairs.
__device__ __forceinline__ dd cv_thresh(dd c, dd t, int hardness) {
  const bool neg = c.hi < 0.f || (c.hi == 0.f && c.lo < 0.f);
  const dd m = neg ? dd{-c.hi, -c.lo} : c;
  if (m.hi < t.hi || (m.hi == t.hi && m.lo < t.lo)) return dd{0.f, 0.f};
  if (hardness != 1) return c;
  const dd r = PDD::sub(m, t);
  return neg ? dd{-r.hi, -r.lo} : r;
}

template <class P>
__device__ __forceinline__ typename P::V cv_tval(double t) {
  if constexpr (std::is_same<P, PDD>::value) return dd_from_double(t);
  else return (typename P::V)t;
}

// Thresholds the staged detail values of levels [minl, maxl] (MODWT tiles).
template <class P>
struct CvDMap {
  static constexpr bool kIdentity = false;
  typename P::V t;
  int minl, maxl, hardness;
  __device__ __forceinline__ typename P::V operator()(typename P::V v, int level) const {
    if (level < minl || level > maxl) return v;
    return cv_thresh(v, t, hardness);
  }
};

// Loss term j of interp_mse (thresh.cpp:363-382) with the reference's
// roundings: (yie - xn[2j])^2 + (yio - xn[2j+1])^2, where the interpolants
// average neighbouring values of the other half (ends special-cased).
template <class T>
__device__ __forceinline__ double cv_term(const T* __restrict__ ye, const T* __restrict__ yo,
                                          const double* __restrict__ xn, int64_t lenh, int64_t j) {
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
  return __dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b));
}

// Inclusive prefix sum of a double over the CTA (an estimate: any order).
__device__ __forceinline__ double cv_block_scan_d(double x, double* wt) {
  const int l = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    const double y = __shfl_up_sync(0xffffffffu, x, o);
    if (l >= o) x += y;
  }
  if (l == 31) wt[w] = x;
  __syncthreads();
  if (w == 0) {
    double t = (l < nw) ? wt[l] : 0.0;
    for (int o = 1; o < 32; o <<= 1) {
      const double y = __shfl_up_sync(0xffffffffu, t, o);
      if (l >= o) t += y;
    }
    wt[l] = t;
  }
  __syncthreads();
  const double r = x + (w > 0 ? wt[w - 1] : 0.0);
  __syncthreads();
  return r;
}

template <int F, class P, int TT>
__global__ void __launch_bounds__(kCvThreads, 3) cv_fused_kernel(const CvFusedArgs a) {
  using T = typename P::T;
  using V = typename P::V;
  constexpr int HH = filter_len(F) / 2;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ long long s_sub[kSeqSubs * 3];
  __shared__ double s_wd[32];
  __shared__ unsigned long long s_m0;

  unsigned int gen = 0;
  const unsigned int nb = gridDim.x;
  const int64_t lenh = a.lenh;
  const int J1 = a.J1;
  // phase timer (CTA 0, thread 0)
  const bool tracing = a.trace != nullptr && blockIdx.x == 0 && threadIdx.x == 0;
  unsigned long long t_last = 0, t_acc[kCvTraceSlots];
  if (tracing) {
    for (int k = 0; k < kCvTraceSlots; k++) t_acc[k] = 0;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_last));
  }
  auto mark = [&](int slot) {
    if (tracing) {
      unsigned long long t;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
      t_acc[slot] += t - t_last;
      t_last = t;
    }
  };

  // ---- 1. thresholded inverse transforms of both halves -------------------
  auto dwt_step = [&](double t, int pair) -> bool {
    PairTaps<F, P> tp;  // synthesis taps of the packed double-float products
    tp.init();
    const T tT = (T)t;
    auto det = [&](int h, int l0, int64_t k) -> V {
      T c = static_cast<const T*>(a.wcoef[h])[((int64_t)1 << l0) + (k << (l0 + 1))];
      if (l0 >= a.minl && l0 <= a.maxl1) c = cv_thresh(c, tT, a.hardness);
      return P::ld(c);
    };
    auto topv = [&](int h, int64_t k) -> V {
      if (k == 0) return P::ld(static_cast<const T*>(a.wcoef[h])[0]);
      return P::ld(static_cast<const T*>(a.top[2 * pair + h])[k]);
    };
    int cur = 0;
    bool from_top = true;
    const int lc = a.dwt_lc;
    if (lc <= J1 - 1) {
      if (blockIdx.x < 2) {
        const int h = blockIdx.x;
        V* sA = reinterpret_cast<V*>(smem);
        V* sB = sA + kCvCoarseMax;
        const int64_t n0 = lenh >> J1;
        for (int64_t k = threadIdx.x; k < n0; k += blockDim.x) sA[k] = topv(h, k);
        __syncthreads();
        for (int l0 = J1 - 1; l0 >= lc; l0--) {
          const int64_t Pl = lenh >> (l0 + 1);
          for (int64_t q = threadIdx.x; q < Pl; q += blockDim.x) {
            V sv[HH], dv[HH];
#pragma unroll
            for (int j = 0; j < HH; j++) {
              const int64_t k = (q - j) & (Pl - 1);
              sv[j] = sA[k];
              dv[j] = det(h, l0, k);
            }
            V e, o;
            inv_pair<F, P>(sv, dv, e, o, tp);
            sB[2 * q] = e;
            sB[2 * q + 1] = o;
          }
          __syncthreads();
          V* tsw = sA;
          sA = sB;
          sB = tsw;
        }
        T* dst = (lc == 0) ? static_cast<T*>(a.rec[2 * pair + h]) : static_cast<T*>(a.tmp[h][0]);
        const int64_t nout = lenh >> lc;
        for (int64_t k = threadIdx.x; k < nout; k += blockDim.x) dst[k] = P::st(sA[k]);
      }
      if (!grid_sync(a.bar, nb, gen, a.status)) return false;
      mark(0);
      from_top = false;
    }
    const int lstart = (lc < J1 ? lc : J1) - 1;
    for (int l0 = lstart; l0 >= 0; l0--) {
      const int64_t Pl = lenh >> (l0 + 1);
      const int64_t stride = (int64_t)gridDim.x * blockDim.x;
      for (int64_t it = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; it < 2 * Pl; it += stride) {
        const int h = it >= Pl ? 1 : 0;
        const int64_t q = it - h * Pl;
        const T* src = static_cast<const T*>(a.tmp[h][cur]);
        V sv[HH], dv[HH];
#pragma unroll
        for (int j = 0; j < HH; j++) {
          const int64_t k = (q - j) & (Pl - 1);
          sv[j] = from_top ? topv(h, k) : P::ld(src[k]);
          dv[j] = det(h, l0, k);
        }
        V e, o;
        inv_pair<F, P>(sv, dv, e, o, tp);
        T* dst = (l0 == 0) ? static_cast<T*>(a.rec[2 * pair + h]) : static_cast<T*>(a.tmp[h][cur ^ 1]);
        dst[2 * q] = P::st(e);
        dst[2 * q + 1] = P::st(o);
      }
      if (!grid_sync(a.bar, nb, gen, a.status)) return false;
      mark(1 + (l0 < kCvMaxGroups - 2 ? l0 : kCvMaxGroups - 2));
      cur ^= 1;
      from_top = false;
    }
    return true;
  };

  auto modwt_step = [&](double t, int pair) -> bool {
    CvDMap<P> dm;
    dm.t = cv_tval<P>(t);
    dm.minl = a.minl;
    dm.maxl = a.maxl1;
    dm.hardness = a.hardness;
    for (int g = 0; g < a.ngroups; g++) {
      const CvModGroup G = a.grp[g];
      for (int64_t tile = blockIdx.x; tile < 2 * G.ntiles; tile += gridDim.x) {
        const int h = tile >= G.ntiles ? 1 : 0;
        const int64_t tl = tile - h * G.ntiles;
        const T* w = static_cast<const T*>(a.wcoef[h]);
        const T* Stop = (g == 0) ? w + (int64_t)2 * (J1 - 1) * lenh
                                 : static_cast<const T*>(a.tmp[h][(g - 1) & 1]);
        T* out = (G.l0 == 0) ? static_cast<T*>(a.rec[2 * pair + h])
                             : static_cast<T*>(a.tmp[h][g & 1]);
        if (G.ni == 1) {
          modwt_inv_tile<F, P, 1>(tl, Stop, w, out, lenh, G.l0, G.C, G.M, smem, dm);
        } else if (G.ni == 2) {
          modwt_inv_tile<F, P, 2>(tl, Stop, w, out, lenh, G.l0, G.C, G.M, smem, dm);
        } else {
          if constexpr (F == 1) modwt_inv_tile<F, P, 3>(tl, Stop, w, out, lenh, G.l0, G.C, G.M, smem, dm);
        }
        __syncthreads();
      }
      if (!grid_sync(a.bar, nb, gen, a.status)) return false;
      mark(g);
    }
    return true;
  };

  auto step = [&](double t, int pair) -> bool {
    if (!a.thr_on) return true;  // the reference never inverts: reconstructions stay zero
    if constexpr (TT == 0) return dwt_step(t, pair);
    else return modwt_step(t, pair);
  };

  // ---- 2-4. loss of a pair of reconstructions ----------------------------
  int evals = 0;  // loss evaluations so far (parity of the chunk-sum buffer)
  auto loss = [&](int pair, double& m) -> bool {
    const T* ye = static_cast<const T*>(a.rec[2 * pair]);
    const T* yo = static_cast<const T*>(a.rec[2 * pair + 1]);
    const int64_t Cn = (lenh + kSeqChunk - 1) / kSeqChunk;
    if constexpr (!std::is_same<P, PExact>::value) {
      // Double-float and FP32 reconstructions already differ from the
      // reference's, so their loss needs no serial replay: FP64 chunk sums
      // in a fixed order, then every CTA adds the chunk sums in the same
      // fixed order and gets the same loss, with one barrier.  The two
      // chunk-sum buffers alternate, so a CTA still reading the previous
      // loss's sums never sees them overwritten.
      double* cs = a.chunk_s + (int64_t)(evals & 1) * Cn;
      evals++;
      for (int64_t c = blockIdx.x; c < Cn; c += gridDim.x) {
        const int64_t base = c * kSeqChunk;
        const int len = (int)(lenh - base < kSeqChunk ? lenh - base : kSeqChunk);
        double acc = 0.0;
        for (int k = threadIdx.x; k < len; k += blockDim.x) acc += cv_term(ye, yo, a.x, lenh, base + k);
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if ((threadIdx.x & 31) == 0) s_wd[threadIdx.x >> 5] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
          double t = 0.0;
          for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += s_wd[w];
          cs[c] = t;
        }
        __syncthreads();
      }
      if constexpr (TT == 0) {
        // the coarse slots of this pair's reconstructions, for its next step
        const int64_t ns = lenh >> J1;
        const int64_t stride = (int64_t)gridDim.x * blockDim.x;
        for (int64_t it = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; it < 2 * ns; it += stride) {
          const int h = it >= ns ? 1 : 0;
          const int64_t k = it - h * ns;
          static_cast<T*>(a.top[2 * pair + h])[k] =
              static_cast<const T*>(a.rec[2 * pair + h])[k << J1];
        }
      }
      if (!grid_sync(a.bar, nb, gen, a.status)) return false;
      mark(kCvTraceTerms);
      double acc = 0.0;
      for (int64_t c = threadIdx.x; c < Cn; c += blockDim.x) acc += cs[c];
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
      if ((threadIdx.x & 31) == 0) s_wd[threadIdx.x >> 5] = acc;
      __syncthreads();
      double tot = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); w++) tot += s_wd[w];
      __syncthreads();
      m = __dmul_rn(tot, 0.5);
      return true;
    }
    // (2) the terms and per-chunk FP64 sums
    double* s_chunk0 = reinterpret_cast<double*>(smem);  // CTA 0: the first chunk's terms
    for (int64_t c = blockIdx.x; c < Cn; c += gridDim.x) {
      const int64_t base = c * kSeqChunk;
      const int len = (int)(lenh - base < kSeqChunk ? lenh - base : kSeqChunk);
      double acc = 0.0;
      for (int k = threadIdx.x; k < len; k += blockDim.x) {
        const double v = cv_term(ye, yo, a.x, lenh, base + k);
        a.terms[base + k] = v;
        if (c == 0) s_chunk0[k] = v;
        acc += v;
      }
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
      if ((threadIdx.x & 31) == 0) s_wd[threadIdx.x >> 5] = acc;
      __syncthreads();
      if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += s_wd[w];
        a.chunk_s[c] = t;
      }
      __syncthreads();
    }
    if (blockIdx.x == 0) {
      // The first chunk starts from m = 0 and crosses many binades; it needs
      // nothing from the other chunks, so CTA 0 replays it now (from shared
      // memory), while the other CTAs compute their terms.
      if (threadIdx.x < 32) {
        unsigned long long mb = 0ull;
        const int len0 = (int)(lenh < kSeqChunk ? lenh : kSeqChunk);
        seq_replay_chunk_warp(s_chunk0, len0, nullptr, 0, mb);
        if (threadIdx.x == 0) s_m0 = mb;
      }
      __syncthreads();
    }
    if constexpr (TT == 0) {
      // the coarse slots of this pair's reconstructions, for its next step
      const int64_t ns = lenh >> J1;
      const int64_t stride = (int64_t)gridDim.x * blockDim.x;
      for (int64_t it = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; it < 2 * ns; it += stride) {
        const int h = it >= ns ? 1 : 0;
        const int64_t k = it - h * ns;
        static_cast<T*>(a.top[2 * pair + h])[k] =
            static_cast<const T*>(a.rec[2 * pair + h])[k << J1];
      }
    }
    if (!grid_sync(a.bar, nb, gen, a.status)) return false;
    mark(kCvTraceTerms);
    // (3) binade estimates of this CTA's chunks (FP64 prefix of the chunk
    //     sums), then their and their sub-chunks' increments for the three
    //     candidate binades
    double carry = 0.0;
    for (int64_t s0 = 0; s0 < Cn; s0 += blockDim.x) {
      const int64_t c = s0 + threadIdx.x;
      const double v = (c < Cn) ? a.chunk_s[c] : 0.0;
      const double incl = cv_block_scan_d(v, s_wd);
      const double excl = carry + (incl - v);
      if (c < Cn && (c % gridDim.x) == blockIdx.x)
        a.chunk_e[c] = (int)(((unsigned long long)__double_as_longlong(excl) >> 52) & 0x7FF);
      if ((int)threadIdx.x == (int)blockDim.x - 1) s_wd[0] = incl;  // the segment's total
      __syncthreads();
      carry += s_wd[0];
      __syncthreads();
    }
    for (int64_t c = blockIdx.x; c < Cn; c += gridDim.x) {
      const int64_t base = c * kSeqChunk;
      const int len = (int)(lenh - base < kSeqChunk ? lenh - base : kSeqChunk);
      seq_chunk_q_subs(a.terms, base, len, a.chunk_e[c], s_sub, a.sub_q + 3 * kSeqSubs * c,
                       a.chunk_q + 3 * c);
    }
    if (!grid_sync(a.bar, nb, gen, a.status)) return false;
    mark(kCvTraceQ);
    // (4) CTA 0: one warp walks the chunks (staged in shared memory a segment
    //     at a time) and replays, sub-chunk by sub-chunk, those it cannot pass
    //     (reading that chunk's sub-chunk increments and the terms of the
    //     sub-chunks it replays straight from global memory: one round trip
    //     each instead of staging the whole chunk)
    if (blockIdx.x == 0) {
      long long* sQ = reinterpret_cast<long long*>(smem);
      int* sE = reinterpret_cast<int*>(sQ + 3 * kCvSeg);
      unsigned long long mb = s_m0;
      for (int64_t seg = 0; seg < Cn; seg += kCvSeg) {
        const int64_t segend = (seg + kCvSeg < Cn) ? seg + kCvSeg : Cn;
        for (int64_t i = threadIdx.x; i < (segend - seg) * 3; i += blockDim.x)
          sQ[i] = a.chunk_q[seg * 3 + i];
        for (int64_t i = threadIdx.x; i < segend - seg; i += blockDim.x) sE[i] = a.chunk_e[seg + i];
        __syncthreads();
        if (threadIdx.x < 32) {
          int64_t c = (seg == 0) ? 1 : seg;  // chunk 0 was replayed with the terms
          while (c < segend) {
            c = seq_walk(sQ, sE, seg, c, segend, mb);
            if (c >= segend) break;
            const int64_t base = c * kSeqChunk;
            const int len = (int)(lenh - base < kSeqChunk ? lenh - base : kSeqChunk);
            seq_replay_chunk_warp<SeqLdGlobal>(a.terms + base, len, a.sub_q + 3 * kSeqSubs * c,
                                               sE[c - seg], mb);
            c++;
          }
        }
        __syncthreads();
      }
      if (threadIdx.x == 0) a.st->m_new = __dmul_rn(__longlong_as_double((long long)mb), 0.5);
    }
    if (!grid_sync(a.bar, nb, gen, a.status)) return false;
    mark(kCvTraceReplay);
    m = *reinterpret_cast<volatile double*>(&a.st->m_new);
    return true;
  };

  // ---- the golden-section search (thresh.cpp:283-320) --------------------
  const double R = 0.61803399, C = __dsub_rn(1., R);
  double t0 = a.st->t0, t1 = a.st->t1, t2 = a.st->t2, t3 = a.st->t3;
  double m1 = 0.0, m2 = 0.0, mm = INFINITY;
  int iters = 0;
  if (!step(t1, 0) || !loss(0, m1)) return;
  if (!step(t2, 1) || !loss(1, m2)) return;
  while (fabs(__dsub_rn(t3, t0)) > __dmul_rn(a.tol, __dadd_rn(t1, t2))) {
    if (iters > 50) break;
    if (m1 != 0.0) {
      const double mg = __ddiv_rn(fabs(__dsub_rn(m1, m2)), fabs(m1));
      if (mg < mm) mm = mg;
    }
    if (m2 < m1) {
      t0 = t1;
      t1 = t2;
      t2 = __dadd_rn(__dmul_rn(R, t2), __dmul_rn(C, t3));
      m1 = m2;
      if (!step(t2, 1) || !loss(1, m2)) return;
    } else {
      t3 = t2;
      t2 = t1;
      t1 = __dadd_rn(__dmul_rn(R, t1), __dmul_rn(C, t0));
      m2 = m1;
      if (!step(t1, 0) || !loss(0, m1)) return;
    }
    iters++;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.st->t0 = t0;
    a.st->t1 = t1;
    a.st->t2 = t2;
    a.st->t3 = t3;
    a.st->m1 = m1;
    a.st->m2 = m2;
    a.st->min_margin = mm;
    a.st->iters = iters;
  }
  if (tracing)
    for (int k = 0; k < kCvTraceSlots; k++) atomicAdd(a.trace + k, t_acc[k]);
}

template <class P>
void* cv_fused_kernel_ptr(int F, int ttype) {
  switch (F * 2 + ttype) {
    case 2: return (void*)cv_fused_kernel<1, P, 0>;
    case 3: return (void*)cv_fused_kernel<1, P, 1>;
    case 4: return (void*)cv_fused_kernel<2, P, 0>;
    case 5: return (void*)cv_fused_kernel<2, P, 1>;
    case 6: return (void*)cv_fused_kernel<3, P, 0>;
    case 7: return (void*)cv_fused_kernel<3, P, 1>;
    case 8: return (void*)cv_fused_kernel<4, P, 0>;
    case 9: return (void*)cv_fused_kernel<4, P, 1>;
  }
  return nullptr;
}

template <class P>
int cv_fused_launch_p(const CvFusedArgs& a, int F, int ttype, int grid, size_t smem,
                      cudaStream_t s) {
  void* kern = cv_fused_kernel_ptr<P>(F, ttype);
  if (!kern) return fail(WC_ERR_ARG, "fused CV: filter %d / transform %d", F, ttype);
  WC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  CvFusedArgs args = a;
  void* params[] = {&args};
  {
    LaunchTimer lt("cv_fused_search", s);
    WC_CUDA(cudaLaunchCooperativeKernel(kern, dim3(grid), dim3(kCvThreads), params, smem, s));
  }
  return after_launch("cv_fused_kernel");
}

template <class P>
int cv_fused_occupancy_p(int F, int ttype, size_t smem) {
  void* kern = cv_fused_kernel_ptr<P>(F, ttype);
  if (!kern) return 0;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  int per = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, kCvThreads, smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return per;
}

}  // namespace
}  // namespace wc
