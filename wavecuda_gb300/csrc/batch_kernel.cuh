#pragma once
// Batched smoothing kernel: thousands of signals of uneven length, filter, transform
// and level count in one persistent launch.
//
// Each CTA pulls a signal index from a device work queue (atomic counter over
// a host-sorted order, largest work first) and runs that signal's whole
// smoothing pipeline -- forward transform, universal or two-fold CV threshold
// (the reference's CVT, thresh.cpp:203-342, including its device-side
// golden-section search), final threshold and inverse -- with block-level
// code, so no host round trip or extra launch happens per signal or per CV
// iteration.  The pipeline and its quirks are those of smooth.cu; the
// differences are structural:
//  * thresholding is fused into the inverse transforms (the coefficient is
//    thresholded as it is read), so the thresholded copies the reference
//    builds (y1e->x, y1e->xmod) are never written;
//  * the MODWT keeps only d_1..d_J and s_J (what the inverse reads);
//  * log/sqrt constants come from the host's libm (per signal), so the
//    device's threshold arithmetic reproduces the reference's doubles.
// A CTA's scratch is a private slice of one workspace allocation, sized for
// the largest signal of the batch.
#include <math.h>

#include <algorithm>
#include <type_traits>
#include <vector>

#include "wc_batch.h"
#include "wc_bulk.cuh"
#include "wc_common.cuh"
#include "wc_dd.cuh"
#include "wc_grid.cuh"
#include "wc_modwt_vec.cuh"
#include "wc_taps2.cuh"

namespace wc {
namespace {

// (g_k, h_k) tap pairs of the packed double-float MODWT forward level
// (wc_taps2.cuh).
struct BatchModwtTaps {
  TapPairF p[8];
};
constexpr BatchModwtTaps batch_modwt_taps(int F) {
  BatchModwtTaps t{};
  for (int k = 0; k < filter_len(F); k++) t.p[k] = tap_pair_f(tap_g(F, k), tap_h(F, k));
  return t;
}
__constant__ BatchModwtTaps kBatchModwtTaps[5] = {BatchModwtTaps{}, batch_modwt_taps(1),
                                                  batch_modwt_taps(2), batch_modwt_taps(3),
                                                  batch_modwt_taps(4)};

constexpr int BT = 512;               // threads per CTA
constexpr uint64_t kFrac = (1ull << 52) - 1;

// ------------------------------------------------------------ values ----

template <class P>
struct Ops {
  using T = typename P::T;
  using V = typename P::V;
  static __device__ __forceinline__ V load(const T& x) { return P::ld(x); }
};

template <class P, class S>
__device__ __forceinline__ typename P::V rd(const S* p, int64_t i) {
  if constexpr (std::is_same<S, typename P::V>::value) return p[i];
  else return P::ld(p[i]);
}

// Threshold in the value domain.  Exact: thresh_coef (thresh.cpp:142-157) in
// FP64.  FP32: the same in float.  Double-float: |c| < t compared on the
// normalised pair, soft shrink by a double-float subtraction.
template <class P>
struct Th {
  typename P::V t;
  int hardness, minl, maxl;
};

__device__ __forceinline__ double thr(double c, double t, int hard) {
  if (fabs(c) < t) return 0.0;
  if (hard == 1) return __dmul_rn((c < 0) ? -1.0 : 1.0, __dsub_rn(fabs(c), t));
  return c;
}
__device__ __forceinline__ float thr(float c, float t, int hard) {
  if (fabsf(c) < t) return 0.f;
  if (hard == 1) return ((c < 0) ? -1.f : 1.f) * (fabsf(c) - t);
  return c;
}
__device__ __forceinline__ dd thr(dd c, dd t, int hard) {
  dd a = c;
  const bool neg = (c.hi < 0.f) || (c.hi == 0.f && c.lo < 0.f);
  if (neg) a = {-c.hi, -c.lo};
  const bool below = (a.hi < t.hi) || (a.hi == t.hi && a.lo < t.lo);
  if (below) return {0.f, 0.f};
  if (hard == 1) {
    dd r = PDD::sub(a, t);
    return neg ? dd{-r.hi, -r.lo} : r;
  }
  return c;
}

template <class P>
__device__ __forceinline__ typename P::V thr_v(typename P::V c, const Th<P>& th, int l) {
  if (l < th.minl || l > th.maxl) return c;
  return thr(c, th.t, th.hardness);
}

// One soft threshold per level (levels [minl, maxl]); the threshold tuner
// keeps it in shared memory.
constexpr int kLvMax = 24;  // = kFitLevels
template <class P>
struct ThL {
  typename P::V t[kLvMax];
  int minl, maxl;
};

template <class P>
__device__ __forceinline__ typename P::V thr_v(typename P::V c, const ThL<P>& th, int l) {
  if (l < th.minl || l > th.maxl) return c;
  return thr(c, th.t[l], 1);
}

template <class P>
__device__ __forceinline__ typename P::V to_v(double x) {
  if constexpr (std::is_same<typename P::V, dd>::value) return dd_from_double(x);
  else return (typename P::V)x;
}

template <class V>
__device__ __forceinline__ double to_d(V v) {
  if constexpr (std::is_same<V, dd>::value) return dd_to_double(v);
  else return (double)v;
}

// Outputs per thread per sweep of the block-level transform loops: the taps of
// U outputs are loaded before any is combined, so that U * L independent
// loads are in flight per thread (the sequences live in global memory).
// Full sweeps of U outputs carry no bounds checks; the remainder runs one
// output at a time.  FP32 takes 4 outputs; the 8-byte value types (FP64,
// double-float) are arithmetic-bound and keep one (measured: two outputs
// per thread slowed the double-float batch by 30 %).
template <class V>
constexpr int mod_unroll() {
  return sizeof(V) == 4 ? 4 : 1;
}

template <int U, class Fn>
__device__ __forceinline__ void sweep_outputs(int64_t N, Fn fn) {
  const int64_t B = blockDim.x, step = U * B, full = (N / step) * step;
  int64_t i0 = threadIdx.x;
  for (; i0 < full; i0 += step) fn(std::integral_constant<int, U>{}, i0);
  for (; i0 < N; i0 += B) fn(std::integral_constant<int, 1>{}, i0);
}

// ------------------------------------------------------- DWT (block) ----

// Forward DWT of y (compact, N values, type S) into the interleaved T array
// `out`; tA/tB hold N/2 values each.
template <int F, class P, class S>
__device__ void bdwt_fwd(const S* y, typename P::T* out, int64_t N, int J, typename P::V* tA,
                         typename P::V* tB) {
  using V = typename P::V;
  constexpr int L = filter_len(F);
  int64_t Nl = N;
  for (int l = 0; l < J; l++) {
    V* dst = (l & 1) ? tB : tA;
    const int64_t Pq = Nl >> 1, step = (int64_t)2 << l, off = (int64_t)1 << l;
    for (int64_t q = threadIdx.x; q < Pq; q += blockDim.x) {
      V s, d;
      if constexpr (F == 1) {
        const V a = (l == 0) ? rd<P>(y, 2 * q) : ((l & 1) ? tA : tB)[2 * q];
        const V b = (l == 0) ? rd<P>(y, 2 * q + 1) : ((l & 1) ? tA : tB)[2 * q + 1];
        s = haar_sum<P>(a, b);
        d = haar_dif<P>(a, b);
      } else {
        V v[L];
#pragma unroll
        for (int j = 0; j < L; j++) {
          const int64_t idx = (2 * q + j) & (Nl - 1);
          v[j] = (l == 0) ? rd<P>(y, idx) : ((l & 1) ? tA : tB)[idx];
        }
        typename P::Acc as = P::acc_init(v[0], tap_h(F, 0));
        typename P::Acc ad = P::acc_init(v[0], tap_g(F, 0));
#pragma unroll
        for (int j = 1; j < L; j++) {
          as = P::acc_add(as, v[j], tap_h(F, j));
          ad = P::acc_add(ad, v[j], tap_g(F, j));
        }
        s = P::acc_fin(as);
        d = P::acc_fin(ad);
      }
      dst[q] = s;
      out[off + q * step] = P::st(d);
    }
    __syncthreads();
    Nl = Pq;
  }
  const typename P::V* src = ((J - 1) & 1) ? tB : tA;
  for (int64_t q = threadIdx.x; q < Nl; q += blockDim.x) out[q << J] = P::st(src[q]);
  __syncthreads();
}

// Inverse DWT of the interleaved coefficients w into `out` (compact, N
// values, type D), with the details of levels in th's range thresholded as
// they are read.  The coarse scaling slots q*2^J, q > 0, are read from
// `coarse` (the reference's stale slots, thresh.cpp:15-35) or from w when
// coarse == nullptr; slot 0 always from w.
template <int F, class P, class D, class TH>
__device__ void bdwt_inv(const typename P::T* w, const D* coarse, D* out, int64_t N, int J,
                         const TH& th, typename P::V* tA, typename P::V* tB) {
  using V = typename P::V;
  constexpr int L = filter_len(F);
  constexpr int H = L / 2;
  int64_t Nl = N >> J;
  V* top = ((J - 1) & 1) ? tB : tA;  // level J compact buffer
  for (int64_t q = threadIdx.x; q < Nl; q += blockDim.x) {
    if (q == 0 || coarse == nullptr) top[q] = P::ld(w[q << J]);
    else top[q] = rd<P>(coarse, q << J);
  }
  __syncthreads();
  for (int l = J - 1; l >= 0; l--) {
    const V* s = (l & 1) ? tB : tA;   // level l+1 values (Nl of them)
    V* dstv = (l & 1) ? tA : tB;
    const int64_t off = (int64_t)1 << l, step = (int64_t)2 << l;
    const int64_t B = blockDim.x;
    sweep_outputs<mod_unroll<V>()>(Nl, [&](auto uc, int64_t q0) {
      constexpr int UU = decltype(uc)::value;
      V sv[UU][H], dv[UU][H];
#pragma unroll
      for (int u = 0; u < UU; u++) {
#pragma unroll
        for (int j = 0; j < H; j++) {
          const int64_t p = (q0 + u * B - j) & (Nl - 1);
          sv[u][j] = s[p];
          dv[u][j] = P::ld(w[off + p * step]);
        }
      }
#pragma unroll
      for (int u = 0; u < UU; u++) {
        const int64_t q = q0 + u * B;
        V e, o;
        if constexpr (F == 1) {
          const V dq = thr_v<P>(dv[u][0], th, l);
          e = haar_sum<P>(sv[u][0], dq);
          o = haar_dif<P>(sv[u][0], dq);
        } else {
          V dt[H];
#pragma unroll
          for (int j = 0; j < H; j++) dt[j] = thr_v<P>(dv[u][j], th, l);
          typename P::Acc ae = P::acc_init(sv[u][H - 1], tap_h(F, 2 * (H - 1)));
          typename P::Acc ao = P::acc_init(sv[u][H - 1], tap_h(F, 2 * (H - 1) + 1));
          ae = P::acc_add(ae, dt[H - 1], tap_g(F, 2 * (H - 1)));
          ao = P::acc_add(ao, dt[H - 1], tap_g(F, 2 * (H - 1) + 1));
#pragma unroll
          for (int j = H - 2; j >= 0; j--) {
            ae = P::acc_add(ae, sv[u][j], tap_h(F, 2 * j));
            ao = P::acc_add(ao, sv[u][j], tap_h(F, 2 * j + 1));
            ae = P::acc_add(ae, dt[j], tap_g(F, 2 * j));
            ao = P::acc_add(ao, dt[j], tap_g(F, 2 * j + 1));
          }
          e = P::acc_fin(ae);
          o = P::acc_fin(ao);
        }
        if (l == 0) {
          if constexpr (std::is_same<D, typename P::V>::value) {
            out[2 * q] = e;
            out[2 * q + 1] = o;
          } else {
            out[2 * q] = P::st(e);
            out[2 * q + 1] = P::st(o);
          }
        } else {
          dstv[2 * q] = e;
          dstv[2 * q + 1] = o;
        }
      }
    });
    __syncthreads();
    Nl <<= 1;
  }
}

// ----------------------------------------------------- MODWT (block) ----
// Stored coefficients: det = [d_1 | ... | d_J] (J blocks of N), sJ (N).

// Shared-memory tiles of the block-level MODWT levels: two stages of two
// arrays (scaling values, details) of mod_tile<V>() values each.  Kernels
// that run them are launched with mod_tile_smem<V>() bytes of dynamic shared
// memory, WC_MOD_TILE_KB per CTA; each translation unit that instantiates a
// kernel sets it for the CTAs it keeps per SM (the batched smoother runs one
// 512-thread CTA per SM and takes 192 KB, the threshold tuner two 256-thread
// CTAs and 104 KB each).  A tile's rows are a power of two, so three times
// the memory gives four times the rows of a 32-column tile: a quarter of the
// tile steps (two barriers each) and a smaller share of halo rows.
#ifndef WC_MOD_TILE_KB
#define WC_MOD_TILE_KB 64
#endif
template <class V>
constexpr int mod_tile() {
  return WC_MOD_TILE_KB * 1024 / (4 * (int)sizeof(V));
}
template <class V>
constexpr size_t mod_tile_smem() {
  return 4 * (size_t)mod_tile<V>() * sizeof(V);
}

// One forward level (taps 2^l apart) by double-buffered shared-memory tiles
// of the row view (taps are the L-1 rows below an output): the tile's raw
// inputs arrive by per-thread asynchronous copies while the previous tile is
// computed; emit(i, s, d) receives every output's scaling and detail value.
template <int F, class P, class S, class Emit>
__device__ void bfwd_level_tiled(const S* src, int64_t N, int l, Emit&& emit) {
  using V = typename P::V;
  static_assert(sizeof(S) == sizeof(V), "in-place staging");
  constexpr int L = filter_len(F);
  constexpr int HR = L - 1;
  constexpr int KT = mod_tile<V>();
  extern __shared__ __align__(16) unsigned char mod_smem[];
  V* buf = reinterpret_cast<V*>(mod_smem);  // [stage][KT]
  const int64_t d0 = (int64_t)1 << l, rows = N >> l;
  const int C = (int)(d0 < 32 ? d0 : 32);
  const int cs = __ffs(C) - 1;
  int64_t M = rows;
  while (M > 1 && (M + HR) * C > KT) M >>= 1;
  const int64_t nb = d0 / C, ntiles = nb * (rows / M);
  const int tot = (int)((M + HR) * C);
  auto issue = [&](int64_t tile, int stage) {
    S* Vs = reinterpret_cast<S*>(buf + stage * KT);
    const int64_t r0 = (tile % nb) * C, m0 = (tile / nb) * M;
    for (int e = threadIdx.x; e < tot; e += blockDim.x) {
      const int row = e >> cs, c = e & (C - 1);
      cp_async_elem(Vs + e, src + (r0 + c) + ((m0 + row) & (rows - 1)) * d0);
    }
    cp_async_commit();
  };
  issue(0, 0);
  for (int64_t tile = 0; tile < ntiles; tile++) {
    const int stage = (int)(tile & 1);
    if (tile + 1 < ntiles) issue(tile + 1, stage ^ 1);
    else cp_async_commit();  // empty group keeps the wait count uniform
    cp_async_wait_prior_1();
    V* Vs = buf + stage * KT;
    if constexpr (!std::is_same<S, V>::value) {
      for (int e = threadIdx.x; e < tot; e += blockDim.x)
        Vs[e] = P::ld(reinterpret_cast<const S*>(Vs)[e]);
    }
    __syncthreads();
    const int64_t r0 = (tile % nb) * C, m0 = (tile / nb) * M;
    for (int e = threadIdx.x; e < (int)(M * C); e += blockDim.x) {
      const int row = e >> cs, c = e & (C - 1);
      V s, d;
      if constexpr (F == 1) {
        d = haar_dif<P>(Vs[e], Vs[e + C]);
        s = haar_sum<P>(Vs[e], Vs[e + C]);
      } else if constexpr (std::is_same<P, PDD>::value) {
        // d in lane 0, s in lane 1: the operations below, packed
        dd_acc2 A = acc2_init(Vs[e], load_tap2(kBatchModwtTaps[F].p[0]));
#pragma unroll
        for (int k = 1; k < L; k++) A = acc2_add(A, Vs[e + k * C], load_tap2(kBatchModwtTaps[F].p[k]));
        acc2_fin(A, d, s);
      } else {
        typename P::Acc ad = P::acc_init(Vs[e], tap_g(F, 0));
        typename P::Acc as = P::acc_init(Vs[e], tap_h(F, 0));
#pragma unroll
        for (int k = 1; k < L; k++) {
          ad = P::acc_add(ad, Vs[e + k * C], tap_g(F, k));
          as = P::acc_add(as, Vs[e + k * C], tap_h(F, k));
        }
        d = P::acc_fin(ad);
        s = P::acc_fin(as);
      }
      emit((r0 + c) + (m0 + row) * d0, s, d);
    }
    __syncthreads();  // this stage is refilled two tiles later
  }
}

// One FP32 forward level by the 16-byte tiles of wc_modwt_vec.cuh,
// double-buffered like bfwd_level_tiled: a thread computes W = 4 adjacent
// outputs of a row (4 rows of a single-column tile) with the operations of
// bfwd_level_tiled per value, and emit(i, s, d) receives the outputs i ..
// i+3 (consecutive in memory).  Returns false without doing anything when
// the tiles do not apply (other precisions, too few rows, a source not
// 16-byte aligned).
template <int F, class P, class S, class EmitG>
__device__ bool bfwd_level_vec(const S* src, int64_t N, int l, EmitG&& emit) {
  if constexpr (!std::is_same<P, PF32>::value || !std::is_same<S, float>::value) {
    return false;
  } else {
    constexpr int L = filter_len(F);
    constexpr int W = 4;
    constexpr int KT = mod_tile<float>();
    const int64_t d0 = (int64_t)1 << l, rows = N >> l;
    const int C = (int)(d0 < 32 ? d0 : 32);
    int64_t M = rows;
    auto rows_in = [&](int64_t m) { return (int64_t)mvec_fwd_rows(L, 1, 0, (int)m, C, W); };
    while (M > W && rows_in(M) * C > KT) M >>= 1;
    if (!mvec_ok(C, (int)M, W) || rows_in(M) * C > KT || ((uintptr_t)src & 15)) return false;
    extern __shared__ __align__(16) unsigned char mod_smem[];
    float* buf = reinterpret_cast<float*>(mod_smem);  // [stage][KT]
    const int cs = __ffs(C) - 1;
    const int64_t nb = d0 / C, ntiles = nb * (rows / M);
    const int totc = (int)(rows_in(M) * C / W);
    auto issue = [&](int64_t tile, int stage) {
      float* Vs = buf + stage * KT;
      const int64_t r0 = (tile % nb) * C, m0 = (tile / nb) * M;
      for (int j = threadIdx.x; j < totc; j += blockDim.x) {
        const int e = j * W;
        const int row = e >> cs, c = e & (C - 1);
        cp_async16(Vs + e, src + (r0 + c) + ((m0 + row) & (rows - 1)) * d0);
      }
      cp_async_commit();
    };
    issue(0, 0);
    for (int64_t tile = 0; tile < ntiles; tile++) {
      const int stage = (int)(tile & 1);
      if (tile + 1 < ntiles) issue(tile + 1, stage ^ 1);
      else cp_async_commit();  // empty group keeps the wait count uniform
      cp_async_wait_prior_1();
      __syncthreads();
      const float* Vs = buf + stage * KT;
      const int64_t r0 = (tile % nb) * C, m0 = (tile / nb) * M;
      auto group = [&](auto rdc) {
        constexpr int RD = decltype(rdc)::value;
        for (int e = (int)threadIdx.x * W; e < (int)(M * C); e += (int)blockDim.x * W) {
          const int row = e >> cs, c = e & (C - 1);
          float sv[W], dv[W];
          fwd_group<F, P, RD>(Vs, e, C, sv, dv);
          emit((r0 + c) + (m0 + row) * d0, sv, dv);
        }
      };
      if (C == 1) group(std::integral_constant<int, 1>{});
      else group(std::integral_constant<int, 0>{});
      __syncthreads();  // this stage is refilled two tiles later
    }
    return true;
  }
}

template <int F, class P, class S>
__device__ void bmodwt_fwd(const S* x, typename P::T* det, typename P::T* sJ, int64_t N, int J,
                           typename P::V* tA, typename P::V* tB) {
  using V = typename P::V;
  for (int l = 0; l < J; l++) {
    V* dst = (l & 1) ? tB : tA;
    typename P::T* dd_out = det + (int64_t)l * N;
    auto emit = [&](int64_t i, V s, V d) {
      dd_out[i] = P::st(d);
      if (l == J - 1) sJ[i] = P::st(s);
      else dst[i] = s;
    };
    if constexpr (std::is_same<P, PF32>::value) {
      // 16-byte stores of four outputs (scratch slices are 256-byte aligned)
      auto emitg = [&](int64_t i, const float (&s)[4], const float (&d)[4]) {
        *reinterpret_cast<float4*>(dd_out + i) = make_float4(d[0], d[1], d[2], d[3]);
        float* so = (l == J - 1) ? sJ : dst;
        *reinterpret_cast<float4*>(so + i) = make_float4(s[0], s[1], s[2], s[3]);
      };
      const bool al = (((uintptr_t)dd_out | (uintptr_t)sJ | (uintptr_t)dst) & 15) == 0;
      if (al && (l == 0 ? bfwd_level_vec<F, P, S>(x, N, 0, emitg)
                        : bfwd_level_vec<F, P, V>((l & 1) ? tA : tB, N, l, emitg)))
        continue;
    }
    if (l == 0) bfwd_level_tiled<F, P, S>(x, N, 0, emit);
    else bfwd_level_tiled<F, P, V>((l & 1) ? tA : tB, N, l, emit);
  }
}

// Inverse MODWT by tiles of the row view: level l splits the sequence into
// d0 = 2^l interleaved columns whose taps are the rows above; a tile of C
// adjacent columns (C = min(d0, 32)) by M rows plus the L-1 halo rows sits
// in shared memory, so every tap is a shared-memory read.  Each output
// keeps the reference's term order (even taps then odd taps, s before d).
// Tiled inverse with double buffering: the next tile's raw values arrive by
// per-thread asynchronous copies while the current tile is computed, so the
// load latency hides behind arithmetic even with one CTA per SM.  Each
// thread converts (double-float) and thresholds the details it copied,
// once, before the tile's barrier.
// One FP32 inverse level (l, taps 2^l apart) by the 16-byte tiles of
// wc_modwt_vec.cuh, double-buffered like the one-value level below: every
// copy, shared-memory load and store moves 16 bytes and a thread computes W
// adjacent outputs of a row (W rows of a single-column tile), each with the
// operations of the one-value level, so the bits are the same.  S holds the
// level's scaling input (raw T values when top, else V values), dl its
// details (thresholded once per staged value), and the outputs go to dst (V)
// or, on the last level, to out (D).  Returns false without doing anything
// when the tiles do not apply (see bmodwt_inv_tiled2).
template <int F, class P, class D, class TH>
__device__ bool bmod_inv_level_vec(const void* S, bool top, const typename P::T* dl, int64_t N,
                                   int l, const TH& th, typename P::V* dst, D* out) {
  // Not in exact FP64, whose levels are bound by the FP64 pipe.
  if constexpr (std::is_same<P, PExact>::value) {
    return false;
  } else {
    constexpr bool kDD = std::is_same<P, PDD>::value;
    using V = typename P::V;
    using T = typename P::T;
    constexpr int L = filter_len(F);
    constexpr int W = mvec_w<P>();
    constexpr int KT = mod_tile<V>();
    const int64_t d0 = (int64_t)1 << l, rows = N >> l;
    const int C = (int)(d0 < 32 ? d0 : 32);
    const int HRp = mvec_inv_halo(L, 1, C, W);
    int64_t M = rows;
    while (M > 1 && (M + HRp) * C > KT) M >>= 1;
    const bool last = (l == 0);
    if (!mvec_ok(C, (int)M, W) || (M + HRp) * C > KT) return false;
    if (((uintptr_t)S | (uintptr_t)dl | (uintptr_t)dst) & 15) return false;
    if (last && (((uintptr_t)out & 15) || sizeof(D) != sizeof(T))) return false;
    extern __shared__ __align__(16) unsigned char mod_smem[];
    V* buf = reinterpret_cast<V*>(mod_smem);  // [stage][S | D][KT]
    const int cs = __ffs(C) - 1;
    const int64_t nb = d0 / C, ntiles = nb * (rows / M);
    const int tot = (int)((M + HRp) * C), totc = tot / W;
    const unsigned char* Sb = static_cast<const unsigned char*>(S);
    auto issue = [&](int64_t tile, int stage) {
      unsigned char* Ss = reinterpret_cast<unsigned char*>(buf + stage * 2 * KT);
      unsigned char* Ds = Ss + KT * sizeof(V);
      const int64_t r0 = (tile % nb) * C, m0 = (tile / nb) * M;
      for (int j = threadIdx.x; j < totc; j += blockDim.x) {
        const int e = j * W;
        const int row = e >> cs, c = e & (C - 1);
        const int64_t g = (r0 + c) + ((m0 - HRp + row) & (rows - 1)) * d0;
        cp_async16(Ss + (size_t)e * sizeof(V), Sb + (size_t)g * sizeof(V));
        cp_async16(Ds + (size_t)e * sizeof(V), dl + g);
      }
      cp_async_commit();
    };
    issue(0, 0);
    for (int64_t tile = 0; tile < ntiles; tile++) {
      const int stage = (int)(tile & 1);
      if (tile + 1 < ntiles) issue(tile + 1, stage ^ 1);
      else cp_async_commit();  // empty group keeps the wait count uniform
      cp_async_wait_prior_1();
      unsigned char* Ss = reinterpret_cast<unsigned char*>(buf + stage * 2 * KT);
      unsigned char* Ds = Ss + KT * sizeof(V);
      // Each thread converts (and thresholds) the chunks it copied.
      for (int j = threadIdx.x; j < totc; j += blockDim.x) {
        if constexpr (kDD) {
          // pair chunks: scaling values from FP64 (top) or double-float
          // {hi0, lo0, hi1, lo1}; details converted and thresholded
          if (top) {
            to_pair_chunk(Ss, j);
          } else {
            const float4 a = reinterpret_cast<const float4*>(Ss)[j];
            reinterpret_cast<PairChunk*>(Ss)[j] = PairChunk{x2_pack(a.x, a.z), x2_pack(a.y, a.w)};
          }
          const double2 v = reinterpret_cast<const double2*>(Ds)[j];
          const dd a = thr_v<P>(dd_from_double(v.x), th, l);
          const dd b = thr_v<P>(dd_from_double(v.y), th, l);
          reinterpret_cast<PairChunk*>(Ds)[j] = PairChunk{x2_pack(a.hi, b.hi), x2_pack(a.lo, b.lo)};
        } else {
          Chunk<T> c = reinterpret_cast<const Chunk<T>*>(Ds)[j];
#pragma unroll
          for (int i = 0; i < W; i++) c.v[i] = thr_v<P>(c.v[i], th, l);
          reinterpret_cast<Chunk<T>*>(Ds)[j] = c;
        }
      }
      __syncthreads();
      const int64_t r0 = (tile % nb) * C, m0 = (tile / nb) * M;
      auto group = [&](auto rdc) {
        constexpr int RD = decltype(rdc)::value;
        // FP32: two groups per thread in flight (double-float measured slower)
#pragma unroll(kDD ? 1 : 2)
        for (int e = HRp * C + (int)threadIdx.x * W; e < tot; e += (int)blockDim.x * W) {
          const int row = e >> cs, c = e & (C - 1);
          const int64_t i = (r0 + c) + (m0 - HRp + row) * d0;
          if constexpr (kDD) {
            f32x2 hi, lo;
            inv_group_dd<F, RD>(reinterpret_cast<const PairChunk*>(Ss),
                                reinterpret_cast<const PairChunk*>(Ds), e, C, hi, lo);
            float h0, h1, l0, l1;
            x2_unpack(hi, h0, h1);
            x2_unpack(lo, l0, l1);
            if (last && !std::is_same<D, V>::value) {
              *reinterpret_cast<double2*>(out + i) =
                  make_double2(dd_to_double(dd{h0, l0}), dd_to_double(dd{h1, l1}));
            } else {
              V* o = last ? reinterpret_cast<V*>(out) : dst;
              *reinterpret_cast<float4*>(o + i) = make_float4(h0, l0, h1, l1);
            }
          } else {
            V r[W];
            inv_group<F, P, RD>(reinterpret_cast<const V*>(Ss), reinterpret_cast<const V*>(Ds), e,
                                C, r);
            Chunk<T> ch;
#pragma unroll
            for (int q = 0; q < W; q++) ch.v[q] = r[q];
            T* o = last ? reinterpret_cast<T*>(out) : reinterpret_cast<T*>(dst);
            *reinterpret_cast<Chunk<T>*>(o + i) = ch;
          }
        }
      };
      if (C == 1) group(std::integral_constant<int, 1>{});
      else group(std::integral_constant<int, 0>{});
      __syncthreads();  // this stage is refilled two tiles later
    }
    return true;
  }
}

template <int F, class P, class D, class TH>
__device__ void bmodwt_inv_tiled2(const typename P::T* det, const typename P::T* sJ, D* out,
                                  int64_t N, int J, const TH& th, typename P::V* tA,
                                  typename P::V* tB) {
  using V = typename P::V;
  using T = typename P::T;
  static_assert(sizeof(V) == sizeof(T), "in-place staging");
  constexpr int L = filter_len(F);
  constexpr int HR = L - 1;
  constexpr int KT = mod_tile<V>();
  extern __shared__ __align__(16) unsigned char mod_smem[];
  V* buf = reinterpret_cast<V*>(mod_smem);  // [stage][S | D][KT]
  for (int l = J - 1; l >= 0; l--) {
    const bool top = (l == J - 1);
    const V* src = ((J - 1 - l) & 1) ? tA : tB;
    V* dst = ((J - 1 - l) & 1) ? tB : tA;
    const T* dl = det + (int64_t)l * N;
    if (bmod_inv_level_vec<F, P, D, TH>(top ? (const void*)sJ : (const void*)src, top, dl, N, l,
                                        th, dst, out))
      continue;
    const int64_t d0 = (int64_t)1 << l, rows = N >> l;
    const int C = (int)(d0 < 32 ? d0 : 32);
    const int cs = __ffs(C) - 1;
    int64_t M = rows;
    while (M > 1 && (M + HR) * C > KT) M >>= 1;
    const int64_t nb = d0 / C, ntiles = nb * (rows / M);
    const int tot = (int)((M + HR) * C);
    auto issue = [&](int64_t tile, int stage) {
      V* Ss = buf + stage * 2 * KT;
      V* Ds = Ss + KT;
      const int64_t r0 = (tile % nb) * C, m0 = (tile / nb) * M;
      for (int e = threadIdx.x; e < tot; e += blockDim.x) {
        const int row = e >> cs, c = e & (C - 1);
        const int64_t g = (r0 + c) + ((m0 - HR + row) & (rows - 1)) * d0;
        if (top) cp_async_elem(reinterpret_cast<T*>(Ss) + e, sJ + g);
        else cp_async_elem(Ss + e, src + g);
        cp_async_elem(reinterpret_cast<T*>(Ds) + e, dl + g);
      }
      cp_async_commit();
    };
    issue(0, 0);
    for (int64_t tile = 0; tile < ntiles; tile++) {
      const int stage = (int)(tile & 1);
      if (tile + 1 < ntiles) issue(tile + 1, stage ^ 1);
      else cp_async_commit();  // empty group keeps the wait count uniform
      cp_async_wait_prior_1();
      V* Ss = buf + stage * 2 * KT;
      V* Ds = Ss + KT;
      for (int e = threadIdx.x; e < tot; e += blockDim.x) {
        if constexpr (!std::is_same<V, T>::value) {
          if (top) Ss[e] = P::ld(reinterpret_cast<const T*>(Ss)[e]);
        }
        Ds[e] = thr_v<P>(P::ld(reinterpret_cast<const T*>(Ds)[e]), th, l);
      }
      __syncthreads();
      const int64_t r0 = (tile % nb) * C, m0 = (tile / nb) * M;
      for (int e = HR * C + threadIdx.x; e < tot; e += blockDim.x) {
        const int row = e >> cs, c = e & (C - 1);
        V r;
        if constexpr (F == 1) {
          V acc = P::add(Ss[e], Ds[e]);
          acc = P::add(acc, Ss[e - C]);
          acc = P::sub(acc, Ds[e - C]);
          r = P::mul(acc, kHInvR2);
        } else {
          typename P::Acc acc;
#pragma unroll
          for (int t = 0; t < L; t++) {
            const int k = (t < L / 2) ? (L - 2 - 2 * t) : (L - 1 - 2 * (t - L / 2));
            if (t == 0) acc = P::acc_init(Ss[e - k * C], tap_h(F, k));
            else acc = P::acc_add(acc, Ss[e - k * C], tap_h(F, k));
            acc = P::acc_add(acc, Ds[e - k * C], tap_g(F, k));
          }
          r = P::half(P::acc_fin(acc));
        }
        const int64_t i = (r0 + c) + (m0 - HR + row) * d0;
        if (l == 0) {
          if constexpr (std::is_same<D, V>::value) out[i] = r;
          else out[i] = P::st(r);
        } else {
          dst[i] = r;
        }
      }
      __syncthreads();  // this stage is refilled two tiles later
    }
  }
}

template <int F, class P, class D, class TH>
__device__ void bmodwt_inv(const typename P::T* det, const typename P::T* sJ, D* out, int64_t N,
                           int J, const TH& th, typename P::V* tA, typename P::V* tB) {
  bmodwt_inv_tiled2<F, P, D, TH>(det, sJ, out, N, J, th, tA, tB);
}

// ------------------------------------------------- radix select (block) --

__device__ __forceinline__ uint64_t key_of(double v) {
  uint64_t u = (uint64_t)__double_as_longlong(v);
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double val_of(uint64_t k) {
  uint64_t u = (k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
  return __longlong_as_double((long long)u);
}

// Source of the universal threshold's values: `nseg` segments of `seg_len`
// values `seg_stride` apart, or (dwt_J > 0) the DWT details i in [1, len)
// with level ctz(i) in [minl, maxl].
template <class T>
struct Src {
  const T* base;
  int64_t seg_len, seg_stride, nseg;
  int dwt_J, minl, maxl;
  int64_t count;
};

struct SelShared {
  unsigned int h[2][256];
  uint64_t prefix[2], mask[2];
  long long rank[2];
};

template <class T, class Fn>
__device__ __forceinline__ void for_each_src(const Src<T>& s, Fn fn) {
  if (s.dwt_J > 0) {
    const int64_t len = s.seg_len;
    for (int64_t i = 1 + threadIdx.x; i < len; i += blockDim.x) {
      const int l = __ffsll((long long)i) - 1;
      if (l >= s.dwt_J || l < s.minl || l > s.maxl) continue;
      fn((double)s.base[i]);
    }
  } else {
    const int64_t total = s.seg_len * s.nseg;
    for (int64_t e = threadIdx.x; e < total; e += blockDim.x) {
      const int64_t seg = e / s.seg_len, off = e - seg * s.seg_len;
      fn((double)s.base[seg * s.seg_stride + off]);
    }
  }
}

// Values of ranks ka and kb (0-based) of the source, into *va, *vb (valid in
// every thread on return).
template <class T>
__device__ void bselect(const Src<T>& src, long long ka, long long kb, SelShared& sh, double* va,
                        double* vb) {
  if (threadIdx.x == 0) {
    sh.prefix[0] = sh.prefix[1] = 0;
    sh.mask[0] = sh.mask[1] = 0;
    sh.rank[0] = ka;
    sh.rank[1] = kb;
  }
  __syncthreads();
  for (int shift = 56; shift >= 0; shift -= 8) {
    for (int i = threadIdx.x; i < 512; i += blockDim.x) (&sh.h[0][0])[i] = 0;
    __syncthreads();
    const uint64_t p0 = sh.prefix[0], p1 = sh.prefix[1], m0 = sh.mask[0], m1 = sh.mask[1];
    for_each_src(src, [&](double v) {
      const uint64_t k = key_of(v);
      const int d = (int)((k >> shift) & 255);
      // Lanes of a warp that hit the same bin add once (the values of a
      // selection cluster in few bins, so per-lane atomics serialise).
      const unsigned act = __activemask();
      const unsigned b0 = ((k & m0) == p0) ? (unsigned)d : 256u;
      const unsigned b1 = ((k & m1) == p1) ? (unsigned)d : 256u;
      const unsigned g0 = __match_any_sync(act, b0), g1 = __match_any_sync(act, b1);
      const int lane = threadIdx.x & 31;
      if (b0 < 256u && lane == __ffs(g0) - 1) atomicAdd(&sh.h[0][b0], (unsigned)__popc(g0));
      if (b1 < 256u && lane == __ffs(g1) - 1) atomicAdd(&sh.h[1][b1], (unsigned)__popc(g1));
    });
    __syncthreads();
    if (threadIdx.x < 2) {
      const int r = threadIdx.x;
      unsigned long long cum = 0;
      int d = 0;
      for (; d < 255; d++) {
        if ((unsigned long long)sh.rank[r] < cum + sh.h[r][d]) break;
        cum += sh.h[r][d];
      }
      sh.rank[r] -= (long long)cum;
      sh.prefix[r] |= (uint64_t)d << shift;
      sh.mask[r] |= (uint64_t)255 << shift;
    }
    __syncthreads();
  }
  *va = val_of(sh.prefix[0]);
  *vb = val_of(sh.prefix[1]);
  __syncthreads();
}

// median / mad of the source (utils.cpp:166-203); dev_buf holds count doubles.
template <class T>
__device__ void bmedian_mad(const Src<T>& src, double* dev_buf, SelShared& sh, double* med,
                            double* mad) {
  const long long n = src.count;
  double a, b;
  bselect(src, (n - 1) / 2, n / 2, sh, &a, &b);
  const double m = __dmul_rn(0.5, __dadd_rn(a, b));
  // |x - med| compactly (order irrelevant to the median)
  __shared__ unsigned long long pos;
  if (threadIdx.x == 0) pos = 0;
  __syncthreads();
  for_each_src(src, [&](double v) {
    // one atomic per warp; lanes take consecutive slots
    const unsigned act = __activemask();
    const int lane = threadIdx.x & 31, leader = __ffs(act) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(&pos, (unsigned long long)__popc(act));
    base = __shfl_sync(act, base, leader);
    const unsigned long long k = base + __popc(act & ((1u << lane) - 1u));
    dev_buf[k] = fabs(__dsub_rn(v, m));
  });
  __syncthreads();
  Src<double> ds{dev_buf, n, n, 1, 0, 0, 0, n};
  bselect(ds, (n - 1) / 2, n / 2, sh, &a, &b);
  *med = m;
  *mad = __dmul_rn(1.4826, __dmul_rn(0.5, __dadd_rn(a, b)));
}

// -------------------------------------------------- exact loss sum (block) --
// Same replay as cv_sum.cu with chunks of blockDim terms.

__device__ __forceinline__ void q_of(double v, int eb_m, long long& q, bool& bad) {
  const uint64_t vb = (uint64_t)__double_as_longlong(v);
  const int ebv = (int)((vb >> 52) & 0x7FF);
  q = 0;
  bad = false;
  if (eb_m <= 0 || eb_m >= 0x7FF || ebv == 0x7FF || ebv >= eb_m) {
    bad = true;
    return;
  }
  const uint64_t M = (vb & kFrac) | (ebv ? (1ull << 52) : 0ull);
  if (M == 0) return;
  const int s = eb_m - (ebv ? ebv : 1);
  if (s == 0) {
    q = (long long)M;
    return;
  }
  if (s > 63) return;
  const uint64_t rem = M & ((1ull << s) - 1), half = 1ull << (s - 1);
  if (rem == half) {
    bad = true;
    return;
  }
  q = (long long)((M >> s) + (rem > half ? 1 : 0));
}

struct SumShared {
  float red_hi[32], red_lo[32];  // per-warp double-float partial sums
  long long warp_tot[32];
  unsigned long long mb;
  long long add;
  int kstar;
};

__device__ __forceinline__ long long bscan_incl(long long x, SumShared& sh) {
  const int l = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    const long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (l >= o) x += y;
  }
  if (l == 31) sh.warp_tot[w] = x;
  __syncthreads();
  if (w == 0) {
    long long t = (l < nw) ? sh.warp_tot[l] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, t, o);
      if (l >= o) t += y;
    }
    if (l < nw) sh.warp_tot[l] = t;
  }
  __syncthreads();
  const long long r = x + (w > 0 ? sh.warp_tot[w - 1] : 0);
  __syncthreads();
  return r;
}

// Serial-order FP64 sum of v[0..n) (all >= 0); result in every thread.
// Chunks are blockDim terms; each chunk is added with one integer add when
// the whole chunk stays in m's binade with no tie, else replayed with a
// block prefix sum up to the first crossing / tie.
__device__ double bseq_sum(const double* v, int64_t n, SumShared& sh) {
  const int B = blockDim.x;
  if (threadIdx.x == 0) sh.mb = 0ull;
  __syncthreads();
  for (int64_t base = 0; base < n; base += B) {
    const int len = (int)((n - base < B) ? (n - base) : B);
    const double myv = (threadIdx.x < len) ? v[base + threadIdx.x] : 0.0;
    int pos = 0;
    while (pos < len) {
      const unsigned long long mb = sh.mb;
      long long q = 0;
      bool bad = false;
      const bool active = threadIdx.x >= pos && threadIdx.x < len;
      if (active) q_of(myv, (int)(mb >> 52), q, bad);
      if (!active || bad) q = 0;
      const long long incl = bscan_incl(q, sh);
      const bool stop = active && (bad || (mb & kFrac) + (unsigned long long)incl >= (1ull << 52));
      if (threadIdx.x == 0) sh.kstar = len;
      __syncthreads();
      if (stop) atomicMin(&sh.kstar, (int)threadIdx.x);
      __syncthreads();
      const int kstar = sh.kstar;
      if (kstar == len) {
        if ((int)threadIdx.x == len - 1) sh.add = incl;
      } else if ((int)threadIdx.x == kstar) {
        sh.add = incl - q;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        unsigned long long m2 = sh.mb + (unsigned long long)sh.add;
        if (kstar < len)
          m2 = (unsigned long long)__double_as_longlong(
              __dadd_rn(__longlong_as_double((long long)m2), v[base + kstar]));
        sh.mb = m2;
      }
      __syncthreads();
      pos = kstar + 1;
    }
  }
  const double m = __longlong_as_double((long long)sh.mb);
  __syncthreads();
  return m;
}

// ------------------------------------------------------ CV loss (block) --

// Terms j0 .. j1-1 of the loss.
template <class Y>
__device__ void bcv_terms(const Y* ye, const Y* yo, const double* xn, int64_t lenh, int64_t j0,
                          int64_t j1, double* terms) {
  for (int64_t j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
    double yie, yio;
    if (j == 0) {
      yie = to_d(yo[0]);
      yio = __dmul_rn(0.5, __dadd_rn(to_d(ye[0]), to_d(ye[1])));
    } else if (j == lenh - 1) {
      yio = to_d(ye[lenh - 1]);
      yie = __dmul_rn(0.5, __dadd_rn(to_d(yo[j]), to_d(yo[j - 1])));
    } else {
      yio = __dmul_rn(0.5, __dadd_rn(to_d(ye[j]), to_d(ye[j + 1])));
      yie = __dmul_rn(0.5, __dadd_rn(to_d(yo[j]), to_d(yo[j - 1])));
    }
    const double a = __dsub_rn(yie, xn[2 * j]);
    const double b = __dsub_rn(yio, xn[2 * j + 1]);
    terms[j] = __dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b));
  }
  __syncthreads();
}

// |v| < t for t >= 0 and v not NaN, by comparing the magnitude bits as
// unsigned integers (the same answer as the floating-point compare, without
// an FP64 instruction).
__device__ __forceinline__ bool abs_less(double v, double t) {
  return ((unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull) <
         (unsigned long long)__double_as_longlong(t);
}
__device__ __forceinline__ bool abs_less(float v, float t) {
  return (__float_as_uint(v) & 0x7FFFFFFFu) < __float_as_uint(t);
}

// Double-float values of the working types (exact for float and dd).
template <class V>
__device__ __forceinline__ dd as_dd(V v) {
  if constexpr (std::is_same<V, dd>::value) return v;
  else return dd{(float)v, 0.f};
}

__device__ __forceinline__ dd dd_sqr(dd a) {
  const float p = __fmul_rn(a.hi, a.hi);
  float e = __fmaf_rn(a.hi, a.hi, -p);
  e = __fmaf_rn(2.f * a.hi, a.lo, e);
  dd r;
  fast_two_sum(p, e, r.hi, r.lo);
  return r;
}

// Sum over the block of one double-float value per thread; the result is
// valid in every thread.
__device__ dd bdd_reduce(dd v, SumShared& sh) {
  for (int o = 16; o > 0; o >>= 1) {
    const dd w{__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o)};
    v = PDD::add(v, w);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) {
    sh.red_hi[warp] = v.hi;
    sh.red_lo[warp] = v.lo;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    dd t{0.f, 0.f};
    for (int w = 0; w < nw; w++) t = PDD::add(t, dd{sh.red_hi[w], sh.red_lo[w]});
    sh.red_hi[0] = t.hi;
    sh.red_lo[0] = t.lo;
  }
  __syncthreads();
  const dd r{sh.red_hi[0], sh.red_lo[0]};
  __syncthreads();
  return r;
}

// Double-float sum of the loss terms j0 .. j1-1, in block order (the
// precisions other than exact FP64; the result is valid in every thread).
// FP32: each term from the FP32 reconstructions and the FP32 copy of the
// signal xt in FP32 arithmetic (its rounding is that of the reconstructions
// it is made of), added into a per-thread double-float sum; double-float:
// every step in double-float from the FP64 signal xn.
template <class P>
__device__ dd bcv_part(const typename P::V* ye, const typename P::V* yo, const double* xn,
                       const typename P::T* xt, int64_t lenh, int64_t j0, int64_t j1,
                       SumShared& sh) {
  if constexpr (std::is_same<P, PF32>::value) {
    float sh_ = 0.f, sl = 0.f;  // running double-float sum (hi, lo)
#pragma unroll 4
    for (int64_t j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
      float yie, yio;
      if (j == 0) {
        yie = yo[0];
        yio = 0.5f * (ye[0] + ye[1]);
      } else if (j == lenh - 1) {
        yio = ye[lenh - 1];
        yie = 0.5f * (yo[j] + yo[j - 1]);
      } else {
        yio = 0.5f * (ye[j] + ye[j + 1]);
        yie = 0.5f * (yo[j] + yo[j - 1]);
      }
      const float a = yie - xt[2 * j], b = yio - xt[2 * j + 1];
      const float t = __fmaf_rn(a, a, b * b);
      float s, e;
      two_sum(sh_, t, s, e);
      sh_ = s;
      sl += e;
    }
    dd acc;
    fast_two_sum(sh_, sl, acc.hi, acc.lo);
    return bdd_reduce(acc, sh);
  } else {
  const dd half{0.5f, 0.f};
  dd acc{0.f, 0.f};
  for (int64_t j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
    dd yie, yio;
    if (j == 0) {
      yie = as_dd(yo[0]);
      yio = PDD::add(as_dd(ye[0]), as_dd(ye[1]));
      yio = dd{yio.hi * half.hi, yio.lo * half.hi};
    } else if (j == lenh - 1) {
      yio = as_dd(ye[lenh - 1]);
      yie = PDD::add(as_dd(yo[j]), as_dd(yo[j - 1]));
      yie = dd{yie.hi * half.hi, yie.lo * half.hi};
    } else {
      yio = PDD::add(as_dd(ye[j]), as_dd(ye[j + 1]));
      yio = dd{yio.hi * half.hi, yio.lo * half.hi};
      yie = PDD::add(as_dd(yo[j]), as_dd(yo[j - 1]));
      yie = dd{yie.hi * half.hi, yie.lo * half.hi};
    }
    const dd a = PDD::sub(yie, dd_from_double(xn[2 * j]));
    const dd b = PDD::sub(yio, dd_from_double(xn[2 * j + 1]));
    acc = PDD::add(acc, PDD::add(dd_sqr(a), dd_sqr(b)));
  }
  return bdd_reduce(acc, sh);
  }
}

// Sum of the interpolation loss terms (the quantity bcv_terms + bseq_sum
// give).  Exact FP64: the reference's roundings and serial order.  The other
// precisions already differ from the reference in the reconstructions, so
// there the terms and their sum run in double-float on the FP32 pipes
// (GB300's FP64 pipe is about 1/64 of its FP32 rate), in block order.
template <class P>
__device__ double bcv_sum(const typename P::V* ye, const typename P::V* yo, const double* xn,
                          const typename P::T* xt, int64_t lenh, double* terms, SumShared& sh) {
  using V = typename P::V;
  if constexpr (std::is_same<P, PExact>::value) {
    bcv_terms<V>(ye, yo, xn, lenh, 0, lenh, terms);
    return bseq_sum(terms, lenh, sh);
  } else {
    return dd_to_double(bcv_part<P>(ye, yo, xn, xt, lenh, 0, lenh, sh));
  }
}

// ------------------------------------------------------------ pipeline --

struct CtaScratch {
  char* base;
  size_t off;
  template <class T>
  __device__ T* take(int64_t n) {
    T* p = reinterpret_cast<T*>(base + off);
    off += ((sizeof(T) * (size_t)n + 255) / 256) * 256;
    return p;
  }
};

struct PipeShared {
  SelShared sel;
  SumShared sum;
};

// Forward transform of a compact signal s (length n) into the coefficient
// store: DWT -> w (interleaved, n); MODWT -> det (J*n) and sJ (n).
template <int F, class P, class S>
__device__ void fwd_any(int ttype, const S* s, typename P::T* w, typename P::T* sJ, int64_t n,
                        int J, typename P::V* tA, typename P::V* tB) {
  if (ttype == 0) bdwt_fwd<F, P, S>(s, w, n, J, tA, tB);
  else bmodwt_fwd<F, P, S>(s, w, sJ, n, J, tA, tB);
}

template <int F, class P, class D, class TH>
__device__ void inv_any(int ttype, const typename P::T* w, const typename P::T* sJ,
                        const D* coarse, D* out, int64_t n, int J, const TH& th,
                        typename P::V* tA, typename P::V* tB) {
  if (ttype == 0) bdwt_inv<F, P, D, TH>(w, coarse, out, n, J, th, tA, tB);
  else bmodwt_inv<F, P, D, TH>(w, sJ, out, n, J, th, tA, tB);
}

// univ_thresh (thresh.cpp:170-201) on the stored coefficients.
template <class T>
__device__ double buniv(int ttype, const T* w, int64_t n, int J, int minl, int maxl,
                        double sq_nm1, double sq_n, double* devbuf, PipeShared& sh) {
  Src<T> src;
  double scale;
  if (ttype == 0) {
    if (minl == 0 && maxl == J - 1) {
      src = Src<T>{w + 1, n - 1, n - 1, 1, 0, 0, 0, n - 1};
      scale = sq_nm1;
    } else {
      int64_t cnt = 0;
      for (int l = minl; l <= maxl; l++) cnt += n >> (l + 1);
      src = Src<T>{w, n, n, 1, J, minl, maxl, cnt};
      scale = sq_n;
    }
  } else {
    const int64_t nb = maxl - minl + 1;  // blocks 0 .. maxl-minl (wavutils.cpp:716-722)
    src = Src<T>{w, n, n, nb, 0, 0, 0, nb * n};
    scale = sq_n;
  }
  double med, mad;
  bmedian_mad(src, devbuf, sh.sel, &med, &mad);
  return __dmul_rn(mad, scale);
}

__device__ __forceinline__ bool range_ok(int64_t n, int J, int minl, int maxl, int L) {
  int maxlev = 0;
  while (((int64_t)L << maxlev) <= n) maxlev++;
  if (J < 1 || J > maxlev || minl < 0 || maxl < 0) return false;
  return minl <= maxl && maxl < J;
}

// ------------------------------------------------------- paired CTAs --

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Longest wait at a pair barrier before it gives up.  The partner's first
// wait spans the leader's forward transform and universal threshold of the
// whole signal (a fraction of a second for 2^20 samples in one CTA).
constexpr unsigned long long kPairWaitNs = 20ull * 1000000000ull;

// Barrier of the two CTAs of a pair; nb counts the barriers this CTA has
// passed.  Writes before it are visible to the other CTA after it (fence,
// atomic arrival, acquire poll, fence).  Returns false in every thread when
// the wait gave up (the status word then has its timeout bit).
__device__ bool pair_sync(BatchPair* pr, unsigned int& nb, unsigned int* status) {
  __syncthreads();
  int ok = 1;
  nb++;
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(&pr->arrive, 1u);
    const unsigned long long t0 = global_ns();
    while (ld_acquire_gpu(&pr->arrive) < 2u * nb) {
      if (global_ns() - t0 > kPairWaitNs) {
        if (status) atomicOr(status, kStatusTimeout);
        ok = 0;
        break;
      }
      __nanosleep(128);
    }
    __threadfence();
  }
  return __syncthreads_and(ok) != 0;
}

// A signal's buffers in its (leader's) CTA scratch, in take order.  The
// partner of a pair finds them by replaying the same takes on the leader's
// scratch.
template <class P>
struct SigBufs {
  typename P::T *xt, *w, *wsJ;
  typename P::V *tA, *tB;
  double* devbuf;
  typename P::T *we, *weJ, *wo, *woJ;  // CV: coefficient stores of the halves
  typename P::V* y[4];                 // CV: the four work vectors
  double* terms;                       // CV: loss terms
};

template <class P>
__device__ SigBufs<P> take_bufs(CtaScratch& cs, const BatchDesc& d) {
  using T = typename P::T;
  using V = typename P::V;
  const int64_t n = d.n, lenh = n / 2;
  const int J = d.J;
  const bool mod = d.ttype == 1;
  SigBufs<P> b{};
  b.xt = cs.take<T>(n);
  b.w = cs.take<T>(mod ? (int64_t)J * n : n);
  b.wsJ = cs.take<T>(mod ? n : 1);
  b.tA = cs.take<V>(n);
  b.tB = cs.take<V>(n);
  b.devbuf = cs.take<double>(mod ? (int64_t)J * n : n);
  if (d.threshtype == 2) {
    const int lv1 = J - 1;
    b.we = cs.take<T>(mod ? (int64_t)lv1 * lenh : lenh);
    b.weJ = cs.take<T>(mod ? lenh : 1);
    b.wo = cs.take<T>(mod ? (int64_t)lv1 * lenh : lenh);
    b.woJ = cs.take<T>(mod ? lenh : 1);
    for (int k = 0; k < 4; k++) b.y[k] = cs.take<V>(lenh);
    b.terms = cs.take<double>(lenh);
  }
  return b;
}

// Whether a CV signal searches at all (thresh.cpp:223-231 returns early).
__device__ __forceinline__ bool cv_runs(const BatchDesc& d, int L) {
  return range_ok(d.n, d.J, d.minl, d.maxl, L) && d.J > 1;
}

// The two-fold CV golden-section search (thresh.cpp:240-325) on the
// forwarded halves in b: each step thresholds and inverts both halves for a
// candidate and evaluates the interpolation loss.  role 0: one CTA does it
// all.  role 1 / 2: the leader / partner of a pair invert the even / odd
// half and compute the first / second half of the loss terms, meeting at
// two barriers per step (after the inverses, after the terms); both reduce
// the same values the same way, so they take the same branches.  tA, tB:
// this CTA's level buffers; nb: pair barriers passed so far.  Returns false
// when a pair barrier gave up.
template <int F, class P>
__device__ bool cv_search(const BatchDesc& d, int role, BatchPair* pr, unsigned int* status,
                          unsigned int nb, const SigBufs<P>& b, typename P::V* tA,
                          typename P::V* tB, const double* x, double t_univ, PipeShared& sh,
                          double& t_out, int& iters_out, double& mm_out) {
  using T = typename P::T;
  using V = typename P::V;
  const int64_t lenh = d.n / 2;
  const int tt = d.ttype, L = filter_len(F), lv1 = d.J - 1, maxl1 = d.maxl - 1;
  const bool half_ok = range_ok(lenh, lv1, d.minl, maxl1, L);
  auto step = [&](int k, double tk) {
    // threshold(we|wo, y_k, tk) then transform(y_k, BWD)
    if (!half_ok) return;  // never thresholded: y_k stays zero
    if ((role == 1 && (k & 1)) || (role == 2 && !(k & 1))) return;  // the other CTA's half
    Th<P> th{to_v<P>(tk), d.hardness, d.minl, maxl1};
    const bool even = (k & 1) == 0;
    const T* ws = even ? b.we : b.wo;
    const T* wJ = even ? b.weJ : b.woJ;
    // DWT: coarse slots k*2^(J-1), k>0, come from y's previous content
    inv_any<F, P, V>(tt, ws, wJ, (tt == 0) ? b.y[k] : nullptr, b.y[k], lenh, lv1, th, tA, tB);
  };
  bool ok = true;
  auto loss = [&](int p) -> double {
    const V* ye = b.y[2 * p];
    const V* yo = b.y[2 * p + 1];
    if (role == 0) return __dmul_rn(bcv_sum<P>(ye, yo, x, b.xt, lenh, b.terms, sh.sum), 0.5);
    ok = pair_sync(pr, nb, status);  // both halves inverted
    if (!ok) return 0.0;
    const int64_t mid = lenh / 2;
    const int64_t j0 = (role == 1) ? 0 : mid, j1 = (role == 1) ? mid : lenh;
    if constexpr (std::is_same<P, PExact>::value) {
      bcv_terms<V>(ye, yo, x, lenh, j0, j1, b.terms);
      ok = pair_sync(pr, nb, status);  // all terms written
      if (!ok) return 0.0;
      return __dmul_rn(bseq_sum(b.terms, lenh, sh.sum), 0.5);
    } else {
      const dd part = bcv_part<P>(ye, yo, x, b.xt, lenh, j0, j1, sh.sum);
      if (threadIdx.x == 0) {
        pr->part[role - 1][0] = part.hi;
        pr->part[role - 1][1] = part.lo;
      }
      ok = pair_sync(pr, nb, status);  // both partial sums written
      if (!ok) return 0.0;
      const dd tot = PDD::add(dd{pr->part[0][0], pr->part[0][1]}, dd{pr->part[1][0], pr->part[1][1]});
      return __dmul_rn(dd_to_double(tot), 0.5);
    }
  };
  const double R = 0.61803399, C = __dsub_rn(1.0, R);
  double ta = 0., tc = t_univ;
  double tb = __dmul_rn(tc, 0.5);
  double t0 = ta, t2 = tb, t1 = __dsub_rn(tb, __dmul_rn(C, __dsub_rn(tb, ta))), t3 = tc;
  double min_margin = 1e300;
  int iters = 0;
  step(0, t1);
  step(1, t1);
  step(2, t2);
  step(3, t2);
  double m1 = loss(0);
  if (!ok) return false;
  double m2 = loss(1);
  if (!ok) return false;
  while (fabs(__dsub_rn(t3, t0)) > __dmul_rn(d.tol, __dadd_rn(t1, t2))) {
    if (iters > 50) break;
    if (m1 != 0.0) min_margin = fmin(min_margin, fabs(__dsub_rn(m1, m2)) / fabs(m1));
    if (m2 < m1) {
      t0 = t1; t1 = t2; t2 = __dadd_rn(__dmul_rn(R, t2), __dmul_rn(C, t3));
      m1 = m2;
      step(2, t2);
      step(3, t2);
      m2 = loss(1);
      if (!ok) return false;
    } else {
      t3 = t2; t2 = t1; t1 = __dadd_rn(__dmul_rn(R, t1), __dmul_rn(C, t0));
      m2 = m1;
      step(0, t1);
      step(1, t1);
      m1 = loss(0);
      if (!ok) return false;
    }
    iters++;
  }
  t_out = m1 < m2 ? t1 : t2;
  iters_out = iters;
  mm_out = min_margin;
  return true;
}

template <int F, class P>
__device__ __noinline__ void smooth_one(const BatchArgs& a, int idx, CtaScratch cs, PipeShared& sh) {
  using T = typename P::T;
  using V = typename P::V;
  const BatchDesc d = a.desc[idx];
  BatchResult* res = a.res + idx;
  double* x = a.data + d.off;
  const int64_t n = d.n, lenh = n / 2;
  const int J = d.J, tt = d.ttype, L = filter_len(F);
  const bool mod = (tt == 1);
  BatchPair* pr = (d.pair > 0) ? a.pairs + (d.pair - 1) : nullptr;
  if (pr && threadIdx.x == 0) atomicExch(&pr->leader, blockIdx.x + 1u);  // the partner's way in

  const SigBufs<P> b = take_bufs<P>(cs, d);
  T* xt = b.xt;
  T* w = b.w;
  T* wsJ = b.wsJ;
  V* tA = b.tA;
  V* tB = b.tB;
  double* devbuf = b.devbuf;
  // x in the working precision
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) xt[i] = (T)x[i];
  __syncthreads();

  double t = d.thresh, t_univ = 0.0, min_margin = 1e300;
  int iters = 0;
  fwd_any<F, P, T>(tt, xt, w, wsJ, n, J, tA, tB);

  if (d.threshtype == 2) {
    if (!cv_runs(d, L)) {
      if (threadIdx.x == 0) {
        res->thresh = 0.0;
        res->iterations = 0;
        res->status = 0;
        res->thresh_univ = 0.0;
        res->kept = res->zeroed = 0;
        res->min_margin = 0.0;
      }
      return;  // thresh.cpp:223-231: x untouched (never paired)
    }
    const int lv1 = J - 1;
    t_univ = buniv<T>(tt, w, n, J, d.minl, d.maxl, d.sq_nm1, d.sq_n, devbuf, sh);
    for (int64_t i = threadIdx.x; i < 4 * lenh; i += blockDim.x) {
      // zero the work vectors (fresh zero-filled pages in the reference)
      (b.y[i / lenh])[i % lenh] = to_v<P>(0.0);
    }
    for (int64_t j = threadIdx.x; j < lenh; j += blockDim.x) {
      reinterpret_cast<T*>(tA)[j] = (T)x[2 * j];
      if (!pr) reinterpret_cast<T*>(tB)[j] = (T)x[2 * j + 1];
    }
    __syncthreads();
    // even/odd halves live in tA/tB's first halves as T; transform them
    // with the upper halves of tA/tB as level buffers (the partner of a
    // pair forwards the odd half)
    {
      T* ev = reinterpret_cast<T*>(tA);
      T* od = reinterpret_cast<T*>(tB);
      V* uA = tA + lenh;
      V* uB = tB + lenh;
      fwd_any<F, P, T>(tt, ev, b.we, b.weJ, lenh, lv1, uA, uB);
      if (!pr) {
        // the odd half moves to devbuf so that uA/uB stay free for levels
        T* od2 = reinterpret_cast<T*>(devbuf);
        for (int64_t j = threadIdx.x; j < lenh; j += blockDim.x) od2[j] = od[j];
        __syncthreads();
        fwd_any<F, P, T>(tt, od2, b.wo, b.woJ, lenh, lv1, uA, uB);
      }
    }
    bool ok = true;
    unsigned int nb = 0;
    if (pr) {
      if (threadIdx.x == 0) pr->t_univ = t_univ;
      ok = pair_sync(pr, nb, a.status);  // both halves forwarded, work vectors zeroed
    }
    if (ok)
      ok = cv_search<F, P>(d, pr ? 1 : 0, pr, a.status, nb, b, tA, tB, x, t_univ, sh, t, iters,
                           min_margin);
    if (!ok) {
      if (threadIdx.x == 0) res->status = 1;
      return;  // a pair barrier gave up: x untouched
    }
    t = __ddiv_rn(t, d.rescale);
  } else if (d.threshtype == 1) {
    t_univ = buniv<T>(tt, w, n, J, 0, 0, d.sq_nm1, d.sq_n, devbuf, sh);
    t = t_univ;
  }

  // kept / zeroed over [minl, maxl] on the unthresholded coefficients
  long long kept = 0, zeroed = 0;
  const bool ok = range_ok(n, J, d.minl, d.maxl, L);
  if (ok) {
    __shared__ unsigned long long cnt[2];
    if (threadIdx.x == 0) cnt[0] = cnt[1] = 0;
    __syncthreads();
    unsigned long long k0 = 0, z0 = 0;
    const T t_cmp = (T)t;
    if (!mod) {
      for (int64_t i = 1 + threadIdx.x; i < n; i += blockDim.x) {
        const int l = __ffsll((long long)i) - 1;
        if (l >= J || l < d.minl || l > d.maxl) continue;
        if (abs_less(w[i], t_cmp)) z0++; else k0++;
      }
    } else {
      for (int64_t e = threadIdx.x; e < (int64_t)(d.maxl - d.minl + 1) * n; e += blockDim.x) {
        if (abs_less(w[(int64_t)d.minl * n + e], t_cmp)) z0++; else k0++;
      }
    }
    atomicAdd(&cnt[0], k0);
    atomicAdd(&cnt[1], z0);
    __syncthreads();
    kept = (long long)cnt[0];
    zeroed = (long long)cnt[1];
  }
  // final threshold + inverse straight into x (FP64 out)
  Th<P> th{to_v<P>(t), d.hardness, ok ? d.minl : 1 << 30, ok ? d.maxl : -1};
  if constexpr (std::is_same<T, double>::value) {
    inv_any<F, P, double>(tt, w, wsJ, nullptr, x, n, J, th, tA, tB);
  } else {
    inv_any<F, P, T>(tt, w, wsJ, nullptr, xt, n, J, th, tA, tB);
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) x[i] = (double)xt[i];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    res->thresh = t;
    res->thresh_univ = t_univ;
    res->iterations = iters;
    res->status = 0;
    res->kept = kept;
    res->zeroed = zeroed;
    res->min_margin = (d.threshtype == 2) ? min_margin : 0.0;
  }
}

// The partner's share of a paired signal's CV search: it forwards the odd
// half into the leader's coefficient store, then runs the search with the
// leader (cv_search, role 2) and leaves; the leader finishes the signal.
template <int F, class P>
__device__ __noinline__ void partner_one(const BatchArgs& a, int idx, CtaScratch cs,
                                         PipeShared& sh) {
  using T = typename P::T;
  using V = typename P::V;
  const BatchDesc d = a.desc[idx];
  if (d.threshtype != 2 || d.pair <= 0 || !cv_runs(d, filter_len(F))) return;
  BatchPair* pr = a.pairs + (d.pair - 1);
  const double* x = a.data + d.off;
  const int64_t n = d.n, lenh = n / 2;
  __shared__ unsigned int s_leader;
  if (threadIdx.x == 0) {
    const unsigned long long t0 = global_ns();
    unsigned int l;
    while ((l = ld_acquire_gpu(&pr->leader)) == 0u) {
      if (global_ns() - t0 > kPairWaitNs) {
        if (a.status) atomicOr(a.status, kStatusTimeout);
        break;
      }
      __nanosleep(128);
    }
    s_leader = l;
  }
  __syncthreads();
  const unsigned int leader = s_leader;
  __syncthreads();
  if (leader == 0u) return;
  CtaScratch lcs{a.scratch + (size_t)(leader - 1u) * a.scratch_per_cta, 0};
  const SigBufs<P> b = take_bufs<P>(lcs, d);
  T* od = cs.take<T>(lenh);
  V* pA = cs.take<V>(n);
  V* pB = cs.take<V>(n);
  for (int64_t j = threadIdx.x; j < lenh; j += blockDim.x) od[j] = (T)x[2 * j + 1];
  __syncthreads();
  fwd_any<F, P, T>(d.ttype, od, b.wo, b.woJ, lenh, d.J - 1, pA, pB);
  unsigned int nb = 0;
  if (!pair_sync(pr, nb, a.status)) return;  // both halves forwarded
  const double t_univ = pr->t_univ;
  double t = 0.0, mm = 0.0;
  int iters = 0;
  cv_search<F, P>(d, 2, pr, a.status, nb, b, pA, pB, x, t_univ, sh, t, iters, mm);
}

template <class P>
__global__ void __launch_bounds__(BT) smooth_batch_kernel(BatchArgs a) {
  __shared__ PipeShared sh;
  __shared__ int s_unit;
  CtaScratch cs{a.scratch + (size_t)blockIdx.x * a.scratch_per_cta, 0};
  while (true) {
    if (threadIdx.x == 0) s_unit = atomicAdd(a.counter, 1);
    __syncthreads();
    const int k = s_unit;
    __syncthreads();
    if (k >= a.nunits) break;
    const unsigned long long t_start = (a.trace && threadIdx.x == 0) ? global_ns() : 0ull;
    const int u = a.order[k];
    const bool partner = u < 0;
    const int idx = partner ? -u - 1 : u;
    cs.off = 0;
    switch (a.desc[idx].F * 2 + (partner ? 1 : 0)) {
      case 2: smooth_one<1, P>(a, idx, cs, sh); break;
      case 3: partner_one<1, P>(a, idx, cs, sh); break;
      case 4: smooth_one<2, P>(a, idx, cs, sh); break;
      case 5: partner_one<2, P>(a, idx, cs, sh); break;
      case 6: smooth_one<3, P>(a, idx, cs, sh); break;
      case 7: partner_one<3, P>(a, idx, cs, sh); break;
      case 8: smooth_one<4, P>(a, idx, cs, sh); break;
      case 9: partner_one<4, P>(a, idx, cs, sh); break;
    }
    __syncthreads();
    if (a.trace && threadIdx.x == 0) {
      a.trace[3 * (size_t)k] = t_start;
      a.trace[3 * (size_t)k + 1] = global_ns();
      a.trace[3 * (size_t)k + 2] = blockIdx.x;
    }
  }
}

}  // namespace

// One precision's launch and occupancy query.  Each precision is compiled in
// its own translation unit (batch_exact.cu, batch_fast.cu, batch_f32.cu) so
// the three instantiations of the pipeline build in parallel.
template <class P>
int batch_launch_p(const BatchArgs& a, int grid, cudaStream_t s) {
  constexpr size_t smem = mod_tile_smem<typename P::V>();
  WC_CUDA(cudaFuncSetAttribute(smooth_batch_kernel<P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem));
  smooth_batch_kernel<P><<<grid, BT, smem, s>>>(a);
  return after_launch("smooth_batch_kernel");
}

template <class P>
int batch_blocks_per_sm_p() {
  constexpr size_t smem = mod_tile_smem<typename P::V>();
  int per = 0;
  if (cudaFuncSetAttribute(smooth_batch_kernel<P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, smooth_batch_kernel<P>, BT, smem) !=
          cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return per < 1 ? 1 : per;
}

}  // namespace wc
