// Shared device/host definitions of the GB300 wavelet library.
//
// Filter taps are the reference's literal decimal constants
// (haarcoeffs.h:4-5, daub4coeffs.h:13-16, c6coeffs.h:6-11, la8coeffs.h:6-13):
// the exact-precision kernels must reproduce the reference's roundings, so
// the taps have to be the same doubles.  Wavelet taps are g_k = (-1)^k
// h_{L-1-k}, which is the sign/order pattern of every detail expression in
// daub4.cpp:31, c6.cpp:45, la8.cpp:41.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "wc_internal.h"

namespace wc {

// ------------------------------------------------------------------ taps --

__host__ __device__ constexpr int filter_len(int F) {
  return F == 1 ? 2 : F == 2 ? 4 : F == 3 ? 6 : F == 4 ? 8 : 0;
}

// Scaling filter h_k of filter F (1 Haar, 2 D4, 3 C6, 4 LA8).
__host__ __device__ constexpr double tap_h(int F, int k) {
  return F == 1 ? 0.70710678118654752440
       : F == 2 ? (k == 0 ? 0.4829629131445341 : k == 1 ? 0.8365163037378079
                 : k == 2 ? 0.2241438680420134 : -0.1294095225512604)
       : F == 3 ? (k == 0 ? -7.273261951252645e-2 : k == 1 ? 3.378976624574818e-1
                 : k == 2 ? 8.525720202116004e-1 : k == 3 ? 3.848648468648577e-1
                 : k == 4 ? -7.273261951252645e-2 : -1.565572813579199e-2)
       : (k == 0 ? -7.576571478950221e-2 : k == 1 ? -2.963552764600249e-2
        : k == 2 ? 4.976186676327750e-1 : k == 3 ? 8.037387518051321e-1
        : k == 4 ? 2.978577956053061e-1 : k == 5 ? -9.921954357663353e-2
        : k == 6 ? -1.260396726203130e-2 : 3.222310060405147e-2);
}

// Wavelet filter g_k = (-1)^k h_{L-1-k}.
__host__ __device__ constexpr double tap_g(int F, int k) {
  return (k & 1) ? -tap_h(F, filter_len(F) - 1 - k) : tap_h(F, filter_len(F) - 1 - k);
}

// max(|c0|, |c1|) with a relative margin of 1e-6 (the sigma bound of the
// extraction dot products).
__host__ __device__ constexpr float tap_pair_max(double c0, double c1) {
  const double a = c0 < 0 ? -c0 : c0, b = c1 < 0 ? -c1 : c1;
  return (float)((a > b ? a : b) * (1.0 + 1e-6));
}
__host__ __device__ constexpr float tap_hg_max(int F, int j) {
  return tap_pair_max(tap_h(F, j), tap_g(F, j));
}

constexpr double kInvR2 = 0.70710678118654752440;   // haarcoeffs.h:4
constexpr double kHInvR2 = 0.35355339059327376220;  // haarcoeffs.h:5

// ----------------------------------------------------- arithmetic policies --
//
// Every kernel is written once against a policy P:
//   P::T   element type in memory,   P::V  value type in registers,
//   ld/st  conversions,  mul(v, c)  product with a filter tap (c a double
//   constant known at compile time), add/sub, and the Haar butterfly.
// PExact rounds every product and sum separately in IEEE FP64 (no
// contraction), which is what makes its results bit-identical to the
// reference's CPU code.

// Dot products (a filter applied to L values) go through an accumulator:
//   Acc a = acc_init(v0, c0);  a = acc_add(a, v_k, c_k) ...;  V r = acc_fin(a)
// which for PExact is exactly mul, then add(acc, mul) in order -- the
// reference's expression order -- and lets the double-float policy defer
// its renormalisation to the end of the dot product.
struct PExact {
  using T = double;
  using V = double;
  using Acc = double;
  static __device__ __forceinline__ Acc acc_init(V a, double c) { return __dmul_rn(a, c); }
  static __device__ __forceinline__ Acc acc_add(Acc s, V a, double c) {
    return __dadd_rn(s, __dmul_rn(a, c));
  }
  static __device__ __forceinline__ V acc_fin(Acc s) { return s; }
  static __device__ __forceinline__ V ld(T x) { return x; }
  static __device__ __forceinline__ T st(V v) { return v; }
  static __device__ __forceinline__ V mul(V a, double c) { return __dmul_rn(a, c); }
  static __device__ __forceinline__ V add(V a, V b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ V sub(V a, V b) { return __dsub_rn(a, b); }
  // acc + a*c with both roundings.
  static __device__ __forceinline__ V madd(V acc, V a, double c) {
    return __dadd_rn(acc, __dmul_rn(a, c));
  }
  static __device__ __forceinline__ V half(V a) { return __dmul_rn(a, 0.5); }
};

struct PF32 {
  using T = float;
  using V = float;
  using Acc = float;
  static __device__ __forceinline__ Acc acc_init(V a, double c) { return a * (float)c; }
  static __device__ __forceinline__ Acc acc_add(Acc s, V a, double c) {
    return __fmaf_rn(a, (float)c, s);
  }
  static __device__ __forceinline__ V acc_fin(Acc s) { return s; }
  static __device__ __forceinline__ V ld(T x) { return x; }
  static __device__ __forceinline__ T st(V v) { return v; }
  static __device__ __forceinline__ V mul(V a, double c) { return a * (float)c; }
  static __device__ __forceinline__ V add(V a, V b) { return a + b; }
  static __device__ __forceinline__ V sub(V a, V b) { return a - b; }
  static __device__ __forceinline__ V madd(V acc, V a, double c) {
    return __fmaf_rn(a, (float)c, acc);
  }
  static __device__ __forceinline__ V half(V a) { return a * 0.5f; }
};

// Element-wise helpers used by all precisions.
template <class P>
__device__ __forceinline__ typename P::V haar_sum(typename P::V a, typename P::V b) {
  return P::mul(P::add(a, b), kInvR2);
}
template <class P>
__device__ __forceinline__ typename P::V haar_dif(typename P::V a, typename P::V b) {
  return P::mul(P::sub(a, b), kInvR2);
}

// Periodic index into a power-of-two length.
__device__ __forceinline__ int64_t wrap(int64_t i, int64_t n) { return i & (n - 1); }

}  // namespace wc
