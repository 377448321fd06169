// Double-float ("float-float") arithmetic policy for the FP64 data path.
//
// GB300's FP64 pipe is a small fraction of its FP32 rate, so WC_F64_FAST keeps
// the data as FP64 in HBM but computes on the FP32 pipes with unevaluated
// float pairs (hi + lo).  The building blocks are the error-free transforms
// of Dekker (1971) and Knuth (TAOCP vol. 2): TwoSum, FastTwoSum and the
// FMA-based TwoProd; products with a filter tap c use c split at compile time
// into (ch, cl) = (fl32(c), fl32(c - ch)).  A value carries about 48
// significant bits (relative error near 2^-47 per operation), and the
// exponent range is that of FP32: the fast kernels are only used for inputs
// whose magnitudes lie well inside it (see range checks at the ABI).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace wc {

struct dd {
  float hi, lo;
};

__device__ __forceinline__ dd two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

__device__ __forceinline__ dd fast_two_sum(float a, float b) {  // |a| >= |b|
  float s = __fadd_rn(a, b);
  float e = __fsub_rn(b, __fsub_rn(s, a));
  return {s, e};
}

// Exact split of a double into hi = fl32(x) and lo = fl32(x - hi).
__device__ __forceinline__ dd dd_from_double(double x) {
  float hi = __double2float_rn(x);
  float lo = __double2float_rn(x - (double)hi);
  return {hi, lo};
}

__device__ __forceinline__ double dd_to_double(dd v) {
  return (double)v.hi + (double)v.lo;
}

struct PDD {
  using T = double;
  using V = dd;
  static __device__ __forceinline__ V ld(T x) { return dd_from_double(x); }
  static __device__ __forceinline__ T st(V v) { return dd_to_double(v); }
  static __device__ __forceinline__ V mul(V a, double c) {
    const float ch = (float)c;
    const float cl = (float)(c - (double)ch);
    float p = __fmul_rn(a.hi, ch);
    float e = __fmaf_rn(a.hi, ch, -p);
    e = __fmaf_rn(a.hi, cl, e);
    e = __fmaf_rn(a.lo, ch, e);
    return fast_two_sum(p, e);
  }
  static __device__ __forceinline__ V add(V a, V b) {
    dd s = two_sum(a.hi, b.hi);
    float e = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
    return fast_two_sum(s.hi, e);
  }
  static __device__ __forceinline__ V sub(V a, V b) { return add(a, {-b.hi, -b.lo}); }
  static __device__ __forceinline__ V madd(V acc, V a, double c) { return add(acc, mul(a, c)); }
  static __device__ __forceinline__ V half(V a) { return {a.hi * 0.5f, a.lo * 0.5f}; }
};

}  // namespace wc
