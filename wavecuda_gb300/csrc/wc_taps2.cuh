// Filter-tap pairs of the packed double-float dot products (wc_dd.cuh) in
// constant memory.
//
// A tap pair built from immediates (make_tap2) is two 32-bit constants that
// the compiler rebuilds with two moves before every packed instruction that
// uses it.  A pair read from a __constant__ table is either kept in
// registers or used directly as a constant-bank operand, which removes those
// moves from the dot products' inner loops.  Each translation unit defines
// its own table of the pairings it uses, built at compile time by
// tap_pair_f (the split of make_tap2: ch = fl32(c), cl = fl32(c - ch),
// stored with the negated copies the packed accumulators take).
#pragma once

#include "wc_common.cuh"
#include "wc_dd.cuh"

namespace wc {

struct alignas(8) TapPairF {
  float ch[2], nch[2], ncl[2];
};

constexpr TapPairF tap_pair_f(double c0, double c1) {
  const float h0 = (float)c0, h1 = (float)c1;
  const float l0 = (float)(c0 - (double)h0), l1 = (float)(c1 - (double)h1);
  return {{h0, h1}, {-h0, -h1}, {-l0, -l1}};
}

__device__ __forceinline__ tap2 load_tap2(const TapPairF& t) {
  return {*reinterpret_cast<const f32x2*>(t.ch), *reinterpret_cast<const f32x2*>(t.nch),
          *reinterpret_cast<const f32x2*>(t.ncl)};
}

}  // namespace wc
