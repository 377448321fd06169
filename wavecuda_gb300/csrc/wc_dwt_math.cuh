// DWT arithmetic shared by the transform passes (dwt.cu) and the fused
// cross-validation search (cv_fused_kernel.cuh): one analysis step (a pair of
// scaling/detail outputs from L inputs, daub4.cpp:20-56, c6.cpp:32-80,
// la8.cpp:27-80) and one synthesis step (an even/odd output pair from L/2
// scaling and L/2 detail values, daub4.cpp:58-88) in each arithmetic policy,
// every product and sum in the reference's order.
#pragma once

#include <type_traits>

#include "wc_common.cuh"
#include "wc_dd.cuh"
#include "wc_taps2.cuh"

namespace wc {
namespace {

// Two adjacent values p[0], p[1] with one vector shared-memory access (p is
// aligned to two values: every pair below starts at an even index of a
// 16-byte-aligned buffer).
template <class V>
__device__ __forceinline__ void ld2(const V* p, V& a, V& b) {
  if constexpr (std::is_same<V, dd>::value) {
    const float4 t = *reinterpret_cast<const float4*>(p);
    a = dd{t.x, t.y};
    b = dd{t.z, t.w};
  } else if constexpr (std::is_same<V, float>::value) {
    const float2 t = *reinterpret_cast<const float2*>(p);
    a = t.x;
    b = t.y;
  } else {
    const double2 t = *reinterpret_cast<const double2*>(p);
    a = t.x;
    b = t.y;
  }
}

template <class V>
__device__ __forceinline__ void st2(V* p, V a, V b) {
  if constexpr (std::is_same<V, dd>::value) {
    *reinterpret_cast<float4*>(p) = make_float4(a.hi, a.lo, b.hi, b.lo);
  } else if constexpr (std::is_same<V, float>::value) {
    *reinterpret_cast<float2*>(p) = make_float2(a, b);
  } else {
    *reinterpret_cast<double2*>(p) = make_double2(a, b);
  }
}

// Tap pairs of the packed double-float dot products (empty for the other
// policies), loaded once at the start of a kernel from constant memory
// (wc_taps2.cuh): forward (h_j, g_j); inverse (h_2j, h_2j+1) and
// (g_2j, g_2j+1).
struct DwtTapTable {
  TapPairF f[8], ih[4], ig[4];
};
constexpr DwtTapTable dwt_tap_table(int F) {
  DwtTapTable t{};
  for (int j = 0; j < filter_len(F); j++) t.f[j] = tap_pair_f(tap_h(F, j), tap_g(F, j));
  for (int j = 0; j < filter_len(F) / 2; j++) {
    t.ih[j] = tap_pair_f(tap_h(F, 2 * j), tap_h(F, 2 * j + 1));
    t.ig[j] = tap_pair_f(tap_g(F, 2 * j), tap_g(F, 2 * j + 1));
  }
  return t;
}
__constant__ DwtTapTable kDwtTaps[5] = {DwtTapTable{}, dwt_tap_table(1), dwt_tap_table(2),
                                        dwt_tap_table(3), dwt_tap_table(4)};

template <int F, class P>
struct PairTaps {
  __device__ __forceinline__ void init() {}
};
template <int F>
struct PairTaps<F, PDD> {
  static constexpr int L = filter_len(F);
  tap2 f[L], ih[L / 2], ig[L / 2];
  __device__ __forceinline__ void init() {
#pragma unroll
    for (int j = 0; j < L; j++) f[j] = load_tap2(kDwtTaps[F].f[j]);
#pragma unroll
    for (int j = 0; j < L / 2; j++) {
      ih[j] = load_tap2(kDwtTaps[F].ih[j]);
      ig[j] = load_tap2(kDwtTaps[F].ig[j]);
    }
  }
};

template <int F, class P>
__device__ __forceinline__ void fwd_pair(const typename P::V* src, typename P::V& s,
                                         typename P::V& d, const PairTaps<F, P>& tp) {
  using V = typename P::V;
  constexpr int L = filter_len(F);
  V v[L];
#pragma unroll
  for (int j = 0; j < L; j += 2) ld2(src + j, v[j], v[j + 1]);
  if constexpr (F == 1) {
    s = haar_sum<P>(v[0], v[1]);
    d = haar_dif<P>(v[0], v[1]);
  } else if constexpr (std::is_same<P, PDD>::value) {
    // s in lane 0, d in lane 1: the same operations as below, packed.
    // By extraction (wc_dd.cuh); sigma from sum_j |v_j| max(|h_j|, |g_j|).
    float as = 0.f;
#pragma unroll
    for (int j = 0; j < L; j++) as = __fmaf_rn(fabsf(v[j].hi), tap_hg_max(F, j), as);
    const f32x2 sig = extract_sigma(as);
    dd_accx A = accx_init(v[0], tp.f[0], sig);
#pragma unroll
    for (int j = 1; j < L; j++) A = accx_add(A, v[j], tp.f[j], sig);
    accx_fin(A, s, d);
  } else {
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
}

// Inverse step of one pair: even and odd outputs from s[-j] and d[-j]
// (sv/dv in ascending j), taps in descending j as daub4.cpp:58-88.
template <int F, class P>
__device__ __forceinline__ void inv_pair(const typename P::V* sv, const typename P::V* dv,
                                         typename P::V& e, typename P::V& o,
                                         const PairTaps<F, P>& tp) {
  constexpr int HH = filter_len(F) / 2;
  if constexpr (F == 1) {
    e = haar_sum<P>(sv[0], dv[0]);
    o = haar_dif<P>(sv[0], dv[0]);
  } else if constexpr (std::is_same<P, PDD>::value) {
    // e in lane 0, o in lane 1: the same operations as below, packed.
    // By extraction (wc_dd.cuh); sigma from the inputs' |.| times the
    // larger of the two lanes' taps.
    float as = 0.f;
#pragma unroll
    for (int j = 0; j < HH; j++) {
      as = __fmaf_rn(fabsf(sv[j].hi), tap_pair_max(tap_h(F, 2 * j), tap_h(F, 2 * j + 1)), as);
      as = __fmaf_rn(fabsf(dv[j].hi), tap_pair_max(tap_g(F, 2 * j), tap_g(F, 2 * j + 1)), as);
    }
    const f32x2 sig = extract_sigma(as);
    dd_accx A = accx_init(sv[HH - 1], tp.ih[HH - 1], sig);
    A = accx_add(A, dv[HH - 1], tp.ig[HH - 1], sig);
#pragma unroll
    for (int j = HH - 2; j >= 0; j--) {
      A = accx_add(A, sv[j], tp.ih[j], sig);
      A = accx_add(A, dv[j], tp.ig[j], sig);
    }
    accx_fin(A, e, o);
  } else {
    typename P::Acc ae = P::acc_init(sv[HH - 1], tap_h(F, 2 * (HH - 1)));
    typename P::Acc ao = P::acc_init(sv[HH - 1], tap_h(F, 2 * (HH - 1) + 1));
    ae = P::acc_add(ae, dv[HH - 1], tap_g(F, 2 * (HH - 1)));
    ao = P::acc_add(ao, dv[HH - 1], tap_g(F, 2 * (HH - 1) + 1));
#pragma unroll
    for (int j = HH - 2; j >= 0; j--) {
      ae = P::acc_add(ae, sv[j], tap_h(F, 2 * j));
      ao = P::acc_add(ao, sv[j], tap_h(F, 2 * j + 1));
      ae = P::acc_add(ae, dv[j], tap_g(F, 2 * j));
      ao = P::acc_add(ao, dv[j], tap_g(F, 2 * j + 1));
    }
    e = P::acc_fin(ae);
    o = P::acc_fin(ao);
  }
}

}  // namespace
}  // namespace wc
