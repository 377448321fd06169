// MODWT arithmetic shared by the transform kernels (modwt.cu) and the fused
// cross-validation search (cv_fused_kernel.cuh): the a-trous analysis and
// synthesis of one output in each arithmetic policy (daub4.cpp:561-589 term
// order) and the row-view tile of the inverse levels.
#pragma once

#include <type_traits>

#include "wc_bulk.cuh"
#include "wc_common.cuh"
#include "wc_dd.cuh"
#include "wc_taps2.cuh"

namespace wc {
namespace {

// Detail values pass through unchanged.
struct NoDMap {
  static constexpr bool kIdentity = true;
  template <class V>
  __device__ __forceinline__ V operator()(V v, int) const {
    return v;
  }
};

// Tap pairs of the packed double-float paths (wc_taps2.cuh): forward
// (g_k, h_k); inverse (h_k, h_k) and (g_k, g_k).
struct ModwtTapTable {
  TapPairF f[8], h[8], g[8];
};
constexpr ModwtTapTable modwt_tap_table(int F) {
  ModwtTapTable t{};
  for (int k = 0; k < filter_len(F); k++) {
    t.f[k] = tap_pair_f(tap_g(F, k), tap_h(F, k));
    t.h[k] = tap_pair_f(tap_h(F, k), tap_h(F, k));
    t.g[k] = tap_pair_f(tap_g(F, k), tap_g(F, k));
  }
  return t;
}
__constant__ ModwtTapTable kModwtTaps[5] = {ModwtTapTable{}, modwt_tap_table(1),
                                            modwt_tap_table(2), modwt_tap_table(3),
                                            modwt_tap_table(4)};

// Forward analysis of one output from taps v[k * stride], k < L.
template <int F, class P>
__device__ __forceinline__ void fwd_taps(const typename P::V* v, int stride, typename P::V& s,
                                         typename P::V& d) {
  if constexpr (F == 1) {
    s = haar_sum<P>(v[0], v[stride]);
    d = haar_dif<P>(v[0], v[stride]);
  } else if constexpr (std::is_same<P, PDD>::value) {
    // d in lane 0, s in lane 1: the same operations as below, packed.
    constexpr int L = filter_len(F);
    dd_acc2 A = acc2_init(v[0], load_tap2(kModwtTaps[F].f[0]));
#pragma unroll
    for (int k = 1; k < L; k++) A = acc2_add(A, v[k * stride], load_tap2(kModwtTaps[F].f[k]));
    acc2_fin(A, d, s);
  } else {
    constexpr int L = filter_len(F);
    typename P::Acc ad = P::acc_init(v[0], tap_g(F, 0));
    typename P::Acc as = P::acc_init(v[0], tap_h(F, 0));
#pragma unroll
    for (int k = 1; k < L; k++) {
      ad = P::acc_add(ad, v[k * stride], tap_g(F, k));
      as = P::acc_add(as, v[k * stride], tap_h(F, k));
    }
    d = P::acc_fin(ad);
    s = P::acc_fin(as);
  }
}

// Inverse synthesis of one output from S[-k * stride], D[-k * stride].
template <int F, class P>
__device__ __forceinline__ typename P::V inv_taps(const typename P::V* S, const typename P::V* D,
                                                   int stride) {
  if constexpr (F == 1) {
    typename P::V acc = P::add(S[0], D[0]);
    acc = P::add(acc, S[-stride]);
    acc = P::sub(acc, D[-stride]);
    return P::mul(acc, kHInvR2);
  } else {
    constexpr int L = filter_len(F);
    typename P::Acc acc;
#pragma unroll
    for (int t = 0; t < L; t++) {
      // even taps L-2, ..., 0 then odd taps L-1, ..., 1
      const int k = (t < L / 2) ? (L - 2 - 2 * t) : (L - 1 - 2 * (t - L / 2));
      if (t == 0) acc = P::acc_init(S[-k * stride], tap_h(F, k));
      else acc = P::acc_add(acc, S[-k * stride], tap_h(F, k));
      acc = P::acc_add(acc, D[-k * stride], tap_g(F, k));
    }
    return P::half(P::acc_fin(acc));
  }
}

// Two adjacent inverse outputs (S, D and S + 1, D + 1) in double-float with
// packed pairs: per lane the operations of inv_taps, so the same bits.
template <int F>
__device__ __forceinline__ void inv_taps2_dd(const dd* S, const dd* D, int stride, dd& r0, dd& r1) {
  constexpr int L = filter_len(F);
  dd_acc2 A;
#pragma unroll
  for (int t = 0; t < L; t++) {
    const int k = (t < L / 2) ? (L - 2 - 2 * t) : (L - 1 - 2 * (t - L / 2));
    const tap2 h = load_tap2(kModwtTaps[F].h[k]), g = load_tap2(kModwtTaps[F].g[k]);
    const dd* s = S - k * stride;
    const dd* d = D - k * stride;
    if (t == 0) A = acc2_init_xy(s[0], s[1], h);
    else A = acc2_add_xy(A, s[0], s[1], h);
    A = acc2_add_xy(A, d[0], d[1], g);
  }
  acc2_fin(A, r0, r1);
  r0 = PDD::half(r0);
  r1 = PDD::half(r1);
}

// Inverse levels l0+NI-1 down to l0 (row unit d0 = 2^l0) of one tile (the
// tile-th C x M block of the row view).  Stop holds the scaling sequence the
// group starts from (s block of level l0+NI-1, or the previous group's
// output); the detail blocks come from xmod, each staged value passed once
// through dmap(value, level) (the identity for a plain inverse, a threshold
// in cross-validation); out receives the group's reconstruction for rows
// m0 .. m0+M-1.  Array row a of the tile is global row m0 - HR + a
// (periodic).  Shared memory: smem_raw, (M + HR) * C * (2 NI) values.  The
// caller synchronises the CTA before reusing smem_raw.
template <int F, class P, int NI, class DMap>
__device__ __forceinline__ void modwt_inv_tile(int64_t tile, const typename P::T* __restrict__ Stop,
                                               const typename P::T* __restrict__ xmod,
                                               typename P::T* __restrict__ out, int64_t n, int l0,
                                               int C, int M, unsigned char* smem_raw,
                                               const DMap& dmap) {
  using V = typename P::V;
  constexpr int L = filter_len(F);
  constexpr int HR = (L - 1) * ((1 << NI) - 1);
  const int R = M + HR;
  V* St = reinterpret_cast<V*>(smem_raw);
  V* Db = St + R * C;           // NI detail tiles
  V* A = Db + NI * R * C;       // intermediates (NI > 1)
  V* B = A + R * C;
  const int64_t d0 = (int64_t)1 << l0, nrows = n >> l0;
  const int64_t nb = d0 / C;
  const int64_t r0 = (tile % nb) * C, m0 = (tile / nb) * M;
  const int cs = __ffs(C) - 1;
  const int tot = R * C;
  // Raw values arrive by per-thread asynchronous copies (every copy of the
  // tile in flight at once), then each thread converts its own in place.
  using T = typename P::T;
  static_assert(sizeof(T) == sizeof(V), "in-place staging");
  T* St_raw = reinterpret_cast<T*>(St);
  T* Db_raw = reinterpret_cast<T*>(Db);
  for (int e = threadIdx.x; e < tot; e += blockDim.x) {
    const int row = e >> cs, c = e & (C - 1);
    const int64_t g = (r0 + c) + ((m0 - HR + row) & (nrows - 1)) * d0;
    cp_async_elem(St_raw + e, Stop + g);
#pragma unroll
    for (int t = 0; t < NI; t++)
      cp_async_elem(Db_raw + t * tot + e, xmod + (int64_t)(2 * (l0 + t) + 1) * n + g);
  }
  cp_async_wait_all();
  if constexpr (!std::is_same<T, V>::value || !DMap::kIdentity) {
    for (int e = threadIdx.x; e < tot; e += blockDim.x) {
      if constexpr (!std::is_same<T, V>::value) St[e] = P::ld(St_raw[e]);
#pragma unroll
      for (int t = 0; t < NI; t++) Db[t * tot + e] = dmap(P::ld(Db_raw[t * tot + e]), l0 + t);
    }
  }
  __syncthreads();
  const V* cur = St;
#pragma unroll
  for (int t = NI - 1; t >= 0; t--) {
    const int rd = 1 << t;
    const int a_lo = HR - (L - 1) * ((1 << t) - 1);
    V* dst = ((NI - 1 - t) & 1) ? B : A;
    const V* Dt = Db + t * tot;
    auto put = [&](int e, V v) {
      if (t == 0) {
        const int row = e >> cs, c = e & (C - 1);
        out[(r0 + c) + (m0 - HR + row) * d0] = P::st(v);
      } else {
        dst[e] = v;
      }
    };
    if constexpr (std::is_same<P, PDD>::value && F != 1) {
      // outputs in adjacent pairs, one packed dot product per pair
      const int e0 = a_lo * C;
      int e = e0 + 2 * (int)threadIdx.x;
      for (; e + 1 < tot; e += 2 * blockDim.x) {
        V v0, v1;
        inv_taps2_dd<F>(cur + e, Dt + e, rd * C, v0, v1);
        put(e, v0);
        put(e + 1, v1);
      }
      if (((tot - e0) & 1) && threadIdx.x == 0) put(tot - 1, inv_taps<F, P>(cur + tot - 1, Dt + tot - 1, rd * C));
    } else {
      for (int e = a_lo * C + threadIdx.x; e < tot; e += blockDim.x)
        put(e, inv_taps<F, P>(cur + e, Dt + e, rd * C));
    }
    if (t > 0) {
      __syncthreads();
      cur = dst;
    }
  }
}

}  // namespace
}  // namespace wc
