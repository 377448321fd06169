// Vectorised row-view tiles of the time-ordered MODWT (modwt.cu).
//
// The scalar tiles (wc_modwt_math.cuh) move one value per instruction: one
// 4- or 8-byte asynchronous copy per staged value, one shared-memory load
// per tap and one global store per output, each with its own 64-bit address
// arithmetic.  On a GB300 that makes the FP32 inverse issue-bound (ncu at
// n = 2^24: 80 % issue active, 44 % DRAM throughput).  Here every copy, load
// and store moves 16 bytes: a thread owns W = 16 / sizeof(T) consecutive
// values of the flattened tile (four FP32 values, two FP64 or double-float
// values), which are W adjacent columns of one row when C >= W, or W
// consecutive rows when the tile has a single column (C == 1, the finest
// level, whose row-view sequence is the signal itself).
//
// Each of the W outputs is computed with exactly the operations of the
// scalar tile (the reference's term order, daub4.cpp:578-582), so results
// are bit-identical to it in every precision.  Double-float values are kept
// in shared memory as "pair" chunks {hi_a, hi_b, lo_a, lo_b} of two adjacent
// values, which are the packed operands of the two-lane dot products
// (wc_dd.cuh) as loaded: no register moves to assemble them.
//
// Halo: C >= W tiles use the scalar tile's (L-1)(2^NI - 1) rows.  A C == 1
// tile rounds every level's first output down to a multiple of W and reads a
// window of whole chunks around each output group, so it stages
// mvec_inv_halo() rows: the exact halo plus 2(W-1), rounded up to a multiple
// of W (every read stays inside the tile; outputs below a level's exact start
// are garbage that no kept output reads).
#pragma once

#include <type_traits>

#include "wc_bulk.cuh"
#include "wc_common.cuh"
#include "wc_dd.cuh"
#include "wc_modwt_math.cuh"

namespace wc {
namespace {

__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gsrc) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(smem_dst)), "l"(gsrc)
               : "memory");
}

// Values per 16-byte chunk of the memory type.
template <class P>
__host__ __device__ constexpr int mvec_w() {
  return 16 / (int)sizeof(typename P::T);
}

// Halo rows of a vectorised inverse tile of NI levels (see the file comment).
__host__ __device__ constexpr int mvec_inv_halo(int L, int NI, int C, int W) {
  const int hr = (L - 1) * ((1 << NI) - 1);
  return C >= W ? hr : ((hr + 2 * (W - 1) + W - 1) / W) * W;
}

// Arrays of an inverse tile: the scaling tile, NI detail tiles and the
// intermediates (one for NI == 2, two alternating for NI >= 3).
__host__ __device__ constexpr int mvec_inv_arrays(int NI) {
  return NI + 1 + (NI - 1 < 2 ? NI - 1 : 2);
}

// Whether the vectorised tile applies: C == 1 or C a multiple of W, and at
// least W rows per tile.
__host__ __device__ constexpr bool mvec_ok(int C, int M, int W) {
  return (C == 1 || C % W == 0) && M >= W && M % W == 0;
}

template <class T>
struct alignas(16) Chunk {
  T v[16 / sizeof(T)];
};
struct alignas(16) PairChunk {
  f32x2 hi, lo;  // {hi_a, hi_b}, {lo_a, lo_b}
};

// Two-lane Dot2 steps on packed operands (acc2_*_xy of wc_dd.cuh with the
// hi and lo pairs given directly): the same operations, so the same bits.
__device__ __forceinline__ dd_acc2 acc2_init_p(f32x2 ah, f32x2 al, const tap2& c) {
  const f32x2 p = x2_mul(ah, c.ch);
  f32x2 ne = x2_fma(ah, c.nch, p);
  ne = x2_fma(ah, c.ncl, ne);
  ne = x2_fma(al, c.nch, ne);
  return {p, ne};
}
__device__ __forceinline__ dd_acc2 acc2_add_p(dd_acc2 A, f32x2 ah, f32x2 al, const tap2& c) {
  const f32x2 p = x2_mul(ah, c.ch);
  f32x2 npe = x2_fma(ah, c.nch, p);
  npe = x2_fma(ah, c.ncl, npe);
  npe = x2_fma(al, c.nch, npe);
  const f32x2 s = x2_add(A.s, p);
  const f32x2 bb = x2_sub(s, A.s);
  const f32x2 t = x2_add(x2_sub(A.s, x2_sub(s, bb)), x2_sub(p, bb));
  return {s, x2_add(A.ne, x2_sub(npe, t))};
}
// acc2_fin with the result left packed: hi = {hi_0, hi_1}, lo = {lo_0, lo_1}.
__device__ __forceinline__ void acc2_fin_p(dd_acc2 A, f32x2& hi, f32x2& lo) {
  hi = x2_sub(A.s, A.ne);
  const f32x2 bb = x2_sub(hi, A.s);
  lo = x2_sub(x2_sub(A.s, x2_sub(hi, bb)), x2_add(A.ne, bb));
}

// Inverse term order of the reference: even taps L-2, ..., 0, then odd taps
// L-1, ..., 1 (daub4.cpp:578-582).
__host__ __device__ constexpr int inv_k(int L, int t) {
  return (t < L / 2) ? (L - 2 - 2 * t) : (L - 1 - 2 * (t - L / 2));
}

// ---------------------------------------------------------------- FP32/FP64
// The W values of tap k of an output group starting at element e: chunk
// e - k*stride (aligned: stride a multiple of W) or, for a single-column
// tile with tap distance RD < W, the values of a window of whole chunks.
template <class P, int L, int RD>
struct Gather {
  static constexpr int W = mvec_w<P>();
  static constexpr int kBack = RD ? ((L - 1) * RD + W - 1) / W : 0;
  typename P::T w[(kBack + 1) * W];
  __device__ __forceinline__ void load(const typename P::T* X, int e) {
#pragma unroll
    for (int j = 0; j <= kBack; j++) {
      const Chunk<typename P::T> c =
          *reinterpret_cast<const Chunk<typename P::T>*>(X + e - (kBack - j) * W);
#pragma unroll
      for (int i = 0; i < W; i++) w[j * W + i] = c.v[i];
    }
  }
  __device__ __forceinline__ typename P::T at(int k, int i) const { return w[kBack * W + i - k * RD]; }
};

// One inverse output group (W values) of level tap distance `stride`
// (elements; RD > 0: single column, stride == RD), from cur (scaling) and
// Dt (details), exactly as inv_taps<F, P> per value.
template <int F, class P, int RD>
__device__ __forceinline__ void inv_group(const typename P::V* cur, const typename P::V* Dt, int e,
                                          int stride, typename P::V (&o)[mvec_w<P>()]) {
  using V = typename P::V;
  using T = typename P::T;
  constexpr int L = filter_len(F);
  constexpr int W = mvec_w<P>();
  const T* S = reinterpret_cast<const T*>(cur);
  const T* D = reinterpret_cast<const T*>(Dt);
  if constexpr (RD) {
    Gather<P, L, RD> gs, gd;
    gs.load(S, e);
    gd.load(D, e);
    if constexpr (F == 1) {
#pragma unroll
      for (int i = 0; i < W; i++) {
        V acc = P::add(gs.at(0, i), gd.at(0, i));
        acc = P::add(acc, gs.at(1, i));
        acc = P::sub(acc, gd.at(1, i));
        o[i] = P::mul(acc, kHInvR2);
      }
    } else {
      typename P::Acc acc[W];
#pragma unroll
      for (int t = 0; t < L; t++) {
        const int k = inv_k(L, t);
#pragma unroll
        for (int i = 0; i < W; i++) {
          acc[i] = (t == 0) ? P::acc_init(gs.at(k, i), tap_h(F, k))
                            : P::acc_add(acc[i], gs.at(k, i), tap_h(F, k));
          acc[i] = P::acc_add(acc[i], gd.at(k, i), tap_g(F, k));
        }
      }
#pragma unroll
      for (int i = 0; i < W; i++) o[i] = P::half(P::acc_fin(acc[i]));
    }
  } else {
    using Ch = Chunk<T>;
    if constexpr (F == 1) {
      const Ch s0 = *reinterpret_cast<const Ch*>(S + e), d0 = *reinterpret_cast<const Ch*>(D + e);
      const Ch s1 = *reinterpret_cast<const Ch*>(S + e - stride);
      const Ch d1 = *reinterpret_cast<const Ch*>(D + e - stride);
#pragma unroll
      for (int i = 0; i < W; i++) {
        V acc = P::add(s0.v[i], d0.v[i]);
        acc = P::add(acc, s1.v[i]);
        acc = P::sub(acc, d1.v[i]);
        o[i] = P::mul(acc, kHInvR2);
      }
    } else {
      typename P::Acc acc[W];
#pragma unroll
      for (int t = 0; t < L; t++) {
        const int k = inv_k(L, t);
        const Ch s = *reinterpret_cast<const Ch*>(S + e - k * stride);
        const Ch d = *reinterpret_cast<const Ch*>(D + e - k * stride);
#pragma unroll
        for (int i = 0; i < W; i++) {
          acc[i] = (t == 0) ? P::acc_init(s.v[i], tap_h(F, k)) : P::acc_add(acc[i], s.v[i], tap_h(F, k));
          acc[i] = P::acc_add(acc[i], d.v[i], tap_g(F, k));
        }
      }
#pragma unroll
      for (int i = 0; i < W; i++) o[i] = P::half(P::acc_fin(acc[i]));
    }
  }
}

// ------------------------------------------------------------ double-float
// Packed operands of values (j, j+1) of a pair-chunk array X (j even: one
// chunk; j odd: lanes of two chunks).
template <bool ODD>
__device__ __forceinline__ void pair_at(const PairChunk* X, int j, f32x2& hi, f32x2& lo) {
  if constexpr (!ODD) {
    const PairChunk c = X[j >> 1];
    hi = c.hi;
    lo = c.lo;
  } else {
    const PairChunk a = X[j >> 1], b = X[(j >> 1) + 1];
    float ah0, ah1, al0, al1, bh0, bh1, bl0, bl1;
    x2_unpack(a.hi, ah0, ah1);
    x2_unpack(a.lo, al0, al1);
    x2_unpack(b.hi, bh0, bh1);
    x2_unpack(b.lo, bl0, bl1);
    hi = x2_pack(ah1, bh0);
    lo = x2_pack(al1, bl0);
  }
}

__device__ __forceinline__ dd pc_lane(const PairChunk& c, int i) {
  float h0, h1, l0, l1;
  x2_unpack(c.hi, h0, h1);
  x2_unpack(c.lo, l0, l1);
  return i ? dd{h1, l1} : dd{h0, l0};
}

// One double-float inverse output pair (values e, e+1; e even) as
// inv_taps2_dd (F > 1) or inv_taps<F, PDD> per value (Haar).
template <int F, int RD>
__device__ __forceinline__ void inv_group_dd(const PairChunk* S, const PairChunk* D, int e,
                                             int stride, f32x2& hi, f32x2& lo) {
  constexpr int L = filter_len(F);
  if constexpr (F == 1) {
    // stride is even unless RD == 1
    const PairChunk s0 = S[e >> 1], d0 = D[e >> 1];
    f32x2 s1h, s1l, d1h, d1l;
    if constexpr (RD == 1) {
      pair_at<true>(S, e - 1, s1h, s1l);
      pair_at<true>(D, e - 1, d1h, d1l);
    } else {
      pair_at<false>(S, e - stride, s1h, s1l);
      pair_at<false>(D, e - stride, d1h, d1l);
    }
    const PairChunk s1{s1h, s1l}, d1{d1h, d1l};
    dd r[2];
#pragma unroll
    for (int i = 0; i < 2; i++) {
      dd acc = PDD::add(pc_lane(s0, i), pc_lane(d0, i));
      acc = PDD::add(acc, pc_lane(s1, i));
      acc = PDD::sub(acc, pc_lane(d1, i));
      r[i] = PDD::mul(acc, kHInvR2);
    }
    hi = x2_pack(r[0].hi, r[1].hi);
    lo = x2_pack(r[0].lo, r[1].lo);
  } else {
    dd_acc2 A;
#pragma unroll
    for (int t = 0; t < L; t++) {
      const int k = inv_k(L, t);
      const tap2 h = load_tap2(kModwtTaps[F].h[k]), g = load_tap2(kModwtTaps[F].g[k]);
      f32x2 sh, sl, dh, dl;
      if constexpr (RD == 1) {
        if (k & 1) {
          pair_at<true>(S, e - k, sh, sl);
          pair_at<true>(D, e - k, dh, dl);
        } else {
          pair_at<false>(S, e - k, sh, sl);
          pair_at<false>(D, e - k, dh, dl);
        }
      } else {
        pair_at<false>(S, e - k * stride, sh, sl);
        pair_at<false>(D, e - k * stride, dh, dl);
      }
      A = (t == 0) ? acc2_init_p(sh, sl, h) : acc2_add_p(A, sh, sl, h);
      A = acc2_add_p(A, dh, dl, g);
    }
    acc2_fin_p(A, hi, lo);
    const f32x2 half2 = x2_pack(0.5f, 0.5f);
    hi = x2_mul(hi, half2);
    lo = x2_mul(lo, half2);
  }
}

// Converts the calling thread's raw FP64 chunk (two values) at X[j] into a
// pair chunk in place.
__device__ __forceinline__ void to_pair_chunk(unsigned char* X, int j) {
  double2 v = reinterpret_cast<const double2*>(X)[j];
  const dd a = dd_from_double(v.x), b = dd_from_double(v.y);
  reinterpret_cast<PairChunk*>(X)[j] = PairChunk{x2_pack(a.hi, b.hi), x2_pack(a.lo, b.lo)};
}

// --------------------------------------------------------------- the tile
// Inverse levels l0+NI-1 down to l0 of one C x M tile (HRp halo rows,
// mvec_inv_halo) of the row view with unit d0 = 2^l0, as modwt_inv_tile but
// vectorised.  Stop, xmod and out must be 16-byte aligned.  Shared memory:
// (M + HRp) * C * mvec_inv_arrays(NI) values.
template <int F, class P, int NI>
struct InvVecTile {
  using T = typename P::T;
  using V = typename P::V;
  static constexpr int L = filter_len(F);
  static constexpr int W = mvec_w<P>();
  static constexpr bool kDD = std::is_same<P, PDD>::value;

  const T* __restrict__ xmod;
  T* __restrict__ out;
  int64_t n, d0, nrows, r0, m0;
  int C, cs, HRp, R, tot;
  unsigned char* sm;

  __device__ __forceinline__ unsigned char* arr(int a) const {
    return sm + (size_t)a * tot * sizeof(T);
  }

  template <int t>
  __device__ __forceinline__ void level() {
    constexpr int rd = 1 << t;
    // arrays: 0 St, 1..NI details, NI+1 A, NI+2 B
    constexpr int src_a = (t == NI - 1) ? 0 : ((((NI - 2 - t) & 1) ? NI + 2 : NI + 1));
    constexpr int dst_a = ((NI - 1 - t) & 1) ? NI + 2 : NI + 1;
    const int a_lo = HRp - (L - 1) * (rd - 1);
    const int e0 = (a_lo * C) & ~(W - 1);
    const int stride = rd * C;
    const unsigned char* S = arr(src_a);
    const unsigned char* D = arr(1 + t);
    unsigned char* Dst = arr(dst_a);
    if constexpr (rd < W) {
      if (C == 1) {
        run<t, rd>(S, D, Dst, e0, stride);
        return;
      }
    }
    run<t, 0>(S, D, Dst, e0, stride);
  }

  template <int t, int RD>
  __device__ __forceinline__ void run(const unsigned char* S, const unsigned char* D,
                                      unsigned char* Dst, int e0, int stride) {
    for (int e = e0 + (int)threadIdx.x * W; e < tot; e += (int)blockDim.x * W) {
      if constexpr (kDD) {
        f32x2 hi, lo;
        inv_group_dd<F, RD>(reinterpret_cast<const PairChunk*>(S),
                            reinterpret_cast<const PairChunk*>(D), e, stride, hi, lo);
        if constexpr (t == 0) {
          float h0, h1, l0, l1;
          x2_unpack(hi, h0, h1);
          x2_unpack(lo, l0, l1);
          const double2 v = make_double2(dd_to_double(dd{h0, l0}), dd_to_double(dd{h1, l1}));
          *reinterpret_cast<double2*>(out + gaddr(e)) = v;
        } else {
          reinterpret_cast<PairChunk*>(Dst)[e >> 1] = PairChunk{hi, lo};
        }
      } else {
        V o[W];
        inv_group<F, P, RD>(reinterpret_cast<const V*>(S), reinterpret_cast<const V*>(D), e,
                            stride, o);
        Chunk<T> c;
#pragma unroll
        for (int i = 0; i < W; i++) c.v[i] = o[i];
        if constexpr (t == 0) {
          *reinterpret_cast<Chunk<T>*>(out + gaddr(e)) = c;
        } else {
          reinterpret_cast<Chunk<T>*>(Dst)[e / W] = c;
        }
      }
    }
  }

  // Global index of tile element e (a kept output row: no wrap).
  __device__ __forceinline__ int64_t gaddr(int e) const {
    const int row = e >> cs, c = e & (C - 1);
    return (r0 + c) + (m0 - HRp + row) * d0;
  }

  template <int t>
  __device__ __forceinline__ void levels() {
    level<t>();
    if constexpr (t > 0) {
      __syncthreads();
      levels<t - 1>();
    }
  }

  __device__ __forceinline__ void run_tile(int64_t tile, const T* __restrict__ Stop) {
    const int64_t nb = d0 / C;
    r0 = (tile % nb) * C;
    m0 = (tile / nb) * M_;
    const int totc = tot / W;
    for (int j = threadIdx.x; j < totc; j += blockDim.x) {
      const int e = j * W;
      const int row = e >> cs, c = e & (C - 1);
      const int64_t g = (r0 + c) + ((m0 - HRp + row) & (nrows - 1)) * d0;
      cp_async16(arr(0) + (size_t)e * sizeof(T), Stop + g);
#pragma unroll
      for (int t = 0; t < NI; t++)
        cp_async16(arr(1 + t) + (size_t)e * sizeof(T), xmod + (int64_t)(2 * (l0_ + t) + 1) * n + g);
    }
    cp_async_wait_all();
    if constexpr (kDD) {
      for (int j = threadIdx.x; j < totc; j += blockDim.x) {
#pragma unroll
        for (int a = 0; a <= NI; a++) to_pair_chunk(arr(a), j);
      }
    }
    __syncthreads();
    levels<NI - 1>();
  }

  int M_, l0_;
};

template <int F, class P, int NI>
__global__ void __launch_bounds__(256)
modwt_inv_vec(const typename P::T* __restrict__ Stop, const typename P::T* __restrict__ xmod,
              typename P::T* __restrict__ out, int64_t n, int l0, int C, int M, int HRp) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  InvVecTile<F, P, NI> tl;
  tl.xmod = xmod;
  tl.out = out;
  tl.n = n;
  tl.d0 = (int64_t)1 << l0;
  tl.nrows = n >> l0;
  tl.C = C;
  tl.cs = __ffs(C) - 1;
  tl.HRp = HRp;
  tl.R = M + HRp;
  tl.tot = tl.R * C;
  tl.sm = smem_raw;
  tl.M_ = M;
  tl.l0_ = l0;
  tl.run_tile(blockIdx.x, Stop);
}

// ------------------------------------------------------------ forward
// Forward levels l0 .. l0+NF-1 of one C x M tile, as modwt_fwd_tiled but
// vectorised and with up to three fused levels.  Level t of the group (taps
// 2^t rows apart) needs its input on rows 0 .. M + H_t - 1 of the tile,
// H_t = (L-1)(2^NF - 2^t) rows of halo below the kept rows (computed
// redundantly, as the scalar tile does).  A single-column tile rounds each
// level's row counts up to whole chunks (mvec_fwd_rows).
//
// Rows of level t's input held by a tile (t = NF: the last level's output
// rows, i.e. M).
__host__ __device__ constexpr int mvec_fwd_rows(int L, int NF, int t, int M, int C, int W) {
  int out = M;  // rows the last level produces
  for (int u = NF - 1; u >= t; u--) {
    const int rd = 1 << u;
    int in = out + (L - 1) * rd;
    if (C < W) in = ((in + W - 1) / W) * W;
    if (u == t) return in;
    out = in;
  }
  return M;
}
// Shared memory of a forward tile in values: the staged input and, for NF >=
// 2, the intermediate scaling rows of levels 0 and 1.
__host__ __device__ constexpr int mvec_fwd_values(int L, int NF, int M, int C, int W) {
  return C * (mvec_fwd_rows(L, NF, 0, M, C, W) + (NF >= 2 ? mvec_fwd_rows(L, NF, 1, M, C, W) : 0) +
              (NF >= 3 ? mvec_fwd_rows(L, NF, 2, M, C, W) : 0));
}

// The W values of tap k (rows below) of an output group starting at element
// e, for the forward: chunk e + k*stride, or a window of whole chunks from e
// on for a single-column tile with tap distance RD < W.
template <class P, int L, int RD>
struct GatherF {
  static constexpr int W = mvec_w<P>();
  static constexpr int kFwd = RD ? ((L - 1) * RD + W - 1) / W : 0;
  typename P::T w[(kFwd + 1) * W];
  __device__ __forceinline__ void load(const typename P::T* X, int e) {
#pragma unroll
    for (int j = 0; j <= kFwd; j++) {
      const Chunk<typename P::T> c = *reinterpret_cast<const Chunk<typename P::T>*>(X + e + j * W);
#pragma unroll
      for (int i = 0; i < W; i++) w[j * W + i] = c.v[i];
    }
  }
  __device__ __forceinline__ typename P::T at(int k, int i) const { return w[i + k * RD]; }
};

// One forward output group: s and d of W values, exactly as fwd_taps<F, P>
// per value.
template <int F, class P, int RD>
__device__ __forceinline__ void fwd_group(const typename P::T* X, int e, int stride,
                                          typename P::V (&s)[mvec_w<P>()],
                                          typename P::V (&d)[mvec_w<P>()]) {
  using T = typename P::T;
  constexpr int L = filter_len(F);
  constexpr int W = mvec_w<P>();
  T v[L][W];
  if constexpr (RD) {
    GatherF<P, L, RD> gw;
    gw.load(X, e);
#pragma unroll
    for (int k = 0; k < L; k++)
#pragma unroll
      for (int i = 0; i < W; i++) v[k][i] = gw.at(k, i);
  } else {
#pragma unroll
    for (int k = 0; k < L; k++) {
      const Chunk<T> c = *reinterpret_cast<const Chunk<T>*>(X + e + k * stride);
#pragma unroll
      for (int i = 0; i < W; i++) v[k][i] = c.v[i];
    }
  }
#pragma unroll
  for (int i = 0; i < W; i++) {
    if constexpr (F == 1) {
      s[i] = haar_sum<P>(v[0][i], v[1][i]);
      d[i] = haar_dif<P>(v[0][i], v[1][i]);
    } else {
      typename P::Acc ad = P::acc_init(v[0][i], tap_g(F, 0));
      typename P::Acc as = P::acc_init(v[0][i], tap_h(F, 0));
#pragma unroll
      for (int k = 1; k < L; k++) {
        ad = P::acc_add(ad, v[k][i], tap_g(F, k));
        as = P::acc_add(as, v[k][i], tap_h(F, k));
      }
      d[i] = P::acc_fin(ad);
      s[i] = P::acc_fin(as);
    }
  }
}

// Double-float forward group (values e, e+1): per value the operations of
// fwd_taps<F, PDD> (one two-lane Dot2 per output kind, lanes = the two
// values); Haar per value with the scalar double-float operations.
template <int F, int RD>
__device__ __forceinline__ void fwd_group_dd(const PairChunk* X, int e, int stride, f32x2& sh,
                                             f32x2& sl, f32x2& dh, f32x2& dl) {
  constexpr int L = filter_len(F);
  if constexpr (F == 1) {
    const PairChunk a = X[e >> 1];
    f32x2 bh, bl;
    if constexpr (RD == 1) pair_at<true>(X, e + 1, bh, bl);
    else pair_at<false>(X, e + stride, bh, bl);
    const PairChunk b{bh, bl};
    dd rs[2], rdv[2];
#pragma unroll
    for (int i = 0; i < 2; i++) {
      rs[i] = haar_sum<PDD>(pc_lane(a, i), pc_lane(b, i));
      rdv[i] = haar_dif<PDD>(pc_lane(a, i), pc_lane(b, i));
    }
    sh = x2_pack(rs[0].hi, rs[1].hi);
    sl = x2_pack(rs[0].lo, rs[1].lo);
    dh = x2_pack(rdv[0].hi, rdv[1].hi);
    dl = x2_pack(rdv[0].lo, rdv[1].lo);
  } else {
    dd_acc2 As, Ad;
#pragma unroll
    for (int k = 0; k < L; k++) {
      const tap2 h = load_tap2(kModwtTaps[F].h[k]), g = load_tap2(kModwtTaps[F].g[k]);
      f32x2 ah, al;
      if constexpr (RD == 1) {
        if (k & 1) pair_at<true>(X, e + k, ah, al);
        else pair_at<false>(X, e + k, ah, al);
      } else {
        pair_at<false>(X, e + k * stride, ah, al);
      }
      if (k == 0) {
        Ad = acc2_init_p(ah, al, g);
        As = acc2_init_p(ah, al, h);
      } else {
        Ad = acc2_add_p(Ad, ah, al, g);
        As = acc2_add_p(As, ah, al, h);
      }
    }
    acc2_fin_p(Ad, dh, dl);
    acc2_fin_p(As, sh, sl);
  }
}

template <int F, class P, int NF>
struct FwdVecTile {
  using T = typename P::T;
  using V = typename P::V;
  static constexpr int L = filter_len(F);
  static constexpr int W = mvec_w<P>();
  static constexpr bool kDD = std::is_same<P, PDD>::value;

  T* __restrict__ xmod;
  int64_t n, d0, nrows, r0, m0;
  int C, cs, M, l0;
  unsigned char* sm;
  int rows[4];  // input rows of level t (rows[NF] = M)

  __device__ __forceinline__ unsigned char* buf(int b) const {
    // b = 0: staged input; 1: level-0 scaling rows; 2: level-1 scaling rows
    size_t off = 0;
    for (int u = 0; u < b; u++) off += (size_t)rows[u] * C;
    return sm + off * sizeof(T);
  }

  __device__ __forceinline__ void store_out(int t, int e, const T (&sv)[W], const T (&dv)[W]) {
    const int row = e >> cs, c = e & (C - 1);
    const int64_t g = (r0 + c) + (m0 + row) * d0;
    T* S = xmod + (int64_t)2 * (l0 + t) * n;
    Chunk<T> a, b;
#pragma unroll
    for (int i = 0; i < W; i++) {
      a.v[i] = sv[i];
      b.v[i] = dv[i];
    }
    *reinterpret_cast<Chunk<T>*>(S + g) = a;
    *reinterpret_cast<Chunk<T>*>(S + n + g) = b;
  }

  template <int t, int RD>
  __device__ __forceinline__ void run(const unsigned char* X, unsigned char* Dst, int stride) {
    const int nout = rows[t + 1] * C;  // values level t produces
    const int keep = M * C;            // values that go to HBM
    for (int e = (int)threadIdx.x * W; e < nout; e += (int)blockDim.x * W) {
      if constexpr (kDD) {
        f32x2 sh, sl, dh, dl;
        fwd_group_dd<F, RD>(reinterpret_cast<const PairChunk*>(X), e, stride, sh, sl, dh, dl);
        if (e < keep) {
          float s0h, s1h, s0l, s1l, d0h, d1h, d0l, d1l;
          x2_unpack(sh, s0h, s1h);
          x2_unpack(sl, s0l, s1l);
          x2_unpack(dh, d0h, d1h);
          x2_unpack(dl, d0l, d1l);
          const double sv[2] = {dd_to_double(dd{s0h, s0l}), dd_to_double(dd{s1h, s1l})};
          const double dv[2] = {dd_to_double(dd{d0h, d0l}), dd_to_double(dd{d1h, d1l})};
          store_out(t, e, sv, dv);
        }
        if constexpr (t < NF - 1) reinterpret_cast<PairChunk*>(Dst)[e >> 1] = PairChunk{sh, sl};
      } else {
        V s[W], d[W];
        fwd_group<F, P, RD>(reinterpret_cast<const T*>(X), e, stride, s, d);
        if (e < keep) store_out(t, e, s, d);
        if constexpr (t < NF - 1) {
          Chunk<T> c;
#pragma unroll
          for (int i = 0; i < W; i++) c.v[i] = s[i];
          reinterpret_cast<Chunk<T>*>(Dst)[e / W] = c;
        }
      }
    }
  }

  template <int t>
  __device__ __forceinline__ void level() {
    constexpr int rd = 1 << t;
    const unsigned char* X = buf(t == 0 ? 0 : (t == 1 ? 1 : 2));
    unsigned char* Dst = buf(t == 0 ? 1 : 2);
    const int stride = rd * C;
    if constexpr (rd < W) {
      if (C == 1) {
        run<t, rd>(X, Dst, stride);
        return;
      }
    }
    run<t, 0>(X, Dst, stride);
  }

  template <int t>
  __device__ __forceinline__ void levels() {
    level<t>();
    if constexpr (t + 1 < NF) {
      __syncthreads();
      levels<t + 1>();
    }
  }

  __device__ __forceinline__ void run_tile(int64_t tile, const T* __restrict__ X) {
    const int64_t nb = d0 / C;
    r0 = (tile % nb) * C;
    m0 = (tile / nb) * M;
    const int totc = rows[0] * C / W;
    for (int j = threadIdx.x; j < totc; j += blockDim.x) {
      const int e = j * W;
      const int row = e >> cs, c = e & (C - 1);
      const int64_t g = (r0 + c) + ((m0 + row) & (nrows - 1)) * d0;
      cp_async16(buf(0) + (size_t)e * sizeof(T), X + g);
    }
    cp_async_wait_all();
    if constexpr (kDD) {
      for (int j = threadIdx.x; j < totc; j += blockDim.x) to_pair_chunk(buf(0), j);
    }
    __syncthreads();
    levels<0>();
  }
};

template <int F, class P, int NF>
__global__ void __launch_bounds__(256)
modwt_fwd_vec(const typename P::T* __restrict__ X, typename P::T* __restrict__ xmod, int64_t n,
              int l0, int C, int M) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int L = filter_len(F), W = mvec_w<P>();
  FwdVecTile<F, P, NF> tl;
  tl.xmod = xmod;
  tl.n = n;
  tl.d0 = (int64_t)1 << l0;
  tl.nrows = n >> l0;
  tl.C = C;
  tl.cs = __ffs(C) - 1;
  tl.M = M;
  tl.l0 = l0;
  tl.sm = smem_raw;
#pragma unroll
  for (int t = 0; t < 4; t++) tl.rows[t] = t <= NF ? mvec_fwd_rows(L, NF, t, M, C, W) : 0;
  tl.run_tile(blockIdx.x, X);
}

}  // namespace
}  // namespace wc
