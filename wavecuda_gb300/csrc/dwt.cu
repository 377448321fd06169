// Periodic DWT (Haar, D4, C6, LA8), forward and inverse, in the reference's
// interleaved layout (haar.cpp:9-30) with the reference's convolution
// alignment (daub4.cpp:20-88, c6.cpp:32-111, la8.cpp:27-115, haar.cpp:47-93).
//
// Design.  A transform of J levels runs as a few "passes"; a pass applies G
// consecutive levels to a compact sequence y (length N) whose elements sit at
// stride S in the interleaved array.  One CTA owns a tile of Tt consecutive
// y values plus the periodic halo its G levels need, keeps every level's
// intermediate in shared memory, assembles the tile's interleaved result in
// shared memory and writes it back with one coalesced sweep.  The tile's
// level-G scaling coefficients also go, compact, to a scratch array that the
// next pass reads contiguously; the last pass handles the short coarse tail
// in a single CTA.  The inverse runs the same passes in reverse order.
//
// Forward halo: a level-l scaling value at index k reads level l-1 values
// 2k .. 2k+L-1, so G fused levels need H_0 = (L-2)(2^G - 1) values to the
// right of the tile (computed redundantly; G is chosen per filter to keep
// this near a tenth of the tile).  Inverse halo: an output pair q reads
// (s,d)[q-j], j < L/2, so the left halo is need_l = ceil(need_{l-1}/2) + L/2-1
// coefficients at level l.
#include <algorithm>
#include <mutex>
#include <type_traits>
#include <vector>

#include "wc_bulk.cuh"
#include "wc_common.cuh"
#include "wc_dd.cuh"
#include "wc_taps2.cuh"
#include "wc_dwt_math.cuh"

namespace wc {
namespace {

constexpr int kThreads = 256;

// Element counts rounded up to a 16-byte multiple (bulk-copy granularity and
// alignment of the shared-memory regions).
template <class X>
__host__ __device__ constexpr int64_t pad16(int64_t n) {
  constexpr int64_t k = 16 / (int64_t)sizeof(X) > 0 ? 16 / (int64_t)sizeof(X) : 1;
  return ((n + k - 1) / k) * k;
}

// Right halo of the forward pass at level l of G (in level-l values).
__host__ __device__ constexpr int64_t fwd_halo(int L, int G, int l) {
  return (int64_t)(L - 2) * (((int64_t)1 << (G - l)) - 1);
}

// Forward pass.  y[m] = in[m] (m < N, compact).  Writes the tile's
// interleaved result to out[(t0+m)*S] and its level-G scaling values to
// coarse[t0/2^G + k] (when coarse != nullptr).  With bit 0 of `bulk` set,
// the tile and its halo arrive by bulk copies (one or two: the halo of the
// last tile wraps to the start); with bit 1 set and S == 1, the result leaves
// by one bulk store (plain stores otherwise, e.g. into host memory).  Block b
// handles tile tile0 + b.
template <int F, class P>
__global__ void __launch_bounds__(kThreads)
dwt_fwd_pass(const typename P::T* __restrict__ in, int64_t N, int G, int64_t Tt,
             typename P::T* __restrict__ out, int64_t S,
             typename P::T* __restrict__ coarse, int write_coarse_slots, int bulk,
             unsigned int* status, int64_t tile0) {
  using V = typename P::V;
  PairTaps<F, P> tp;
  tp.init();
  using T = typename P::T;
  constexpr int L = filter_len(F);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar;
  const int64_t H0 = pad16<T>(fwd_halo(L, G, 0));
  V* A = reinterpret_cast<V*>(smem_raw);
  V* B = A + pad16<V>(Tt + H0);
  V* Z = B + pad16<V>(Tt / 2 + fwd_halo(L, G, 1));
  const int64_t t0 = (tile0 + (int64_t)blockIdx.x) * Tt;

  if (bulk & 1) {
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
      mbar_expect_tx(&bar, (uint32_t)((Tt + H0) * sizeof(T)));
      if (t0 + Tt + H0 <= N) {
        bulk_g2s(A, in + t0, (uint32_t)((Tt + H0) * sizeof(T)), &bar);
      } else {
        bulk_g2s(A, in + t0, (uint32_t)(Tt * sizeof(T)), &bar);
        if (H0 > 0) bulk_g2s(reinterpret_cast<T*>(A) + Tt, in, (uint32_t)(H0 * sizeof(T)), &bar);
      }
    }
    const bool ok = mbar_wait(&bar, 0, status);
    if (__syncthreads_or(!ok)) return;
    if constexpr (!std::is_same<T, V>::value) {
      for (int m = threadIdx.x; m < (int)(Tt + H0); m += blockDim.x)
        A[m] = P::ld(reinterpret_cast<const T*>(A)[m]);
      __syncthreads();
    }
  } else {
    for (int m = threadIdx.x; m < (int)(Tt + H0); m += blockDim.x)
      A[m] = P::ld(in[wrap(t0 + m, N)]);
    __syncthreads();
  }

  V* src = A;
  V* dst = B;
  for (int l = 1; l <= G; l++) {
    const int nD = (int)(Tt >> l);
    const int nS = nD + (int)fwd_halo(L, G, l);
    const int dstep = 1 << l, doff = 1 << (l - 1);
    for (int k = threadIdx.x; k < nS; k += blockDim.x) {
      V s, d;
      fwd_pair<F, P>(src + 2 * k, s, d, tp);
      dst[k] = s;
      if (k < nD) Z[doff + k * dstep] = d;
    }
    __syncthreads();
    V* t = src; src = dst; dst = t;
  }
  const int nC = (int)(Tt >> G);
  for (int k = threadIdx.x; k < nC; k += blockDim.x) {
    Z[k << G] = src[k];
    if (coarse) coarse[(t0 >> G) + k] = P::st(src[k]);
  }
  __syncthreads();
  if ((bulk & 2) && S == 1) {
    T* Zt = reinterpret_cast<T*>(Z);
    if constexpr (!std::is_same<T, V>::value) {
      for (int m = threadIdx.x; m < (int)Tt; m += blockDim.x) {
        const V v = Z[m];
        Zt[m] = P::st(v);
      }
    }
    fence_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
      bulk_s2g(out + t0, Zt, (uint32_t)(Tt * sizeof(T)));
      bulk_commit();
      bulk_wait_read();
    }
    return;
  }
  const int64_t cmask = ((int64_t)1 << G) - 1;
  for (int m = threadIdx.x; m < (int)Tt; m += blockDim.x) {
    if (write_coarse_slots || (m & cmask) != 0) out[(t0 + m) * S] = P::st(Z[m]);
  }
}

// Inverse pass: reconstructs y[t0 .. t0+Tt) of the compact level sequence
// (length N) from the level-G scaling values (coarse, length N/2^G, stride
// cstride) and the details of levels 1..G stored at det[m*S] (m = 2^(l-1) mod
// 2^l).  Writes outp[(t0+m)*ostride].  `bulk` bit 0: bulk-copy staging of
// det (S == 1); bit 1: bulk store of the tile (ostride == 1).  Block b
// handles tile tile0 + b.
struct InvGeom {
  int need[24];  // left halo at level l (coefficients)
  int off[24];   // buffer offset of level l
  int offmax;    // max over l of off[l]
};

// Shared memory of an inverse pass: the staged interleaved range
// [t0 - H, t0 + Tt) (W = Tt + H values of T; two buffers in the pipelined
// kernel), its details de-interleaved per level (D, W values of V), and the
// scaling values of the even (SA) and odd (SB) levels.  The pipelined kernel
// keeps the staging buffers, D, SA and SB apart; the per-tile kernel puts D
// first and SA/SB in the staging space, which is dead once split.  D holds level l's
// details d_l[i] = staged[2^(l-1) + i*2^l], i < W >> l, at offset
// W - (W >> (l-1)): the level loops then read consecutive details from
// consecutive addresses instead of at stride 2^l (a 2^l-way bank conflict
// up to 32-way).
__host__ __device__ inline int64_t inv_sa_len(const InvGeom& g, int64_t Tt) {
  return Tt + 2 * g.off[0] + 16;
}
__host__ __device__ inline int64_t inv_sb_len(const InvGeom& g, int64_t Tt) {
  return Tt / 2 + 2 * g.offmax + 16;
}

// Splits the staged details into D (all levels 1..G; the level-G scaling
// slots, m % 2^G == 0, are skipped), converting them to V.
template <class P, class Get>
__device__ __forceinline__ void deinterleave(typename P::V* D, int W, int G, Get&& get) {
  const int gmask = (1 << G) - 1;
  for (int m = threadIdx.x; m < W; m += blockDim.x) {
    if (m & gmask) {
      const int l = __ffs(m);
      D[W - (W >> (l - 1)) + (m >> l)] = P::ld(get(m));
    }
  }
}

template <int F, class P>
__global__ void __launch_bounds__(kThreads)
dwt_inv_pass(const typename P::T* __restrict__ coarse, int64_t cstride,
             const typename P::T* __restrict__ det, int64_t S, int64_t N, int G,
             int64_t Tt, typename P::T* __restrict__ outp, int64_t ostride,
             InvGeom geo, int bulk, unsigned int* status, int64_t tile0) {
  using V = typename P::V;
  PairTaps<F, P> tp;
  tp.init();
  using T = typename P::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar;
  const int64_t H = (int64_t)geo.need[G] << G;  // left halo of the staged array
  const int W = (int)(Tt + H);
  // D first; the staged range Z is dead once split into D, so SA and SB
  // reuse its space.
  V* D = reinterpret_cast<V*>(smem_raw);
  T* Z = reinterpret_cast<T*>(D + pad16<V>(W));
  V* SA = reinterpret_cast<V*>(Z);
  V* SB = SA + pad16<V>(inv_sa_len(geo, Tt));
  const int64_t t0 = (tile0 + (int64_t)blockIdx.x) * Tt;

  if (bulk & 1) {
    // S == 1: the staged range [t0-H, t0+Tt) is contiguous except that the
    // first tile's halo wraps to the end of the array.
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
      mbar_expect_tx(&bar, (uint32_t)((Tt + H) * sizeof(T)));
      if (t0 >= H) {
        bulk_g2s(Z, det + (t0 - H), (uint32_t)((Tt + H) * sizeof(T)), &bar);
      } else {
        bulk_g2s(Z, det + (N - H), (uint32_t)(H * sizeof(T)), &bar);
        bulk_g2s(Z + H, det + t0, (uint32_t)(Tt * sizeof(T)), &bar);
      }
    }
    const bool ok = mbar_wait(&bar, 0, status);
    if (__syncthreads_or(!ok)) return;
    deinterleave<P>(D, W, G, [&](int m) { return Z[m]; });
  } else {
    deinterleave<P>(D, W, G, [&](int m) { return det[wrap(t0 - H + m, N) * S]; });
  }
  __syncthreads();  // Z is read; SA and SB overwrite it
  {
    const int64_t NG = N >> G, q0 = t0 >> G;
    const int cnt = (int)(Tt >> G) + geo.need[G];
    V* buf = (G & 1) ? SB : SA;  // level-G buffer; level 0 ends in SA
    for (int k = threadIdx.x; k < cnt; k += blockDim.x)
      buf[k] = P::ld(coarse[wrap(q0 - geo.need[G] + k, NG) * cstride]);
  }
  __syncthreads();

  for (int l = G; l >= 1; l--) {
    V* src = (l & 1) ? SB : SA;
    V* dst = (l & 1) ? SA : SB;
    const int P_l = (geo.need[l - 1] + 1) >> 1;
    const int nq = (int)(Tt >> l) + P_l;
    const V* Dl = D + (W - (W >> (l - 1))) + (int)(H >> l);
    for (int k = threadIdx.x; k < nq; k += blockDim.x) {
      const int qr = k - P_l;  // q - q0
      constexpr int HH = filter_len(F) / 2;
      V sv[HH], dv[HH];
#pragma unroll
      for (int j = 0; j < HH; j++) {
        sv[j] = src[qr - j + geo.off[l]];
        dv[j] = Dl[qr - j];
      }
      V e, o;
      inv_pair<F, P>(sv, dv, e, o, tp);
      st2(dst + 2 * qr + geo.off[l - 1], e, o);
    }
    __syncthreads();
  }
  if ((bulk & 2) && ostride == 1) {
    T* St = reinterpret_cast<T*>(SA);
    if constexpr (!std::is_same<T, V>::value) {
      for (int m = threadIdx.x; m < (int)Tt; m += blockDim.x) {
        const V v = SA[m];
        St[m] = P::st(v);
      }
    }
    fence_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
      bulk_s2g(outp + t0, St, (uint32_t)(Tt * sizeof(T)));
      bulk_commit();
      bulk_wait_read();
    }
    return;
  }
  for (int m = threadIdx.x; m < (int)Tt; m += blockDim.x)
    outp[(t0 + m) * ostride] = P::st(SA[m + geo.off[0]]);
}

// Pipelined first forward pass (S == 1, compact input, contiguous output).
// A persistent CTA walks tiles blockIdx.x, blockIdx.x + gridDim.x, ...:
// thread 0 issues the bulk copy of the next tile (and its halo) into the
// second staging buffer before the block computes the current one, and the
// previous tile's bulk store drains while the block computes, so loads,
// stores and arithmetic overlap inside one CTA.  Staging buffers hold T
// values and are converted to V in place (same size).
template <int F, class P, int NT>
__global__ void __launch_bounds__(NT)
dwt_fwd_pipe(const typename P::T* __restrict__ in, int64_t N, int G, int64_t Tt,
             typename P::T* __restrict__ out, typename P::T* __restrict__ coarse,
             unsigned int* status, int64_t ntiles) {
  using V = typename P::V;
  PairTaps<F, P> tp;
  tp.init();
  using T = typename P::T;
  static_assert(sizeof(V) == sizeof(T) || std::is_same<V, T>::value, "in-place staging");
  constexpr int L = filter_len(F);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar[2];
  const int64_t H0 = pad16<T>(fwd_halo(L, G, 0));
  V* const R0 = reinterpret_cast<V*>(smem_raw);
  V* const R1 = R0 + pad16<V>(Tt + H0);
  V* B = R1 + pad16<V>(Tt + H0);
  V* Z = B + pad16<V>(Tt / 2 + fwd_halo(L, G, 1));
  int64_t tile = blockIdx.x;
  if (tile >= ntiles) return;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
  }
  __syncthreads();
  auto issue = [&](int64_t tl, int b) {
    const int64_t t0 = tl * Tt;
    T* dst = reinterpret_cast<T*>(b ? R1 : R0);
    mbar_expect_tx(&bar[b], (uint32_t)((Tt + H0) * sizeof(T)));
    if (t0 + Tt + H0 <= N) {
      bulk_g2s(dst, in + t0, (uint32_t)((Tt + H0) * sizeof(T)), &bar[b]);
    } else {
      bulk_g2s(dst, in + t0, (uint32_t)(Tt * sizeof(T)), &bar[b]);
      if (H0 > 0) bulk_g2s(dst + Tt, in, (uint32_t)(H0 * sizeof(T)), &bar[b]);
    }
  };
  if (threadIdx.x == 0) issue(tile, 0);
  uint32_t ph0 = 0u, ph1 = 0u;
  int b = 0;
  for (; tile < ntiles; tile += gridDim.x) {
    const int64_t t0 = tile * Tt;
    const int64_t next = tile + gridDim.x;
    if (threadIdx.x == 0) {
      if (next < ntiles) issue(next, b ^ 1);
      bulk_wait_read();  // the previous tile's store has finished reading Z
    }
    const bool ok = mbar_wait(b ? &bar[1] : &bar[0], b ? ph1 : ph0, status);
    if (b) ph1 ^= 1u; else ph0 ^= 1u;
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) bulk_wait_read();
      return;
    }
    V* A = b ? R1 : R0;
    if constexpr (!std::is_same<T, V>::value) {
      for (int m = threadIdx.x; m < (int)(Tt + H0); m += blockDim.x)
        A[m] = P::ld(reinterpret_cast<const T*>(A)[m]);
      __syncthreads();
    }
    V* src = A;
    V* dst = B;
    for (int l = 1; l <= G; l++) {
      const int nD = (int)(Tt >> l);
      const int nS = nD + (int)fwd_halo(L, G, l);
      const int dstep = 1 << l, doff = 1 << (l - 1);
      for (int k = threadIdx.x; k < nS; k += blockDim.x) {
        V s, d;
        fwd_pair<F, P>(src + 2 * k, s, d, tp);
        dst[k] = s;
        if (k < nD) Z[doff + k * dstep] = d;
      }
      __syncthreads();
      V* t = src; src = dst; dst = t;
    }
    const int nC = (int)(Tt >> G);
    for (int k = threadIdx.x; k < nC; k += blockDim.x) {
      Z[k << G] = src[k];
      if (coarse) coarse[(t0 >> G) + k] = P::st(src[k]);
    }
    __syncthreads();
    T* Zt = reinterpret_cast<T*>(Z);
    if constexpr (!std::is_same<T, V>::value) {
      for (int m = threadIdx.x; m < (int)Tt; m += blockDim.x) {
        const V v = Z[m];
        Zt[m] = P::st(v);
      }
    }
    // Order this thread's generic shared-memory accesses before the async
    // proxy reads Z (store below) and refills this staging buffer (the load
    // issued two tiles later).
    fence_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
      bulk_s2g(out + t0, Zt, (uint32_t)(Tt * sizeof(T)));
      bulk_commit();
    }
    b ^= 1;
  }
  if (threadIdx.x == 0) bulk_wait_read();
}

// Pipelined last inverse pass (S == 1): reconstructs tiles of the signal from
// the interleaved coefficients `det` (the staged range [t0 - H, t0 + Tt) is
// double-buffered by bulk copies) and the compact level-G scaling values
// `coarse`; the tile leaves by one bulk store from SA.  Same tile arithmetic
// as dwt_inv_pass.
template <int F, class P, int NT>
__global__ void __launch_bounds__(NT)
dwt_inv_pipe(const typename P::T* __restrict__ coarse, int64_t cstride,
             const typename P::T* __restrict__ det, int64_t N, int G, int64_t Tt,
             typename P::T* __restrict__ outp, InvGeom geo, unsigned int* status,
             int64_t ntiles) {
  using V = typename P::V;
  PairTaps<F, P> tp;
  tp.init();
  using T = typename P::T;
  constexpr int HH = filter_len(F) / 2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar[2];
  const int64_t H = (int64_t)geo.need[G] << G;
  const int W = (int)(Tt + H);
  T* const Z0 = reinterpret_cast<T*>(smem_raw);
  T* const Z1 = Z0 + pad16<T>(W);
  V* const D = reinterpret_cast<V*>(Z1 + pad16<T>(W));
  V* SA = D + pad16<V>(W);
  V* SB = SA + pad16<V>(inv_sa_len(geo, Tt));
  int64_t tile = blockIdx.x;
  if (tile >= ntiles) return;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
  }
  __syncthreads();
  auto issue = [&](int64_t tl, int b) {
    const int64_t t0 = tl * Tt;
    T* dst = b ? Z1 : Z0;
    mbar_expect_tx(&bar[b], (uint32_t)((Tt + H) * sizeof(T)));
    if (t0 >= H) {
      bulk_g2s(dst, det + (t0 - H), (uint32_t)((Tt + H) * sizeof(T)), &bar[b]);
    } else {
      bulk_g2s(dst, det + (N - H), (uint32_t)(H * sizeof(T)), &bar[b]);
      bulk_g2s(dst + H, det + t0, (uint32_t)(Tt * sizeof(T)), &bar[b]);
    }
  };
  if (threadIdx.x == 0) issue(tile, 0);
  uint32_t ph0 = 0u, ph1 = 0u;
  int b = 0;
  const int64_t NG = N >> G;
  for (; tile < ntiles; tile += gridDim.x) {
    const int64_t t0 = tile * Tt;
    const int64_t next = tile + gridDim.x;
    if (threadIdx.x == 0) {
      if (next < ntiles) issue(next, b ^ 1);
      bulk_wait_read();  // the previous tile's store has finished reading SA
    }
    const bool ok = mbar_wait(b ? &bar[1] : &bar[0], b ? ph1 : ph0, status);
    if (b) ph1 ^= 1u; else ph0 ^= 1u;
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) bulk_wait_read();
      return;
    }
    const T* Z = b ? Z1 : Z0;
    deinterleave<P>(D, W, G, [&](int m) { return Z[m]; });
    {
      const int64_t q0 = t0 >> G;
      const int cnt = (int)(Tt >> G) + geo.need[G];
      V* buf = (G & 1) ? SB : SA;
      for (int k = threadIdx.x; k < cnt; k += blockDim.x)
        buf[k] = P::ld(coarse[wrap(q0 - geo.need[G] + k, NG) * cstride]);
    }
    __syncthreads();
    for (int l = G; l >= 1; l--) {
      V* src = (l & 1) ? SB : SA;
      V* dst = (l & 1) ? SA : SB;
      const int P_l = (geo.need[l - 1] + 1) >> 1;
      const int nq = (int)(Tt >> l) + P_l;
      const V* Dl = D + (W - (W >> (l - 1))) + (int)(H >> l);
      for (int k = threadIdx.x; k < nq; k += blockDim.x) {
        const int qr = k - P_l;
        V sv[HH], dv[HH];
#pragma unroll
        for (int j = 0; j < HH; j++) {
          sv[j] = src[qr - j + geo.off[l]];
          dv[j] = Dl[qr - j];
        }
        V e, o;
        inv_pair<F, P>(sv, dv, e, o, tp);
        st2(dst + 2 * qr + geo.off[l - 1], e, o);
      }
      __syncthreads();
    }
    T* St = reinterpret_cast<T*>(SA);
    if constexpr (!std::is_same<T, V>::value) {
      for (int m = threadIdx.x; m < (int)Tt; m += blockDim.x) {
        const V v = SA[m];
        St[m] = P::st(v);
      }
    }
    fence_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
      bulk_s2g(outp + t0, St, (uint32_t)(Tt * sizeof(T)));
      bulk_commit();
    }
    b ^= 1;
  }
  if (threadIdx.x == 0) bulk_wait_read();
}

bool aligned16_host(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

struct PassPlan {
  int64_t N, S, Tt;
  int G;
};

constexpr size_t kSmemBudget = 100 * 1024;
constexpr int kHostChunksMax = 16;  // chunks of a host-streamed DWT

template <class P>
size_t fwd_smem(int L, int G, int64_t Tt) {
  using V = typename P::V;
  using T = typename P::T;
  return sizeof(V) * (size_t)(pad16<V>(Tt + pad16<T>(fwd_halo(L, G, 0))) +
                              pad16<V>(Tt / 2 + fwd_halo(L, G, 1)) + pad16<V>(Tt));
}

InvGeom inv_geom(int L, int G) {
  InvGeom g{};
  g.need[0] = 0;
  for (int l = 1; l <= G; l++) g.need[l] = (g.need[l - 1] + 1) / 2 + L / 2 - 1;
  g.off[G] = g.need[G];
  for (int l = 0; l < G; l++) g.off[l] = 2 * ((g.need[l] + 1) / 2);
  g.offmax = 0;
  for (int l = 0; l <= G; l++) g.offmax = std::max(g.offmax, g.off[l]);
  return g;
}

template <class P>
size_t inv_smem(int L, int G, int64_t Tt) {
  InvGeom g = inv_geom(L, G);
  int64_t H = (int64_t)g.need[G] << G;
  using V = typename P::V;
  using T = typename P::T;
  const size_t staged = sizeof(T) * (size_t)pad16<T>(Tt + H);
  const size_t scal =
      sizeof(V) * (size_t)(pad16<V>(inv_sa_len(g, Tt)) + pad16<V>(inv_sb_len(g, Tt)));
  return sizeof(V) * (size_t)pad16<V>(Tt + H) + std::max(staged, scal);
}

template <class P>
std::vector<PassPlan> plan_passes(int64_t n, int J, int F) {
  const int L = filter_len(F);
  const int64_t TT = (int64_t)(4096 * 8 / sizeof(typename P::V));
  const int gmax = F == 1 ? 30 : F == 2 ? 8 : F == 3 ? 7 : 6;
  std::vector<PassPlan> plan;
  int64_t N = n, S = 1;
  int l = 0;
  while (l < J) {
    const int64_t Tt = std::min(N, TT);
    int G = std::min(J - l, (Tt == N) ? 30 : gmax);
    while (G > 1 && ((((int64_t)1 << G) > Tt) || fwd_smem<P>(L, G, Tt) > kSmemBudget ||
                     inv_smem<P>(L, G, Tt) > kSmemBudget))
      G--;
    plan.push_back({N, S, Tt, G});
    N >>= G;
    S <<= G;
    l += G;
  }
  return plan;
}

// ------------------------------------------------------ tile configuration --
// First-pass tiling of the main DWT path, per (filter, precision): tile size,
// levels fused in the first pass, threads per CTA and whether the pipelined
// persistent kernels are used.  Defaults below; wc_tune_dwt() replaces them
// with the fastest measured candidate.
struct TileCfg {
  int tile, g0, threads, pipe;
};

std::mutex g_cfg_mu;
TileCfg g_cfg[5][3];
bool g_cfg_set[5][3] = {};

int gmax_of(int F) { return F == 1 ? 12 : F == 2 ? 8 : F == 3 ? 7 : 6; }

// Defaults: the fastest candidates of wc_tune_dwt on a GB300 at n = 2^24
// (forward + inverse), per filter and precision (exact, fast, FP32).
TileCfg default_cfg(int F, int prec) {
  static const TileCfg table[5][3] = {
      {{4096, 8, 512, 1}, {4096, 8, 512, 1}, {8192, 8, 512, 1}},
      {{2048, 11, 256, 0}, {2048, 11, 512, 0}, {4096, 12, 256, 1}},  // Haar
      {{4096, 7, 512, 0}, {2048, 7, 256, 0}, {4096, 8, 256, 1}},     // D4
      {{4096, 7, 512, 0}, {2048, 6, 512, 0}, {4096, 6, 256, 1}},     // C6
      {{4096, 5, 256, 0}, {2048, 5, 512, 0}, {4096, 5, 512, 0}},     // LA8
  };
  if (F < 1 || F > 4 || prec < 0 || prec > 2) return TileCfg{4096, gmax_of(F), 512, 1};
  return table[F][prec];
}

TileCfg get_cfg(int F, int prec) {
  std::lock_guard<std::mutex> lk(g_cfg_mu);
  if (!g_cfg_set[F][prec]) {
    g_cfg[F][prec] = default_cfg(F, prec);
    g_cfg_set[F][prec] = true;
  }
  return g_cfg[F][prec];
}

void set_cfg(int F, int prec, TileCfg c) {
  std::lock_guard<std::mutex> lk(g_cfg_mu);
  g_cfg[F][prec] = c;
  g_cfg_set[F][prec] = true;
}

template <class P>
size_t fwd_pipe_smem(int L, int G, int64_t Tt) {
  using V = typename P::V;
  using T = typename P::T;
  return sizeof(V) * (size_t)(2 * pad16<V>(Tt + pad16<T>(fwd_halo(L, G, 0))) +
                              pad16<V>(Tt / 2 + fwd_halo(L, G, 1)) + pad16<V>(Tt));
}

template <class P>
size_t inv_pipe_smem(int L, int G, int64_t Tt) {
  InvGeom g = inv_geom(L, G);
  const int64_t H = (int64_t)g.need[G] << G;
  using V = typename P::V;
  using T = typename P::T;
  return 2 * sizeof(T) * (size_t)pad16<T>(Tt + H) +
         sizeof(V) * (size_t)(pad16<V>(Tt + H) + pad16<V>(inv_sa_len(g, Tt)) +
                              pad16<V>(inv_sb_len(g, Tt)));
}

constexpr size_t kPipeSmemMax = 200 * 1024;

// Passes with the first pass taken from cfg; later passes as plan_passes.
template <class P>
std::vector<PassPlan> plan_passes_cfg(int64_t n, int J, int F, const TileCfg& c) {
  const int L = filter_len(F);
  const int64_t TT = (int64_t)(4096 * 8 / sizeof(typename P::V));
  const int gmax = gmax_of(F);
  std::vector<PassPlan> plan;
  int64_t N = n, S = 1;
  int l = 0;
  while (l < J) {
    const bool first = plan.empty();
    int64_t Tt = std::min(N, first ? (int64_t)c.tile : TT);
    // Later passes are short: smaller tiles keep every SM busy.
    while (!first && Tt > 1024 && N / Tt < 2 * 152) Tt >>= 1;
    int G = std::min(J - l, (Tt == N) ? 30 : (first ? c.g0 : gmax));
    auto fits = [&](int g) {
      if (first && c.pipe && Tt < N)
        return fwd_pipe_smem<P>(L, g, Tt) <= kPipeSmemMax &&
               inv_pipe_smem<P>(L, g, Tt) <= kPipeSmemMax;
      return fwd_smem<P>(L, g, Tt) <= kSmemBudget && inv_smem<P>(L, g, Tt) <= kSmemBudget;
    };
    while (G > 1 && ((((int64_t)1 << G) > Tt) || !fits(G))) G--;
    plan.push_back({N, S, Tt, G});
    N >>= G;
    S <<= G;
    l += G;
  }
  return plan;
}

template <class P>
constexpr int prec_of() {
  return std::is_same<P, PExact>::value ? WC_F64_EXACT
         : std::is_same<P, PDD>::value  ? WC_F64_FAST
                                        : WC_F32;
}

int sm_count() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  return sms;
}

// Persistent grid: every CTA that fits at once, at most one per tile.
template <class K>
int persistent_grid(K kern, int threads, size_t smem, int64_t ntiles) {
  int per = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, threads, smem) != cudaSuccess ||
      per < 1) {
    cudaGetLastError();
    per = 1;
  }
  return (int)std::min<int64_t>(ntiles, (int64_t)per * sm_count());
}

template <int F, class P, int NT>
int launch_fwd_pipe_nt(const typename P::T* src, const PassPlan& pp, typename P::T* out,
                       typename P::T* coarse, unsigned int* status, cudaStream_t s) {
  const size_t smem = fwd_pipe_smem<P>(filter_len(F), pp.G, pp.Tt);
  auto kern = dwt_fwd_pipe<F, P, NT>;
  WC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t ntiles = pp.N / pp.Tt;
  const int grid = persistent_grid(kern, NT, smem, ntiles);
  {
    LaunchTimer lt("dwt_fwd_pass0", s);
    kern<<<grid, NT, smem, s>>>(src, pp.N, pp.G, pp.Tt, out, coarse, status, ntiles);
  }
  return after_launch("dwt_fwd_pipe");
}

template <int F, class P>
int launch_fwd_pipe(int threads, const typename P::T* src, const PassPlan& pp,
                    typename P::T* out, typename P::T* coarse, unsigned int* status,
                    cudaStream_t s) {
  if (threads == 256) return launch_fwd_pipe_nt<F, P, 256>(src, pp, out, coarse, status, s);
  return launch_fwd_pipe_nt<F, P, 512>(src, pp, out, coarse, status, s);
}

template <int F, class P, int NT>
int launch_inv_pipe_nt(const typename P::T* coarse, int64_t cstride, const typename P::T* det,
                       const PassPlan& pp, typename P::T* dst, const InvGeom& geo,
                       unsigned int* status, cudaStream_t s) {
  const size_t smem = inv_pipe_smem<P>(filter_len(F), pp.G, pp.Tt);
  auto kern = dwt_inv_pipe<F, P, NT>;
  WC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t ntiles = pp.N / pp.Tt;
  const int grid = persistent_grid(kern, NT, smem, ntiles);
  {
    LaunchTimer lt("dwt_inv_pass0", s);
    kern<<<grid, NT, smem, s>>>(coarse, cstride, det, pp.N, pp.G, pp.Tt, dst, geo, status,
                                ntiles);
  }
  return after_launch("dwt_inv_pipe");
}

template <int F, class P>
int launch_inv_pipe(int threads, const typename P::T* coarse, int64_t cstride,
                    const typename P::T* det, const PassPlan& pp, typename P::T* dst,
                    const InvGeom& geo, unsigned int* status, cudaStream_t s) {
  if (threads == 256)
    return launch_inv_pipe_nt<F, P, 256>(coarse, cstride, det, pp, dst, geo, status, s);
  return launch_inv_pipe_nt<F, P, 512>(coarse, cstride, det, pp, dst, geo, status, s);
}

template <int F, class P>
int run_dwt(const void* vin, void* vout, int64_t n, int sense, int J, cudaStream_t s) {
  using T = typename P::T;
  const int L = filter_len(F);
  const T* in = static_cast<const T*>(vin);
  T* out = static_cast<T*>(vout);
  const TileCfg cfg = get_cfg(F, prec_of<P>());
  std::vector<PassPlan> plan = plan_passes_cfg<P>(n, J, F, cfg);
  unsigned int* status = device_status_word();
  if (!status) return workspace_error();
  const int np = (int)plan.size();
  T* scratch[2] = {nullptr, nullptr};
  if (np > 1) {
    size_t cbytes = sizeof(T) * (size_t)(plan[0].N >> plan[0].G);
    scratch[0] = static_cast<T*>(workspace(kSlotCoarse0, cbytes));
    scratch[1] = static_cast<T*>(workspace(kSlotCoarse1, cbytes));
    if (!scratch[0] || !scratch[1]) return workspace_error();
  }
  if (sense == 1) {
    const T* src = in;
    for (int p = 0; p < np; p++) {
      const PassPlan& pp = plan[p];
      const bool last = (p == np - 1);
      T* coarse = last ? nullptr : scratch[p & 1];
      size_t smem = fwd_smem<P>(L, pp.G, pp.Tt);
      // Bulk staging needs 16-byte aligned tiles and a halo that wraps at
      // most once.
      const int64_t H0 = pad16<T>(fwd_halo(L, pp.G, 0));
      const int bulk = aligned16_host(src) && aligned16_host(out) && H0 <= pp.N &&
                       (pp.Tt * (int64_t)sizeof(T)) % 16 == 0;
      if (p == 0 && cfg.pipe && bulk && pp.Tt < pp.N) {
        WC_TRY((launch_fwd_pipe<F, P>(cfg.threads, src, pp, out, coarse, status, s)));
        src = coarse;
        continue;
      }
      auto kern = dwt_fwd_pass<F, P>;
      WC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      {
        LaunchTimer lt(p == 0 ? "dwt_fwd_pass0" : "dwt_fwd_pass", s);
        kern<<<(unsigned)(pp.N / pp.Tt), kThreads, smem, s>>>(src, pp.N, pp.G, pp.Tt, out, pp.S,
                                                             coarse, (last || pp.S == 1) ? 1 : 0,
                                                             bulk ? 3 : 0, status, 0);
      }
      WC_TRY(after_launch("dwt_fwd_pass"));
      src = coarse;
    }
  } else {
    // Passes in reverse order; pass p reads its coarse input from the
    // interleaved array (top pass) or from the scratch written by pass p+1.
    const T* coarse = in;
    int64_t cstride = plan[np - 1].S << plan[np - 1].G;
    for (int p = np - 1; p >= 0; p--) {
      const PassPlan& pp = plan[p];
      T* dst = (p == 0) ? out : scratch[p & 1];
      InvGeom geo = inv_geom(L, pp.G);
      size_t smem = inv_smem<P>(L, pp.G, pp.Tt);
      const int64_t H = (int64_t)geo.need[pp.G] << pp.G;
      const int bulk = pp.S == 1 && H <= pp.N && aligned16_host(in) && aligned16_host(dst) &&
                       (H * (int64_t)sizeof(T)) % 16 == 0 && (pp.Tt * (int64_t)sizeof(T)) % 16 == 0;
      if (p == 0 && cfg.pipe && bulk && pp.Tt < pp.N) {
        WC_TRY((launch_inv_pipe<F, P>(cfg.threads, coarse, cstride, in, pp, dst, geo, status, s)));
        coarse = dst;
        cstride = 1;
        continue;
      }
      auto kern = dwt_inv_pass<F, P>;
      WC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      {
        LaunchTimer lt(p == 0 ? "dwt_inv_pass0" : "dwt_inv_pass", s);
        kern<<<(unsigned)(pp.N / pp.Tt), kThreads, smem, s>>>(coarse, cstride, in, pp.S, pp.N,
                                                             pp.G, pp.Tt, dst, 1, geo, bulk ? 3 : 0,
                                                             status, 0);
      }
      WC_TRY(after_launch("dwt_inv_pass"));
      coarse = dst;
      cstride = 1;
    }
  }
  return WC_OK;
}

template <class P>
int dispatch_dwt(const void* in, void* out, int64_t n, int sense, int J, int F, cudaStream_t s) {
  switch (F) {
    case 1: return run_dwt<1, P>(in, out, n, sense, J, s);
    case 2: return run_dwt<2, P>(in, out, n, sense, J, s);
    case 3: return run_dwt<3, P>(in, out, n, sense, J, s);
    case 4: return run_dwt<4, P>(in, out, n, sense, J, s);
  }
  return fail(WC_ERR_ARG, "unknown filter %d", F);
}

}  // namespace

int dwt(const void* in, void* out, int64_t n, int sense, int J, int F, int prec,
        cudaStream_t s) {
  switch (prec) {
    case WC_F64_EXACT: return dispatch_dwt<PExact>(in, out, n, sense, J, F, s);
    case WC_F64_FAST: return dispatch_dwt<PDD>(in, out, n, sense, J, F, s);
    case WC_F32: return dispatch_dwt<PF32>(in, out, n, sense, J, F, s);
  }
  return fail(WC_ERR_ARG, "unknown precision %d", prec);
}

// ---------------------------------------------------------------------------
// Host-resident signals (the R entry points' case).  Copying the whole signal
// in, transforming, and copying it back serialises two host-link transfers;
// here the signal streams in by chunks on a second stream while the first
// (forward) or last (inverse) pass of earlier chunks runs, and that pass
// stores its tiles straight into host memory, so the link carries both
// directions at once.  The coarse passes read (inverse) or write (forward)
// their strided slots of the host array directly.  Needs a host array the
// GPU can address (pinned, or pageable memory on a system whose GPU uses the
// host page tables, such as Grace); callers check that.
namespace {

template <class T>
__global__ void gather_stride_kernel(const T* __restrict__ src, T* __restrict__ dst, int64_t count,
                                     int shift) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride)
    dst[i] = src[i << shift];
}

struct HostStreamState {
  cudaStream_t up = nullptr;
  cudaEvent_t ev[kHostChunksMax] = {};
};
std::mutex g_hs_mu;
HostStreamState g_hs[64];

int host_stream_state(HostStreamState** out) {
  int dev = 0;
  WC_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(WC_ERR_UNSUPPORTED, "device ordinal %d", dev);
  std::lock_guard<std::mutex> lk(g_hs_mu);
  HostStreamState& st = g_hs[dev];
  if (!st.up) {
    WC_CUDA(cudaStreamCreateWithFlags(&st.up, cudaStreamNonBlocking));
    for (int k = 0; k < kHostChunksMax; k++)
      WC_CUDA(cudaEventCreateWithFlags(&st.ev[k], cudaEventDisableTiming));
  }
  *out = &st;
  return WC_OK;
}

template <int F, class P>
int run_dwt_host(typename P::T* x, int64_t n, int sense, int J, cudaStream_t s) {
  using T = typename P::T;
  const int L = filter_len(F);
  TileCfg cfg = get_cfg(F, prec_of<P>());
  cfg.pipe = 0;  // tile-offset launches of the per-tile kernels
  std::vector<PassPlan> plan = plan_passes_cfg<P>(n, J, F, cfg);
  const int np = (int)plan.size();
  const PassPlan& p0 = plan[0];
  const int64_t ntiles = p0.N / p0.Tt;
  if (ntiles < 2) return WC_ERR_UNSUPPORTED;
  const int K = (int)std::min<int64_t>(kHostChunksMax, ntiles);
  const int64_t ct = ntiles / K, cs = ct * p0.Tt;  // tiles and values per chunk
  const int64_t H0 = pad16<T>(fwd_halo(L, p0.G, 0));
  const InvGeom geo0 = inv_geom(L, p0.G);
  const int64_t HI = (int64_t)geo0.need[p0.G] << p0.G;
  if (H0 > cs || HI > cs) return WC_ERR_UNSUPPORTED;
  HostStreamState* hs = nullptr;
  WC_TRY(host_stream_state(&hs));
  unsigned int* status = device_status_word();
  if (!status) return workspace_error();
  T* A = static_cast<T*>(workspace(kSlotStageA, sizeof(T) * (size_t)n));
  if (!A) return workspace_error();
  T* scratch[2] = {nullptr, nullptr};
  if (np > 1) {
    const size_t cbytes = sizeof(T) * (size_t)(p0.N >> p0.G);
    scratch[0] = static_cast<T*>(workspace(kSlotCoarse0, cbytes));
    scratch[1] = static_cast<T*>(workspace(kSlotCoarse1, cbytes));
    if (!scratch[0] || !scratch[1]) return workspace_error();
  }
  // The upload stream must not start before earlier work on s that may
  // still read the staging buffer.
  WC_CUDA(cudaEventRecord(hs->ev[0], s));
  WC_CUDA(cudaStreamWaitEvent(hs->up, hs->ev[0], 0));
  for (int k = 0; k < K; k++) {
    WC_CUDA(cudaMemcpyAsync(A + k * cs, x + k * cs, sizeof(T) * (size_t)cs,
                            cudaMemcpyHostToDevice, hs->up));
    WC_CUDA(cudaEventRecord(hs->ev[k], hs->up));
  }
  const int ld_bulk = (aligned16_host(A) && (p0.Tt * (int64_t)sizeof(T)) % 16 == 0) ? 1 : 0;
  if (sense == 1) {
    T* coarse = (np > 1) ? scratch[0] : nullptr;
    const size_t smem = fwd_smem<P>(L, p0.G, p0.Tt);
    auto kern = dwt_fwd_pass<F, P>;
    WC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    for (int k = 0; k < K; k++) {
      WC_CUDA(cudaStreamWaitEvent(s, hs->ev[k], 0));
      WC_CUDA(cudaStreamWaitEvent(s, hs->ev[(k + 1) % K], 0));  // right halo
      {
        LaunchTimer lt("dwt_fwd_pass0", s);
        kern<<<(unsigned)ct, kThreads, smem, s>>>(A, p0.N, p0.G, p0.Tt, x, 1, coarse, 1,
                                                  (ld_bulk && H0 <= p0.N) ? 1 : 0, status,
                                                  (int64_t)k * ct);
      }
      WC_TRY(after_launch("dwt_fwd_pass"));
    }
    const T* src = coarse;
    for (int p = 1; p < np; p++) {
      const PassPlan& pp = plan[p];
      const bool last = (p == np - 1);
      T* cn = last ? nullptr : scratch[p & 1];
      const size_t sm = fwd_smem<P>(L, pp.G, pp.Tt);
      const int64_t h0 = pad16<T>(fwd_halo(L, pp.G, 0));
      const int b = (aligned16_host(src) && h0 <= pp.N && (pp.Tt * (int64_t)sizeof(T)) % 16 == 0)
                        ? 1 : 0;
      WC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
      {
        LaunchTimer lt("dwt_fwd_pass", s);
        kern<<<(unsigned)(pp.N / pp.Tt), kThreads, sm, s>>>(src, pp.N, pp.G, pp.Tt, x, pp.S, cn,
                                                            last ? 1 : 0, b, status, 0);
      }
      WC_TRY(after_launch("dwt_fwd_pass"));
      src = cn;
    }
    return WC_OK;
  }
  // Inverse: coarse passes straight from the host array, then the first
  // pass chunk by chunk (chunk 0 last: its left halo wraps to the end).
  // The coarse passes read only the slots q 2^G0 of the host array: one
  // gather kernel with many reads in flight brings them to the device first.
  auto ikern = dwt_inv_pass<F, P>;
  const T* cin = x;
  int sh = 0;
  if (np > 1) {
    const int64_t cnt = p0.N >> p0.G;
    T* C = static_cast<T*>(workspace(kSlotHostCoarse, sizeof(T) * (size_t)cnt));
    if (!C) return workspace_error();
    {
      LaunchTimer lt("gather_stride", s);
      const int64_t blocks = std::min<int64_t>((cnt + kThreads - 1) / kThreads, 152 * 32);
      gather_stride_kernel<T><<<(unsigned)blocks, kThreads, 0, s>>>(x, C, cnt, p0.G);
    }
    WC_TRY(after_launch("gather_stride_kernel"));
    cin = C;
    sh = p0.G;
  }
  const T* coarse = cin;
  int64_t cstride = (plan[np - 1].S << plan[np - 1].G) >> sh;
  for (int p = np - 1; p >= 1; p--) {
    const PassPlan& pp = plan[p];
    T* dst = scratch[p & 1];
    InvGeom geo = inv_geom(L, pp.G);
    const size_t sm = inv_smem<P>(L, pp.G, pp.Tt);
    WC_CUDA(cudaFuncSetAttribute(ikern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    {
      LaunchTimer lt("dwt_inv_pass", s);
      ikern<<<(unsigned)(pp.N / pp.Tt), kThreads, sm, s>>>(coarse, cstride, cin, pp.S >> sh, pp.N,
                                                          pp.G, pp.Tt, dst, 1, geo, 0, status, 0);
    }
    WC_TRY(after_launch("dwt_inv_pass"));
    coarse = dst;
    cstride = 1;
  }
  // A one-pass transform reads its coarse values from the staged copy: the
  // chunks below overwrite the host array.
  if (np == 1) coarse = A;
  const size_t sm0 = inv_smem<P>(L, p0.G, p0.Tt);
  WC_CUDA(cudaFuncSetAttribute(ikern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm0));
  const int b0 = (ld_bulk && HI <= p0.N && (HI * (int64_t)sizeof(T)) % 16 == 0) ? 1 : 0;
  for (int i = 1; i <= K; i++) {
    const int k = i % K;
    WC_CUDA(cudaStreamWaitEvent(s, hs->ev[k], 0));
    WC_CUDA(cudaStreamWaitEvent(s, hs->ev[(k + K - 1) % K], 0));  // left halo
    {
      LaunchTimer lt("dwt_inv_pass0", s);
      ikern<<<(unsigned)ct, kThreads, sm0, s>>>(coarse, cstride, A, 1, p0.N, p0.G, p0.Tt, x, 1,
                                                geo0, b0, status, (int64_t)k * ct);
    }
    WC_TRY(after_launch("dwt_inv_pass"));
  }
  return WC_OK;
}

template <class P>
int dispatch_dwt_host(void* x, int64_t n, int sense, int J, int F, cudaStream_t s) {
  using T = typename P::T;
  T* xt = static_cast<T*>(x);
  switch (F) {
    case 1: return run_dwt_host<1, P>(xt, n, sense, J, s);
    case 2: return run_dwt_host<2, P>(xt, n, sense, J, s);
    case 3: return run_dwt_host<3, P>(xt, n, sense, J, s);
    case 4: return run_dwt_host<4, P>(xt, n, sense, J, s);
  }
  return fail(WC_ERR_ARG, "unknown filter %d", F);
}

}  // namespace

int dwt_host_inplace(double* x, int64_t n, int sense, int J, int F, int prec, cudaStream_t s) {
  switch (prec) {
    case WC_F64_EXACT: return dispatch_dwt_host<PExact>(x, n, sense, J, F, s);
    case WC_F64_FAST: return dispatch_dwt_host<PDD>(x, n, sense, J, F, s);
  }
  return WC_ERR_UNSUPPORTED;
}

}  // namespace wc

// ---------------------------------------------------------------------------
// Allocation-free DWT entry point (wc_dwt_device_noalloc).
//
// Some callers cannot let this library call cudaMalloc: a host framework that
// has already reserved nearly all of HBM for its own memory pool (a
// cudaMalloc from here would fail, or fragment that pool), or a latency-
// critical loop that must not hit the device-wide synchronisation cudaFree
// performs when the workspace grows.  For them the DWT's only scratch -- the
// compact coarse coefficients handed from one pass to the next -- and its
// status word live in one file-scope device array of fixed size, loaded with
// the library and held by every GPU that loads it until the process exits.
// Host code must not use the array's name as a device address (it is a
// host-side stand-in); the device address comes from cudaGetSymbolAddress,
// looked up with the device current.  The first call on a device does that
// set-up, so make it before any stream capture; later calls look the address
// up again (which follows a reload of the module after a device reset) except
// while their stream is capturing, when they use the address found before.
// All calls share the array and it keeps the last call's contents: calls
// whose work overlaps on the GPU (different streams, or threads) race on it.
// The status word is sticky: a timed-out wait sets its bit, and only
// wc_device_status() reads and clears it (the array starts zeroed).
#include <mutex>

namespace wc {
namespace {

// Longest signal the allocation-free entry point accepts, and its scratch.
constexpr int64_t kNoAllocMaxLen = (int64_t)1 << 22;
constexpr size_t kNoAllocStatusBytes = 256;
constexpr size_t kNoAllocCoarseBytes = (size_t)1 << 19;  // per coarse buffer
static __device__ __align__(256) unsigned char
    g_noalloc_scratch[kNoAllocStatusBytes + 2 * kNoAllocCoarseBytes];

std::mutex g_noalloc_mu;
void* g_noalloc_base[256] = {};

// Device address of g_noalloc_scratch on the current device.  Looked up
// afresh unless the caller's stream is capturing (then the address found by
// an earlier call is used; there must be one).
int noalloc_base(unsigned char** base, cudaStream_t s, bool lookup) {
  int dev = 0;
  WC_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 256) return fail(WC_ERR_ARG, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (lookup) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    WC_CUDA(cudaStreamIsCapturing(s, &cs));
    if (cs == cudaStreamCaptureStatusNone || !g_noalloc_base[dev]) {
      if (cs != cudaStreamCaptureStatusNone)
        return fail(WC_ERR_ARG,
                    "allocation-free DWT: the first call on a device must come before stream "
                    "capture (it looks up the static scratch's device address)");
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) {
        cudaGetLastError();
        return fail(WC_ERR_CUDA, "cudaGetSymbolAddress of the static DWT scratch failed: %s",
                    cudaGetErrorString(e));
      }
      g_noalloc_base[dev] = p;
    }
  }
  *base = static_cast<unsigned char*>(g_noalloc_base[dev]);
  return WC_OK;
}

// The DWT of run_dwt with its scratch taken from the static array.
template <int F, class P>
int run_dwt_noalloc(const void* vin, void* vout, int64_t n, int sense, int J, cudaStream_t s,
                    unsigned char* base) {
  using T = typename P::T;
  const int L = filter_len(F);
  const T* in = static_cast<const T*>(vin);
  T* out = static_cast<T*>(vout);
  std::vector<PassPlan> plan = plan_passes<P>(n, J, F);
  const int np = (int)plan.size();
  unsigned int* status = reinterpret_cast<unsigned int*>(base);
  T* scratch[2] = {reinterpret_cast<T*>(base + kNoAllocStatusBytes),
                   reinterpret_cast<T*>(base + kNoAllocStatusBytes + kNoAllocCoarseBytes)};
  if (np > 1 && sizeof(T) * (size_t)(plan[0].N >> plan[0].G) > kNoAllocCoarseBytes)
    return fail(WC_ERR_ARG, "allocation-free DWT: coarse scratch of %zu bytes exceeds %zu",
                sizeof(T) * (size_t)(plan[0].N >> plan[0].G), kNoAllocCoarseBytes);
  // The status word is not cleared here: a timeout of an earlier call stays
  // visible until wc_device_status() reads it.
  if (sense == 1) {
    const T* src = in;
    for (int p = 0; p < np; p++) {
      const PassPlan& pp = plan[p];
      const bool last = (p == np - 1);
      T* coarse = last ? nullptr : scratch[p & 1];
      const size_t smem = fwd_smem<P>(L, pp.G, pp.Tt);
      const int64_t H0 = pad16<T>(fwd_halo(L, pp.G, 0));
      const int bulk = aligned16_host(src) && aligned16_host(out) && H0 <= pp.N &&
                       (pp.Tt * (int64_t)sizeof(T)) % 16 == 0;
      auto kern = dwt_fwd_pass<F, P>;
      WC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      kern<<<(unsigned)(pp.N / pp.Tt), kThreads, smem, s>>>(src, pp.N, pp.G, pp.Tt, out, pp.S,
                                                           coarse, (last || pp.S == 1) ? 1 : 0,
                                                           bulk ? 3 : 0, status, 0);
      WC_TRY(after_launch("dwt_fwd_pass"));
      src = coarse;
    }
  } else {
    const T* coarse = in;
    int64_t cstride = plan[np - 1].S << plan[np - 1].G;
    for (int p = np - 1; p >= 0; p--) {
      const PassPlan& pp = plan[p];
      T* dst = (p == 0) ? out : scratch[p & 1];
      InvGeom geo = inv_geom(L, pp.G);
      const size_t smem = inv_smem<P>(L, pp.G, pp.Tt);
      const int64_t H = (int64_t)geo.need[pp.G] << pp.G;
      const int bulk = pp.S == 1 && H <= pp.N && aligned16_host(in) && aligned16_host(dst) &&
                       (H * (int64_t)sizeof(T)) % 16 == 0 &&
                       (pp.Tt * (int64_t)sizeof(T)) % 16 == 0;
      auto kern = dwt_inv_pass<F, P>;
      WC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      kern<<<(unsigned)(pp.N / pp.Tt), kThreads, smem, s>>>(coarse, cstride, in, pp.S, pp.N,
                                                           pp.G, pp.Tt, dst, 1, geo, bulk ? 3 : 0,
                                                           status, 0);
      WC_TRY(after_launch("dwt_inv_pass"));
      coarse = dst;
      cstride = 1;
    }
  }
  return WC_OK;
}

template <class P>
int dispatch_noalloc(const void* in, void* out, int64_t n, int sense, int J, int F,
                     cudaStream_t s, unsigned char* base) {
  switch (F) {
    case 1: return run_dwt_noalloc<1, P>(in, out, n, sense, J, s, base);
    case 2: return run_dwt_noalloc<2, P>(in, out, n, sense, J, s, base);
    case 3: return run_dwt_noalloc<3, P>(in, out, n, sense, J, s, base);
    case 4: return run_dwt_noalloc<4, P>(in, out, n, sense, J, s, base);
  }
  return fail(WC_ERR_ARG, "unrecognised filter %d", F);
}

}  // namespace

unsigned int* noalloc_status_word_if_known() {
  unsigned char* b = nullptr;
  if (noalloc_base(&b, nullptr, false) != WC_OK) return nullptr;
  return reinterpret_cast<unsigned int*>(b);
}

int noalloc_status_word(unsigned int** w) {
  unsigned char* b = nullptr;
  WC_TRY(noalloc_base(&b, nullptr, true));
  *w = reinterpret_cast<unsigned int*>(b);
  return WC_OK;
}

}  // namespace wc

extern "C" int wc_dwt_device_noalloc(const void* in, void* out, int64_t len, int sense,
                                     int nlevels, int filter, int precision, void* stream) {
  using namespace wc;
  clear_error();
  WC_TRY(ensure_device());
  if (filter < 1 || filter > 4) return fail(WC_ERR_ARG, "unrecognised filter %d", filter);
  if (sense != 0 && sense != 1) return fail(WC_ERR_ARG, "sense must be 1 (FWD) or 0 (BWD)");
  if (precision < 0 || precision > 2) return fail(WC_ERR_ARG, "unknown precision %d", precision);
  if (len <= 0 || (len & (len - 1)) != 0)
    return fail(WC_ERR_ARG, "length %lld is not a power of 2", (long long)len);
  if (len > kNoAllocMaxLen)
    return fail(WC_ERR_ARG,
                "length %lld exceeds the allocation-free DWT's maximum of %lld samples "
                "(use wc_dwt_device for longer signals)",
                (long long)len, (long long)kNoAllocMaxLen);
  const int J = check_levels(len, nlevels, filter_len(filter));
  if (J == 0) return fail(WC_ERR_LEVELS, "nlevels %d invalid for length %lld", nlevels, (long long)len);
  if (!in || !out || in == out) return fail(WC_ERR_ARG, "in and out must be distinct device buffers");
  // No library stream is created here: NULL means the legacy default stream.
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned char* base = nullptr;
  WC_TRY(noalloc_base(&base, s, true));
  switch (precision) {
    case WC_F64_EXACT: return dispatch_noalloc<PExact>(in, out, len, sense, J, filter, s, base);
    case WC_F64_FAST: return dispatch_noalloc<PDD>(in, out, len, sense, J, filter, s, base);
    default: return dispatch_noalloc<PF32>(in, out, len, sense, J, filter, s, base);
  }
}

// ------------------------------------------------------------- autotune --

namespace wc {
namespace {

int check_cfg(int F, int prec, const TileCfg& c) {
  if (F < 1 || F > 4 || prec < 0 || prec > 2) return fail(WC_ERR_ARG, "bad filter/precision");
  if (c.tile < 256 || c.tile > 16384 || (c.tile & (c.tile - 1)) != 0)
    return fail(WC_ERR_ARG, "tile %d must be a power of two in [256, 16384]", c.tile);
  if (c.g0 < 1 || c.g0 > 14 || (1 << c.g0) > c.tile)
    return fail(WC_ERR_ARG, "levels per first pass %d out of range for tile %d", c.g0, c.tile);
  if (c.threads != 256 && c.threads != 512) return fail(WC_ERR_ARG, "threads must be 256 or 512");
  return WC_OK;
}

}  // namespace
}  // namespace wc

extern "C" int wc_set_dwt_tiling(int filter, int precision, int tile, int g0, int threads,
                                 int pipelined) {
  using namespace wc;
  clear_error();
  TileCfg c{tile, g0, threads, pipelined ? 1 : 0};
  WC_TRY(check_cfg(filter, precision, c));
  set_cfg(filter, precision, c);
  return WC_OK;
}

extern "C" int wc_get_dwt_tiling(int filter, int precision, int* tile, int* g0, int* threads,
                                 int* pipelined) {
  using namespace wc;
  clear_error();
  if (filter < 1 || filter > 4 || precision < 0 || precision > 2)
    return fail(WC_ERR_ARG, "bad filter/precision");
  const TileCfg c = get_cfg(filter, precision);
  if (tile) *tile = c.tile;
  if (g0) *g0 = c.g0;
  if (threads) *threads = c.threads;
  if (pipelined) *pipelined = c.pipe;
  return WC_OK;
}

// Times forward+inverse DWT (J = log2n - 2 levels, capped at 16) on a random
// signal of 2^log2n samples for each candidate tiling and keeps the fastest.
extern "C" int wc_tune_dwt(int filter, int precision, int log2n, float* best_ms) {
  using namespace wc;
  clear_error();
  WC_TRY(ensure_device());
  if (filter < 1 || filter > 4 || precision < 0 || precision > 2)
    return fail(WC_ERR_ARG, "bad filter/precision");
  if (log2n < 14 || log2n > 28) return fail(WC_ERR_ARG, "log2n must lie in [14, 28]");
  const int64_t n = (int64_t)1 << log2n;
  const size_t es = (precision == WC_F32) ? 4 : 8;
  const int J = std::min(16, check_levels(n, 0, filter_len(filter)));
  void* a = nullptr;
  void* b = nullptr;
  WC_CUDA(cudaMalloc(&a, es * (size_t)n));
  if (cudaMalloc(&b, es * (size_t)n) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(a);
    return fail(WC_ERR_NOMEM, "tuning buffers");
  }
  cudaStream_t s = lib_stream();
  if (fill_noise(a, n, es, s) != WC_OK) {
    cudaFree(a);
    cudaFree(b);
    return fail(WC_ERR_CUDA, "tuning signal");
  }
  const TileCfg keep = get_cfg(filter, precision);
  const int gm = gmax_of(filter);
  std::vector<TileCfg> cand;
  const int tiles8[3] = {1024, 2048, 4096}, tiles4[3] = {2048, 4096, 8192};
  for (int ti = 0; ti < 3; ti++) {
    const int tile = (precision == WC_F32) ? tiles4[ti] : tiles8[ti];
    for (int g : {gm - 2, gm - 1, gm, gm + 1}) {
      if (g < 1 || (1 << g) > tile) continue;
      for (int th : {256, 512})
        for (int pp : {1, 0}) cand.push_back(TileCfg{tile, g, th, pp});
    }
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  TileCfg best_c = keep;
  int rc = WC_OK;
  for (const TileCfg& c : cand) {
    set_cfg(filter, precision, c);
    float ms_min = 1e30f;
    for (int rep = 0; rep < 4 && rc == WC_OK; rep++) {
      cudaEventRecord(e0, s);
      rc = dwt(a, b, n, 1, J, filter, precision, s);
      if (rc == WC_OK) rc = dwt(b, a, n, 0, J, filter, precision, s);
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0) ms_min = std::min(ms_min, ms);
    }
    if (rc != WC_OK) break;
    if (ms_min < best) {
      best = ms_min;
      best_c = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(a);
  cudaFree(b);
  set_cfg(filter, precision, rc == WC_OK ? best_c : keep);
  if (best_ms) *best_ms = best;
  return rc;
}
