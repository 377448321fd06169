// Device building blocks of the exact replay of the reference's serial FP64
// loss sum m = (((0 + v_0) + v_1) + ... + v_{n-1}) (interp_mse,
// thresh.cpp:363-383) for non-negative terms.
//
// While the running sum m stays in one binade [2^e, 2^(e+1)), every
// representable result is a multiple of u = 2^(e-52) and fl(m + v) =
// m + u * rne(v / u) exactly, unless v / u is exactly half way between two
// integers (round-half-even then looks at m's last bit).  So inside a binade
// a run of terms adds the integer sum of q_k = rne(v_k / u) to m's
// significand: an associative, hence parallel, operation.  Binade crossings,
// ties and a zero m take the serial rule (a real FP64 addition).
//
// Terms are grouped in chunks of kSeqChunk, each split into sub-chunks of
// kSeqSub.  The binade of the running sum at a chunk's start is that of the
// FP64 prefix of the chunk sums or a neighbour (any summation order is far
// closer than a factor of two), so the integer increments Q of every chunk
// and sub-chunk are computed in parallel for those three binades (-1 where a
// term ties).  One warp then walks the chunks 32 at a time with a prefix sum
// of their Q (for the binade the running sum is in); a chunk it cannot pass
// (binade crossing, tie, zero m)
// is walked sub-chunk by sub-chunk, and only a sub-chunk with an event is
// replayed term by term: a warp prefix sum of q finds the first term that
// ties or leaves the binade, everything before it is added at once and that
// one term is added with a real FP64 addition.  The integer q_k come from
// the bit patterns alone.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace wc {

constexpr int kSeqChunk = 1024;                // terms per chunk
constexpr int kSeqSub = 64;                    // terms per sub-chunk
constexpr int kSeqSubs = kSeqChunk / kSeqSub;  // sub-chunks per chunk (16)
constexpr uint64_t kSeqFrac = (1ull << 52) - 1;

// q = rne(v / u) for the binade with biased exponent eb_m; bad when the term
// ties, is not below 2^e, or the binade is not a normal one.
__device__ __forceinline__ void seq_q_of(double v, int eb_m, long long& q, bool& bad) {
  const uint64_t vb = (uint64_t)__double_as_longlong(v);
  const int ebv = (int)((vb >> 52) & 0x7FF);
  q = 0;
  bad = false;
  if (eb_m <= 0 || eb_m >= 0x7FF || ebv == 0x7FF || ebv >= eb_m) {
    bad = true;
    return;
  }
  const uint64_t M = (vb & kSeqFrac) | (ebv ? (1ull << 52) : 0ull);
  if (M == 0) return;
  const int s = eb_m - (ebv ? ebv : 1);
  if (s == 0) {
    q = (long long)M;
    return;
  }
  if (s > 63) return;
  const uint64_t rem = M & ((1ull << s) - 1);
  const uint64_t half = 1ull << (s - 1);
  if (rem == half) {
    bad = true;
    return;
  }
  q = (long long)((M >> s) + (rem > half ? 1 : 0));
}

// Q of one chunk and of its 16 sub-chunks of 64 terms for the binades
// eb0 - 1 .. eb0 + 1 (CTA-wide, blockDim 256: warp w covers sub-chunks 2w and
// 2w + 1, two terms per lane each).  sub_out receives 16 x 3 values,
// chunk_out 3 (-1 where a term ties or reaches the binade's size).
__device__ __forceinline__ void seq_chunk_q_subs(const double* __restrict__ v, int64_t base,
                                                 int len, int eb0, long long* s_sub /* 48 */,
                                                 long long* sub_out, long long* chunk_out) {
  const int l = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < 2; j++) {
    const int sb = 2 * w + j;
    long long tot[3] = {0, 0, 0};
    bool bad[3] = {false, false, false};
#pragma unroll
    for (int r = 0; r < 2; r++) {
      const int k = sb * kSeqSub + r * 32 + l;
      if (k < len) {
        const double x = v[base + k];
#pragma unroll
        for (int d = 0; d < 3; d++) {
          long long q;
          bool b;
          seq_q_of(x, eb0 - 1 + d, q, b);
          tot[d] += q;
          bad[d] |= b;
        }
      }
    }
#pragma unroll
    for (int d = 0; d < 3; d++) {
      long long t = tot[d];
      for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
      const bool anybad = __any_sync(0xffffffffu, bad[d]);
      if (l == 0) s_sub[sb * 3 + d] = anybad ? -1 : t;
    }
  }
  __syncthreads();
  if (threadIdx.x < kSeqSubs * 3) sub_out[threadIdx.x] = s_sub[threadIdx.x];
  if (threadIdx.x < 3) {
    long long t = 0;
    for (int sb = 0; sb < kSeqSubs; sb++) {
      const long long q = s_sub[sb * 3 + threadIdx.x];
      if (q < 0 || t < 0) t = -1;
      else t += q;
    }
    chunk_out[threadIdx.x] = t;
  }
  __syncthreads();
}

// One warp advances the running sum (bit pattern mb) over chunks [c, cend)
// while each chunk's Q for the current binade (candidates sQ[3 (c - base) +
// d] for the binades sE[c - base] - 1 + d) is valid and keeps m inside that
// binade.  Returns the first chunk not passed (cend when all were); every
// lane returns the same value and leaves the same mb.
__device__ __forceinline__ int64_t seq_walk(const long long* sQ, const int* sE, int64_t base,
                                            int64_t c, int64_t cend, unsigned long long& mb) {
  const int lane = threadIdx.x & 31;
  while (c < cend) {
    const int64_t cc = c + lane;
    const int eb = (int)(mb >> 52);
    long long q = 0;
    bool ok = false;
    if (cc < cend && mb != 0ull) {
      const int i = eb - sE[cc - base] + 1;
      if (i >= 0 && i <= 2) {
        q = sQ[(cc - base) * 3 + i];
        ok = q >= 0;
      }
    }
    const unsigned okm = __ballot_sync(0xffffffffu, ok);
    const int nok = (okm == 0xffffffffu) ? 32 : __ffs(~okm) - 1;
    long long s = (lane < nok) ? q : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    const bool over = lane < nok && (mb & kSeqFrac) + (unsigned long long)s >= (1ull << 52);
    const unsigned ovm = __ballot_sync(0xffffffffu, over);
    int k = nok;
    if (ovm) k = min(k, __ffs(ovm) - 1);
    const long long add = __shfl_sync(0xffffffffu, s, k > 0 ? k - 1 : 0);
    if (k > 0) mb += (unsigned long long)add;
    c += k;
    if (k < 32) break;
  }
  return c;
}

// One warp walks the sub-chunks sb .. 15 of one chunk while each one's Q
// (sub[3 s + d] for the binades eb0 - 1 + d) is valid for m's binade and
// keeps m inside it; returns the first sub-chunk not passed (16 when all
// were).  Same rule as seq_walk.
// Loads of the replay helpers: from shared memory, or from global memory
// that other CTAs wrote earlier in the same launch (ld.global.cg: served by
// L2, never by a stale L1 or read-only-cache line).
struct SeqLdShared {
  template <class X>
  __device__ __forceinline__ X operator()(const X* p) const {
    return *p;
  }
};
struct SeqLdGlobal {
  template <class X>
  __device__ __forceinline__ X operator()(const X* p) const {
    return __ldcg(p);
  }
};

template <class Ld = SeqLdShared>
__device__ __forceinline__ int seq_walk_subs(const long long* sub, int eb0, int sb,
                                             unsigned long long& mb) {
  const Ld ld{};
  const int l = threadIdx.x & 31;
  const int s = sb + l;
  const int eb = (int)(mb >> 52);
  long long q = 0;
  bool ok = false;
  if (s < kSeqSubs && mb != 0ull) {
    const int i = eb - eb0 + 1;
    if (i >= 0 && i <= 2) {
      q = ld(sub + 3 * s + i);
      ok = q >= 0;
    }
  }
  const unsigned okm = __ballot_sync(0xffffffffu, ok);
  const int nok = (okm == 0xffffffffu) ? 32 : __ffs(~okm) - 1;
  long long p = (l < nok) ? q : 0;
  for (int o = 1; o < 32; o <<= 1) {
    const long long y = __shfl_up_sync(0xffffffffu, p, o);
    if (l >= o) p += y;
  }
  const bool over = l < nok && (mb & kSeqFrac) + (unsigned long long)p >= (1ull << 52);
  const unsigned ovm = __ballot_sync(0xffffffffu, over);
  int k = nok;
  if (ovm) k = min(k, __ffs(ovm) - 1);
  const long long add = __shfl_sync(0xffffffffu, p, k > 0 ? k - 1 : 0);
  if (k > 0) mb += (unsigned long long)add;
  return sb + k;
}

// One warp replays the 64 terms v[0 .. 64) of a sub-chunk onto the running
// sum (bit pattern mb, the same in every lane), in the serial order: lane l
// holds terms 2l and 2l + 1; a warp prefix sum of their q finds the first
// term that ties or leaves the binade, everything before it is added at
// once, that term with a real FP64 addition, and the rest continues.
// v is 16-byte aligned.
template <class Ld = SeqLdShared>
__device__ __forceinline__ void seq_replay_sub_warp(const double* v, unsigned long long& mb) {
  const int l = threadIdx.x & 31;
  const double2 pr = Ld{}(reinterpret_cast<const double2*>(v) + l);
  const double v0 = pr.x, v1 = pr.y;
  int pos = 0;
  while (pos < kSeqSub) {
    const int eb = (int)(mb >> 52);
    const bool a0 = 2 * l >= pos, a1 = 2 * l + 1 >= pos;
    long long q0 = 0, q1 = 0;
    bool b0 = false, b1 = false;
    if (a0) seq_q_of(v0, eb, q0, b0);
    if (a1) seq_q_of(v1, eb, q1, b1);
    if (!a0 || b0) q0 = 0;
    if (!a1 || b1) q1 = 0;
    long long s = q0 + q1;
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, s, o);
      if (l >= o) s += y;
    }
    const long long ex = s - q0 - q1;  // sum of the terms before 2l
    const unsigned long long fr = mb & kSeqFrac;
    const bool st0 = a0 && (b0 || fr + (unsigned long long)(ex + q0) >= (1ull << 52));
    const bool st1 = a1 && (b1 || fr + (unsigned long long)(ex + q0 + q1) >= (1ull << 52));
    const unsigned sm = __ballot_sync(0xffffffffu, st0 || st1);
    if (sm == 0u) {
      mb += (unsigned long long)__shfl_sync(0xffffffffu, s, 31);
      break;
    }
    const int L = __ffs(sm) - 1;
    const int k = __shfl_sync(0xffffffffu, st0 ? 2 * l : 2 * l + 1, L);
    const long long pre = __shfl_sync(0xffffffffu, (k & 1) ? ex + q0 : ex, L);
    const double vk = __shfl_sync(0xffffffffu, (k & 1) ? v1 : v0, L);
    const unsigned long long m2 = mb + (unsigned long long)pre;
    mb = (unsigned long long)__double_as_longlong(
        __dadd_rn(__longlong_as_double((long long)m2), vk));
    pos = k + 1;
  }
}

// One warp replays a whole chunk onto mb, sub-chunk by sub-chunk: a run of
// sub-chunks whose Q applies is added at once, the others are replayed term
// by term.  v: the chunk's terms, len of them; sub: its 16 x 3 sub-chunk Q
// (binades eb0 - 1 .. eb0 + 1), or nullptr to replay every sub-chunk.  Ld:
// SeqLdShared when v and sub are in shared memory, SeqLdGlobal when they are
// global memory written earlier in the launch.
template <class Ld = SeqLdShared>
__device__ __forceinline__ void seq_replay_chunk_warp(const double* v, int len,
                                                      const long long* sub, int eb0,
                                                      unsigned long long& mb) {
  const Ld ld{};
  const int nsub = (len + kSeqSub - 1) / kSeqSub;
  int sb = 0;
  while (sb < nsub) {
    if (sub && len == kSeqChunk) sb = seq_walk_subs<Ld>(sub, eb0, sb, mb);
    if (sb >= nsub) break;
    if ((sb + 1) * kSeqSub <= len) {
      seq_replay_sub_warp<Ld>(v + sb * kSeqSub, mb);
    } else {
      // ragged tail: one term at a time (the same in every lane)
      for (int k = sb * kSeqSub; k < len; k++)
        mb = (unsigned long long)__double_as_longlong(
            __dadd_rn(__longlong_as_double((long long)mb), ld(v + k)));
    }
    sb++;
  }
}

}  // namespace wc
