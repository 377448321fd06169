// Exact replay of the reference's sequential FP64 loss sum
//     m = (((0 + v_0) + v_1) + ... + v_{n-1}),   result m * 0.5
// (interp_mse, thresh.cpp:363-383) with every addition rounded exactly as the
// serial loop rounds it, computed in parallel.
//
// Why it can be parallel.  Every term is a sum of squares, v_k >= 0, so the
// running sum never decreases.  While m stays inside one binade [2^e, 2^(e+1))
// all representable results are multiples of u = 2^(e-52), m is one of them,
// and fl(m + v) = m + u * rne(v / u) exactly -- unless v/u is exactly half way
// between integers, where round-half-even looks at m's last bit.  So inside a
// binade a run of terms adds the *integer* sum of q_k = rne(v_k / u) to m's
// significand: associative, hence parallel.  Only three events need the
// serial rule: a binade crossing, an exact tie, and a zero/subnormal m.
//
// Kernels (chunks of B = 1024 terms):
//  1. chunk_sums    S_c = sum of chunk c (any order; only an estimate)
//  2. chunk_scan    P_c = exclusive prefix of S_c; the binade of the true m at
//                   chunk start is that of P_c or a neighbour (the serial sum
//                   differs from P_c by far less than a factor of two)
//  3. chunk_q       for the 3 candidate binades of each chunk, Q = sum q_k,
//                   or -1 if a term ties or reaches the binade's size
//  4. replay        one block walks the chunks: when m's binade is a
//                   candidate with a valid Q that keeps m inside the binade,
//                   m's bit pattern advances by Q; otherwise the block replays
//                   that chunk: a block-wide prefix sum of q finds the first
//                   term that ties or leaves the binade, everything before it
//                   is added at once and that one term is added with a real
//                   FP64 addition.
// The integer q_k come from the bit patterns alone (no FP64 arithmetic).
#include "wc_common.cuh"

namespace wc {
namespace {

constexpr int kB = 1024;           // terms per chunk (= replay block size)
constexpr int kSumThreads = 256;   // threads of the per-chunk kernels
constexpr uint64_t kFrac = (1ull << 52) - 1;

// q = rne(v / u) for the binade with biased exponent eb_m; bad when the term
// ties, is not below 2^e, or the binade is not a normal one.
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
  const uint64_t rem = M & ((1ull << s) - 1);
  const uint64_t half = 1ull << (s - 1);
  if (rem == half) {
    bad = true;
    return;
  }
  q = (long long)((M >> s) + (rem > half ? 1 : 0));
}

__device__ __forceinline__ double block_sum_double(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x < 32) {
    t = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  }
  __syncthreads();
  return t;  // valid in thread 0
}

__global__ void __launch_bounds__(kSumThreads)
chunk_sums(const double* __restrict__ v, int64_t n, double* __restrict__ S) {
  __shared__ double sh[32];
  const int64_t base = (int64_t)blockIdx.x * kB;
  double acc = 0.0;
  for (int k = threadIdx.x; k < kB; k += blockDim.x)
    if (base + k < n) acc += v[base + k];
  const double t = block_sum_double(acc, sh);
  if (threadIdx.x == 0) S[blockIdx.x] = t;
}

__global__ void __launch_bounds__(1024)
chunk_scan(const double* __restrict__ S, int64_t C, int* __restrict__ ebhat) {
  __shared__ double sh[1024];
  __shared__ double carry;
  if (threadIdx.x == 0) carry = 0.0;
  __syncthreads();
  for (int64_t seg = 0; seg < C; seg += 1024) {
    const int64_t c = seg + threadIdx.x;
    sh[threadIdx.x] = (c < C) ? S[c] : 0.0;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {  // Hillis-Steele inclusive scan
      const double add = (threadIdx.x >= o) ? sh[threadIdx.x - o] : 0.0;
      __syncthreads();
      sh[threadIdx.x] += add;
      __syncthreads();
    }
    const double excl = carry + ((threadIdx.x > 0) ? sh[threadIdx.x - 1] : 0.0);
    if (c < C) ebhat[c] = (int)(((uint64_t)__double_as_longlong(excl) >> 52) & 0x7FF);
    __syncthreads();
    if (threadIdx.x == 0) carry += sh[1023];
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kSumThreads)
chunk_q(const double* __restrict__ v, int64_t n, const int* __restrict__ ebhat,
        long long* __restrict__ Q) {
  __shared__ long long shq[3][kSumThreads / 32];
  __shared__ int shbad[3];
  const int64_t c = blockIdx.x, base = c * kB;
  const int eb0 = ebhat[c];
  if (threadIdx.x < 3) shbad[threadIdx.x] = 0;
  __syncthreads();
  long long tot[3] = {0, 0, 0};
  bool bad[3] = {false, false, false};
  for (int k = threadIdx.x; k < kB; k += blockDim.x) {
    if (base + k >= n) break;
    const double x = v[base + k];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      long long q;
      bool b;
      q_of(x, eb0 - 1 + d, q, b);
      tot[d] += q;
      bad[d] |= b;
    }
  }
#pragma unroll
  for (int d = 0; d < 3; d++) {
    long long t = tot[d];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if ((threadIdx.x & 31) == 0) shq[d][threadIdx.x >> 5] = t;
    if (bad[d]) shbad[d] = 1;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    long long t = 0;
    for (int w = 0; w < kSumThreads / 32; w++) t += shq[threadIdx.x][w];
    Q[c * 3 + threadIdx.x] = shbad[threadIdx.x] ? -1 : t;
  }
}

// Inclusive block scan of a 64-bit integer over 1024 threads.
__device__ __forceinline__ long long block_incl_scan(long long x, long long* warp_tot) {
  const int l = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    const long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (l >= o) x += y;
  }
  if (l == 31) warp_tot[w] = x;
  __syncthreads();
  if (w == 0) {
    long long t = warp_tot[l];
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, t, o);
      if (l >= o) t += y;
    }
    warp_tot[l] = t;
  }
  __syncthreads();
  const long long r = x + (w > 0 ? warp_tot[w - 1] : 0);
  __syncthreads();
  return r;
}

constexpr int kSeg = 1024;  // chunks staged in shared memory at a time

__global__ void __launch_bounds__(1024)
replay(const double* __restrict__ v, int64_t n, const long long* __restrict__ Q,
       const int* __restrict__ ebhat, int64_t C, double* __restrict__ out) {
  __shared__ long long sQ[kSeg * 3];
  __shared__ int sE[kSeg];
  __shared__ long long warp_tot[32];
  __shared__ unsigned long long s_mb;
  __shared__ long long s_c, s_add;
  __shared__ int s_kstar;
  const int tid = threadIdx.x;
  if (tid == 0) s_mb = 0ull;
  for (int64_t seg = 0; seg < C; seg += kSeg) {
    const int64_t seg_end = (seg + kSeg < C) ? seg + kSeg : C;
    for (int64_t i = tid; i < (seg_end - seg) * 3; i += blockDim.x) sQ[i] = Q[seg * 3 + i];
    for (int64_t i = tid; i < seg_end - seg; i += blockDim.x) sE[i] = ebhat[seg + i];
    __syncthreads();
    int64_t c = seg;
    while (true) {
      if (tid == 0) {
        unsigned long long mb = s_mb;
        int64_t cc = c;
        for (; cc < seg_end; cc++) {
          const int eb = (int)(mb >> 52);
          const int i = eb - sE[cc - seg] + 1;
          if (mb == 0ull || i < 0 || i > 2) break;
          const long long q = sQ[(cc - seg) * 3 + i];
          if (q < 0 || (mb & kFrac) + (unsigned long long)q >= (1ull << 52)) break;
          mb += (unsigned long long)q;
        }
        s_mb = mb;
        s_c = cc;
      }
      __syncthreads();
      c = s_c;
      if (c >= seg_end) break;
      // Replay chunk c with the block: one term per thread.
      const int64_t base = c * kB;
      const int len = (int)((n - base < kB) ? (n - base) : kB);
      const double myv = (tid < len) ? v[base + tid] : 0.0;
      int pos = 0;
      while (pos < len) {
        const unsigned long long mb = s_mb;
        long long q = 0;
        bool bad = false;
        const bool active = (tid >= pos) && (tid < len);
        if (active) q_of(myv, (int)(mb >> 52), q, bad);
        if (!active || bad) q = 0;
        const long long incl = block_incl_scan(q, warp_tot);
        const bool stop = active && (bad || (mb & kFrac) + (unsigned long long)incl >= (1ull << 52));
        if (tid == 0) s_kstar = len;
        __syncthreads();
        if (stop) atomicMin(&s_kstar, tid);
        __syncthreads();
        const int kstar = s_kstar;
        if (kstar == len) {
          if (tid == len - 1) s_add = incl;
        } else if (tid == kstar) {
          s_add = incl - q;
        }
        __syncthreads();
        if (tid == 0) {
          unsigned long long m2 = s_mb + (unsigned long long)s_add;
          if (kstar < len)
            m2 = (unsigned long long)__double_as_longlong(
                __dadd_rn(__longlong_as_double((long long)m2), v[base + kstar]));
          s_mb = m2;
        }
        __syncthreads();
        pos = kstar + 1;
      }
      c++;
    }
    __syncthreads();
  }
  if (tid == 0) *out = __dmul_rn(__longlong_as_double((long long)s_mb), 0.5);
}

}  // namespace

// Scratch: C doubles, C ints, 3C long longs after the terms' own buffer.
size_t cv_sum_scratch_bytes(int64_t count) {
  const int64_t C = (count + kB - 1) / kB;
  return (size_t)C * (sizeof(double) + sizeof(int) + 3 * sizeof(long long)) + 256;
}

int cv_sequential_sum(const double* terms, int64_t count, double* dev_out, void* scratch,
                      cudaStream_t s) {
  const int64_t C = (count + kB - 1) / kB;
  char* p = static_cast<char*>(scratch);
  long long* Q = reinterpret_cast<long long*>(p);
  double* S = reinterpret_cast<double*>(p + (size_t)C * 3 * sizeof(long long));
  int* eb = reinterpret_cast<int*>(p + (size_t)C * 3 * sizeof(long long) + (size_t)C * sizeof(double));
  {
    LaunchTimer lt("cv_sum_chunks", s);
    chunk_sums<<<(unsigned)C, kSumThreads, 0, s>>>(terms, count, S);
  }
  WC_TRY(after_launch("chunk_sums"));
  chunk_scan<<<1, 1024, 0, s>>>(S, C, eb);
  WC_TRY(after_launch("chunk_scan"));
  {
    LaunchTimer lt("cv_sum_q", s);
    chunk_q<<<(unsigned)C, kSumThreads, 0, s>>>(terms, count, eb, Q);
  }
  WC_TRY(after_launch("chunk_q"));
  {
    LaunchTimer lt("cv_sum_replay", s);
    replay<<<1, 1024, 0, s>>>(terms, count, Q, eb, C, dev_out);
  }
  return after_launch("replay");
}

}  // namespace wc
