// Grid-wide barrier for persistent cooperative kernels.
//
// Every CTA of a cooperative launch is resident at once, so the CTAs can
// meet at a barrier in global memory: thread 0 of each CTA makes its CTA's
// writes visible (fence), counts itself in with atomics, and the last CTA
// to arrive resets the counts and advances a generation word that the others
// poll with acquire loads.  The wait is bounded: after kGridMaxSpins polls a
// CTA records a timeout in the status word and the call returns false, so a
// kernel whose CTAs no longer meet ends instead of hanging the GPU.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "wc_bulk.cuh"

namespace wc {

constexpr unsigned int kGridMaxSpins = 1u << 22;

__device__ __forceinline__ unsigned int ld_acquire_gpu(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Two-level arrival: CTAs count themselves in at one of several group
// counters (kGridGroup CTAs each, every counter on its own 128-byte line),
// and only the last CTA of each group counts the group in at the top
// counter, so no address takes more than max(kGridGroup, groups) atomics.
// bar[0]: groups arrived; bar[1]: generation; bar[32 * (1 + g)]: CTAs of
// group g arrived.  All start at zero; the caller provides
// grid_bar_words(nblocks) words.  `gen` is the caller's count of barriers
// passed (the same in every CTA).  Returns false in every thread of the CTA
// when the wait gave up.
constexpr unsigned int kGridGroup = 16;

__host__ __device__ constexpr size_t grid_bar_words(unsigned int nblocks) {
  return 32u * (1u + (nblocks + kGridGroup - 1) / kGridGroup);
}

__device__ __forceinline__ bool grid_sync(unsigned int* bar, unsigned int nblocks,
                                          unsigned int& gen, unsigned int* status) {
  __syncthreads();
  int ok = 1;
  if (threadIdx.x == 0) {
    const unsigned int g = gen;
    const unsigned int grp = blockIdx.x / kGridGroup;
    const unsigned int ngroups = (nblocks + kGridGroup - 1) / kGridGroup;
    const unsigned int in_grp =
        (grp + 1 < ngroups) ? kGridGroup : nblocks - (ngroups - 1) * kGridGroup;
    unsigned int* gc = bar + 32 * (1 + grp);
    __threadfence();
    bool last = false;
    if (atomicAdd(gc, 1u) == in_grp - 1) {
      atomicExch(gc, 0u);
      __threadfence();
      last = atomicAdd(bar, 1u) == ngroups - 1;
    }
    if (last) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicExch(bar + 1, g + 1);
    } else {
      unsigned int it = 0;
      while (ld_acquire_gpu(bar + 1) == g) {
        if (++it > kGridMaxSpins) {
          if (status) atomicOr(status, kStatusTimeout);
          ok = 0;
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
  }
  gen++;
  return __syncthreads_and(ok) != 0;
}

}  // namespace wc
