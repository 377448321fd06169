// Bulk asynchronous copies between global and shared memory (the TMA's
// non-tensor "cp.async.bulk" form) with an mbarrier, written as inline PTX
// for sm_90+ (used here on sm_103a).
//
// Rules the callers keep: global and shared addresses 16-byte aligned, sizes
// multiples of 16 bytes, one mbarrier phase per staged load.  Every wait is
// bounded: after kMaxPolls unsuccessful polls the waiting thread records a
// timeout in the device status word (read with wc_device_status) and the
// kernel skips its work instead of hanging the GPU.  The status word lives in
// the library workspace (wc::device_status_word); every host-buffer call reads
// and clears it after its work and returns WC_ERR_TIMEOUT when the bit is
// set, and wc_device_status() reads it for the asynchronous device-pointer
// calls.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace wc {

// Status word bit: a bounded wait gave up.
constexpr unsigned int kStatusTimeout = 1u;

constexpr unsigned int kMaxPolls = 1u << 26;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

// Global -> shared bulk copy completing on `bar`.
__device__ __forceinline__ void bulk_g2s(void* dst_smem, const void* src_gmem, uint32_t bytes,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst_smem)),
      "l"(src_gmem), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// Bounded wait for phase `parity` of `bar`; false when it gave up after
// max_polls unsuccessful polls (each poll may suspend the thread for a short,
// hardware-defined time).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, unsigned int* status,
                                          unsigned int max_polls = kMaxPolls) {
  const uint32_t a = smem_u32(bar);
  for (unsigned int it = 0; it < max_polls; it++) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  if (status) atomicOr(status, kStatusTimeout);
  return false;
}

// Invalidates an mbarrier whose shared memory is about to be reused.
__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Makes this thread's generic-proxy shared-memory writes visible to the
// async proxy (required before a bulk store reads them).
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Shared -> global bulk copy (bulk-group completion).
__device__ __forceinline__ void bulk_s2g(void* dst_gmem, const void* src_smem, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst_gmem),
               "r"(smem_u32(src_smem)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void bulk_commit() {
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

// Waits until the committed bulk stores have finished reading shared memory.
__device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}

__device__ __forceinline__ bool aligned16(const void* p) {
  return (reinterpret_cast<uintptr_t>(p) & 15) == 0;
}

// Per-thread asynchronous copy of one 4- or 8-byte element from global to
// shared memory (cp.async, sm_80 and later): the load needs no register, so a
// thread can keep all its copies in flight at once.  cp_async_wait_all()
// waits for the calling thread's copies (a hardware wait on plain loads,
// which always complete).
template <class T>
__device__ __forceinline__ void cp_async_elem(T* smem_dst, const T* gsrc) {
  static_assert(sizeof(T) == 4 || sizeof(T) == 8, "4- or 8-byte elements");
  if constexpr (sizeof(T) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(smem_dst)), "l"(gsrc)
                 : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(smem_dst)), "l"(gsrc)
                 : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;" ::: "memory");
}

// Groups of per-thread asynchronous copies: commit closes the copies issued
// since the last commit; wait_prior_1 waits until at most the newest group
// is still in flight (double buffering).
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_prior_1() {
  asm volatile("cp.async.wait_group 1;" ::: "memory");
}

}  // namespace wc
