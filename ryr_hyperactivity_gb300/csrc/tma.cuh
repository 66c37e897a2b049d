// tma.cuh — asynchronous copies from global to shared memory: per-thread
// 16-byte cp.async (completed with cp.async.wait_all) and the TMA unit's 1-D
// cp.async.bulk (completed on an mbarrier, with bounded waits).
//
// Rules kept here: both addresses 16-byte aligned, sizes multiples of 16
// bytes, the mbarrier initialised and fenced before any copy names it, and
// every wait gives up after a fixed number of polls (the caller records the
// timeout and never reads the buffers).
#pragma once

#include <stdint.h>

namespace rh {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

// global -> shared bulk copy of `bytes` (multiple of 16, both ends 16-byte
// aligned), signalling `bar` with the transferred byte count
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// One thread's 16-byte global -> shared copy (both addresses 16-byte
// aligned); L1 is bypassed (.cg), the data goes straight to shared memory.
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_addr(dst)), "l"(src)
               : "memory");
}

// 8- and 4-byte variants (both addresses aligned to the size; cached in L1).
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(smem_addr(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(smem_addr(dst)), "l"(src)
               : "memory");
}

// Waits until every cp.async this thread issued has landed in shared memory
// (other threads' copies need a barrier after their own wait).
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// Copies `bytes` (a multiple of 16) from src to dst with the CTA's NT
// threads, 16 bytes per thread and round.
template <int NT>
__device__ __forceinline__ void cp_async_region(void* dst, const void* src, int bytes, int tid) {
  char* d = static_cast<char*>(dst);
  const char* s = static_cast<const char*>(src);
  for (int i = tid * 16; i < bytes; i += NT * 16) cp_async16(d + i, s + i);
}

// Polls the barrier's phase `parity` at most `max_polls` times; returns 1 when
// the phase completed, 0 on timeout.
__device__ __forceinline__ int mbar_wait(uint64_t* bar, uint32_t parity, uint32_t max_polls) {
  const uint32_t a = smem_addr(bar);
  for (uint32_t i = 0; i < max_polls; ++i) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return 1;
  }
  return 0;
}

}  // namespace rh
