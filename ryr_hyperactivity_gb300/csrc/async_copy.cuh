// async_copy.cuh — per-thread asynchronous copies from global to shared
// memory (cp.async): the copy runs in the background, the issuing thread
// holds no register for the data, and cp.async.wait_all plus a CTA barrier
// make the tile visible to every thread.
#pragma once

#include <stdint.h>

namespace rh {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// 16-byte copy (both addresses 16-byte aligned); bypasses L1 (.cg).
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_addr(dst)), "l"(src)
               : "memory");
}

// 8- and 4-byte copies (both addresses aligned to the size; cached in L1).
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(smem_addr(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(smem_addr(dst)), "l"(src)
               : "memory");
}

// Closes the group of this thread's cp.async copies issued since the last
// commit; cp_async_wait_group<N> waits until at most N of its groups are
// still in flight (again only this thread's copies).
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait_group() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Waits until every cp.async this thread issued has landed in shared memory
// (other threads' copies need a barrier after their own wait).
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

}  // namespace rh
