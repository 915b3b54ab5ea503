// Bulk asynchronous copies global -> shared with mbarrier completion (sm_90+ PTX), used by
// the z passes to stage the next tile's pencils while the current tile computes.
//
// One thread arms the barrier with the byte count of the tile (arrive.expect_tx), then
// the lanes of one warp issue one cp.async.bulk per pencil row; each copy decrements the
// barrier's transaction count as its bytes land. The barrier's phase completes when the
// armed arrival has happened and every byte has landed; consumers wait on the phase
// parity. Copies address only this CTA's own shared memory and this GPU's own global
// memory (no cluster multicast). Every address and size is a multiple of 16 bytes.
#pragma once
#include <stdint.h>

namespace peec {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}

// makes the initialised barrier visible to the async proxy (the bulk copies)
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// waits for the barrier phase of the given parity, giving up after `limit` polls
// (each poll may suspend the thread for a short hardware-chosen time)
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int limit) {
  for (int i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// orders this thread's earlier shared-memory accesses (and, through the barrier that
// precedes it, the block's) before its later async-proxy copies into the same buffer
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// bytes (a multiple of 16) from global src to shared dst (both 16-byte aligned),
// completing on bar
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

}  // namespace peec
