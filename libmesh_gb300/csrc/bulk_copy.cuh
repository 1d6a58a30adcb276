// Bulk asynchronous copies (TMA, non-tensor form) from global into shared
// memory, completed on shared-memory mbarriers, and bounded waits on them.
//
// A copy needs 16-byte aligned source and destination addresses and a size
// that is a multiple of 16 bytes; callers round the source down to its 16-byte
// boundary, copy the slack with it and index past it in shared memory.  No
// wait spins without a limit: mbar_wait gives up after `limit` polls and the
// caller reports an error status instead of hanging.
#pragma once

#include <cstdint>

namespace lmg {

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *m, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(m)), "r"(count) : "memory");
}

// Makes initialised barriers visible to the asynchronous proxy.
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// One arrival that also announces `bytes` of copies completing on m.
__device__ __forceinline__ void mbar_expect_tx(uint64_t *m, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(m)), "r"(bytes) : "memory");
}

// Orders this thread's earlier shared-memory accesses before later accesses of
// the asynchronous proxy (a bulk copy overwriting what was read).
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Copies `bytes` from global `src` into shared `dst`; completion counts on m.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *m) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(m))
               : "memory");
}

// Waits for the phase of m with parity `parity` to complete; false after
// `limit` polls without completion.
__device__ __forceinline__ bool mbar_wait(uint64_t *m, uint32_t parity, int limit) {
  uint32_t done = 0;
  for (int it = 0; it < limit && !done; ++it)
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_addr(m)), "r"(parity)
        : "memory");
  return done != 0;
}

}  // namespace lmg
