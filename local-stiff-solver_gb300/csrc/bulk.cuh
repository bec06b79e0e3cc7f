// Bulk global -> shared copies on the sm_103a copy engine (cp.async.bulk,
// completion counted on an mbarrier) with bounded waits.
//
// A wait polls the barrier a bounded number of times; when the bound runs out
// the caller records an error status and returns instead of spinning on.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace lss {

// polls of an mbarrier before a wait gives up (each poll sleeps ~64 ns)
constexpr uint32_t MBAR_POLL_LIMIT = 1u << 22;

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// makes initialised barriers visible to the copy engine
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// orders this thread's earlier generic shared-memory accesses (after a CTA
// barrier: the whole CTA's) before later bulk copies into the same bytes
__device__ __forceinline__ void proxy_async_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// dst, src 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// true once the phase with the given parity has completed; false when the
// poll limit ran out
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity)
{
    for (uint32_t k = 0; k < MBAR_POLL_LIMIT; ++k) {
        if (mbar_test(bar, parity)) return true;
        __nanosleep(64);
    }
    return false;
}

}  // namespace lss
