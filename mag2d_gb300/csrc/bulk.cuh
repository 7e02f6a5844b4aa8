// Bulk asynchronous copies global -> shared (the TMA engine's untiled form,
// cp.async.bulk) completed on an mbarrier, and the bounded waits on them.
//
// A copy needs 16-byte aligned source and destination addresses and a size
// that is a multiple of 16 bytes.  Waits give up after kBulkWaitLimit polls
// (each poll may suspend the thread for a short, hardware-chosen time), so a
// copy that never lands turns into an error status instead of a hung kernel.
#pragma once
#include <cstdint>

namespace mag {

constexpr long long kBulkWaitLimit = 1ll << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t arrivals)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(arrivals) : "memory");
}

// makes barrier initialisation visible to the async proxy (the copy engine)
__device__ __forceinline__ void mbar_init_fence()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// orders this thread's earlier generic-proxy accesses of shared memory before
// later async-proxy accesses (a buffer read by threads, then refilled by a copy)
__device__ __forceinline__ void async_proxy_fence()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// one arrival that also announces the bytes the phase's copies will deliver
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// true once the barrier's phase with this parity completed, false after the limit
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity)
{
    for (long long it = 0; it < kBulkWaitLimit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

}  // namespace mag
