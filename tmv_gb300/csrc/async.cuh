// async.cuh -- mbarrier, bulk-copy and cluster-store helpers (inline PTX, sm_103a).
#pragma once

#include <stdint.h>

namespace tmvg {

// Polls of a bounded mbarrier wait before it reports a timeout.
constexpr unsigned kTryWaitLimit = 1u << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Makes initialised mbarriers visible to the async proxy and the cluster.
__device__ __forceinline__ void mbar_fence_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// One arrival that also expects `bytes` of transactions in the current phase.
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

// Wait for the phase with the given parity to complete; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity)
{
    for (unsigned spins = 0; spins < kTryWaitLimit; ++spins) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// The shared::cluster address of the same shared variable in CTA `rank`.
__device__ __forceinline__ uint32_t cluster_addr(const void* p, int rank)
{
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_u32(p)), "r"(rank));
    return r;
}

// 16-byte store into another CTA's shared memory that completes `bytes`
// transactions on that CTA's mbarrier (both addresses from cluster_addr).
__device__ __forceinline__ void st_async16(uint32_t dst, const uint4& v, uint32_t mbar)
{
    asm volatile(
        "st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.b32 [%0], {%1, %2, %3, %4}, [%5];" ::"r"(dst),
        "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w), "r"(mbar)
        : "memory");
}

// Wait with cluster-scope acquire (pairs with release arrivals from other
// CTAs of the cluster); false on timeout.
__device__ __forceinline__ bool mbar_wait_cluster(uint64_t* bar, uint32_t parity)
{
    for (unsigned spins = 0; spins < kTryWaitLimit; ++spins) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Arrival on an mbarrier of another CTA (address from cluster_addr) with
// cluster-scope release: this thread's earlier writes, and those it has
// observed, are visible to a thread that acquires the completed phase.
__device__ __forceinline__ void mbar_arrive_remote_release(uint32_t bar)
{
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(bar) : "memory");
}

// 16-byte store into / load from another CTA's shared memory.
__device__ __forceinline__ void st_cluster16(uint32_t dst, const uint4& v)
{
    asm volatile("st.shared::cluster.v4.u32 [%0], {%1, %2, %3, %4};" ::"r"(dst), "r"(v.x), "r"(v.y),
                 "r"(v.z), "r"(v.w)
                 : "memory");
}

// Orders this thread's earlier generic-proxy shared-memory writes before its
// (or, after a warp/CTA barrier, its peers') later async-proxy operations.
__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Bulk copy of `bytes` (a multiple of 16, both addresses 16-byte aligned)
// from this CTA's shared memory to the shared memory of a CTA of the cluster,
// completing `bytes` transactions on that CTA's mbarrier (dst and mbar from
// cluster_addr).
__device__ __forceinline__ void bulk_s2cluster(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.shared::cta.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
        "r"(smem_u32(src)), "r"(bytes), "r"(mbar)
        : "memory");
}

__device__ __forceinline__ uint4 ld_cluster16(uint32_t src)
{
    uint4 v;
    asm volatile("ld.shared::cluster.v4.u32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "r"(src)
                 : "memory");
    return v;
}

}  // namespace tmvg
