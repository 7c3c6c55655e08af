// tc_cluster.cuh -- inline-PTX wrappers for bulk copies with
// transaction-count mbarriers, thread-block clusters (barrier, distributed
// shared memory) and proxy fences, as used by the cluster tensor-core
// kernel (sllg_tcc.cu).
#pragma once
#include <cstdint>
#include "tc_ptx.cuh"

namespace magpy {
namespace tc {

// Arrive on an mbarrier and add `bytes` to the transaction count its current
// phase waits for (the bulk copies that complete_tx on it).
__device__ inline void mbar_arrive_expect_tx(void *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                 :
                 : "r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// Bulk copy global -> this CTA's shared memory (the untiled form: both
// addresses 16-byte aligned, size a multiple of 16), completing `bytes` on
// the mbarrier.
__device__ inline void bulk_g2s(void *dst_smem, const void *src_gmem, uint32_t bytes, void *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        :
        : "r"(smem_addr(dst_smem)), "l"(src_gmem), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ inline uint32_t cluster_ctarank()
{
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

// Every thread of every CTA of the cluster arrives (release) and waits
// (acquire): a hardware barrier that orders each CTA's earlier memory
// operations (shared and global) before the other CTAs' later ones.
__device__ inline void cluster_sync()
{
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
    asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Address of the same shared-memory location in CTA `rank` of the cluster.
__device__ inline uint32_t mapa(uint32_t saddr, uint32_t rank)
{
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(saddr), "r"(rank));
    return r;
}

__device__ inline double ld_cluster_f64(uint32_t caddr)
{
    double v;
    asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(caddr) : "memory");
    return v;
}

__device__ inline int32_t ld_cluster_s32(uint32_t caddr)
{
    int32_t v;
    asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(caddr) : "memory");
    return v;
}

// Orders this thread's generic-proxy global accesses with its async-proxy
// (bulk copy) accesses, both ways.
__device__ inline void fence_proxy_async_global()
{
    asm volatile("fence.proxy.async.global;" ::: "memory");
}

}  // namespace tc
}  // namespace magpy
