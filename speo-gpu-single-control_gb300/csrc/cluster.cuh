// cluster.cuh -- thread-block-cluster helpers (sm_90 and later): this block's rank in its cluster,
// addresses in a peer block's shared memory, remote shared-memory stores, and the cluster barrier.
#pragma once

#include <stdint.h>

namespace speo {

__device__ __forceinline__ uint32_t cluster_rank()
{
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t map_peer(const void *p, uint32_t peer)
{
    uint32_t out;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;"
                 : "=r"(out)
                 : "r"((uint32_t)__cvta_generic_to_shared(p)), "r"(peer));
    return out;
}
__device__ __forceinline__ void st_peer4(uint32_t addr, float4 v)
{
    asm volatile("st.shared::cluster.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "f"(v.x), "f"(v.y), "f"(v.z),
                 "f"(v.w)
                 : "memory");
}
__device__ __forceinline__ void st_peer1(uint32_t addr, float v)
{
    asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(addr), "f"(v) : "memory");
}
// All threads of both blocks: writes before it (local and remote) are visible after it.
__device__ __forceinline__ void cluster_sync()
{
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

}  // namespace speo
