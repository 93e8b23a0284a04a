// Tensor-memory-access (TMA) and mbarrier helpers (sm_90+ PTX, used on sm_103a) and the host-side
// tensor-map encoder.  Every wait on an mbarrier is bounded: it gives up after a fixed number
// of polls and reports it, so a copy that never lands cannot hang a kernel.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace uc {

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

// makes the initialised barriers visible to the async proxy (the TMA unit)
__device__ __forceinline__ void mbar_fence_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// one arrival that also announces `bytes` of transactions the phase must see before completing
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(bar), "r"(parity)
                 : "memory");
    return ok != 0;
}

// waits for the phase with the given parity to complete; false after `polls` unsuccessful polls
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, uint32_t polls)
{
    for (uint32_t i = 0; i < polls; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// orders this thread's earlier generic-proxy accesses of shared memory before later async-proxy
// (TMA) accesses
__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 2-D tiled load of the tensor map's box at (x, y) into shared memory at dst (128-byte aligned),
// completing `box bytes` of transactions on the mbarrier
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar)
{
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
                 ::"r"(dst), "l"((uint64_t)map), "r"(x), "r"(y), "r"(bar)
                 : "memory");
}

// host: a 2-D u8 tensor map over rows x row_bytes bytes at base (16-byte aligned, row pitch a
// multiple of 16) with a box of box_w x box_h bytes, out-of-range samples read as 0
int encode_tensor_map_u8(CUtensorMap *map, const void *base, uint64_t row_bytes, uint64_t rows, uint64_t pitch,
                         uint32_t box_w, uint32_t box_h);

}  // namespace uc
