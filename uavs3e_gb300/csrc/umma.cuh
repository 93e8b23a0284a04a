// 5th-generation tensor-core (tcgen05) helpers for sm_100-family GPUs (sm_103a here): tensor
// memory (TMEM) allocation, the bf16 x bf16 -> f32 MMA with shared-memory operand descriptors,
// commit to an mbarrier, and TMEM -> register loads.
//
// Operand layout used throughout: "K-major, no swizzle".  A tile of R rows x K columns (bf16,
// K a multiple of 16) is stored as 8 x 8 core matrices of 128 contiguous bytes (8 rows of 16
// bytes); core matrices adjacent along K are 128 bytes apart (the descriptor's leading byte
// offset) and 8-row groups are K * 16 bytes apart (its stride byte offset):
//     byte(r, k) = (r / 8) * (K * 16) + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2.
// One MMA consumes 16 columns of K, i.e. the descriptor of step s starts s * 256 bytes in.
//
// "MN-major, no swizzle" (the operand transposed): a core matrix holds 8 MN-consecutive elements
// (16 bytes) for each of 8 consecutive K (128 contiguous bytes); the descriptor's leading byte
// offset is then the distance between core matrices adjacent along K and its stride byte offset
// the distance between core matrices adjacent along MN.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace uc {

__host__ __device__ constexpr uint32_t umma_tile_off(int r, int k, int K)
{
    return (uint32_t)((r >> 3) * (K * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// shared-memory matrix descriptor: start address, leading byte offset (K direction of a K-major
// operand), stride byte offset (its 8-row groups), descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// descriptor of an MN-major, no-swizzle operand (layout above): mn_stride = bytes between core
// matrices adjacent along M (or N), k_stride = bytes between core matrices adjacent along K
__device__ __forceinline__ uint64_t umma_desc_mn(uint32_t saddr, uint32_t mn_stride, uint32_t k_stride)
{
    return umma_desc(saddr, k_stride, mn_stride);
}

// instruction descriptor of kind::f16 with bf16 A and B (both the same type), f32 accumulator,
// M x N; A and B K-major unless a_mn / b_mn (bits 15 / 16: the operand is MN-major)
__host__ __device__ constexpr uint32_t umma_idesc_bf16(int M, int N, bool a_mn = false, bool b_mn = false)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((a_mn ? 1u : 0u) << 15) | ((b_mn ? 1u : 0u) << 16) |
           ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// TMEM allocation of ncols columns (a power of two >= 32) by one whole warp; the address is
// written to shared memory at smem_dst
__device__ __forceinline__ void tmem_alloc(uint32_t smem_dst, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_dst), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread
__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate)
{
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "setp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                 ::"r"(d_tmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
                 : "memory");
}

// the mbarrier receives one arrival once every MMA this thread issued before has completed
__device__ __forceinline__ void umma_commit(uint32_t mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

__device__ __forceinline__ void tc_fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

// 16 consecutive 32-bit TMEM columns of the warp's 32 lanes (lane quarter = warp index % 4)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                 "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                   "=r"(r[15])
                 : "r"(taddr)
                 : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

}  // namespace uc
