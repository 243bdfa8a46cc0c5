// gs_tc.cuh -- tcgen05 (5th-generation tensor core) helpers for sm_103a,
// inline PTX: TMEM allocation, BF16 MMA with FP32 accumulation in TMEM,
// completion through an mbarrier, TMEM -> register loads.
//
// Shared-memory operands use the canonical no-swizzle layout: the matrix is
// cut into "core matrices" of 8 rows x 16 bytes (8 BF16), each stored as
// 128 contiguous bytes, row r at +16 r.
//   K-major   (rows along M/N, the 8 contiguous elements along K)
//   MN-major  (rows along K, the 8 contiguous elements along M/N)
// In both, the descriptor's leading byte offset (LBO) is the distance between
// core matrices adjacent along K and the stride byte offset (SBO) the
// distance between core matrices adjacent along M/N.
#pragma once

#include <cstdint>

#include "gs_ptx.cuh"

namespace gs {

// Byte offset of element (r, k) of an R x K operand stored K-major with
// core matrices laid out K-fastest: lbo = 128, sbo = 128 * (K / 8).
__host__ __device__ __forceinline__ uint32_t kmajor_offset(int r, int k, int K)
{
    return (uint32_t)((r >> 3) * (K * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// Byte offset of element (r, k) (r along M/N, k along K) of an R x K
// operand stored MN-major with core matrices laid out MN-fastest:
// sbo = 128, lbo = 128 * (R / 8).
__host__ __device__ __forceinline__ uint32_t mnmajor_offset(int r, int k, int R)
{
    return (uint32_t)((k >> 3) * (R * 16) + (r >> 3) * 128 + (k & 7) * 16 + (r & 7) * 2);
}

// Shared-memory matrix descriptor (no swizzle).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3fff);
    d |= (uint64_t)((lbo >> 4) & 0x3fff) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3fff) << 32;
    d |= (uint64_t)1 << 46;   // descriptor version of this architecture
    // base offset 0, lbo mode 0, layout type 0 (no swizzle)
    return d;
}

// Instruction descriptor of kind::f16: BF16 x BF16 -> FP32, M x N.
__host__ __device__ __forceinline__ uint32_t idesc_bf16_f32(int M, int N, bool a_mn_major,
                                                            bool b_mn_major)
{
    uint32_t d = 0;
    d |= 1u << 4;                         // D format: F32
    d |= 1u << 7;                         // A format: BF16
    d |= 1u << 10;                        // B format: BF16
    d |= (a_mn_major ? 1u : 0u) << 15;
    d |= (b_mn_major ? 1u : 0u) << 16;
    d |= (uint32_t)(N >> 3) << 17;
    d |= (uint32_t)(M >> 4) << 24;
    return d;
}

// One warp allocates `ncols` TMEM columns (power of two >= 32) and writes the
// base address to *dst (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(dst)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
                 : "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T, one instruction (K = 16 for BF16).
__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc,
                                          uint32_t idesc, uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Arrive on `bar` when all prior MMAs issued by this thread have completed.
__device__ __forceinline__ void umma_commit(uint64_t *bar)
{
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Generic-proxy shared-memory writes -> visible to the tensor core.
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 32 lanes x 16 columns of 32-bit TMEM -> 16 registers per thread.
// Warp w (w = warp index % 4) may only read lanes 32w..32w+31.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace gs
