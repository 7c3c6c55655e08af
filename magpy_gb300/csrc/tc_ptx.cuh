// tc_ptx.cuh -- inline-PTX wrappers for the Blackwell tensor cores (tcgen05),
// tensor memory and mbarriers, as used by the tensor-core sLLG kernel.
//
// Operand layout (both operands K-major, no swizzle): an operand is a grid of
// 8x8 "core matrices" of 16-bit elements, each stored as 128 contiguous bytes
// (8 rows of 16 bytes).  Core matrices adjacent along K are `lbo` bytes apart,
// those adjacent along M (or N) are `sbo` bytes apart.
#pragma once
#include <cstdint>
#include <cuda_fp16.h>

namespace magpy {
namespace tc {

__device__ inline uint32_t smem_addr(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor (64-bit) for tcgen05.mma:
// [0,14) start >> 4, [16,30) leading byte offset >> 4, [32,46) stride byte
// offset >> 4, [46,48) version = 1, [49,52) base offset 0, [52] LBO mode 0,
// [61,64) swizzle = 0 (none).
__device__ inline uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor (32-bit) for kind::f16 with FP16 A and B, FP32
// accumulator, both K-major, dense: [4,6) D format (1 = F32), [7,10) A format
// (0 = F16), [10,13) B format (0 = F16), [15] A major, [16] B major,
// [17,23) N >> 3, [24,29) M >> 4.
__host__ __device__ constexpr uint32_t idesc_f16_f32(uint32_t M, uint32_t N)
{
    return (1u << 4) | (0u << 7) | (0u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread.
__device__ inline void mma_f16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                               uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
        :
        : "r"(d_tmem), "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// D[tmem] (+)= A[tmem] * B[smem]^T: A in tensor memory (row i in lane i, K
// along columns, two 16-bit elements per 32-bit column, the even K index in
// the low half), issued by one thread.
__device__ inline void mma_f16_ta(uint32_t d_tmem, uint32_t a_tmem, uint64_t b_desc,
                                  uint32_t idesc, uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}\n"
        :
        : "r"(d_tmem), "r"(a_tmem), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Arrive on an mbarrier once all prior tcgen05 operations of this thread complete.
__device__ inline void mma_commit(void *mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 :
                 : "r"(smem_addr(mbar))
                 : "memory");
}

// Warp-wide forms: every lane of a fully active warp executes the call with
// the same operands and one lane chosen by elect.sync issues.  The operands
// then stay warp-uniform; measured on GB300, a chain of M = 128, N = 16/32
// MMAs issued this way takes ~20-33 cycles per MMA against ~57 for the same
// chain issued from a lane-0 branch.
__device__ inline void mma_f16_ta_warp(uint32_t d_tmem, uint32_t a_tmem, uint64_t b_desc,
                                       uint32_t idesc, uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p, e;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "elect.sync _|e, 0xffffffff;\n\t"
        "@e tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}\n"
        :
        : "r"(d_tmem), "r"(a_tmem), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ inline void mma_f16_warp(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc,
                                    uint32_t idesc, uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p, e;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "elect.sync _|e, 0xffffffff;\n\t"
        "@e tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
        :
        : "r"(d_tmem), "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ inline void mma_commit_warp(void *mbar)
{
    asm volatile(
        "{\n\t.reg .pred e;\n\t"
        "elect.sync _|e, 0xffffffff;\n\t"
        "@e tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n\t}\n"
        :
        : "r"(smem_addr(mbar))
        : "memory");
}

// Tensor-memory allocation (one full warp).
__device__ inline void tmem_alloc(uint32_t *slot_smem, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :
                 : "r"(smem_addr(slot_smem)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ inline void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                 :
                 : "r"(taddr), "r"(ncols)
                 : "memory");
}

__device__ inline void fence_before_sync()
{
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ inline void fence_after_sync()
{
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Generic-proxy shared-memory writes -> visible to the tensor cores.
__device__ inline void fence_proxy_async()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 8 consecutive 32-bit columns of the warp's 32 TMEM lanes (one lane per thread).
__device__ inline void tmem_ld8(uint32_t taddr, float v[8])
{
    uint32_t r0, r1, r2, r3, r4, r5, r6, r7;
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3), "=r"(r4), "=r"(r5), "=r"(r6),
                   "=r"(r7)
                 : "r"(taddr)
                 : "memory");
    v[0] = __uint_as_float(r0); v[1] = __uint_as_float(r1);
    v[2] = __uint_as_float(r2); v[3] = __uint_as_float(r3);
    v[4] = __uint_as_float(r4); v[5] = __uint_as_float(r5);
    v[6] = __uint_as_float(r6); v[7] = __uint_as_float(r7);
}

// 4 consecutive 32-bit columns of the warp's 32 TMEM lanes.
__device__ inline void tmem_ld4(uint32_t taddr, float v[4])
{
    uint32_t r0, r1, r2, r3;
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(taddr)
                 : "memory");
    v[0] = __uint_as_float(r0); v[1] = __uint_as_float(r1);
    v[2] = __uint_as_float(r2); v[3] = __uint_as_float(r3);
}

// 8 consecutive 32-bit columns of the warp's 32 TMEM lanes from registers.
__device__ inline void tmem_st8(uint32_t taddr, const uint32_t v[8])
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};"
                 :
                 : "r"(taddr), "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]),
                   "r"(v[5]), "r"(v[6]), "r"(v[7])
                 : "memory");
}

__device__ inline void tmem_st_wait()
{
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

__device__ inline void tmem_ld_wait()
{
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// ---- mbarrier ----
__device__ inline void mbar_init(void *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
                 : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ inline bool mbar_try_wait(void *bar, uint32_t parity)
{
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred P1;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n\t"
        "selp.b32 %0, 1, 0, P1;\n\t}\n"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// Bounded wait: returns false if the phase did not complete within `limit`
// polls (each try_wait may itself block for a short, hardware-defined time).
__device__ inline bool mbar_wait_bounded(void *bar, uint32_t parity, uint32_t limit)
{
    for (uint32_t i = 0; i < limit; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// fp16 split of an FP32 value: x ~ hi + lo / 2048 with |lo| <= |x| (scaled
// so that the residual stays in the normal fp16 range).
constexpr float SPLIT_SCALE = 2048.0f;
__device__ inline void split_f16(float x, __half &hi, __half &lo)
{
    hi = __float2half_rn(x);
    lo = __float2half_rn((x - __half2float(hi)) * SPLIT_SCALE);
}

// Element offset of (row, k) in a K-major core-matrix grid with rows grouped
// outermost: [row/8][k/8][row%8][k%8], `kp` (multiple of 8) columns.
__host__ __device__ inline uint32_t cm_offset_rows(uint32_t row, uint32_t k, uint32_t kp)
{
    return (((row >> 3) * (kp >> 3) + (k >> 3)) << 6) + ((row & 7) << 3) + (k & 7);
}

// Element offset of (row, k) in a K-major core-matrix grid with `rows_pad`
// rows (multiple of 8): [k/8][row/8][row%8][k%8].
__host__ __device__ inline uint32_t cm_offset(uint32_t row, uint32_t k, uint32_t rows_pad)
{
    return (((k >> 3) * (rows_pad >> 3) + (row >> 3)) << 6) + ((row & 7) << 3) + (k & 7);
}

}  // namespace tc
}  // namespace magpy
