// pgb_tc.cuh -- inline-PTX helpers for kernels on the 5th-generation tensor
// cores (tcgen05.mma with accumulators in tensor memory, operands in shared
// memory described by matrix descriptors, completion on mbarriers).
//
// Operand layout assumed by tc_desc (no swizzle, K-major): a tile of R rows
// x 16 K values of a 2-byte type is R/8 x 2 core matrices of 8 rows x 16
// bytes; row group g and K half h sit at g * 256 + h * 128 bytes, row r of a
// core matrix at r * 16 (leading byte offset 128 = the next core matrix
// along K, stride byte offset 256 = the next 8-row group).
#pragma once
#include <stdint.h>

namespace pgb {

__device__ __forceinline__ uint32_t tc_smem(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared memory matrix descriptor: start address, LBO 128 B, SBO 256 B, the
// fixed 0b001 at bits 46-48, no swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr)
{
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(256 >> 4) << 32) |
           (1ull << 46);
}

// instruction descriptor of kind::f16 with BF16 A and B (both K-major) and an
// FP32 accumulator, for an M x N tile
__host__ __device__ constexpr uint32_t tc_idesc_bf16(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_bar_init(uint32_t bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ bool tc_bar_try(uint32_t bar, unsigned parity)
{
    uint32_t ok;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait: false when `limit` polls did not see the phase complete
__device__ __forceinline__ bool tc_bar_wait(uint32_t bar, unsigned parity, long limit)
{
    for (long it = 0; it < limit; it++)
        if (tc_bar_try(bar, parity)) return true;
    return false;
}

// D[tmem] (+)= A[ad] B[bd]' with the given instruction descriptor
__device__ __forceinline__ void tc_mma(uint32_t dt, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dt),
        "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
// eight 32-bit columns of this warp's 32 TMEM lanes (one lane per thread)
__device__ __forceinline__ void tc_ld8(uint32_t taddr, uint32_t (&v)[8])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
                 : "r"(taddr)
                 : "memory");
}
__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy writes of shared memory made visible to the tensor core
__device__ __forceinline__ void tc_fence_proxy() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_st16(uint32_t addr, uint4 v)
{
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w)
                 : "memory");
}

}  // namespace pgb
