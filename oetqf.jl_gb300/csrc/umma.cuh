// tcgen05 (fifth-generation tensor core) helpers for sm_100a-family targets, inline PTX: TMEM
// allocation, the instruction and shared-memory descriptors of a BF16 x BF16 -> FP32 MMA with
// K-major operands staged by TMA with 128-byte swizzle, MMA issue, completion to an mbarrier,
// TMEM loads and the thread-sync fences around them.
#pragma once
#include <cstdint>

#include "tma.cuh"

namespace gbc {
namespace umma {

// Instruction descriptor of tcgen05.mma .kind::f16: D in FP32 (bits 4-5 = 1), A and B in BF16
// (bits 7-9 and 10-12 = 1), no negation, both K-major (bits 15 and 16 = 0), N >> 3 in bits 17-22,
// M >> 4 in bits 24-28. M = 128 needs N a multiple of 16 in [16, 256].
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Shared-memory matrix descriptor of a K-major tile that TMA wrote with 128-byte swizzle (rows of
// 128 bytes = 64 BF16, the tile 1024-byte aligned): start address >> 4 in bits 0-13, leading byte
// offset 16 B (>> 4 = 1; not used by this layout) in bits 16-29, stride byte offset 1024 B between
// 8-row groups (>> 4) in bits 32-45, descriptor version 1 in bits 46-47, base offset 0 in bits
// 49-51, swizzle mode 2 (128 B) in bits 61-63. The K-th 16-element slice of a row starts 32 K bytes
// further: the hardware applies the swizzle to the computed address.
__host__ __device__ constexpr uint64_t sdesc_sw128(uint32_t saddr) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

#ifdef __CUDACC__
// one full warp: allocate ncols TMEM columns (a power of two >= 32); the address lands in *slot
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
// one full warp, after every reader and the MMAs are done
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// D[tmem] (+)= A B^T for one 128 x N x 16 slice; accumulate = 0 overwrites D
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// arrive once on bar when every tcgen05.mma this thread issued so far has completed
__device__ __forceinline__ void commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
// three 16-column loads of this warp's 32 TMEM lanes (one row per thread) and the wait for them,
// in one asm statement so that no use of r can be scheduled before the wait
__device__ __forceinline__ void ld3x16(uint32_t t0, uint32_t t1, uint32_t t2, uint32_t (&r)[48]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%48];\n"
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%49];\n"
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%32, %33, %34, %35, %36, %37, %38, %39, %40, %41, %42, %43, %44, %45, %46, %47}, [%50];\n"
        "tcgen05.wait::ld.sync.aligned;\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47])
        : "r"(t0), "r"(t1), "r"(t2)
        : "memory");
}
#endif

}  // namespace umma
}  // namespace gbc
