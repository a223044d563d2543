// pp_tc.cuh -- 5th-generation tensor-core (tcgen05) building blocks for the warm-start MLP.
//
// One CTA multiplies a 128-row bf16 tile A [128 x K] held in shared memory by a bf16 tile
// B [N x K] (also shared memory; i.e. B^T of a K x N operand) into a float32 accumulator
// D [128 x N] in tensor memory: thread 0 issues K/16 tcgen05.mma (kind::f16, bf16 inputs,
// f32 accumulate) and commits them to an mbarrier; every thread then reads its row of D
// (TMEM lane = row) with tcgen05.ld.
//
// Shared-memory tiles use the canonical K-major layout without swizzling: 8-row x 16-byte
// core matrices (128 contiguous bytes), ordered first along K (leading byte offset 128 B),
// then along rows (stride byte offset K/8 * 128 B):
//     byte(row, k) = ((row / 8) * (K / 8) + k / 8) * 128 + (row % 8) * 16 + (k % 8) * 2.
// Descriptor fields (64 bits): start address >> 4 [0,14), leading byte offset >> 4
// [16,30), stride byte offset >> 4 [32,46), descriptor version 1 [46,48), swizzle mode 0
// [61,64).  Instruction descriptor (kind::f16): D format f32 (bit 4), A and B bf16 (bits
// 7 and 10), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
#pragma once

#include <cstdint>

#include <cuda_bf16.h>

namespace ppgpu {

__device__ __forceinline__ uint32_t tc_smem_u32(const void *p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

// Byte offset of element (row, k) in a K-major no-swizzle tile with K columns.
__host__ __device__ __forceinline__ uint32_t tile_off(int row, int k, int K) {
    return (uint32_t)(((row >> 3) * (K >> 3) + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version for tcgen05
    return d;                // base offset 0, swizzle none
}

// kind::f16 instruction descriptor: bf16 x bf16 -> f32, A and B K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// ---- tensor memory allocation (one warp) ----
__device__ __forceinline__ void tmem_alloc(uint32_t *smem_dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem_u32(smem_dst)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// ---- MMA issue (one thread) ----
__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool accumulate) {
    const uint32_t acc = accumulate ? 1u : 0u;
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t *mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(tc_smem_u32(mbar))
                 : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Generic-proxy shared-memory writes made visible to the tensor core (async proxy).
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// D[128 x N] (+)= A[128 x K] . B[N x K]^T, both tiles K-major in shared memory.  One thread.
__device__ __forceinline__ void tc_gemm(uint32_t d_tmem, const void *A, const void *B, int K, int N, bool accumulate) {
    const uint32_t a0 = tc_smem_u32(A), b0 = tc_smem_u32(B);
    const uint32_t sbo = (uint32_t)(K >> 3) * 128u;
    const uint32_t idesc = idesc_bf16(128, N);
    for (int k0 = 0; k0 < K; k0 += 16) {
        const uint32_t step = (uint32_t)(k0 >> 3) * 128u;  // two core matrices along K per step
        tc_mma(d_tmem, smem_desc(a0 + step, 128u, sbo), smem_desc(b0 + step, 128u, sbo), idesc, accumulate || k0 > 0);
    }
}

// ---- mbarrier helpers (bounded wait: ~2 s, then false) ----
__device__ __forceinline__ void tc_mbar_init(uint64_t *bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem_u32(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool tc_mbar_try(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(tc_smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool tc_mbar_wait(uint64_t *bar, uint32_t parity) {
    if (tc_mbar_try(bar, parity)) return true;
    uint64_t t0;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    for (uint32_t i = 0; i < (1u << 26); i++) {
        if (tc_mbar_try(bar, parity)) return true;
        if ((i & 255u) == 255u) {
            uint64_t t;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
            if (t - t0 > 2000000000ull) break;
        }
    }
    return false;
}

// ---- TMEM -> registers: 16 consecutive f32 columns of this thread's lane ----
// Warp w of the CTA reads lanes 32*(w%4) .. +31; taddr = lane << 16 | column.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

}  // namespace ppgpu
