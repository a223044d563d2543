// pp_mlp_dev.cuh -- device side of the warm-start network (shared by the proposal kernel of
// pp_batch.cu and the training kernels of pp_mlp.cu).
//
// Network: x[96] (90 features, 6 zeros) -> 128 -> 128 -> y[16] (3 used), SiLU, bf16 weights and
// activations, float32 accumulation in tensor memory (tcgen05, pp_tc.cuh).  One CTA of 128
// threads runs 128 samples; thread t owns sample t (TMEM lane t).
//
// Features of a probe whose start point (tip + previous converged displacement d) has grid
// coordinate m + s (m the nearest grid node, s in [-1/2, 1/2)^3), with F the force at the
// 3 x 3 x 3 grid nodes around m:
//   f[3 (9 (a+1) + 3 (b+1) + (c+1)) + comp] = tanh(FEAT_FSCALE * F_comp(m + (a, b, c)))   0..80
//   f[81 + k] = 2 s_k                                                                 81..83
//   f[84 + k] = FEAT_DSCALE * (d - rPP0)_k                                            84..86
//   f[87 + k] = OUT_SCALE * (change of the converged displacement at the height above) 87..89
//   f[90..95] = 0.
// Output: y[0..2] = OUT_SCALE * (d_converged - d).
#pragma once

#include <cuda_bf16.h>

#include "pp_common.cuh"
#include "pp_df.cuh"
#include "pp_tc.cuh"

namespace ppgpu {

constexpr int MLP_IN = 96;
constexpr int MLP_FEAT = 90;
constexpr int MLP_H = 128;
constexpr int MLP_OUT = 16;
constexpr int MLP_NOUT = 3;
constexpr float FEAT_FSCALE = 2.0f;   // 1/(0.5 eV/A)
constexpr float FEAT_DSCALE = 10.0f;  // 1/(0.1 A)
constexpr float OUT_SCALE = 10.0f;    // outputs in units of 0.1 A

// bf16 weight tiles in the K-major core-matrix layout of pp_tc.cuh (device memory).
struct MLPTiles {
    const unsigned char *W1t;  // [128 out][96 in]   forward B of layer 1
    const unsigned char *W2t;  // [128 out][128 in]  forward B of layer 2
    const unsigned char *W3t;  // [16 out][128 in]   forward B of layer 3
    const unsigned char *W3;   // [128 in][16 out]   backward B of dY . W3^T
    const unsigned char *W2;   // [128 in][128 out]  backward B of dZ2 . W2^T
    const float *b1, *b2, *b3;
};
constexpr int TILE_W1T = MLP_H * MLP_IN * 2;
constexpr int TILE_W2T = MLP_H * MLP_H * 2;
constexpr int TILE_W3T = MLP_OUT * MLP_H * 2;
constexpr int TILE_W3 = MLP_H * MLP_OUT * 2;
constexpr int TILE_W2 = MLP_H * MLP_H * 2;
constexpr int TILE_ACT = 128 * MLP_H * 2;  // one 128 x 128 bf16 activation tile

// Hardware tanh (MUFU, max relative error ~2^-11): the activations and the force compression
// go through it, sigma(z) = (1 + tanh(z/2)) / 2.
__device__ __forceinline__ float tanh_fast(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float sigmoid_fast(float z) { return fmaf(0.5f, tanh_fast(0.5f * z), 0.5f); }
__device__ __forceinline__ float silu(float z) { return z * sigmoid_fast(z); }
__device__ __forceinline__ float silu_grad(float z) {
    const float s = sigmoid_fast(z);
    return s * (1.f + z * (1.f - s));
}

// Copies `bytes` (multiple of 16) from global to shared memory with all threads of the CTA.
__device__ __forceinline__ void copy_tile(unsigned char *dst, const unsigned char *src, int bytes) {
    const int4 *s = reinterpret_cast<const int4 *>(src);
    int4 *d = reinterpret_cast<int4 *>(dst);
    for (int i = threadIdx.x; i < bytes / 16; i += blockDim.x) d[i] = s[i];
}

// Writes this thread's row (K values) into a K-major tile, 8 values per 16-byte store.
__device__ __forceinline__ void store_row_bf16(unsigned char *tile, int row, const float *v, int K) {
#pragma unroll 4
    for (int k0 = 0; k0 < K; k0 += 8) {
        __align__(16) __nv_bfloat162 p[4];
#pragma unroll
        for (int i = 0; i < 4; i++) p[i] = __floats2bfloat162_rn(v[k0 + 2 * i], v[k0 + 2 * i + 1]);
        *reinterpret_cast<int4 *>(tile + tile_off(row, k0, K)) = *reinterpret_cast<const int4 *>(p);
    }
}

// All threads: wait for the committed MMAs (phase parity ph), then order TMEM reads after it.
__device__ __forceinline__ bool mma_wait(uint64_t *bar, uint32_t &ph) {
    const bool ok = tc_mbar_wait(bar, ph);
    ph ^= 1u;
    tc_fence_after();
    return ok;
}

// Generic-proxy tile writes -> visible to the next MMA; TMEM reads done before it is reused.
__device__ __forceinline__ void cta_handoff() {
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
}

// The same for the 128 threads of warpgroup g alone (named barrier 1 + g), so several
// warpgroups of a CTA can each run their own tile.
__device__ __forceinline__ void wg_sync(int g) { asm volatile("bar.sync %0, 128;" ::"r"(1 + g) : "memory"); }
__device__ __forceinline__ void wg_handoff(int g) {
    fence_async_smem();
    tc_fence_before();
    wg_sync(g);
    tc_fence_after();
}

__device__ __forceinline__ uint32_t lane_addr(uint32_t tmem, int col) {
    const int warp = threadIdx.x >> 5;
    return tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)col;
}

// 16 consecutive values of this thread's row into a K-major tile (two 16-byte stores).
__device__ __forceinline__ void store16_bf16(unsigned char *tile, int row, int k0, const float *v, int K) {
#pragma unroll
    for (int g = 0; g < 2; g++) {
        __align__(16) __nv_bfloat162 p[4];
#pragma unroll
        for (int i = 0; i < 4; i++) p[i] = __floats2bfloat162_rn(v[8 * g + 2 * i], v[8 * g + 2 * i + 1]);
        *reinterpret_cast<int4 *>(tile + tile_off(row, k0 + 8 * g, K)) = *reinterpret_cast<const int4 *>(p);
    }
}

// act row <- bf16(SiLU(D row + b)) over 128 columns, 16 columns at a time (row = the
// thread's index in its warpgroup = its TMEM lane).
__device__ __forceinline__ void silu_epilogue(unsigned char *act, uint32_t tmem, const float *b) {
#pragma unroll 1
    for (int c = 0; c < MLP_H; c += 16) {
        float v[16];
        tmem_ld16(lane_addr(tmem, c), v);
#pragma unroll
        for (int i = 0; i < 16; i++) v[i] = silu(v[i] + b[c + i]);
        store16_bf16(act, threadIdx.x & 127, c, v, MLP_H);
    }
}

// Forward pass of the 128 samples whose inputs are in `act` (K = MLP_IN layout), run by
// warpgroup g (its thread t owns sample t, TMEM lane t; MMAs accumulate at column tmem).
// Leaves the output row (16 floats, bias added) in y.  act is overwritten by the hidden
// activations.  Returns false if an MMA never completed (bounded wait).
__device__ __forceinline__ bool mlp_forward(unsigned char *act, const unsigned char *W1t, const unsigned char *W2t,
                                            const unsigned char *W3t, const float *b1, const float *b2, const float *b3,
                                            uint32_t tmem, uint64_t *bar, uint32_t &ph, float *y, int g = 0) {
    const bool leader = (threadIdx.x & 127) == 0;
    bool ok = true;
    // layer 1
    if (leader) {
        tc_gemm(tmem, act, W1t, MLP_IN, MLP_H, false);
        tc_commit(bar);
    }
    ok &= mma_wait(bar, ph);
    silu_epilogue(act, tmem, b1);
    wg_handoff(g);
    // layer 2
    if (leader) {
        tc_gemm(tmem, act, W2t, MLP_H, MLP_H, false);
        tc_commit(bar);
    }
    ok &= mma_wait(bar, ph);
    silu_epilogue(act, tmem, b2);
    wg_handoff(g);
    // layer 3
    if (leader) {
        tc_gemm(tmem, act, W3t, MLP_H, MLP_OUT, false);
        tc_commit(bar);
    }
    ok &= mma_wait(bar, ph);
    tmem_ld16(lane_addr(tmem, 0), y);
#pragma unroll
    for (int c = 0; c < MLP_OUT; c++) y[c] += b3[c];
    tc_fence_before();
    wg_sync(g);
    tc_fence_after();
    return ok;
}

}  // namespace ppgpu
