// pp_mlp_dev.cuh -- device side of the warm-start network (shared by the proposal kernel of
// pp_batch.cu and the training kernels of pp_mlp.cu).
//
// Network: x[96] (84 features, 12 zeros) -> 128 -> 128 -> y[16] (3 used), SiLU, bf16 weights and
// activations, float32 accumulation in tensor memory (tcgen05, pp_tc.cuh).  One CTA of 128
// threads runs 128 samples; thread t owns sample t (TMEM lane t).
//
// Features of a probe at grid coordinate base + u with previous converged displacement d:
//   f[9*(3*(a+1)+(b+1))+3*(c+1)+comp] = tanh(FEAT_FSCALE * F_comp(u + (a, b, c)))
//       for a, b, c in {-1, 0, 1}: the trilinear force one grid step around the probe;
//   f[81..83] = FEAT_DSCALE * (d - rPP0);   f[84..95] = 0.
// Output: y[0..2] = OUT_SCALE * (d_converged - d).
#pragma once

#include <cuda_bf16.h>

#include "pp_common.cuh"
#include "pp_df.cuh"
#include "pp_tc.cuh"

namespace ppgpu {

constexpr int MLP_IN = 96;
constexpr int MLP_FEAT = 84;
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

// act row <- bf16(SiLU(D row + b)) over 128 columns, 16 columns at a time.
__device__ __forceinline__ void silu_epilogue(unsigned char *act, uint32_t tmem, const float *b) {
#pragma unroll 1
    for (int c = 0; c < MLP_H; c += 16) {
        float v[16];
        tmem_ld16(lane_addr(tmem, c), v);
#pragma unroll
        for (int i = 0; i < 16; i++) v[i] = silu(v[i] + b[c + i]);
        store16_bf16(act, threadIdx.x, c, v, MLP_H);
    }
}

// Forward pass of the 128 samples whose inputs are in `act` (K = 96 layout).  Leaves the
// output row (16 floats, bias added) in y.  act is overwritten by the hidden activations.
// Returns false if an MMA never completed (bounded wait).
__device__ __forceinline__ bool mlp_forward(unsigned char *act, const unsigned char *W1t, const unsigned char *W2t,
                                            const unsigned char *W3t, const float *b1, const float *b2, const float *b3,
                                            uint32_t tmem, uint64_t *bar, uint32_t &ph, float *y) {
    const int tid = threadIdx.x;
    bool ok = true;
    // layer 1
    if (tid == 0) {
        tc_gemm(tmem, act, W1t, MLP_IN, MLP_H, false);
        tc_commit(bar);
    }
    ok &= mma_wait(bar, ph);
    silu_epilogue(act, tmem, b1);
    cta_handoff();
    // layer 2
    if (tid == 0) {
        tc_gemm(tmem, act, W2t, MLP_H, MLP_H, false);
        tc_commit(bar);
    }
    ok &= mma_wait(bar, ph);
    silu_epilogue(act, tmem, b2);
    cta_handoff();
    // layer 3
    if (tid == 0) {
        tc_gemm(tmem, act, W3t, MLP_H, MLP_OUT, false);
        tc_commit(bar);
    }
    ok &= mma_wait(bar, ph);
    tmem_ld16(lane_addr(tmem, 0), y);
#pragma unroll
    for (int c = 0; c < MLP_OUT; c++) y[c] += b3[c];
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    return ok;
}

// Features of one probe (see the header comment) written as row `row` of the K = 96 input
// tile.  FE: float4 grid, n: its size, base + u: the probe's grid coordinate (u
// double-float), dr = d - rPP0.
template <bool NC>
__device__ __forceinline__ void warm_features(const float4 *FE, int n0, int n1, int n2, const int base[3],
                                              const dfl u[3], float3 dr, unsigned char *tile, int row) {
    int ci[3];
    float t[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const dfl tk = split_cell(u[k], ci[k]);
        ci[k] += base[k];
        t[k] = __fadd_rn(tk.h, tk.l);
    }
    float acc[27][3];
#pragma unroll
    for (int s = 0; s < 27; s++) acc[s][0] = acc[s][1] = acc[s][2] = 0.f;
    // the 4x4 node columns around the cell (x, y offsets -1..2), each 4 nodes along z
#pragma unroll
    for (int px = 0; px < 4; px++) {
        const int ix = wrap_index(ci[0] - 1 + px, n0);
#pragma unroll
        for (int py = 0; py < 4; py++) {
            const int iy = wrap_index(ci[1] - 1 + py, n1);
            const long long col = ((long long)ix * n1 + iy) * n2;
            float3 node[4];
#pragma unroll
            for (int pz = 0; pz < 4; pz++) {
                const int iz = wrap_index(ci[2] - 1 + pz, n2);
                const float4 q = NC ? __ldg(FE + col + iz) : FE[col + iz];
                node[pz] = make_float3(q.x, q.y, q.z);
            }
            // z interpolation for the sample offsets -1, 0, 1 (c = 0, 1, 2): nodes c, c+1
            float3 vz[3];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                vz[c].x = fmaf(t[2], node[c + 1].x - node[c].x, node[c].x);
                vz[c].y = fmaf(t[2], node[c + 1].y - node[c].y, node[c].y);
                vz[c].z = fmaf(t[2], node[c + 1].z - node[c].z, node[c].z);
            }
#pragma unroll
            for (int a = 0; a < 3; a++) {
                // sample a uses x nodes a (weight 1-tx) and a+1 (weight tx)
                const float wx = (px == a) ? 1.f - t[0] : ((px == a + 1) ? t[0] : 0.f);
                if (px != a && px != a + 1) continue;
#pragma unroll
                for (int b = 0; b < 3; b++) {
                    if (py != b && py != b + 1) continue;
                    const float w = wx * ((py == b) ? 1.f - t[1] : t[1]);
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        const int s = 9 * a + 3 * b + c;
                        acc[s][0] = fmaf(w, vz[c].x, acc[s][0]);
                        acc[s][1] = fmaf(w, vz[c].y, acc[s][1]);
                        acc[s][2] = fmaf(w, vz[c].z, acc[s][2]);
                    }
                }
            }
        }
    }
    // tanh-compressed forces, the scaled displacement and zero padding: 96 values
    float v[16];
#pragma unroll
    for (int g = 0; g < MLP_IN / 16; g++) {
#pragma unroll
        for (int i = 0; i < 16; i++) {
            const int k = 16 * g + i;
            float x;
            if (k < 81)
                x = tanh_fast(FEAT_FSCALE * acc[k / 3][k % 3]);
            else if (k == 81)
                x = FEAT_DSCALE * dr.x;
            else if (k == 82)
                x = FEAT_DSCALE * dr.y;
            else if (k == 83)
                x = FEAT_DSCALE * dr.z;
            else
                x = 0.f;
            v[i] = x;
        }
        store16_bf16(tile, row, 16 * g, v, MLP_IN);
    }
}

}  // namespace ppgpu
