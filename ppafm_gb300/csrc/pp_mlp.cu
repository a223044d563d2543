// pp_mlp.cu -- the learned warm start: a small MLP on the tcgen05 tensor cores.
//
// No reference counterpart (new in this library).  The network proposes FIRE's starting
// displacement for the next height of a stroke from the force grid around the probe and the
// converged displacement of the height above; plain FIRE then always runs to the same
// convergence criterion, so the network can only save iterations.
//
// Network: 96 (90 features + 6 zero pad) -> 128 -> 128 -> 16 (3 used), SiLU, bf16 weights
// and activations, float32 accumulation in tensor memory.  Every GEMM is a 128-row tile
// issued by one thread with tcgen05.mma (pp_tc.cuh); epilogues (bias, SiLU, its derivative,
// conversions) run on all threads from tcgen05.ld.
#include <cmath>
#include <cstring>

#include <random>
#include <vector>

#include "pp_common.cuh"
#include "pp_mlp_dev.cuh"
#include "pp_tc.cuh"

namespace ppgpu {

// ------------------------------------------------------------- parameters
// Master parameters (float32, one array): W1 [96 in][128 out], W2 [128][128], W3 [128][16],
// b1 [128], b2 [128], b3 [16].  Rows 90..95 of W1 multiply zero padding.
constexpr int OFF_W1 = 0;
constexpr int OFF_W2 = OFF_W1 + MLP_IN * MLP_H;
constexpr int OFF_W3 = OFF_W2 + MLP_H * MLP_H;
constexpr int OFF_B1 = OFF_W3 + MLP_H * MLP_OUT;
constexpr int OFF_B2 = OFF_B1 + MLP_H;
constexpr int OFF_B3 = OFF_B2 + MLP_H;
constexpr int NPARAM = OFF_B3 + MLP_OUT;

struct MLP {
    float *P = nullptr, *G = nullptr, *M = nullptr, *V = nullptr;  // params, grads, Adam moments
    unsigned char *tiles = nullptr;  // W1t | W2t | W3t | W3 | W2
    float *loss = nullptr;           // device scalar
    float lw[3] = {1.f, 1.f, 1.f};   // per-output loss weights
    // per-batch transposed activation tiles for the weight gradients
    unsigned char *xt = nullptr, *h1t = nullptr, *h2t = nullptr, *dyt = nullptr, *dz2t = nullptr, *dz1t = nullptr;
    int cap_tiles = 0;  // CTAs (of 128 samples) the transposed buffers hold
    MLPTiles view() const {
        MLPTiles t;
        t.W1t = tiles;
        t.W2t = t.W1t + TILE_W1T;
        t.W3t = t.W2t + TILE_W2T;
        t.W3 = t.W3t + TILE_W3T;
        t.W2 = t.W3 + TILE_W3;
        t.b1 = P + OFF_B1;
        t.b2 = P + OFF_B2;
        t.b3 = P + OFF_B3;
        return t;
    }
};

// bf16 tiles of the current parameters (all five layouts).
__global__ void mlp_pack_kernel(const float *P, unsigned char *tiles) {
    unsigned char *W1t = tiles, *W2t = W1t + TILE_W1T, *W3t = W2t + TILE_W2T, *W3 = W3t + TILE_W3T, *W2 = W3 + TILE_W3;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < MLP_IN * MLP_H) {  // W1[in][out]
        const int in = i / MLP_H, out = i % MLP_H;
        *(__nv_bfloat16 *)(W1t + tile_off(out, in, MLP_IN)) = __float2bfloat16_rn(P[OFF_W1 + i]);
    }
    if (i < MLP_H * MLP_H) {  // W2[in][out]
        const int in = i / MLP_H, out = i % MLP_H;
        const __nv_bfloat16 w = __float2bfloat16_rn(P[OFF_W2 + i]);
        *(__nv_bfloat16 *)(W2t + tile_off(out, in, MLP_H)) = w;
        *(__nv_bfloat16 *)(W2 + tile_off(in, out, MLP_H)) = w;
    }
    if (i < MLP_H * MLP_OUT) {  // W3[in][out]
        const int in = i / MLP_OUT, out = i % MLP_OUT;
        const __nv_bfloat16 w = __float2bfloat16_rn(P[OFF_W3 + i]);
        *(__nv_bfloat16 *)(W3t + tile_off(out, in, MLP_H)) = w;
        *(__nv_bfloat16 *)(W3 + tile_off(in, out, MLP_OUT)) = w;
    }
}

// Adam (Kingma & Ba) on the master parameters; the gradient buffer is cleared for the next step.
__global__ void mlp_adam_kernel(float *P, float *G, float *M, float *V, float lr, float b1t, float b2t) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= NPARAM) return;
    const float g = G[i];
    const float m = 0.9f * M[i] + 0.1f * g;
    const float v = 0.999f * V[i] + 0.001f * g * g;
    M[i] = m;
    V[i] = v;
    P[i] -= lr * (m / b1t) / (sqrtf(v / b2t) + 1e-8f);
    G[i] = 0.f;
}

// Transposed copy of this thread's row value into tile T[feature][sample] (K = 128 samples).
__device__ __forceinline__ void store_t(unsigned char *T, int feat, int sample, float v) {
    *(__nv_bfloat16 *)(T + tile_off(feat, sample, 128)) = __float2bfloat16_rn(v);
}

// Column sums of a value over the CTA's 128 rows, added into g (warp shuffles + 4 atomics).
__device__ __forceinline__ void col_sum_add(float v, float *g) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(g, v);
}

constexpr int FB_SMEM = TILE_W1T + TILE_W2T + TILE_W3T + TILE_W3 + TILE_W2 + 128 * MLP_IN * 2 + 2 * TILE_ACT;

// Forward + backward of one tile of 128 samples (minibatch rows idx[128 c .. 128 c + 127]).
// Writes the transposed activations/deltas of the tile for the weight gradients, adds the
// bias gradients and the loss.  TMEM columns: Z1 [0,128), Z2 [128,256), Y [256,272),
// dH2 [384,512), dH1 [128,256) (over Z2 once it is consumed).
__global__ void __launch_bounds__(128, 1) mlp_fwd_bwd_kernel(MLPTiles W, const __nv_bfloat16 *X, const float4 *T,
                                                             const int *idx, int nbatch, float3 lw, float *G, float *loss,
                                                             unsigned char *xt, unsigned char *h1t, unsigned char *h2t,
                                                             unsigned char *dyt, unsigned char *dz2t, unsigned char *dz1t,
                                                             int *err) {
    extern __shared__ __align__(128) unsigned char sm[];
    __shared__ uint64_t bar;
    __shared__ uint32_t tbase;
    unsigned char *sW1t = sm, *sW2t = sW1t + TILE_W1T, *sW3t = sW2t + TILE_W2T, *sW3 = sW3t + TILE_W3T,
                  *sW2 = sW3 + TILE_W3, *bufA = sW2 + TILE_W2, *bufB = bufA + 128 * MLP_IN * 2, *bufC = bufB + TILE_ACT;
    const int tid = threadIdx.x, c = blockIdx.x;
    const size_t tb = (size_t)c * TILE_ACT;  // this CTA's transposed tiles
    copy_tile(sW1t, W.W1t, TILE_W1T);
    copy_tile(sW2t, W.W2t, TILE_W2T);
    copy_tile(sW3t, W.W3t, TILE_W3T);
    copy_tile(sW3, W.W3, TILE_W3);
    copy_tile(sW2, W.W2, TILE_W2);
    const int s = idx[c * 128 + tid];
    {
        const int4 *xr = reinterpret_cast<const int4 *>(X + (size_t)s * MLP_IN);
#pragma unroll
        for (int g = 0; g < MLP_IN / 8; g++) {
            const int4 q = xr[g];
            *reinterpret_cast<int4 *>(bufA + tile_off(tid, 8 * g, MLP_IN)) = q;
            const __nv_bfloat16 *e = reinterpret_cast<const __nv_bfloat16 *>(&q);
#pragma unroll
            for (int i = 0; i < 8; i++) *(__nv_bfloat16 *)(xt + tb + tile_off(8 * g + i, tid, 128)) = e[i];
        }
    }
    const float4 tg = T[s];
    if (tid == 0) tc_mbar_init(&bar);
    if (tid < 32) tmem_alloc(&tbase, 512);
    cta_handoff();
    const uint32_t tm = tbase;
    uint32_t ph = 0;
    bool ok = true;
    const float inv = 1.f / (float)nbatch;
    // ---- forward
    if (tid == 0) {
        tc_gemm(tm, bufA, sW1t, MLP_IN, MLP_H, false);
        tc_commit(&bar);
    }
    ok &= mma_wait(&bar, ph);
    for (int c0 = 0; c0 < MLP_H; c0 += 16) {
        float v[16];
        tmem_ld16(lane_addr(tm, c0), v);
        for (int i = 0; i < 16; i++) {
            v[i] = silu(v[i] + W.b1[c0 + i]);
            store_t(h1t + tb, c0 + i, tid, v[i]);
        }
        store16_bf16(bufB, tid, c0, v, MLP_H);
    }
    cta_handoff();
    if (tid == 0) {
        tc_gemm(tm + 128, bufB, sW2t, MLP_H, MLP_H, false);
        tc_commit(&bar);
    }
    ok &= mma_wait(&bar, ph);
    for (int c0 = 0; c0 < MLP_H; c0 += 16) {
        float v[16];
        tmem_ld16(lane_addr(tm, 128 + c0), v);
        for (int i = 0; i < 16; i++) {
            v[i] = silu(v[i] + W.b2[c0 + i]);
            store_t(h2t + tb, c0 + i, tid, v[i]);
        }
        store16_bf16(bufC, tid, c0, v, MLP_H);
    }
    cta_handoff();
    if (tid == 0) {
        tc_gemm(tm + 256, bufC, sW3t, MLP_H, MLP_OUT, false);
        tc_commit(&bar);
    }
    ok &= mma_wait(&bar, ph);
    {
        float y[16], dy[16];
        tmem_ld16(lane_addr(tm, 256), y);
        const float t3[3] = {tg.x, tg.y, tg.z};
        float l = 0.f;
        const float w3[3] = {lw.x, lw.y, lw.z};
        for (int o = 0; o < MLP_OUT; o++) {
            const float e = (o < MLP_NOUT) ? (y[o] + W.b3[o] - t3[o]) : 0.f;
            const float wo = (o < MLP_NOUT) ? w3[o] : 0.f;
            l += wo * e * e;
            dy[o] = 2.f * wo * e * inv;
            store_t(dyt + (size_t)c * 128 * MLP_OUT * 2, o, tid, dy[o]);
            col_sum_add(dy[o], G + OFF_B3 + o);
        }
        col_sum_add(l * inv, loss);
        // dY tile [128 x 16] into bufA (the inputs are no longer needed)
        store16_bf16(bufA, tid, 0, dy, MLP_OUT);
    }
    cta_handoff();
    // ---- backward: dH2 = dY . W3^T -> [384, 512)
    if (tid == 0) {
        tc_gemm(tm + 384, bufA, sW3, MLP_OUT, MLP_H, false);
        tc_commit(&bar);
    }
    ok &= mma_wait(&bar, ph);
    for (int c0 = 0; c0 < MLP_H; c0 += 16) {
        float dh[16], z[16];
        tmem_ld16(lane_addr(tm, 384 + c0), dh);
        tmem_ld16(lane_addr(tm, 128 + c0), z);
        for (int i = 0; i < 16; i++) {
            dh[i] *= silu_grad(z[i] + W.b2[c0 + i]);  // dZ2
            store_t(dz2t + tb, c0 + i, tid, dh[i]);
            col_sum_add(dh[i], G + OFF_B2 + c0 + i);
        }
        store16_bf16(bufB, tid, c0, dh, MLP_H);
    }
    cta_handoff();
    // dH1 = dZ2 . W2^T -> [128, 256)
    if (tid == 0) {
        tc_gemm(tm + 128, bufB, sW2, MLP_H, MLP_H, false);
        tc_commit(&bar);
    }
    ok &= mma_wait(&bar, ph);
    for (int c0 = 0; c0 < MLP_H; c0 += 16) {
        float dh[16], z[16];
        tmem_ld16(lane_addr(tm, 128 + c0), dh);
        tmem_ld16(lane_addr(tm, c0), z);
        for (int i = 0; i < 16; i++) {
            dh[i] *= silu_grad(z[i] + W.b1[c0 + i]);  // dZ1
            store_t(dz1t + tb, c0 + i, tid, dh[i]);
            col_sum_add(dh[i], G + OFF_B1 + c0 + i);
        }
    }
    if (!ok && tid == 0) raise_device_error(err, PPGPU_ERR_DEVICE_TIMEOUT);
    tc_fence_before();
    __syncthreads();
    if (tid < 32) tmem_dealloc(tm, 512);
}

// Weight gradients: dW = A^T-tiles . B-tiles summed over the batch's CTA tiles
// [c0, c1) (K = 128 samples each), added into G.  blockIdx.y: 0 -> dW1 (XT, DZ1T),
// 1 -> dW2 (H1T, DZ2T), 2 -> dW3 (H2T, DYT, N = 16).
__global__ void __launch_bounds__(128, 1) mlp_wgrad_kernel(int ntiles, int per, const unsigned char *xt,
                                                           const unsigned char *h1t, const unsigned char *h2t,
                                                           const unsigned char *dyt, const unsigned char *dz2t,
                                                           const unsigned char *dz1t, float *G, int *err) {
    extern __shared__ __align__(128) unsigned char sm[];
    __shared__ uint64_t bar;
    __shared__ uint32_t tbase;
    const int m = blockIdx.y, tid = threadIdx.x;
    const int c0 = blockIdx.x * per, c1 = min(ntiles, c0 + per);
    if (c0 >= c1) return;
    const int N = (m == 2) ? MLP_OUT : MLP_H;
    const unsigned char *A = (m == 0) ? xt : (m == 1 ? h1t : h2t);
    const unsigned char *B = (m == 0) ? dz1t : (m == 1 ? dz2t : dyt);
    const int bbytes = N * 128 * 2;
    unsigned char *sA = sm, *sB = sm + TILE_ACT;
    if (tid == 0) tc_mbar_init(&bar);
    if (tid < 32) tmem_alloc(&tbase, 128);
    cta_handoff();
    const uint32_t tm = tbase;
    uint32_t ph = 0;
    bool ok = true;
    for (int c = c0; c < c1; c++) {
        copy_tile(sA, A + (size_t)c * TILE_ACT, TILE_ACT);
        copy_tile(sB, B + (size_t)c * bbytes, bbytes);
        cta_handoff();
        if (tid == 0) {
            tc_gemm(tm, sA, sB, 128, N, c > c0);
            tc_commit(&bar);
        }
        ok &= mma_wait(&bar, ph);  // the tiles are reloaded next: wait for the MMAs to read them
        __syncthreads();
    }
    const int row = tid;  // input feature
    const int nrows = (m == 0) ? MLP_IN : MLP_H;
    float *g = G + (m == 0 ? OFF_W1 : (m == 1 ? OFF_W2 : OFF_W3));
    for (int cc = 0; cc < N; cc += 16) {
        float v[16];
        tmem_ld16(lane_addr(tm, cc), v);
        if (row < nrows)
            for (int i = 0; i < 16; i++) atomicAdd(g + (size_t)row * N + cc + i, v[i]);
    }
    if (!ok && tid == 0) raise_device_error(err, PPGPU_ERR_DEVICE_TIMEOUT);
    tc_fence_before();
    __syncthreads();
    if (tid < 32) tmem_dealloc(tm, 128);
}

// Forward only (tests): Y[n][16] for rows X[n][96], n a multiple of 128.
__global__ void __launch_bounds__(128, 1) mlp_forward_kernel(MLPTiles W, const __nv_bfloat16 *X, float *Y, int *err) {
    extern __shared__ __align__(128) unsigned char sm[];
    __shared__ uint64_t bar;
    __shared__ uint32_t tbase;
    unsigned char *sW1t = sm, *sW2t = sW1t + TILE_W1T, *sW3t = sW2t + TILE_W2T, *act = sW3t + TILE_W3T;
    const int tid = threadIdx.x;
    copy_tile(sW1t, W.W1t, TILE_W1T);
    copy_tile(sW2t, W.W2t, TILE_W2T);
    copy_tile(sW3t, W.W3t, TILE_W3T);
    const size_t s = (size_t)blockIdx.x * 128 + tid;
    const int4 *xr = reinterpret_cast<const int4 *>(X + s * MLP_IN);
#pragma unroll
    for (int g = 0; g < MLP_IN / 8; g++) *reinterpret_cast<int4 *>(act + tile_off(tid, 8 * g, MLP_IN)) = xr[g];
    if (tid == 0) tc_mbar_init(&bar);
    if (tid < 32) tmem_alloc(&tbase, 128);
    cta_handoff();
    uint32_t ph = 0;
    float y[16];
    const bool ok = mlp_forward(act, sW1t, sW2t, sW3t, W.b1, W.b2, W.b3, tbase, &bar, ph, y);
    for (int o = 0; o < MLP_OUT; o++) Y[s * MLP_OUT + o] = y[o];
    if (!ok && tid == 0) raise_device_error(err, PPGPU_ERR_DEVICE_TIMEOUT);
    tc_fence_before();
    __syncthreads();
    if (tid < 32) tmem_dealloc(tbase, 128);
}

// ------------------------------------------------------------------ self test
// D[128 x N] = A[128 x K] . B[N x K]^T for one tile, operands given row-major in global memory.
__global__ void __launch_bounds__(128) tc_selftest_kernel(const __nv_bfloat16 *A, const __nv_bfloat16 *B, int K, int N,
                                                          float *D, int *err) {
    extern __shared__ __align__(128) unsigned char sm[];
    __shared__ uint64_t bar;
    __shared__ uint32_t tbase;
    unsigned char *sA = sm;
    unsigned char *sB = sm + 128 * K * 2;
    const int tid = threadIdx.x;
    for (int i = tid; i < 128 * K; i += 128) {
        const int r = i / K, k = i - r * K;
        *(__nv_bfloat16 *)(sA + tile_off(r, k, K)) = A[i];
    }
    for (int i = tid; i < N * K; i += 128) {
        const int r = i / K, k = i - r * K;
        *(__nv_bfloat16 *)(sB + tile_off(r, k, K)) = B[i];
    }
    fence_async_smem();
    const uint32_t ncols = N <= 32 ? 32u : (N <= 64 ? 64u : (N <= 128 ? 128u : 256u));
    if (tid == 0) tc_mbar_init(&bar);
    if (tid < 32) tmem_alloc(&tbase, ncols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tbase;
    if (tid == 0) {
        tc_gemm(tmem, sA, sB, K, N, false);
        tc_commit(&bar);
    }
    const bool ok = tc_mbar_wait(&bar, 0);
    tc_fence_after();
    if (ok) {
        const int warp = tid >> 5;
        const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;
        for (int c = 0; c < N; c += 16) {
            float v[16];
            tmem_ld16(tmem + lane_base + (uint32_t)c, v);
            for (int i = 0; i < 16; i++) D[(long long)tid * N + c + i] = v[i];
        }
    } else if (tid == 0) {
        raise_device_error(err, PPGPU_ERR_DEVICE_TIMEOUT);
    }
    tc_fence_before();
    __syncthreads();
    if (tid < 32) tmem_dealloc(tmem, ncols);
}

static int mlp_repack(MLP *M, cudaStream_t st) {
    mlp_pack_kernel<<<(MLP_H * MLP_H + 255) / 256, 256, 0, st>>>(M->P, M->tiles);
    PPGPU_CHECK_LAUNCH("mlp_pack_kernel");
    return PPGPU_OK;
}

static int mlp_reserve(MLP *M, int ntiles) {
    if (ntiles <= M->cap_tiles) return PPGPU_OK;
    cudaFree(M->xt);
    M->xt = nullptr;
    M->cap_tiles = 0;
    const size_t big = (size_t)ntiles * TILE_ACT, small = (size_t)ntiles * 128 * MLP_OUT * 2;
    unsigned char *p = nullptr;
    cudaError_t e = cudaMalloc(&p, 5 * big + small);
    if (e != cudaSuccess) return cuda_fail(e, "mlp activation tiles");
    e = cudaMemset(p, 0, 5 * big + small);  // rows 96..127 of the input tiles stay zero
    if (e != cudaSuccess) {
        cudaFree(p);
        return cuda_fail(e, "mlp activation tiles");
    }
    M->xt = p;
    M->h1t = p + big;
    M->h2t = p + 2 * big;
    M->dz2t = p + 3 * big;
    M->dz1t = p + 4 * big;
    M->dyt = p + 5 * big;
    M->cap_tiles = ntiles;
    return PPGPU_OK;
}


}  // namespace ppgpu

using namespace ppgpu;

extern "C" int ppgpu_tc_selftest(const void *A, const void *B, int K, int N, float *D, void *stream) {
    if (!A || !B || !D) return set_error(PPGPU_ERR_ARG, "tc_selftest: null argument");
    if (K <= 0 || K > 128 || (K % 16) != 0 || N < 16 || N > 256 || (N % 16) != 0)
        return set_error(PPGPU_ERR_ARG, "tc_selftest: K in 16..128 (multiple of 16), N in 16..256 (multiple of 16)");
    const size_t smem = (size_t)(128 + N) * K * 2;
    PPGPU_CUDA(cudaFuncSetAttribute(tc_selftest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
               "tc_selftest smem");
    tc_selftest_kernel<<<1, 128, smem, (cudaStream_t)stream>>>((const __nv_bfloat16 *)A, (const __nv_bfloat16 *)B, K, N,
                                                               D, device_error_word());
    PPGPU_CHECK_LAUNCH("tc_selftest_kernel");
    return set_ok();
}


extern "C" int ppgpu_mlp_create(unsigned long long seed, void **handle) {
    if (!handle) return set_error(PPGPU_ERR_ARG, "mlp_create: null handle");
    MLP *M = new MLP();
    float *p = nullptr;
    cudaError_t e = cudaMalloc(&p, 4 * NPARAM * sizeof(float) + sizeof(float) * 4);
    if (e != cudaSuccess) {
        delete M;
        return cuda_fail(e, "mlp parameters");
    }
    M->P = p;
    M->G = p + NPARAM;
    M->M = p + 2 * NPARAM;
    M->V = p + 3 * NPARAM;
    M->loss = p + 4 * NPARAM;
    e = cudaMalloc(&M->tiles, TILE_W1T + TILE_W2T + TILE_W3T + TILE_W3 + TILE_W2);
    if (e != cudaSuccess) {
        cudaFree(p);
        delete M;
        return cuda_fail(e, "mlp tiles");
    }
    // He-uniform weights for the SiLU layers, small last layer, zero biases
    std::vector<float> h(NPARAM, 0.f);
    std::mt19937_64 rng(seed);
    auto fill = [&](int off, int fan_in, int n, float gain) {
        const float a = gain * std::sqrt(6.f / (float)fan_in);
        std::uniform_real_distribution<float> U(-a, a);
        for (int i = 0; i < n; i++) h[off + i] = U(rng);
    };
    fill(OFF_W1, MLP_FEAT, MLP_IN * MLP_H, 1.f);
    for (int r = MLP_FEAT; r < MLP_IN; r++)
        for (int c = 0; c < MLP_H; c++) h[OFF_W1 + r * MLP_H + c] = 0.f;
    fill(OFF_W2, MLP_H, MLP_H * MLP_H, 1.f);
    fill(OFF_W3, MLP_H, MLP_H * MLP_OUT, 0.1f);
    for (int r = 0; r < MLP_H; r++)
        for (int c = MLP_NOUT; c < MLP_OUT; c++) h[OFF_W3 + r * MLP_OUT + c] = 0.f;
    e = cudaMemcpy(M->P, h.data(), NPARAM * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(M->G, 0, 3 * NPARAM * sizeof(float) + sizeof(float) * 4);
    if (e != cudaSuccess) {
        cudaFree(M->tiles);
        cudaFree(p);
        delete M;
        return cuda_fail(e, "mlp init");
    }
    int st = mlp_repack(M, 0);
    if (st) return st;
    PPGPU_CUDA(cudaDeviceSynchronize(), "mlp init");
    *handle = M;
    return set_ok();
}

extern "C" int ppgpu_mlp_destroy(void *handle) {
    MLP *M = (MLP *)handle;
    if (!M) return set_ok();
    cudaFree(M->P);
    cudaFree(M->tiles);
    cudaFree(M->xt);
    delete M;
    return set_ok();
}

extern "C" int ppgpu_mlp_nparams(void) { return NPARAM; }

/* which: 0 parameters, 1 gradients (read), 2 Adam first moments, 3 second moments. */
extern "C" int ppgpu_mlp_get(void *handle, int which, float *host) {
    MLP *M = (MLP *)handle;
    if (!M || !host || which < 0 || which > 3) return set_error(PPGPU_ERR_ARG, "mlp_get: bad arguments");
    const float *src = which == 0 ? M->P : (which == 1 ? M->G : (which == 2 ? M->M : M->V));
    PPGPU_CUDA(cudaMemcpy(host, src, NPARAM * sizeof(float), cudaMemcpyDeviceToHost), "mlp_get");
    return set_ok();
}

extern "C" int ppgpu_mlp_set(void *handle, const float *host) {
    MLP *M = (MLP *)handle;
    if (!M || !host) return set_error(PPGPU_ERR_ARG, "mlp_set: bad arguments");
    PPGPU_CUDA(cudaMemcpy(M->P, host, NPARAM * sizeof(float), cudaMemcpyHostToDevice), "mlp_set");
    PPGPU_CUDA(cudaMemset(M->G, 0, 3 * NPARAM * sizeof(float)), "mlp_set");
    int st = mlp_repack(M, 0);
    if (st) return st;
    PPGPU_CUDA(cudaDeviceSynchronize(), "mlp_set");
    return set_ok();
}

extern "C" int ppgpu_mlp_forward(void *handle, const void *X, int n, float *Y, void *stream) {
    MLP *M = (MLP *)handle;
    if (!M || !X || !Y || n <= 0 || n % 128) return set_error(PPGPU_ERR_ARG, "mlp_forward: n must be a positive multiple of 128");
    const int smem = TILE_W1T + TILE_W2T + TILE_W3T + TILE_ACT;
    PPGPU_CUDA(cudaFuncSetAttribute(mlp_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem), "mlp smem");
    mlp_forward_kernel<<<n / 128, 128, smem, (cudaStream_t)stream>>>(M->view(), (const __nv_bfloat16 *)X, Y,
                                                                     device_error_word());
    PPGPU_CHECK_LAUNCH("mlp_forward_kernel");
    return set_ok();
}

/* Gradients of the mean squared error over the minibatch rows idx[0..nbatch) of X [.][96] bf16
 * and T [.][4] f32 (3 used) are ADDED to the gradient buffer; the batch loss is added to the
 * device loss scalar.  nbatch: multiple of 128. */
extern "C" int ppgpu_mlp_backward(void *handle, const void *X, const float *T, const int *idx, int nbatch, void *stream) {
    MLP *M = (MLP *)handle;
    if (!M || !X || !T || !idx || nbatch <= 0 || nbatch % 128)
        return set_error(PPGPU_ERR_ARG, "mlp_backward: nbatch must be a positive multiple of 128");
    const int ntiles = nbatch / 128;
    int st = mlp_reserve(M, ntiles);
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    PPGPU_CUDA(cudaFuncSetAttribute(mlp_fwd_bwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, FB_SMEM), "mlp smem");
    mlp_fwd_bwd_kernel<<<ntiles, 128, FB_SMEM, s>>>(M->view(), (const __nv_bfloat16 *)X, (const float4 *)T, idx, nbatch,
                                                    make_float3(M->lw[0], M->lw[1], M->lw[2]), M->G, M->loss, M->xt, M->h1t, M->h2t, M->dyt, M->dz2t, M->dz1t,
                                                    device_error_word());
    PPGPU_CHECK_LAUNCH("mlp_fwd_bwd_kernel");
    const int per = 8;
    const int wsmem = 2 * TILE_ACT;
    PPGPU_CUDA(cudaFuncSetAttribute(mlp_wgrad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, wsmem), "mlp smem");
    mlp_wgrad_kernel<<<dim3((ntiles + per - 1) / per, 3), 128, wsmem, s>>>(ntiles, per, M->xt, M->h1t, M->h2t, M->dyt,
                                                                         M->dz2t, M->dz1t, M->G, device_error_word());
    PPGPU_CHECK_LAUNCH("mlp_wgrad_kernel");
    return set_ok();
}

/* One Adam step (lr, step t >= 1) from the accumulated gradients, which are then cleared. */
extern "C" int ppgpu_mlp_adam(void *handle, double lr, int step, void *stream) {
    MLP *M = (MLP *)handle;
    if (!M || step < 1) return set_error(PPGPU_ERR_ARG, "mlp_adam: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    const float b1t = (float)(1.0 - std::pow(0.9, step)), b2t = (float)(1.0 - std::pow(0.999, step));
    mlp_adam_kernel<<<(NPARAM + 255) / 256, 256, 0, s>>>(M->P, M->G, M->M, M->V, (float)lr, b1t, b2t);
    PPGPU_CHECK_LAUNCH("mlp_adam_kernel");
    return mlp_repack(M, s);
}

/* Reads and clears the accumulated loss (synchronises the stream). */
extern "C" int ppgpu_mlp_take_loss(void *handle, double *out, void *stream) {
    MLP *M = (MLP *)handle;
    if (!M || !out) return set_error(PPGPU_ERR_ARG, "mlp_take_loss: bad arguments");
    float v = 0.f;
    cudaStream_t s = (cudaStream_t)stream;
    PPGPU_CUDA(cudaMemcpyAsync(&v, M->loss, sizeof(float), cudaMemcpyDeviceToHost, s), "mlp loss");
    PPGPU_CUDA(cudaMemsetAsync(M->loss, 0, sizeof(float), s), "mlp loss");
    PPGPU_CUDA(cudaStreamSynchronize(s), "mlp loss");
    *out = v;
    return set_ok();
}

/* Device views for the proposal kernel: 5 tile pointers + 3 bias pointers (void *[8]). */
extern "C" int ppgpu_mlp_views(void *handle, void **out8) {
    MLP *M = (MLP *)handle;
    if (!M || !out8) return set_error(PPGPU_ERR_ARG, "mlp_views: bad arguments");
    const MLPTiles t = M->view();
    out8[0] = (void *)t.W1t;
    out8[1] = (void *)t.W2t;
    out8[2] = (void *)t.W3t;
    out8[3] = (void *)t.W3;
    out8[4] = (void *)t.W2;
    out8[5] = (void *)t.b1;
    out8[6] = (void *)t.b2;
    out8[7] = (void *)t.b3;
    return set_ok();
}

/* Loss weights of the three outputs (default 1, 1, 1): the loss is mean(sum_o w_o (y_o - t_o)^2). */
extern "C" int ppgpu_mlp_set_loss_weights(void *handle, const double *w3) {
    MLP *M = (MLP *)handle;
    if (!M || !w3) return set_error(PPGPU_ERR_ARG, "mlp_set_loss_weights: bad arguments");
    for (int k = 0; k < 3; k++) {
        if (!(w3[k] >= 0.0)) return set_error(PPGPU_ERR_ARG, "mlp_set_loss_weights: weights must be >= 0");
        M->lw[k] = (float)w3[k];
    }
    return set_ok();
}
