// pp_mlp.cu -- the learned warm start: a small MLP on the tcgen05 tensor cores.
//
// No reference counterpart (new in this library).  The network proposes FIRE's starting
// displacement for the next height of a stroke from the force grid around the probe and the
// converged displacement of the height above; plain FIRE then always runs to the same
// convergence criterion, so the network can only save iterations.
//
// Network: 96 (84 features + 12 zero pad) -> 128 -> 128 -> 16 (3 used), SiLU, bf16 weights
// and activations, float32 accumulation in tensor memory.  Every GEMM is a 128-row tile
// issued by one thread with tcgen05.mma (pp_tc.cuh); epilogues (bias, SiLU, its derivative,
// conversions) run on all threads from tcgen05.ld.
#include <cmath>
#include <cstring>

#include "pp_common.cuh"
#include "pp_tc.cuh"

namespace ppgpu {

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
