// pp_grid.cu -- elementwise grid kernels and the FP32 peak probe.
//
//   ppgpu_fz2df       Fz2df (ppafm/common.py:421-430) as a standalone per-column kernel
//   ppgpu_clamp_grid  limit_vec_field (ppafm/io.py:766-778)
//   ppgpu_axpby_grid  the FF composition FF = FFLJ + Q*FFel (ppafm/HighLevel.py:143-145)
//   conversions between the reference's float64 [n,3] (+[n]) grids and float4 grids.
// All are HBM-streaming kernels: grid-stride loops over 16-byte elements, sized to a
// multiple of the SM count.
#include <cstring>

#include "pp_common.cuh"

namespace ppgpu {

constexpr int GRID_THREADS = 256;

static unsigned stream_blocks(long long n) {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long want = (n + GRID_THREADS - 1) / GRID_THREADS;
    long long cap = (long long)sms * 8;
    if (want > cap) want = cap;
    if (want < 1) want = 1;
    return (unsigned)want;
}

struct DfW {
    float w[64];
};

__global__ void fz2df_kernel(const float *__restrict__ F, long long ncol, int nz, int nw, DfW W, float scale,
                             float *__restrict__ out) {
    const int nout = nz - nw + 1;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncol; c += (long long)gridDim.x * blockDim.x) {
        const float *f = F + c * nz;
        float *o = out + c * nout;
        for (int j = 0; j < nout; j++) {
            float acc = 0.f;
            for (int i = 0; i < nw; i++) acc = fmaf(f[j + i], W.w[nw - 1 - i], acc);
            o[j] = acc * scale;
        }
    }
}

__global__ void clamp_kernel(float4 *FE, long long n, float Fmax) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float4 v = FE[i];
        const float m = fmaxf(fabsf(v.x), fmaxf(fabsf(v.y), fabsf(v.z)));
        if (m > 0.f) {
            const float s = 1.f / m;
            const float fr = m * sqrtf((v.x * s) * (v.x * s) + (v.y * s) * (v.y * s) + (v.z * s) * (v.z * s));
            if (fr > Fmax) {
                const float k = Fmax / fr;
                v.x *= k;
                v.y *= k;
                v.z *= k;
                FE[i] = v;
            }
        }
    }
}

__global__ void axpby_kernel(float4 *out, const float4 *a, float ca, const float4 *b, float cb, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float4 x = a[i];
        const float4 y = b ? b[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        out[i] = make_float4(fmaf(ca, x.x, cb * y.x), fmaf(ca, x.y, cb * y.y), fmaf(ca, x.z, cb * y.z),
                             fmaf(ca, x.w, cb * y.w));
    }
}

__global__ void from_f64_kernel(float4 *FE, const double *F3, const double *E, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        FE[i] = make_float4((float)F3[3 * i], (float)F3[3 * i + 1], (float)F3[3 * i + 2], E ? (float)E[i] : 0.f);
    }
}

__global__ void to_f64_kernel(double *F3, double *E, const float4 *FE, long long n, int acc) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float4 v = FE[i];
        if (F3) {
            if (acc) {
                F3[3 * i] += v.x;
                F3[3 * i + 1] += v.y;
                F3[3 * i + 2] += v.z;
            } else {
                F3[3 * i] = v.x;
                F3[3 * i + 1] = v.y;
                F3[3 * i + 2] = v.z;
            }
        }
        if (E) E[i] = acc ? E[i] + v.w : (double)v.w;
    }
}

// Dependent FFMA chains, 8 independent chains per thread: a pure FP32-pipe load.
__global__ void __launch_bounds__(256) ffma_kernel(float *sink, int iters) {
    float a[8];
#pragma unroll
    for (int k = 0; k < 8; k++) a[k] = threadIdx.x * 1e-6f + k;
    const float b = 0.999999f, c = 1e-7f;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 8; k++) a[k] = fmaf(a[k], b, c);
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; k++) s += a[k];
    if (s == 12345.678f) sink[threadIdx.x] = s;  // keeps the chains alive
}

}  // namespace ppgpu

using namespace ppgpu;

extern "C" int ppgpu_fz2df(const float *F, long long ncol, int nz, int nw, const double *W, double scale, float *out,
                           void *stream) {
    if (!F || !out || !W) return set_error(PPGPU_ERR_ARG, "fz2df: null argument");
    if (nw <= 0 || nw > 64 || nw > nz) return set_error(PPGPU_ERR_ARG, "fz2df: need 1 <= nw <= min(64, nz)");
    if (ncol <= 0) return set_ok();
    DfW w;
    memset(&w, 0, sizeof(w));
    for (int i = 0; i < nw; i++) w.w[i] = (float)W[i];
    fz2df_kernel<<<stream_blocks(ncol), GRID_THREADS, 0, (cudaStream_t)stream>>>(F, ncol, nz, nw, w, (float)scale, out);
    PPGPU_CHECK_LAUNCH("fz2df_kernel");
    return set_ok();
}

extern "C" int ppgpu_clamp_grid(float *FE, long long npts, double Fmax, void *stream) {
    if (!FE) return set_error(PPGPU_ERR_ARG, "clamp_grid: null grid");
    if (npts <= 0) return set_ok();
    clamp_kernel<<<stream_blocks(npts), GRID_THREADS, 0, (cudaStream_t)stream>>>(reinterpret_cast<float4 *>(FE), npts,
                                                                                 (float)Fmax);
    PPGPU_CHECK_LAUNCH("clamp_kernel");
    return set_ok();
}

extern "C" int ppgpu_axpby_grid(float *FE_out, const float *FE_a, double a, const float *FE_b, double b,
                                long long npts, void *stream) {
    if (!FE_out || !FE_a) return set_error(PPGPU_ERR_ARG, "axpby_grid: null grid");
    if (npts <= 0) return set_ok();
    axpby_kernel<<<stream_blocks(npts), GRID_THREADS, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<float4 *>(FE_out), reinterpret_cast<const float4 *>(FE_a), (float)a,
        reinterpret_cast<const float4 *>(FE_b), (float)b, npts);
    PPGPU_CHECK_LAUNCH("axpby_kernel");
    return set_ok();
}

extern "C" int ppgpu_grid_from_f64(float *FE, const double *F3, const double *E, long long npts, void *stream) {
    if (!FE || !F3) return set_error(PPGPU_ERR_ARG, "grid_from_f64: null argument");
    if (npts <= 0) return set_ok();
    from_f64_kernel<<<stream_blocks(npts), GRID_THREADS, 0, (cudaStream_t)stream>>>(reinterpret_cast<float4 *>(FE), F3,
                                                                                    E, npts);
    PPGPU_CHECK_LAUNCH("from_f64_kernel");
    return set_ok();
}

extern "C" int ppgpu_grid_to_f64(double *F3, double *E, const float *FE, long long npts, int accumulate, void *stream) {
    if (!FE) return set_error(PPGPU_ERR_ARG, "grid_to_f64: null grid");
    if (npts <= 0) return set_ok();
    to_f64_kernel<<<stream_blocks(npts), GRID_THREADS, 0, (cudaStream_t)stream>>>(
        F3, E, reinterpret_cast<const float4 *>(FE), npts, accumulate);
    PPGPU_CHECK_LAUNCH("to_f64_kernel");
    return set_ok();
}

extern "C" int ppgpu_ffma_peak(float *scratch, int iters, long long *fma_count, void *stream) {
    if (!scratch || iters <= 0) return set_error(PPGPU_ERR_ARG, "ffma_peak: bad arguments");
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const unsigned nblk = (unsigned)sms * 8;  // 8 x 256 threads = 64 warps per SM
    ffma_kernel<<<nblk, 256, 0, (cudaStream_t)stream>>>(scratch, iters);
    PPGPU_CHECK_LAUNCH("ffma_kernel");
    if (fma_count) *fma_count = (long long)nblk * 256 * 8 * (long long)iters;
    return set_ok();
}
