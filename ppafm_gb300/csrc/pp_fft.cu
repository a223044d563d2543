// pp_fft.cu -- the FFT density-overlap route on sm_103a (cuFFT + fused k-space kernels).
//
//   potential2forces_mem (ppafm/fieldFFT.py:268-319) with getMGrid (:32-49),
//   getForceTransform (:198-210), getNormalizedBasisMatrix (:213-217):
//     E   = Re ifft( FFT(V) conj(FFT(rho)) dV / det Linv )
//     F_a = Re ifft( zeta_a FFT(V) conj(FFT(rho)) (-2 pi i) dV / det Linv )
//   getProbeDensity (fieldFFT.py:99-118): normalised Gaussian tip with multipoles
//   handle_negative_density + rho^B (ppafm/cli/conv_rho.py:18-22, 57-64)
//   a Poisson solve for a Hartree potential (no reference counterpart)
//
// A handle computes in float32 complex (cufft R2C/C2R) or, created with PPGPU_FFT_F64, in
// float64 (D2Z/Z2D): float32 transforms leave an error of ~1e-6 of the field's maximum at
// every point, which the weak lateral spring turns into ~1e-3 A probe displacements where
// the field is small; the float64 handle removes it at a higher cost.
//
// Design: real-to-complex transforms of V and rho, one fused kernel that forms the four
// output spectra (E, Fx, Fy, Fz) on the half spectrum, one batched complex-to-real
// transform of the four, and an epilogue that writes the interleaved float4 grid the
// relaxation reads (scaled, optionally accumulated).  numpy takes Re(ifftn(Y)) of a full
// spectrum; with a half spectrum that equals ifft of the Hermitian part of Y, which for
// Y = zeta C (-2 pi i) uses the odd part of the rolled coordinate grid zeta -- exact for
// even and odd sizes (the reference's grid is not antisymmetric for odd sizes).
#include <cufft.h>

#include <cmath>
#include <cstring>

#include "pp_common.cuh"

namespace ppgpu {

constexpr int FFT_THREADS = 256;

struct FFTPlan {
    int n[3];
    long long N, Nh;  // real points, half-spectrum points
    bool f64;         // transforms and spectra in float64 (cufft D2Z/Z2D)
    cufftHandle r2c = 0, c2r4 = 0, c2r1 = 0;
    void *Vk = nullptr, *Rk = nullptr, *S4 = nullptr;  // cufftComplex or cufftDoubleComplex
    void *Tk = nullptr;  // spectrum of the last correlation kernel (ppgpu_fft_correlate)
    void *planar = nullptr;  // 4 real planes (float or double)
    double *sums = nullptr;  // reduction scratch
};

static int cufft_fail(cufftResult r, const char *what) {
    return set_error(PPGPU_ERR_CUDA, "%s: cuFFT error %d", what, (int)r);
}

#define PPGPU_CUFFT(call, what)                         \
    do {                                                \
        cufftResult _r = (call);                        \
        if (_r != CUFFT_SUCCESS) return cufft_fail(_r, what); \
    } while (0)

static unsigned blocks_for(long long n) {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long want = (n + FFT_THREADS - 1) / FFT_THREADS;
    long long cap = (long long)sms * 8;
    return (unsigned)(want < 1 ? 1 : (want > cap ? cap : want));
}

// One thread per half-spectrum element over a 1-D grid.
static unsigned spec_blocks(const FFTPlan *P) { return (unsigned)((P->Nh + FFT_THREADS - 1) / FFT_THREADS); }

// Rolled coordinate index of getMGrid (fieldFFT.py:32-49): i for i < n/2, i - n above.
__device__ __forceinline__ double rolled(int i, int n) { return (double)(i < n / 2 ? i : i - n); }
// Twice the odd part of the rolled index, rolled(i) - rolled(-i mod n): an integer, so the
// spectra kernel needs no float64 arithmetic in its float32 form.
__device__ __forceinline__ int rolled_odd2(int i, int n) {
    const int j = (i == 0) ? 0 : n - i;
    return (i < n / 2 ? i : i - n) - (j < n / 2 ? j : j - n);
}

struct GaussCell {
    double cell[9], inv[9];  // rows a, b, c and the inverse (fractional = r . inv columns)
};

struct SpecPrm {
    int n0, n1, n2, nh2;
    long long Nh;   // elements of one half spectrum
    double z[9];    // zeta_a = sum_j z[3a+j] * Xodd_j   (Linv[a][j] * dzeta_j * d_j)
    double sE, sF;  // dV/detLinv/N and 2 pi dV/detLinv/N
    float zf[9], sEf, sFf;  // the same rounded to float32 (the float32 kernel's copies)
};

// The coefficients in the kernel's precision (no float64 -> float32 conversions per thread).
template <typename R>
__device__ __forceinline__ R spec_z(const SpecPrm &P, int i);
template <>
__device__ __forceinline__ float spec_z<float>(const SpecPrm &P, int i) { return P.zf[i]; }
template <>
__device__ __forceinline__ double spec_z<double>(const SpecPrm &P, int i) { return P.z[i]; }
template <typename R>
__device__ __forceinline__ R spec_s(const SpecPrm &P, bool force) {
    if constexpr (sizeof(R) == 4) return force ? P.sFf : P.sEf;
    else return force ? P.sF : P.sE;
}

template <typename C>
struct Cx;
template <>
struct Cx<cufftComplex> {
    using real = float;
    static __device__ __forceinline__ cufftComplex make(float x, float y) { return make_cuComplex(x, y); }
};
template <>
struct Cx<cufftDoubleComplex> {
    using real = double;
    static __device__ __forceinline__ cufftDoubleComplex make(double x, double y) { return make_cuDoubleComplex(x, y); }
};

// Four output spectra from FFT(V) and FFT(rho).  One thread per half-spectrum element, the
// elements numbered q = (i * n1 + j) * nh2 + k over a 1-D grid.  The arithmetic is done in
// the precision of the transforms (float32 spectra: float; float64 spectra: double).
template <typename C>
__global__ void spectra_kernel(const C *__restrict__ Vk, const C *__restrict__ Rk, C *__restrict__ S4, SpecPrm P) {
    using R = typename Cx<C>::real;
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= P.Nh) return;
    const long long row = q / P.nh2;
    const int k = (int)(q - row * P.nh2);
    const int i = (int)(row / P.n1), j = (int)(row - (long long)i * P.n1);
    const C a = Vk[q], b = Rk[q];
    // C = a conj(b)
    const R cr = a.x * b.x + a.y * b.y;
    const R ci = a.y * b.x - a.x * b.y;
    const R xo = (R)0.5 * (R)rolled_odd2(i, P.n0), yo = (R)0.5 * (R)rolled_odd2(j, P.n1),
            zo = (R)0.5 * (R)rolled_odd2(k, P.n2);
    const R sE = spec_s<R>(P, false), sF = spec_s<R>(P, true);
    S4[q] = Cx<C>::make(cr * sE, ci * sE);
#pragma unroll
    for (int ax = 0; ax < 3; ax++) {
        const R zeta = (spec_z<R>(P, 3 * ax) * xo + spec_z<R>(P, 3 * ax + 1) * yo + spec_z<R>(P, 3 * ax + 2) * zo) * sF;
        // zeta C (-2 pi i) = zeta (2 pi ci, -2 pi cr)
        S4[(ax + 1) * P.Nh + q] = Cx<C>::make(zeta * ci, -zeta * cr);
    }
}

// FE[p] = (acc ? FE[p] : 0) + scale * (Fx, Fy, Fz, E)[p] from the four real planes.
template <typename R>
__global__ void pack_fe_kernel(float4 *FE, const R *__restrict__ planes, long long N, double scale, int with_e,
                               int acc) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < N; p += (long long)gridDim.x * blockDim.x) {
        const R s = (R)scale;
        R x = s * planes[N + p], y = s * planes[2 * N + p], z = s * planes[3 * N + p], e = with_e ? s * planes[p] : (R)0;
        if (acc) {
            const float4 o = FE[p];
            x += o.x;
            y += o.y;
            z += o.z;
            e += o.w;
        }
        FE[p] = make_float4((float)x, (float)y, (float)z, (float)e);
    }
}

__global__ void f32_to_f64_kernel(double *out, const float *in, long long N) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < N; p += (long long)gridDim.x * blockDim.x)
        out[p] = (double)in[p];
}

__global__ void f64_to_f32_kernel(float *out, const double *in, long long N) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < N; p += (long long)gridDim.x * blockDim.x)
        out[p] = (float)in[p];
}

// ------------------------------------------------------------------ tip density

struct TipPrm {
    int n0, n1, n2;
    double dd[3];
    double mat[9];  // rows: normalised basis matrix transposed (getProbeDensity's `mat`)
    double sigma;
    double coef[10];  // s, px, py, pz, dz2, dx2, dy2, dxy, dxz, dyz
};

__device__ __forceinline__ void tip_coords(const TipPrm &P, long long p, double &rx, double &ry, double &rz) {
    const int k = (int)(p % P.n2);
    const int j = (int)((p / P.n2) % P.n1);
    const int i = (int)(p / ((long long)P.n2 * P.n1));
    const double X = P.dd[0] * rolled(i, P.n0), Y = P.dd[1] * rolled(j, P.n1), Z = P.dd[2] * rolled(k, P.n2);
    rx = X * P.mat[0] + Y * P.mat[1] + Z * P.mat[2];
    ry = X * P.mat[3] + Y * P.mat[4] + Z * P.mat[5];
    rz = X * P.mat[6] + Y * P.mat[7] + Z * P.mat[8];
}

__device__ __forceinline__ void block_sum_to(double v, double *out) {
    __shared__ double sh[FFT_THREADS / 32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = (threadIdx.x < blockDim.x / 32) ? sh[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) atomicAdd(out, v);
    }
}

__global__ void tip_radial_sum_kernel(TipPrm P, long long N, double *sum) {
    double s = 0.0;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < N; p += (long long)gridDim.x * blockDim.x) {
        double rx, ry, rz;
        tip_coords(P, p, rx, ry, rz);
        s += exp(-(rx * rx + ry * ry + rz * rz) / (2 * P.sigma * P.sigma));
    }
    block_sum_to(s, sum);
}

__global__ void tip_density_kernel(float *rho, TipPrm P, long long N, const double *sum, double norm_extra) {
    const double inv = 1.0 / (sum[0] * norm_extra);
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < N; p += (long long)gridDim.x * blockDim.x) {
        double rx, ry, rz;
        tip_coords(P, p, rx, ry, rz);
        const double radial = exp(-(rx * rx + ry * ry + rz * rz) / (2 * P.sigma * P.sigma)) * inv;
        const double x = rx / P.sigma, y = ry / P.sigma, z = rz / P.sigma;
        const double h = P.coef[0] + P.coef[1] * x + P.coef[2] * y + P.coef[3] * z +
                         P.coef[4] * 0.25 * (2 * z * z - x * x - y * y) + P.coef[5] * 0.25 * (2 * x * x - y * y - z * z) +
                         P.coef[6] * 0.25 * (2 * y * y - x * x - z * z) + P.coef[7] * x * y + P.coef[8] * x * z +
                         P.coef[9] * y * z;
        rho[p] = (float)(radial * h);
    }
}

// ------------------------------------------------------------- density pre-processing

// Sum and positive sum of a float grid: compensated float32 sums per thread (a few dozen
// values each), float64 across threads.
__global__ void density_sums_kernel(const float *rho, long long N, double *sums) {
    float s = 0.f, sc = 0.f, sp = 0.f, spc = 0.f;  // Neumaier running compensations
    auto add = [](float &acc, float &c, float v) {
        const float t = acc + v;
        c += (fabsf(acc) >= fabsf(v)) ? (acc - t) + v : (v - t) + acc;
        acc = t;
    };
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < N; p += (long long)gridDim.x * blockDim.x) {
        const float v = rho[p];
        add(s, sc, v);
        add(sp, spc, v > 0.f ? v : 0.f);
    }
    block_sum_to((double)s + (double)sc, sums);
    __syncthreads();
    block_sum_to((double)sp + (double)spc, sums + 1);
}

__global__ void density_power_kernel(float *rho, long long N, const double *sums, int fix_negative, float B) {
    const float f = fix_negative ? (float)(sums[0] / sums[1]) : 1.f;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < N; p += (long long)gridDim.x * blockDim.x) {
        float v = rho[p];
        if (fix_negative) v = (v < 0.f ? 0.f : v) * f;
        if (B != 1.f) v = powf(v, B);
        rho[p] = v;
    }
}

// ------------------------------------------------------------------ Poisson

struct PoissonPrm {
    int n0, n1, n2, nh2;
    long long Nh;
    double b[9];  // reciprocal basis rows b_j (2 pi included): G = sum_j m_j b_j
    double s;     // 4 pi k_e / N
    float bf[9], sf;  // the same rounded to float32
};

// numpy fftfreq index: 0..(n-1)/2 then negative.
__device__ __forceinline__ int freq(int i, int n) { return i <= (n - 1) / 2 ? i : i - n; }

template <typename R>
__device__ __forceinline__ R pois_b(const PoissonPrm &P, int i) {
    if constexpr (sizeof(R) == 4) return P.bf[i];
    else return P.b[i];
}

template <typename C>
__global__ void poisson_kernel(C *Rk, PoissonPrm P) {
    using R = typename Cx<C>::real;
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= P.Nh) return;
    const long long row = q / P.nh2;
    const int k = (int)(q - row * P.nh2);
    const int i = (int)(row / P.n1), j = (int)(row - (long long)i * P.n1);
    const R m0 = (R)freq(i, P.n0), m1 = (R)freq(j, P.n1), m2 = (R)freq(k, P.n2);
    const R gx = m0 * pois_b<R>(P, 0) + m1 * pois_b<R>(P, 3) + m2 * pois_b<R>(P, 6);
    const R gy = m0 * pois_b<R>(P, 1) + m1 * pois_b<R>(P, 4) + m2 * pois_b<R>(P, 7);
    const R gz = m0 * pois_b<R>(P, 2) + m1 * pois_b<R>(P, 5) + m2 * pois_b<R>(P, 8);
    const R g2 = gx * gx + gy * gy + gz * gz;
    const C r = Rk[q];
    const R sc = (sizeof(R) == 4) ? (R)P.sf : (R)P.s;
    const R f = (q == 0) ? (R)0 : sc / g2;
    Rk[q] = Cx<C>::make(r.x * f, r.y * f);
}

// ------------------------------------------------------------ cross-correlation

// S = conj(R) V s over the half spectrum (the AFMulator's FFTCrossCorrelation,
// ppafm/ocl/field.py:707-840: conj_mult then the scaled inverse transform).
template <typename C>
__global__ void corr_mul_kernel(const C *__restrict__ Vk, const C *__restrict__ Rk, C *__restrict__ Sk, long long Nh,
                                typename Cx<C>::real s) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= Nh) return;
    const C a = Vk[q], b = Rk[q];
    Sk[q] = Cx<C>::make((b.x * a.x + b.y * a.y) * s, (b.x * a.y - b.y * a.x) * s);
}

// ------------------------------------------------------------- Gaussian densities

// rho[p] (+)= sum_i w_i g(|p - R_i|; s_i), normalised 3-D Gaussians, minimum-image distance
// on the periodic cell; atoms: [natoms][5] = (x, y, z, sigma, weight), relative to the origin.
__global__ void gauss_density_kernel(float *rho, int n0, int n1, int n2, GaussCell C, const double *atoms, int natoms,
                                     int accumulate) {
    const long long N = (long long)n0 * n1 * n2;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < N; p += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(p % n2);
        const int j = (int)((p / n2) % n1);
        const int i = (int)(p / ((long long)n2 * n1));
        // fractional coordinates of the point
        const double f0 = (double)i / n0, f1 = (double)j / n1, f2 = (double)k / n2;
        double s = 0.0;
        for (int a = 0; a < natoms; a++) {
            const double *A = atoms + 5 * a;
            double g0 = f0 - (A[0] * C.inv[0] + A[1] * C.inv[3] + A[2] * C.inv[6]);
            double g1 = f1 - (A[0] * C.inv[1] + A[1] * C.inv[4] + A[2] * C.inv[7]);
            double g2 = f2 - (A[0] * C.inv[2] + A[1] * C.inv[5] + A[2] * C.inv[8]);
            g0 -= rint(g0);
            g1 -= rint(g1);
            g2 -= rint(g2);
            const double dx = g0 * C.cell[0] + g1 * C.cell[3] + g2 * C.cell[6];
            const double dy = g0 * C.cell[1] + g1 * C.cell[4] + g2 * C.cell[7];
            const double dz = g0 * C.cell[2] + g1 * C.cell[5] + g2 * C.cell[8];
            const double sg = A[3];
            const double t = (dx * dx + dy * dy + dz * dz) / (2 * sg * sg);
            // exp(-t) < 1e-17 beyond t = 40: below float32 resolution of any sum it joins
            if (t < 40.0) s += A[4] * (double)expf(-(float)t) / (15.749609945722419 * sg * sg * sg);  // (2 pi)^1.5
        }
        rho[p] = accumulate ? rho[p] + (float)s : (float)s;
    }
}

// ------------------------------------------------------------------ host helpers

static void inv3(const double *m, double *o, double *det) {
    const double a = m[0], b = m[1], c = m[2], d = m[3], e = m[4], f = m[5], g = m[6], h = m[7], i = m[8];
    const double A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;
    *det = a * A + b * B + c * C;
    const double id = 1.0 / *det;
    o[0] = A * id;
    o[1] = -(b * i - c * h) * id;
    o[2] = (b * f - c * e) * id;
    o[3] = B * id;
    o[4] = (a * i - c * g) * id;
    o[5] = -(a * f - c * d) * id;
    o[6] = C * id;
    o[7] = -(a * h - b * g) * id;
    o[8] = (a * e - b * d) * id;
}

// Normalised basis (rows a/|a|, b/|b|, c/|c|) and grid steps dd_j = |l_j|/n_j.
static void basis(const int *n, const double *lvec, double *L, double *dd) {
    for (int r = 0; r < 3; r++) {
        const double *v = lvec + 3 * (r + 1);
        const double nv = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        for (int c = 0; c < 3; c++) L[3 * r + c] = v[c] / nv;
        dd[r] = nv / n[r];
    }
}

}  // namespace ppgpu

using namespace ppgpu;

extern "C" int ppgpu_fft_create(const int *n, int flags, void **handle) {
    if (!n || !handle) return set_error(PPGPU_ERR_ARG, "fft_create: null argument");
    for (int k = 0; k < 3; k++)
        if (n[k] <= 0) return set_error(PPGPU_ERR_ARG, "fft_create: sizes must be positive");
    if (n[0] > 65535 || n[1] > 65535) return set_error(PPGPU_ERR_ARG, "fft_create: n0, n1 must be at most 65535");
    if (flags & ~PPGPU_FFT_F64) return set_error(PPGPU_ERR_ARG, "fft_create: unknown flags %d", flags);
    FFTPlan *P = new FFTPlan();
    for (int k = 0; k < 3; k++) P->n[k] = n[k];
    P->N = (long long)n[0] * n[1] * n[2];
    P->Nh = (long long)n[0] * n[1] * (n[2] / 2 + 1);
    P->f64 = (flags & PPGPU_FFT_F64) != 0;
    auto fail = [&](int st) {
        if (P->r2c) cufftDestroy(P->r2c);
        if (P->c2r4) cufftDestroy(P->c2r4);
        if (P->c2r1) cufftDestroy(P->c2r1);
        cudaFree(P->Vk);
        cudaFree(P->Rk);
        cudaFree(P->S4);
        cudaFree(P->planar);
        cudaFree(P->sums);
        delete P;
        return st;
    };
    const cufftType fwd = P->f64 ? CUFFT_D2Z : CUFFT_R2C, inv = P->f64 ? CUFFT_Z2D : CUFFT_C2R;
    cufftResult r = cufftPlan3d(&P->r2c, n[0], n[1], n[2], fwd);
    if (r != CUFFT_SUCCESS) return fail(cufft_fail(r, "cufftPlan3d forward"));
    r = cufftPlan3d(&P->c2r1, n[0], n[1], n[2], inv);
    if (r != CUFFT_SUCCESS) return fail(cufft_fail(r, "cufftPlan3d inverse"));
    int dims[3] = {n[0], n[1], n[2]};
    // NULL embeds: natural layout, batch distance = one grid (spectrum / real)
    r = cufftPlanMany(&P->c2r4, 3, dims, nullptr, 1, 0, nullptr, 1, 0, inv, 4);
    if (r != CUFFT_SUCCESS) return fail(cufft_fail(r, "cufftPlanMany inverse x4"));
    const size_t cs = P->f64 ? sizeof(cufftDoubleComplex) : sizeof(cufftComplex);
    const size_t rs = P->f64 ? sizeof(double) : sizeof(float);
    cudaError_t e;
    if ((e = cudaMalloc(&P->Vk, P->Nh * cs)) != cudaSuccess) return fail(cuda_fail(e, "fft buffers"));
    if ((e = cudaMalloc(&P->Rk, P->Nh * cs)) != cudaSuccess) return fail(cuda_fail(e, "fft buffers"));
    if ((e = cudaMalloc(&P->S4, 4 * P->Nh * cs)) != cudaSuccess) return fail(cuda_fail(e, "fft buffers"));
    if ((e = cudaMalloc(&P->planar, 4 * P->N * rs)) != cudaSuccess) return fail(cuda_fail(e, "fft buffers"));
    if ((e = cudaMalloc(&P->sums, 8 * sizeof(double))) != cudaSuccess) return fail(cuda_fail(e, "fft buffers"));
    *handle = P;
    return set_ok();
}

extern "C" int ppgpu_fft_destroy(void *handle) {
    FFTPlan *P = (FFTPlan *)handle;
    if (!P) return set_ok();
    cufftDestroy(P->r2c);
    cufftDestroy(P->c2r4);
    cufftDestroy(P->c2r1);
    cudaFree(P->Vk);
    cudaFree(P->Rk);
    cudaFree(P->S4);
    cudaFree(P->Tk);
    cudaFree(P->planar);
    cudaFree(P->sums);
    delete P;
    return set_ok();
}

// Forward transform of a float32 real grid into the spectrum buffer `out` (float64 plans
// widen the grid into `stage` first).
static int forward(FFTPlan *P, const float *x, void *out, double *stage, cudaStream_t st, const char *what) {
    if (P->f64) {
        f32_to_f64_kernel<<<blocks_for(P->N), FFT_THREADS, 0, st>>>(stage, x, P->N);
        PPGPU_CHECK_LAUNCH("f32_to_f64_kernel");
        PPGPU_CUFFT(cufftExecD2Z(P->r2c, stage, (cufftDoubleComplex *)out), what);
    } else {
        PPGPU_CUFFT(cufftExecR2C(P->r2c, (cufftReal *)x, (cufftComplex *)out), what);
    }
    return PPGPU_OK;
}

extern "C" int ppgpu_fft_potential2forces(void *handle, const float *V, const float *rho, const double *lvec,
                                          double scale, int flags, float *FE, void *stream) {
    FFTPlan *P = (FFTPlan *)handle;
    if (!P || !V || !rho || !lvec || !FE) return set_error(PPGPU_ERR_ARG, "potential2forces: null argument");
    cudaStream_t st = (cudaStream_t)stream;
    PPGPU_CUFFT(cufftSetStream(P->r2c, st), "cufftSetStream");
    PPGPU_CUFFT(cufftSetStream(P->c2r4, st), "cufftSetStream");
    double *stage = (double *)P->planar;  // the planes are free until the inverse transform
    int rc;
    if ((rc = forward(P, V, P->Vk, stage, st, "forward V")) != PPGPU_OK) return rc;
    if ((rc = forward(P, rho, P->Rk, stage, st, "forward rho")) != PPGPU_OK) return rc;
    double L[9], dd[3], Li[9], det;
    basis(P->n, lvec, L, dd);
    inv3(L, Li, &det);  // LmatInv
    const double detLinv = fabs(1.0 / det);
    SpecPrm sp;
    sp.n0 = P->n[0];
    sp.n1 = P->n[1];
    sp.n2 = P->n[2];
    sp.nh2 = P->n[2] / 2 + 1;
    for (int a = 0; a < 3; a++)
        for (int j = 0; j < 3; j++) sp.z[3 * a + j] = Li[3 * a + j] / (P->n[j] * dd[j] * dd[j]) * dd[j];
    const double dV = dd[0] * dd[1] * dd[2];
    sp.sE = dV / detLinv / (double)P->N;
    sp.sF = 2 * M_PI * dV / detLinv / (double)P->N;
    sp.Nh = P->Nh;
    for (int a = 0; a < 9; a++) sp.zf[a] = (float)sp.z[a];
    sp.sEf = (float)sp.sE;
    sp.sFf = (float)sp.sF;
    const int with_e = (flags & PPGPU_FF_WITH_E) ? 1 : 0, acc = (flags & PPGPU_FF_ACCUMULATE) ? 1 : 0;
    if (P->f64) {
        spectra_kernel<cufftDoubleComplex><<<spec_blocks(P), FFT_THREADS, 0, st>>>(
            (const cufftDoubleComplex *)P->Vk, (const cufftDoubleComplex *)P->Rk, (cufftDoubleComplex *)P->S4, sp);
        PPGPU_CHECK_LAUNCH("spectra_kernel");
        PPGPU_CUFFT(cufftExecZ2D(P->c2r4, (cufftDoubleComplex *)P->S4, (double *)P->planar), "inverse x4");
        pack_fe_kernel<double><<<blocks_for(P->N), FFT_THREADS, 0, st>>>((float4 *)FE, (const double *)P->planar, P->N,
                                                                          scale, with_e, acc);
    } else {
        spectra_kernel<cufftComplex><<<spec_blocks(P), FFT_THREADS, 0, st>>>(
            (const cufftComplex *)P->Vk, (const cufftComplex *)P->Rk, (cufftComplex *)P->S4, sp);
        PPGPU_CHECK_LAUNCH("spectra_kernel");
        PPGPU_CUFFT(cufftExecC2R(P->c2r4, (cufftComplex *)P->S4, (cufftReal *)P->planar), "inverse x4");
        pack_fe_kernel<float><<<blocks_for(P->N), FFT_THREADS, 0, st>>>((float4 *)FE, (const float *)P->planar, P->N,
                                                                         scale, with_e, acc);
    }
    PPGPU_CHECK_LAUNCH("pack_fe_kernel");
    return set_ok();
}

extern "C" int ppgpu_fft_probe_density(void *handle, float *rho, const double *lvec, double sigma,
                                       const double *multipole, void *stream) {
    FFTPlan *P = (FFTPlan *)handle;
    if (!P || !rho || !lvec) return set_error(PPGPU_ERR_ARG, "probe_density: null argument");
    if (!(sigma > 0)) return set_error(PPGPU_ERR_ARG, "probe_density: sigma must be positive");
    cudaStream_t st = (cudaStream_t)stream;
    TipPrm tp;
    tp.n0 = P->n[0];
    tp.n1 = P->n[1];
    tp.n2 = P->n[2];
    double L[9];
    basis(P->n, lvec, L, tp.dd);
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) tp.mat[3 * r + c] = L[3 * c + r];  // getNormalizedBasisMatrix(...).getT()
    tp.sigma = sigma;
    for (int k = 0; k < 10; k++) tp.coef[k] = multipole ? multipole[k] : (k == 0 ? 1.0 : 0.0);
    const double det = tp.mat[0] * (tp.mat[4] * tp.mat[8] - tp.mat[5] * tp.mat[7]) -
                       tp.mat[1] * (tp.mat[3] * tp.mat[8] - tp.mat[5] * tp.mat[6]) +
                       tp.mat[2] * (tp.mat[3] * tp.mat[7] - tp.mat[4] * tp.mat[6]);
    PPGPU_CUDA(cudaMemsetAsync(P->sums, 0, sizeof(double), st), "clear sums");
    tip_radial_sum_kernel<<<blocks_for(P->N), FFT_THREADS, 0, st>>>(tp, P->N, P->sums);
    PPGPU_CHECK_LAUNCH("tip_radial_sum_kernel");
    tip_density_kernel<<<blocks_for(P->N), FFT_THREADS, 0, st>>>(rho, tp, P->N, P->sums,
                                                                 fabs(det) * tp.dd[0] * tp.dd[1] * tp.dd[2]);
    PPGPU_CHECK_LAUNCH("tip_density_kernel");
    return set_ok();
}

extern "C" int ppgpu_fft_density_power(void *handle, float *rho, double B, int fix_negative, void *stream) {
    FFTPlan *P = (FFTPlan *)handle;
    if (!P || !rho) return set_error(PPGPU_ERR_ARG, "density_power: null argument");
    cudaStream_t st = (cudaStream_t)stream;
    if (fix_negative) {
        PPGPU_CUDA(cudaMemsetAsync(P->sums, 0, 2 * sizeof(double), st), "clear sums");
        density_sums_kernel<<<blocks_for(P->N), FFT_THREADS, 0, st>>>(rho, P->N, P->sums);
        PPGPU_CHECK_LAUNCH("density_sums_kernel");
    }
    if (!fix_negative && B == 1.0) return set_ok();
    density_power_kernel<<<blocks_for(P->N), FFT_THREADS, 0, st>>>(rho, P->N, P->sums, fix_negative, (float)B);
    PPGPU_CHECK_LAUNCH("density_power_kernel");
    return set_ok();
}

extern "C" int ppgpu_fft_poisson(void *handle, const float *rho_charge, const double *lvec, float *V, void *stream) {
    FFTPlan *P = (FFTPlan *)handle;
    if (!P || !rho_charge || !lvec || !V) return set_error(PPGPU_ERR_ARG, "poisson: null argument");
    cudaStream_t st = (cudaStream_t)stream;
    PPGPU_CUFFT(cufftSetStream(P->r2c, st), "cufftSetStream");
    PPGPU_CUFFT(cufftSetStream(P->c2r1, st), "cufftSetStream");
    double *stage = (double *)P->planar;
    int rc;
    if ((rc = forward(P, rho_charge, P->Rk, stage, st, "forward rho")) != PPGPU_OK) return rc;
    // reciprocal basis: rows of inv(cell)^T times 2 pi
    double cell[9], ci[9], det;
    for (int k = 0; k < 9; k++) cell[k] = lvec[3 + k];
    inv3(cell, ci, &det);
    if (!(det != 0.0)) return set_error(PPGPU_ERR_ARG, "poisson: singular cell");
    PoissonPrm pp;
    pp.n0 = P->n[0];
    pp.n1 = P->n[1];
    pp.n2 = P->n[2];
    pp.nh2 = P->n[2] / 2 + 1;
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) pp.b[3 * r + c] = 2 * M_PI * ci[3 * c + r];
    pp.s = 4 * M_PI * 14.399645 / (double)P->N;
    pp.Nh = P->Nh;
    for (int a = 0; a < 9; a++) pp.bf[a] = (float)pp.b[a];
    pp.sf = (float)pp.s;
    if (P->f64) {
        poisson_kernel<cufftDoubleComplex><<<spec_blocks(P), FFT_THREADS, 0, st>>>((cufftDoubleComplex *)P->Rk, pp);
        PPGPU_CHECK_LAUNCH("poisson_kernel");
        PPGPU_CUFFT(cufftExecZ2D(P->c2r1, (cufftDoubleComplex *)P->Rk, stage), "inverse V");
        f64_to_f32_kernel<<<blocks_for(P->N), FFT_THREADS, 0, st>>>(V, stage, P->N);
        PPGPU_CHECK_LAUNCH("f64_to_f32_kernel");
    } else {
        poisson_kernel<cufftComplex><<<spec_blocks(P), FFT_THREADS, 0, st>>>((cufftComplex *)P->Rk, pp);
        PPGPU_CHECK_LAUNCH("poisson_kernel");
        PPGPU_CUFFT(cufftExecC2R(P->c2r1, (cufftComplex *)P->Rk, (cufftReal *)V), "inverse V");
    }
    return set_ok();
}

extern "C" int ppgpu_gaussian_density(float *rho, const int *n, const double *lvec, int natoms, const double *atoms,
                                      int accumulate, void *stream) {
    if (!rho || !n || !lvec || (natoms > 0 && !atoms)) return set_error(PPGPU_ERR_ARG, "gaussian_density: null argument");
    for (int k = 0; k < 3; k++)
        if (n[k] <= 0) return set_error(PPGPU_ERR_ARG, "gaussian_density: sizes must be positive");
    GaussCell C;
    for (int k = 0; k < 9; k++) C.cell[k] = lvec[3 + k];
    double det;
    inv3(C.cell, C.inv, &det);
    if (!(det != 0.0)) return set_error(PPGPU_ERR_ARG, "gaussian_density: singular cell");
    const long long N = (long long)n[0] * n[1] * n[2];
    gauss_density_kernel<<<blocks_for(N), FFT_THREADS, 0, (cudaStream_t)stream>>>(rho, n[0], n[1], n[2], C, atoms,
                                                                                natoms, accumulate);
    PPGPU_CHECK_LAUNCH("gauss_density_kernel");
    return set_ok();
}

/* E = IFFT(conj(FFT(rho)) FFT(V)) * scale / N: the circular cross-correlation of the AFMulator's
 * Hartree route (FFTCrossCorrelation.correlate, ppafm/ocl/field.py:800-840, with reikna's
 * normalised inverse).  V, rho, E: float32 grids of the plan's size.  The spectrum of rho is
 * kept with the plan: rho NULL reuses the last one (like the reference, which transforms the
 * tip density once, FFTCrossCorrelation._set_rho). */
extern "C" int ppgpu_fft_correlate(void *handle, const float *V, const float *rho, double scale, float *E, void *stream) {
    FFTPlan *P = (FFTPlan *)handle;
    if (!P || !V || !E) return set_error(PPGPU_ERR_ARG, "correlate: null argument");
    if (!rho && !P->Tk) return set_error(PPGPU_ERR_STATE, "correlate: no kernel spectrum yet (pass rho)");
    cudaStream_t st = (cudaStream_t)stream;
    PPGPU_CUFFT(cufftSetStream(P->r2c, st), "cufftSetStream");
    PPGPU_CUFFT(cufftSetStream(P->c2r1, st), "cufftSetStream");
    double *stage = (double *)P->planar;
    int rc;
    if (rho) {
        if (!P->Tk) {
            const size_t cs = P->f64 ? sizeof(cufftDoubleComplex) : sizeof(cufftComplex);
            cudaError_t e = cudaMalloc(&P->Tk, P->Nh * cs);
            if (e != cudaSuccess) {
                P->Tk = nullptr;
                return cuda_fail(e, "correlation spectrum");
            }
        }
        if ((rc = forward(P, rho, P->Tk, stage, st, "forward rho")) != PPGPU_OK) return rc;
    }
    if ((rc = forward(P, V, P->Vk, stage, st, "forward V")) != PPGPU_OK) return rc;
    const double s = scale / (double)P->N;
    if (P->f64) {
        corr_mul_kernel<cufftDoubleComplex><<<spec_blocks(P), FFT_THREADS, 0, st>>>(
            (const cufftDoubleComplex *)P->Vk, (const cufftDoubleComplex *)P->Tk, (cufftDoubleComplex *)P->S4, P->Nh, s);
        PPGPU_CHECK_LAUNCH("corr_mul_kernel");
        PPGPU_CUFFT(cufftExecZ2D(P->c2r1, (cufftDoubleComplex *)P->S4, stage), "inverse E");
        f64_to_f32_kernel<<<blocks_for(P->N), FFT_THREADS, 0, st>>>(E, stage, P->N);
        PPGPU_CHECK_LAUNCH("f64_to_f32_kernel");
    } else {
        corr_mul_kernel<cufftComplex><<<spec_blocks(P), FFT_THREADS, 0, st>>>(
            (const cufftComplex *)P->Vk, (const cufftComplex *)P->Tk, (cufftComplex *)P->S4, P->Nh, (float)s);
        PPGPU_CHECK_LAUNCH("corr_mul_kernel");
        PPGPU_CUFFT(cufftExecC2R(P->c2r1, (cufftComplex *)P->S4, E), "inverse E");
    }
    return set_ok();
}
