// pp_grid.cu -- elementwise grid kernels and the FP32 peak probe.
//
//   ppgpu_fz2df       Fz2df (ppafm/common.py:421-430) as a standalone per-column kernel
//   ppgpu_clamp_grid  limit_vec_field (ppafm/io.py:766-778)
//   ppgpu_axpby_grid  the FF composition FF = FFLJ + Q*FFel (ppafm/HighLevel.py:143-145)
//   conversions between the reference's float64 [n,3] (+[n]) grids and float4 grids.
// All are HBM-streaming kernels: grid-stride loops over 16-byte elements, sized to a
// multiple of the SM count.
#include <algorithm>
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

// The same convolution with the columns staged in shared memory: a warp takes 32
// consecutive columns, whose samples are one contiguous run of 32*nz floats (and whose outputs
// one run of 32*nout), loads the run with coalesced float4 reads, convolves each column from
// shared memory in the order of fz2df_kernel (bit for bit its result), and stores the outputs
// coalesced.  Columns of at most FZ2DF_TILE_NZ samples; F and out 16-byte aligned.
constexpr int FZ2DF_TILE_NZ = 64;
constexpr int FZ2DF_WARPS = 4;

__global__ void __launch_bounds__(32 * FZ2DF_WARPS) fz2df_tiled_kernel(const float *__restrict__ F, long long ncol,
                                                                       int nz, int nw, DfW W, float scale,
                                                                       float *__restrict__ out) {
    extern __shared__ __align__(16) float fz_smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nout = nz - nw + 1;
    float *sin = fz_smem + (size_t)warp * 32 * (nz + nout);
    float *sout = sin + 32 * nz;
    const long long ntile = (ncol + 31) / 32;
    for (long long t = (long long)blockIdx.x * FZ2DF_WARPS + warp; t < ntile; t += (long long)gridDim.x * FZ2DF_WARPS) {
        const long long c0 = t * 32;
        const int ncl = (int)min(32LL, ncol - c0);
        const float *src = F + c0 * nz;
        const int nin = ncl * nz;
        if (ncl == 32 && (nz & 3) == 0) {  // whole tile: float4 (32*nz floats from a 16-byte boundary)
            const float4 *s4 = reinterpret_cast<const float4 *>(src);
            float4 *d4 = reinterpret_cast<float4 *>(sin);
            for (int i = lane; i < nin / 4; i += 32) d4[i] = __ldcs(s4 + i);
        } else {
            for (int i = lane; i < nin; i += 32) sin[i] = __ldcs(src + i);
        }
        __syncwarp();
        if (lane < ncl) {
            const float *f = sin + lane * nz;
            float *o = sout + lane * nout;
            for (int j = 0; j < nout; j++) {
                float acc = 0.f;
                for (int i = 0; i < nw; i++) acc = fmaf(f[j + i], W.w[nw - 1 - i], acc);
                o[j] = acc * scale;
            }
        }
        __syncwarp();
        float *dst = out + c0 * nout;
        const int nres = ncl * nout;
        if (ncl == 32 && (nout & 3) == 0) {
            const float4 *s4 = reinterpret_cast<const float4 *>(sout);
            float4 *d4 = reinterpret_cast<float4 *>(dst);
            for (int i = lane; i < nres / 4; i += 32) __stcs(d4 + i, s4[i]);
        } else {
            for (int i = lane; i < nres; i += 32) __stcs(dst + i, sout[i]);
        }
        __syncwarp();
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

// ------------------------------------------------ grids of the AFMulator's Hartree route

// The voxel of a periodic grid that holds point pos, and the offsets in it (linearInterpB,
// ppafm/ocl/cl/FF.cl:34-72): lattice coordinate (pos - origin) . T rows, float32.
struct LerpCell {
    long long c[8];  // corners 000, 001, 010, 011, 100, 101, 110, 111 (i, j, k bits)
    float dx, dy, dz;
};

__device__ __forceinline__ LerpCell lerp_cell(int3 n, float3 o, float3 TA, float3 TB, float3 TC, float3 pos) {
    const float3 c = make_float3(pos.x - o.x, pos.y - o.y, pos.z - o.z);
    const float3 g = make_float3(c.x * TA.x + c.y * TA.y + c.z * TA.z, c.x * TB.x + c.y * TB.y + c.z * TB.z,
                                 c.x * TC.x + c.y * TC.y + c.z * TC.z);
    const float fx = floorf(g.x), fy = floorf(g.y), fz = floorf(g.z);
    LerpCell L;
    // fract(): x - floor(x), kept below 1
    L.dx = fminf(g.x - fx, 0x1.fffffep-1f);
    L.dy = fminf(g.y - fy, 0x1.fffffep-1f);
    L.dz = fminf(g.z - fz, 0x1.fffffep-1f);
    // periodic index; the integer remainder only for points outside the home cell
    auto wrap = [](int i, int m) {
        if ((unsigned)i < (unsigned)m) return i;
        const int r = i % m;
        return r >= 0 ? r : r + m;
    };
    const int i0 = wrap((int)fx, n.x), j0 = wrap((int)fy, n.y), k0 = wrap((int)fz, n.z);
    const int i1 = i0 + 1 == n.x ? 0 : i0 + 1, j1 = j0 + 1 == n.y ? 0 : j0 + 1, k1 = k0 + 1 == n.z ? 0 : k0 + 1;
    const long long nyz = (long long)n.y * n.z;
    const long long I[2] = {i0 * nyz, i1 * nyz}, J[2] = {(long long)j0 * n.z, (long long)j1 * n.z};
    const int K[2] = {k0, k1};
#pragma unroll
    for (int b = 0; b < 8; b++) L.c[b] = I[b >> 2] + J[(b >> 1) & 1] + K[b & 1];
    return L;
}

__device__ __forceinline__ float lerp_mix(const LerpCell &L, const float v[8]) {
    const float dx = L.dx, dy = L.dy, dz = L.dz;
    return (1 - dx) * (1 - dy) * (1 - dz) * v[0] + (1 - dx) * (1 - dy) * dz * v[1] + (1 - dx) * dy * (1 - dz) * v[2] +
           (1 - dx) * dy * dz * v[3] + dx * (1 - dy) * (1 - dz) * v[4] + dx * (1 - dy) * dz * v[5] +
           dx * dy * (1 - dz) * v[6] + dx * dy * dz * v[7];
}

// Periodic trilinear interpolation of a scalar grid (linearInterpB).
__device__ __forceinline__ float lin_interp_b(const float *in, int3 n, float3 o, float3 TA, float3 TB, float3 TC,
                                              float3 pos) {
    const LerpCell L = lerp_cell(n, o, TA, TB, TC, pos);
    float v[8];
#pragma unroll
    for (int b = 0; b < 8; b++) v[b] = in[L.c[b]];
    return lerp_mix(L, v);
}

// The same for a float4 grid, component by component (linearInterpB4, FF.cl:74-113).
__device__ __forceinline__ float4 lin_interp_b4(const float4 *in, int3 n, float3 o, float3 TA, float3 TB, float3 TC,
                                                float3 pos) {
    const LerpCell L = lerp_cell(n, o, TA, TB, TC, pos);
    float4 q[8];
#pragma unroll
    for (int b = 0; b < 8; b++) q[b] = in[L.c[b]];
    float vx[8], vy[8], vz[8], vw[8];
#pragma unroll
    for (int b = 0; b < 8; b++) {
        vx[b] = q[b].x;
        vy[b] = q[b].y;
        vz[b] = q[b].z;
        vw[b] = q[b].w;
    }
    return make_float4(lerp_mix(L, vx), lerp_mix(L, vy), lerp_mix(L, vz), lerp_mix(L, vw));
}

struct InterpPrm {
    int3 nin, nout;
    float3 TA, TB, TC, oin;          // input lattice transform rows, input origin
    float3 sA, sB, sC, oout;         // output grid steps and origin
    float3 rA, rB, rC, rc;           // rotation rows and centre
};

// interp_at (ppafm/ocl/cl/FF.cl:1010-1046): output point (i, j, k), C order, rotated about rc.
__global__ void interp_at_kernel(const float *__restrict__ in, float *__restrict__ out, InterpPrm P, long long nout) {
    for (long long ind = blockIdx.x * (long long)blockDim.x + threadIdx.x; ind < nout;
         ind += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(ind / ((long long)P.nout.y * P.nout.z));
        const int j = (int)((ind / P.nout.z) % P.nout.y);
        const int k = (int)(ind % P.nout.z);
        float3 pos = make_float3(P.oout.x + i * P.sA.x + j * P.sB.x + k * P.sC.x, P.oout.y + i * P.sA.y + j * P.sB.y + k * P.sC.y,
                                 P.oout.z + i * P.sA.z + j * P.sB.z + k * P.sC.z);
        const float3 d = make_float3(pos.x - P.rc.x, pos.y - P.rc.y, pos.z - P.rc.z);
        pos = make_float3(P.rc.x + (P.rA.x * d.x + P.rA.y * d.y + P.rA.z * d.z), P.rc.y + (P.rB.x * d.x + P.rB.y * d.y + P.rB.z * d.z),
                          P.rc.z + (P.rC.x * d.x + P.rC.y * d.y + P.rC.z * d.z));
        out[ind] = lin_interp_b(in, P.nin, P.oin, P.TA, P.TB, P.TC, pos);
    }
}

// grad (ppafm/ocl/cl/FF.cl:920-961) in C order: FE = scale * (dE/dx, dE/dy, dE/dz, E) by
// periodic centred differences; accumulate adds to FE.
__global__ void grad_fd_kernel(const float *__restrict__ E, float4 *__restrict__ FE, int3 n, float3 step, float4 scale,
                               int accumulate, long long npts) {
    for (long long ind = blockIdx.x * (long long)blockDim.x + threadIdx.x; ind < npts;
         ind += (long long)gridDim.x * blockDim.x) {
        const long long nyz = (long long)n.y * n.z;
        const int i = (int)(ind / nyz), j = (int)((ind % nyz) / n.z), k = (int)(ind % n.z);
        const long long ip = i > 0 ? ind - nyz : ind + (long long)(n.x - 1) * nyz;
        const long long jp = j > 0 ? ind - n.z : ind + (long long)(n.y - 1) * n.z;
        const long long kp = k > 0 ? ind - 1 : ind + (n.z - 1);
        const long long in_ = i < n.x - 1 ? ind + nyz : ind - (long long)(n.x - 1) * nyz;
        const long long jn = j < n.y - 1 ? ind + n.z : ind - (long long)(n.y - 1) * n.z;
        const long long kn = k < n.z - 1 ? ind + 1 : ind - (n.z - 1);
        float4 f = make_float4(scale.x * (0.5f * (E[in_] - E[ip]) / step.x), scale.y * (0.5f * (E[jn] - E[jp]) / step.y),
                               scale.z * (0.5f * (E[kn] - E[kp]) / step.z), scale.w * E[ind]);
        if (accumulate) {
            const float4 o = FE[ind];
            f = make_float4(f.x + o.x, f.y + o.y, f.z + o.z, f.w + o.w);
        }
        FE[ind] = f;
    }
}

// gradPotentialGrid (ppafm/ocl/cl/FF.cl:964-1008): the electric field -grad V on a target
// grid by centred differences (step h) of the potential interpolated at the six neighbours;
// w = V at the point.  C order over the target grid.
struct GradPotPrm {
    int3 nin, nout;
    float3 TA, TB, TC, oin;   // potential lattice transform rows and origin
    float3 sA, sB, sC, oout;  // target grid steps and origin
    float3 h;
};

__global__ void grad_pot_grid_kernel(const float *__restrict__ pot, float4 *__restrict__ field, GradPotPrm P,
                                     long long nout) {
    for (long long ind = blockIdx.x * (long long)blockDim.x + threadIdx.x; ind < nout;
         ind += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(ind / ((long long)P.nout.y * P.nout.z));
        const int j = (int)((ind / P.nout.z) % P.nout.y);
        const int k = (int)(ind % P.nout.z);
        const float3 p = make_float3(P.oout.x + i * P.sA.x + j * P.sB.x + k * P.sC.x, P.oout.y + i * P.sA.y + j * P.sB.y + k * P.sC.y,
                                     P.oout.z + i * P.sA.z + j * P.sB.z + k * P.sC.z);
        auto V = [&](float ax, float ay, float az) {
            return lin_interp_b(pot, P.nin, P.oin, P.TA, P.TB, P.TC, make_float3(p.x + ax, p.y + ay, p.z + az));
        };
        const float v0 = V(0.f, 0.f, 0.f);
        const float vip = V(-P.h.x, 0.f, 0.f), vjp = V(0.f, -P.h.y, 0.f), vkp = V(0.f, 0.f, -P.h.z);
        const float vin = V(P.h.x, 0.f, 0.f), vjn = V(0.f, P.h.y, 0.f), vkn = V(0.f, 0.f, P.h.z);
        field[ind] = make_float4(0.5f * (vip - vin) / P.h.x, 0.5f * (vjp - vjn) / P.h.y, 0.5f * (vkp - vkn) / P.h.z, v0);
    }
}

// The tip charges' part of evalLJC_Hartree (ppafm/ocl/cl/FF.cl:860-915): at every grid point,
// FE += sum_q Q_q * field(point + (0, 0, QZ_q)), the field (float4, C order, on the same
// grid) interpolated periodically.  Charges of zero add nothing and are skipped.
struct TipQPrm {
    int3 n;
    float3 TA, TB, TC, o;  // grid lattice transform rows and origin
    float3 sA, sB, sC;     // grid steps
    float Q[4], QZ[4];
};

__global__ void tip_charges_kernel(const float4 *__restrict__ field, float4 *__restrict__ FE, TipQPrm P, int accumulate,
                                   long long npts) {
    for (long long ind = blockIdx.x * (long long)blockDim.x + threadIdx.x; ind < npts;
         ind += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(ind / ((long long)P.n.y * P.n.z));
        const int j = (int)((ind / P.n.z) % P.n.y);
        const int k = (int)(ind % P.n.z);
        const float3 p = make_float3(P.o.x + P.sA.x * i + P.sB.x * j + P.sC.x * k, P.o.y + P.sA.y * i + P.sB.y * j + P.sC.y * k,
                                     P.o.z + P.sA.z * i + P.sB.z * j + P.sC.z * k);
        float4 fe = accumulate ? FE[ind] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int q = 0; q < 4; q++) {
            if (P.Q[q] == 0.f) continue;
            const float4 e = lin_interp_b4(field, P.n, P.o, P.TA, P.TB, P.TC, make_float3(p.x, p.y, p.z + P.QZ[q]));
            fe = make_float4(fe.x + P.Q[q] * e.x, fe.y + P.Q[q] * e.y, fe.z + P.Q[q] * e.z, fe.w + P.Q[q] * e.w);
        }
        FE[ind] = fe;
    }
}

// interp_tip_at (ppafm/ocl/cl/FF.cl:1049-1093): a tip density centred on the grid origin
// resampled onto another grid.  Output indices past the middle wrap to negative positions,
// points beyond half of the input cell along any lattice vector are zero (the input's
// fractional coordinate f = pos . Linv rows, Linv = inverse of the input cell, as the
// reference forms it), the rest interpolated periodically about origin 0.
struct TipInterpPrm {
    int3 nin, nout;
    float3 TA, TB, TC;  // input lattice transform rows
    float3 LA, LB, LC;  // rows of the inverse input cell
    float3 sA, sB, sC;  // output grid steps
};

__global__ void interp_tip_kernel(const float *__restrict__ in, float *__restrict__ out, TipInterpPrm P, long long nout) {
    for (long long ind = blockIdx.x * (long long)blockDim.x + threadIdx.x; ind < nout;
         ind += (long long)gridDim.x * blockDim.x) {
        int i = (int)(ind / ((long long)P.nout.y * P.nout.z));
        int j = (int)((ind / P.nout.z) % P.nout.y);
        int k = (int)(ind % P.nout.z);
        if (i > P.nout.x / 2) i -= P.nout.x;
        if (j > P.nout.y / 2) j -= P.nout.y;
        if (k > P.nout.z / 2) k -= P.nout.z;
        const float3 pos = make_float3(i * P.sA.x + j * P.sB.x + k * P.sC.x, i * P.sA.y + j * P.sB.y + k * P.sC.y,
                                       i * P.sA.z + j * P.sB.z + k * P.sC.z);
        const float fa = P.LA.x * pos.x + P.LA.y * pos.y + P.LA.z * pos.z;
        const float fb = P.LB.x * pos.x + P.LB.y * pos.y + P.LB.z * pos.z;
        const float fc = P.LC.x * pos.x + P.LC.y * pos.y + P.LC.z * pos.z;
        if (fabsf(fa) > 0.5f || fabsf(fb) > 0.5f || fabsf(fc) > 0.5f)
            out[ind] = 0.f;
        else
            out[ind] = lin_interp_b(in, P.nin, make_float3(0.f, 0.f, 0.f), P.TA, P.TB, P.TC, pos);
    }
}

// Elementwise scalar-grid operations of DataGrid (ppafm/ocl/field.py:288-452; kernels
// clamp_hard, clamp_soft, addMult, power, normalizeSumReduce of FF.cl:1095-1223).
__global__ void scalar_clamp_kernel(const float *__restrict__ in, float *__restrict__ out, long long n, float lo, float hi,
                                    int soft, float width) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float v = in[i];
        if (!soft) {
            v = fmaxf(lo, fminf(hi, v));
        } else {
            // sigmoid blend towards the bound over the width (clamp_soft)
            if (hi < INFINITY) v = (v - hi) / (1.f + expf((v - hi) / width)) + hi;
            if (lo > -INFINITY) v = (v - lo) / (1.f + expf((v - lo) / -width)) + lo;
        }
        out[i] = v;
    }
}

__global__ void scalar_add_mult_kernel(const float *__restrict__ a, const float *__restrict__ b, float *__restrict__ out,
                                       long long n, float s) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = a[i] + s * b[i];
}

// (sum of all values, sum of the positive ones) in float64: block partials, then one atomic
// add per block.
__global__ void scalar_sums_kernel(const float *__restrict__ in, long long n, double *sums) {
    double t = 0.0, p = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float v = in[i];
        t += v;
        if (v > 0.f) p += v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        t += __shfl_xor_sync(0xffffffffu, t, o);
        p += __shfl_xor_sync(0xffffffffu, p, o);
    }
    __shared__ double st[GRID_THREADS / 32], sp[GRID_THREADS / 32];
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        st[w] = t;
        sp[w] = p;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double T = 0.0, Pp = 0.0;
        for (int k = 0; k < GRID_THREADS / 32; k++) {
            T += st[k];
            Pp += sp[k];
        }
        atomicAdd(sums, T);
        atomicAdd(sums + 1, Pp);
    }
}

__global__ void scalar_power_kernel(const float *__restrict__ in, float *__restrict__ out, long long n, float p, float scale) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = scale * powf(fmaxf(0.f, in[i]), p);
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
    const bool aligned = (((uintptr_t)F | (uintptr_t)out) & 15u) == 0;
    if (nz <= FZ2DF_TILE_NZ && aligned) {
        const int nout = nz - nw + 1;
        const size_t smem = (size_t)FZ2DF_WARPS * 32 * (nz + nout) * sizeof(float);
        int dev = 0, sms = 152;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const long long ntile = (ncol + 31) / 32;
        const long long want = (ntile + FZ2DF_WARPS - 1) / FZ2DF_WARPS;
        const unsigned nblk = (unsigned)std::max(1LL, std::min(want, (long long)sms * 8));
        PPGPU_CUDA(cudaFuncSetAttribute(fz2df_tiled_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        FZ2DF_WARPS * 32 * 2 * FZ2DF_TILE_NZ * (int)sizeof(float)),
                   "fz2df shared memory");
        fz2df_tiled_kernel<<<nblk, 32 * FZ2DF_WARPS, smem, (cudaStream_t)stream>>>(F, ncol, nz, nw, w, (float)scale, out);
        PPGPU_CHECK_LAUNCH("fz2df_tiled_kernel");
        return set_ok();
    }
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

static float3 f3(const double *v) { return make_float3((float)v[0], (float)v[1], (float)v[2]); }

// T = inv(step)^T as rows (lattice coordinate = coordinate . T rows); false when singular.
static bool lattice_transform(const double *m, double T[9]) {
    const double A = m[4] * m[8] - m[5] * m[7], B = -(m[3] * m[8] - m[5] * m[6]), C = m[3] * m[7] - m[4] * m[6];
    const double det = m[0] * A + m[1] * B + m[2] * C;
    if (!(det != 0.0)) return false;
    const double inv[9] = {A / det, -(m[1] * m[8] - m[2] * m[7]) / det, (m[1] * m[5] - m[2] * m[4]) / det,
                           B / det, (m[0] * m[8] - m[2] * m[6]) / det, -(m[0] * m[5] - m[2] * m[3]) / det,
                           C / det, -(m[0] * m[7] - m[1] * m[6]) / det, (m[0] * m[4] - m[1] * m[3]) / det};
    const double Tt[9] = {inv[0], inv[3], inv[6], inv[1], inv[4], inv[7], inv[2], inv[5], inv[8]};
    memcpy(T, Tt, sizeof(Tt));
    return true;
}

/* interp_at (ppafm/ocl/cl/FF.cl:1010-1046, DataGrid.interp_at, ppafm/ocl/field.py:515-572):
 * out[nout0][nout1][nout2] = periodic trilinear interpolation of in[nin0][nin1][nin2] (lattice
 * origin origin_in, steps step_in rows) at origin_out + i a + j b + k c (step_out rows), rotated
 * about rot_center by rot (rows).  float32 arithmetic like the reference. */
extern "C" int ppgpu_interp_grid(const float *in, const int *nin, const double *origin_in, const double *step_in,
                                 float *out, const int *nout, const double *origin_out, const double *step_out,
                                 const double *rot, const double *rot_center, void *stream) {
    if (!in || !nin || !origin_in || !step_in || !out || !nout || !origin_out || !step_out)
        return set_error(PPGPU_ERR_ARG, "interp_grid: null argument");
    for (int k = 0; k < 3; k++)
        if (nin[k] <= 0 || nout[k] <= 0) return set_error(PPGPU_ERR_ARG, "interp_grid: sizes must be positive");
    double T[9];
    if (!lattice_transform(step_in, T)) return set_error(PPGPU_ERR_ARG, "interp_grid: singular input cell");
    const double I[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1}, Z[3] = {0, 0, 0};
    const double *R = rot ? rot : I, *rc = rot_center ? rot_center : Z;
    InterpPrm P;
    P.nin = make_int3(nin[0], nin[1], nin[2]);
    P.nout = make_int3(nout[0], nout[1], nout[2]);
    P.TA = f3(T);
    P.TB = f3(T + 3);
    P.TC = f3(T + 6);
    P.oin = f3(origin_in);
    P.sA = f3(step_out);
    P.sB = f3(step_out + 3);
    P.sC = f3(step_out + 6);
    P.oout = f3(origin_out);
    P.rA = f3(R);
    P.rB = f3(R + 3);
    P.rC = f3(R + 6);
    P.rc = f3(rc);
    const long long n = (long long)nout[0] * nout[1] * nout[2];
    interp_at_kernel<<<stream_blocks(n), GRID_THREADS, 0, (cudaStream_t)stream>>>(in, out, P, n);
    PPGPU_CHECK_LAUNCH("interp_at_kernel");
    return set_ok();
}

/* grad (ppafm/ocl/cl/FF.cl:920-961, DataGrid.grad, ppafm/ocl/field.py:454-513) in C order:
 * FE[n0][n1][n2] float4 = scale[0..3] * (dE/dx, dE/dy, dE/dz, E), periodic centred differences
 * with the grid steps step[3]; accumulate adds to FE. */
extern "C" int ppgpu_grad_fd(const float *E, const int *n, const double *step, const double *scale, float *FE,
                             int accumulate, void *stream) {
    if (!E || !n || !step || !scale || !FE) return set_error(PPGPU_ERR_ARG, "grad_fd: null argument");
    for (int k = 0; k < 3; k++)
        if (n[k] <= 0) return set_error(PPGPU_ERR_ARG, "grad_fd: sizes must be positive");
    const long long npts = (long long)n[0] * n[1] * n[2];
    grad_fd_kernel<<<stream_blocks(npts), GRID_THREADS, 0, (cudaStream_t)stream>>>(
        E, reinterpret_cast<float4 *>(FE), make_int3(n[0], n[1], n[2]), f3(step),
        make_float4((float)scale[0], (float)scale[1], (float)scale[2], (float)scale[3]), accumulate, npts);
    PPGPU_CHECK_LAUNCH("grad_fd_kernel");
    return set_ok();
}

/* gradPotentialGrid (ppafm/ocl/cl/FF.cl:964-1008, ppafm/ocl/field.py:1225-1317): field
 * [nout0][nout1][nout2] float4 = (-dV/dx, -dV/dy, -dV/dz, V) at origin_out + i a + j b + k c
 * (step_out rows), centred differences with steps h[3] of the periodic trilinear interpolation
 * of pot[nin0][nin1][nin2] (origin origin_in, steps step_in rows).  float32 like the kernel. */
extern "C" int ppgpu_grad_potential_grid(const float *pot, const int *nin, const double *origin_in, const double *step_in,
                                         float *field, const int *nout, const double *origin_out,
                                         const double *step_out, const double *h, void *stream) {
    if (!pot || !nin || !origin_in || !step_in || !field || !nout || !origin_out || !step_out || !h)
        return set_error(PPGPU_ERR_ARG, "grad_potential_grid: null argument");
    for (int k = 0; k < 3; k++) {
        if (nin[k] <= 0 || nout[k] <= 0) return set_error(PPGPU_ERR_ARG, "grad_potential_grid: sizes must be positive");
        if (!(h[k] > 0.0)) return set_error(PPGPU_ERR_ARG, "grad_potential_grid: steps h must be positive");
    }
    double T[9];
    if (!lattice_transform(step_in, T)) return set_error(PPGPU_ERR_ARG, "grad_potential_grid: singular potential cell");
    GradPotPrm P;
    P.nin = make_int3(nin[0], nin[1], nin[2]);
    P.nout = make_int3(nout[0], nout[1], nout[2]);
    P.TA = f3(T);
    P.TB = f3(T + 3);
    P.TC = f3(T + 6);
    P.oin = f3(origin_in);
    P.sA = f3(step_out);
    P.sB = f3(step_out + 3);
    P.sC = f3(step_out + 6);
    P.oout = f3(origin_out);
    P.h = f3(h);
    const long long n = (long long)nout[0] * nout[1] * nout[2];
    grad_pot_grid_kernel<<<stream_blocks(n), GRID_THREADS, 0, (cudaStream_t)stream>>>(pot, reinterpret_cast<float4 *>(field), P, n);
    PPGPU_CHECK_LAUNCH("grad_pot_grid_kernel");
    return set_ok();
}

/* The tip charges of evalLJC_Hartree (ppafm/ocl/cl/FF.cl:860-915, ppafm/ocl/field.py:1168-1223):
 * FE[n0][n1][n2] float4 (+)= sum_q Qs[q] * field(p + (0, 0, QZs[q])) at every grid point
 * p = origin + i a + j b + k c (step rows), field [n0][n1][n2] float4 on the same grid,
 * interpolated periodically.  accumulate adds to FE (which then holds the Lennard-Jones part,
 * the reference's order of summation). */
extern "C" int ppgpu_tip_charges_field(const float *field, const int *n, const double *origin, const double *step,
                                       const double *Qs, const double *QZs, float *FE, int accumulate, void *stream) {
    if (!field || !n || !origin || !step || !Qs || !QZs || !FE) return set_error(PPGPU_ERR_ARG, "tip_charges_field: null argument");
    for (int k = 0; k < 3; k++)
        if (n[k] <= 0) return set_error(PPGPU_ERR_ARG, "tip_charges_field: sizes must be positive");
    if (field == FE) return set_error(PPGPU_ERR_ARG, "tip_charges_field: field and FE must be different buffers");
    double T[9];
    if (!lattice_transform(step, T)) return set_error(PPGPU_ERR_ARG, "tip_charges_field: singular cell");
    TipQPrm P;
    P.n = make_int3(n[0], n[1], n[2]);
    P.TA = f3(T);
    P.TB = f3(T + 3);
    P.TC = f3(T + 6);
    P.o = f3(origin);
    P.sA = f3(step);
    P.sB = f3(step + 3);
    P.sC = f3(step + 6);
    for (int q = 0; q < 4; q++) {
        P.Q[q] = (float)Qs[q];
        P.QZ[q] = (float)QZs[q];
    }
    const long long npts = (long long)n[0] * n[1] * n[2];
    tip_charges_kernel<<<stream_blocks(npts), GRID_THREADS, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const float4 *>(field), reinterpret_cast<float4 *>(FE), P, accumulate, npts);
    PPGPU_CHECK_LAUNCH("tip_charges_kernel");
    return set_ok();
}

/* TipDensity.interp_at (ppafm/ocl/field.py:606-650, kernel interp_tip_at, FF.cl:1049-1093):
 * the tip density in[nin0][nin1][nin2] (grid steps step_in rows, cell cell_in rows), centred
 * on the origin, resampled onto out[nout0][nout1][nout2] with steps step_out rows; output
 * indices past the middle are negative positions, points beyond half of the input cell are 0. */
extern "C" int ppgpu_interp_tip_grid(const float *in, const int *nin, const double *step_in, const double *cell_in,
                                     float *out, const int *nout, const double *step_out, void *stream) {
    if (!in || !nin || !step_in || !cell_in || !out || !nout || !step_out)
        return set_error(PPGPU_ERR_ARG, "interp_tip_grid: null argument");
    for (int k = 0; k < 3; k++)
        if (nin[k] <= 0 || nout[k] <= 0) return set_error(PPGPU_ERR_ARG, "interp_tip_grid: sizes must be positive");
    double T[9], LT[9];
    if (!lattice_transform(step_in, T) || !lattice_transform(cell_in, LT))
        return set_error(PPGPU_ERR_ARG, "interp_tip_grid: singular input cell");
    // lattice_transform gives inv(m)^T as rows; the reference takes the rows of inv(cell)
    const double L[9] = {LT[0], LT[3], LT[6], LT[1], LT[4], LT[7], LT[2], LT[5], LT[8]};
    TipInterpPrm P;
    P.nin = make_int3(nin[0], nin[1], nin[2]);
    P.nout = make_int3(nout[0], nout[1], nout[2]);
    P.TA = f3(T);
    P.TB = f3(T + 3);
    P.TC = f3(T + 6);
    P.LA = f3(L);
    P.LB = f3(L + 3);
    P.LC = f3(L + 6);
    P.sA = f3(step_out);
    P.sB = f3(step_out + 3);
    P.sC = f3(step_out + 6);
    const long long n = (long long)nout[0] * nout[1] * nout[2];
    interp_tip_kernel<<<stream_blocks(n), GRID_THREADS, 0, (cudaStream_t)stream>>>(in, out, P, n);
    PPGPU_CHECK_LAUNCH("interp_tip_kernel");
    return set_ok();
}

/* DataGrid.clamp (ppafm/ocl/field.py:288-340; clamp_hard, clamp_soft, FF.cl:1179-1210):
 * out[i] = in[i] clipped to [minimum, maximum] (soft = 0), or blended into the bounds by a
 * sigmoid of the given width (soft = 1).  in == out is allowed. */
extern "C" int ppgpu_scalar_clamp(const float *in, float *out, long long n, double minimum, double maximum, int soft,
                                  double width, void *stream) {
    if (!in || !out) return set_error(PPGPU_ERR_ARG, "scalar_clamp: null argument");
    if (n <= 0) return set_ok();
    scalar_clamp_kernel<<<stream_blocks(n), GRID_THREADS, 0, (cudaStream_t)stream>>>(in, out, n, (float)minimum, (float)maximum,
                                                                                     soft, (float)width);
    PPGPU_CHECK_LAUNCH("scalar_clamp_kernel");
    return set_ok();
}

/* DataGrid.add_mult (ppafm/ocl/field.py:342-376; addMult, FF.cl:1213-1223): out = a + scale*b. */
extern "C" int ppgpu_scalar_add_mult(const float *a, const float *b, float *out, long long n, double scale, void *stream) {
    if (!a || !b || !out) return set_error(PPGPU_ERR_ARG, "scalar_add_mult: null argument");
    if (n <= 0) return set_ok();
    scalar_add_mult_kernel<<<stream_blocks(n), GRID_THREADS, 0, (cudaStream_t)stream>>>(a, b, out, n, (float)scale);
    PPGPU_CHECK_LAUNCH("scalar_add_mult_kernel");
    return set_ok();
}

/* The normalisation sums of DataGrid.power_positive (ppafm/ocl/field.py:431-452;
 * normalizeSumReduce, FF.cl:1108-1150): sums[0] = sum of all values, sums[1] = sum of the
 * positive ones, float64, into the device array sums[2] (cleared here). */
extern "C" int ppgpu_scalar_sums(const float *in, long long n, double *sums, void *stream) {
    if (!in || !sums) return set_error(PPGPU_ERR_ARG, "scalar_sums: null argument");
    PPGPU_CUDA(cudaMemsetAsync(sums, 0, 2 * sizeof(double), (cudaStream_t)stream), "clear sums");
    if (n <= 0) return set_ok();
    scalar_sums_kernel<<<stream_blocks(n), GRID_THREADS, 0, (cudaStream_t)stream>>>(in, n, sums);
    PPGPU_CHECK_LAUNCH("scalar_sums_kernel");
    return set_ok();
}

/* DataGrid.power_positive's power (ppafm/ocl/field.py:378-429; power, FF.cl:1095-1106):
 * out[i] = scale * max(0, in[i])^p.  in == out is allowed. */
extern "C" int ppgpu_scalar_power(const float *in, float *out, long long n, double p, double scale, void *stream) {
    if (!in || !out) return set_error(PPGPU_ERR_ARG, "scalar_power: null argument");
    if (n <= 0) return set_ok();
    scalar_power_kernel<<<stream_blocks(n), GRID_THREADS, 0, (cudaStream_t)stream>>>(in, out, n, (float)p, (float)scale);
    PPGPU_CHECK_LAUNCH("scalar_power_kernel");
    return set_ok();
}
