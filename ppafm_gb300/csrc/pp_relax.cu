// pp_relax.cu -- probe-particle relaxation on sm_103a.
//
// CPU-core semantics (ppafm/cpp/ProbeParticle.cpp):
//   relaxTipStrokes_omp 682-701, relaxTipStroke 633-676, relaxProbe 297-313,
//   getPPforce 282-294, FIREstate::move 142-174, RELAX::move 84-88,
//   interpolate3DvecWrap + SET_GRID_IND (ppafm/cpp/Grid.h:66-69, 93-111),
//   forceRSpring (ppafm/cpp/Forces.h:85-89);
//   Fz2df (ppafm/common.py:421-430) fused as a per-pixel epilogue.
// AFMulator semantics (ppafm/ocl/cl/relax.cl):
//   relaxStrokesTilted 391-464, update_FIRE 105-126, tipForce 37-41, convolveZ 571-608.
//
// Design (GB300):
//  * One lane per stroke (pixel column).  A lane's whole z-walk is a single flattened
//    loop in which every trip does exactly one trilinear gather (8 x 16-byte __ldg of
//    the interleaved float4 grid), so lanes that converge early at one height move on
//    to their next height instead of idling; the warp leaves the loop on a
//    __any_sync vote once all of its lanes have finished their strokes.
//  * Precision, chosen by measurement against the float64 reference on a GB300, whose
//    float64 rate is 1/64 of its float32 rate: the probe displacement d = r - r_tip, the grid
//    coordinate, the trilinear weights and interpolation sum, the springs and the force sum
//    are double-float (pp_df.cuh: two floats, ~48 significant bits); the FIRE state
//    (velocity, dt, mixing coefficient) and the residual force it consumes are float32.
//    Rounding noise in the interpolated force of ~3e-8 relative (plain float32) moves the
//    stopping point of a few pixel heights in 1e5 by more than 1e-3 A inside the
//    |F| < 1e-4 eV/A ball (the soft lateral spring leaves it ~6e-3 A wide); 1e-9 relative
//    noise moves none, and neither does a float32 FIRE state.  The only difference from the
//    reference left is the float32 storage of the grid values.  Float64 is used once per
//    height (tip grid coordinate), not per iteration.
//  * Trilinear weights are explicit (no texture filtering).
#include <cmath>
#include <cstring>

#include "pp_common.cuh"
#include "pp_df.cuh"

namespace ppgpu {

constexpr int RELAX_THREADS = 64;  // small blocks spread the strokes evenly over the SMs
constexpr int MAX_DF_TAPS = 64;
constexpr unsigned FULL = 0xffffffffu;

struct RelaxPrm {
    const float4 *FE;
    int n0, n1, n2;
    double dicd[9];  // grid coordinate rows: g_k = r . dicd[3k..3k+2]
    int maxIters;
    double convF2, dtmax, acoef0, finc, fdec, falpha;
    double lRad, kRad;
    double rPP0[3], kSpring[3];
    int relaxAlg, probeStart;
    unsigned long long *iter_total;
    int *err;
    // per-iteration constants
    dfl dic[9];  // dicd as double-floats
    int diag;    // dicd is diagonal
    dfl kRadf, nl0;        // kRad, -lRad
    dfl nr0[3], kSf[3];    // -rPP0, kSpring
    dfl r0[3];             // rPP0
    float convF2f, dtmaxf, acoef0f, fincf, fdecf, falphaf;
};

struct StrokeIO {  // relaxTipStrokes semantics (float64 in/out)
    int nstroke, nstep;
    const double *rTips;
    double *rs, *fs;
    int *iters, *itrsum;
};

struct ScanIO {  // regular scan semantics
    int nx, ny, nz;
    const double *xs, *ys, *zs;
    double off[3];
    dfl offd[3];
    float *fzs, *ppos, *df;
    int *iters;
    int nw;
    float W[MAX_DF_TAPS];
};

// ----------------------------------------------------------- interpolation

// Periodic trilinear interpolation of the force (Grid.h:93-111) at the grid coordinate
// base + u (base integer, u double-float): float32 grid values, double-float weights and
// compensated sums, so the only rounding left is that of the stored grid values.
__device__ __forceinline__ void interp_force_df(const float4 *__restrict__ FE, int n0, int n1, int n2,
                                                const int base[3], const dfl u[3], dfl F[3]) {
    int ci[3];
    dfl t[3], m[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        t[k] = split_cell(u[k], ci[k]);
        ci[k] += base[k];
        const dfl o = two_sum(1.f, -t[k].h);
        m[k] = {o.h, __fsub_rn(o.l, t[k].l)};
    }
    const int ix0 = wrap_index(ci[0], n0), iy0 = wrap_index(ci[1], n1), iz0 = wrap_index(ci[2], n2);
    const int ix1 = (ix0 + 1 == n0) ? 0 : ix0 + 1;
    const int iy1 = (iy0 + 1 == n1) ? 0 : iy0 + 1;
    const int iz1 = (iz0 + 1 == n2) ? 0 : iz0 + 1;
    const long long r00 = ((long long)ix0 * n1 + iy0) * n2, r01 = ((long long)ix0 * n1 + iy1) * n2;
    const long long r10 = ((long long)ix1 * n1 + iy0) * n2, r11 = ((long long)ix1 * n1 + iy1) * n2;
    // corner order (x, y, z bits): 000 001 010 011 100 101 110 111
    const float4 c[8] = {ldg4(FE + r00 + iz0), ldg4(FE + r00 + iz1), ldg4(FE + r01 + iz0), ldg4(FE + r01 + iz1),
                         ldg4(FE + r10 + iz0), ldg4(FE + r10 + iz1), ldg4(FE + r11 + iz0), ldg4(FE + r11 + iz1)};
    const dfl wxy[4] = {df_mul(m[0], m[1]), df_mul(m[0], t[1]), df_mul(t[0], m[1]), df_mul(t[0], t[1])};
    dfl w[8];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        w[2 * k] = df_mul(wxy[k], m[2]);
        w[2 * k + 1] = df_mul(wxy[k], t[2]);
    }
#pragma unroll
    for (int comp = 0; comp < 3; comp++) {
        dfl p[8];
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const float v = comp == 0 ? c[k].x : (comp == 1 ? c[k].y : c[k].z);
            p[k] = two_prod(w[k].h, v);
            p[k].l = __fmaf_rn(w[k].l, v, p[k].l);
        }
        const dfl a0 = df_add_raw(p[0], p[1]), a1 = df_add_raw(p[2], p[3]);
        const dfl a2 = df_add_raw(p[4], p[5]), a3 = df_add_raw(p[6], p[7]);
        const dfl r = df_add_raw(df_add_raw(a0, a1), df_add_raw(a2, a3));
        F[comp] = two_sum(r.h, r.l);
    }
}

// Same, all four channels, at a float grid coordinate (AFMulator path).
__device__ __forceinline__ float4 interp_fe4(const float4 *__restrict__ FE, int n0, int n1, int n2, float3 g) {
    const float fx = floorf(g.x), fy = floorf(g.y), fz = floorf(g.z);
    const float tx = g.x - fx, ty = g.y - fy, tz = g.z - fz;
    const float mx = 1.f - tx, my = 1.f - ty, mz = 1.f - tz;
    const int ix0 = wrap_index((int)fx, n0), iy0 = wrap_index((int)fy, n1), iz0 = wrap_index((int)fz, n2);
    const int ix1 = (ix0 + 1 == n0) ? 0 : ix0 + 1;
    const int iy1 = (iy0 + 1 == n1) ? 0 : iy0 + 1;
    const int iz1 = (iz0 + 1 == n2) ? 0 : iz0 + 1;
    const long long r00 = ((long long)ix0 * n1 + iy0) * n2, r01 = ((long long)ix0 * n1 + iy1) * n2;
    const long long r10 = ((long long)ix1 * n1 + iy0) * n2, r11 = ((long long)ix1 * n1 + iy1) * n2;
    const float4 c000 = ldg4(FE + r00 + iz0), c001 = ldg4(FE + r00 + iz1);
    const float4 c010 = ldg4(FE + r01 + iz0), c011 = ldg4(FE + r01 + iz1);
    const float4 c100 = ldg4(FE + r10 + iz0), c101 = ldg4(FE + r10 + iz1);
    const float4 c110 = ldg4(FE + r11 + iz0), c111 = ldg4(FE + r11 + iz1);
    float4 o;
#define PP_LERP3(c)                                                                                \
    {                                                                                              \
        const float v00 = fmaf(c100.c, tx, c000.c * mx), v10 = fmaf(c110.c, tx, c010.c * mx);     \
        const float v01 = fmaf(c101.c, tx, c001.c * mx), v11 = fmaf(c111.c, tx, c011.c * mx);     \
        const float v0 = fmaf(v10, ty, v00 * my), v1 = fmaf(v11, ty, v01 * my);                   \
        o.c = fmaf(v1, tz, v0 * mz);                                                               \
    }
    PP_LERP3(x) PP_LERP3(y) PP_LERP3(z) PP_LERP3(w)
#undef PP_LERP3
    return o;
}

// Grid coordinate g_k = r . dicell_row_k of a float64 position (Grid.h:46-50).
__device__ __forceinline__ double3 to_grid(const RelaxPrm &P, double x, double y, double z) {
    return make_double3(fma(z, P.dicd[2], fma(y, P.dicd[1], x * P.dicd[0])),
                        fma(z, P.dicd[5], fma(y, P.dicd[4], x * P.dicd[3])),
                        fma(z, P.dicd[8], fma(y, P.dicd[7], x * P.dicd[6])));
}

// Grid coordinate of the displacement d relative to tf (double-float): u_k = tf_k + dic_k . d.
__device__ __forceinline__ void grid_coord_df(const RelaxPrm &P, const dfl tf[3], const dfl d[3], dfl u[3]) {
    if (P.diag) {
#pragma unroll
        for (int k = 0; k < 3; k++) u[k] = df_add(tf[k], df_mul(P.dic[4 * k], d[k]));
    } else {
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const dfl a = df_add_raw(df_mul(P.dic[3 * k], d[0]), df_mul(P.dic[3 * k + 1], d[1]));
            u[k] = df_add(tf[k], df_add(a, df_mul(P.dic[3 * k + 2], d[2])));
        }
    }
}

// Probe-particle force = grid force + radial spring + lateral spring (getPPforce,
// ProbeParticle.cpp:282-294; forceRSpring, Forces.h:85-89) in double-float, returned as the
// float32 residual: the radial spring is stiff, so l - l0 is a small difference of ~4 A
// lengths, and the force is a small difference of the grid force and the springs.
__device__ __forceinline__ float3 pp_force_df(const RelaxPrm &P, const dfl F[3], const dfl d[3]) {
    const dfl l2 = df_add(df_add(df_sq(d[0]), df_sq(d[1])), df_sq(d[2]));
    // l = sqrt(l2) and 1/l: approximate float32 root, then one correction from the exact
    // residual l2 - L^2 (error ~ the square of the approximation's)
    const float rs = rsqrt_approx(l2.h);
    const float L = __fmul_rn(l2.h, rs);
    const dfl LL = two_prod(L, L);
    const float res = __fadd_rn(__fsub_rn(__fsub_rn(l2.h, LL.h), LL.l), l2.l);
    const dfl l = fast_two_sum(L, __fmul_rn(res, __fmul_rn(0.5f, rs)));
    const dfl x = df_add(l, P.nl0);  // l - l0
    // q = (l - l0) / l: approximate quotient plus the correction from its exact remainder
    const float qh = __fmul_rn(x.h, rs);
    const dfl ql = two_prod(qh, l.h);
    const float rem = __fsub_rn(__fadd_rn(__fsub_rn(__fsub_rn(x.h, ql.h), ql.l), x.l), __fmul_rn(qh, l.l));
    const dfl s = df_mul(P.kRadf, two_sum(qh, __fmul_rn(rem, rs)));
    // f = F + d s + (d - r0) kS: the three high parts summed error-free, every low part and
    // product error added once at the end (the result is rounded to float32)
    float f[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const dfl b = two_prod(d[k].h, s.h);
        const float bl = __fmaf_rn(d[k].l, s.h, __fmaf_rn(d[k].h, s.l, b.l));
        const dfl r = two_sum(d[k].h, P.nr0[k].h);  // d - r0
        const float rl = __fadd_rn(r.l, __fadd_rn(d[k].l, P.nr0[k].l));
        const dfl c = two_prod(r.h, P.kSf[k].h);
        const float cl = __fmaf_rn(rl, P.kSf[k].h, __fmaf_rn(r.h, P.kSf[k].l, c.l));
        const dfl s1 = two_sum(F[k].h, b.h);
        const dfl s2 = two_sum(s1.h, c.h);
        f[k] = __fadd_rn(s2.h, __fadd_rn(__fadd_rn(s1.l, s2.l), __fadd_rn(F[k].l, __fadd_rn(bl, cl))));
    }
    return make_float3(f[0], f[1], f[2]);
}

// One FIRE move (FIREstate::move, ProbeParticle.cpp:153-172; relaxAlg 1) or damped
// leap-frog (RELAX::move, ProbeParticle.cpp:84-88; relaxAlg 0): float32 velocity, dt and
// mixing coefficient; the displacement d += v dt is accumulated in double-float.
// Returns |f|^2.
__device__ __forceinline__ float relax_move_df(const RelaxPrm &P, float3 f, dfl d[3], float3 &v, float &dt,
                                               float &acoef) {
    const float ff = f.x * f.x + f.y * f.y + f.z * f.z;
    float h;
    if (P.relaxAlg == 1) {
        const float vv = v.x * v.x + v.y * v.y + v.z * v.z;
        const float vf = f.x * v.x + f.y * v.y + f.z * v.z;
        if (vf < 0.f) {
            v = make_float3(0.f, 0.f, 0.f);
            dt = dt * P.fdecf;
            acoef = P.acoef0f;
        } else {
            // cf f has length acoef |v|; vv ff below 1e-30 gives cf = 0 instead of an
            // overflow (the reference divides by zero at ff == 0, and cf = 0 at vv == 0)
            const float vf2 = vv * ff;  // sqrt(vv/ff) = vv / sqrt(vv ff)
            const float cf = (vf2 > 1e-30f) ? acoef * vv * rsqrt_approx(vf2) : 0.f;
            const float cv = 1.f - acoef;
            v.x = fmaf(f.x, cf, v.x * cv);
            v.y = fmaf(f.y, cf, v.y * cv);
            v.z = fmaf(f.z, cf, v.z * cv);
            dt = fminf(dt * P.fincf, P.dtmaxf);
            acoef = acoef * P.falphaf;
        }
        h = dt;
    } else {
        const float c = 1.f - P.acoef0f;
        v.x *= c;
        v.y *= c;
        v.z *= c;
        h = P.dtmaxf;
    }
    v.x = fmaf(f.x, h, v.x);
    v.y = fmaf(f.y, h, v.y);
    v.z = fmaf(f.z, h, v.z);
    d[0] = df_add_f(d[0], v.x * h);
    d[1] = df_add_f(d[1], v.y * h);
    d[2] = df_add_f(d[2], v.z * h);
    return ff;
}

__device__ __forceinline__ void add_iterations(unsigned long long *total, unsigned long long mine) {
    if (!total) return;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(FULL, mine, o);
    if ((threadIdx.x & 31) == 0 && mine) atomicAdd(total, mine);
}

// --------------------------------------------------------- CPU-core semantics

// Tip grid coordinate g = dic . tip split into an integer cell (base) and a fraction (tf).
__device__ __forceinline__ void tip_cell(const RelaxPrm &P, const dfl g[3], int base[3], dfl tf[3]) {
#pragma unroll
    for (int k = 0; k < 3; k++) tf[k] = split_cell(g[k], base[k]);
}

__device__ __forceinline__ void grid_of(const RelaxPrm &P, const dfl r[3], dfl g[3]) {
    if (P.diag) {
#pragma unroll
        for (int k = 0; k < 3; k++) g[k] = df_mul(P.dic[4 * k], r[k]);
    } else {
#pragma unroll
        for (int k = 0; k < 3; k++)
            g[k] = df_add(df_add(df_mul(P.dic[3 * k], r[0]), df_mul(P.dic[3 * k + 1], r[1])), df_mul(P.dic[3 * k + 2], r[2]));
    }
}

// Scan mode keeps a per-height table in shared memory: (z, g_z0, g_z1, g_z2) as
// double-floats, g_z = dic . (0, 0, z), so a height change needs no float64.
constexpr int ZTAB = 4;

template <bool SCAN>
__global__ void __launch_bounds__(RELAX_THREADS) relax_kernel(const RelaxPrm P, const StrokeIO S, const ScanIO C) {
    extern __shared__ dfl ztab[];
    const int s = blockIdx.x * RELAX_THREADS + threadIdx.x;
    const int nstroke = SCAN ? C.nx * C.ny : S.nstroke;
    const int nstep = SCAN ? C.nz : S.nstep;
    if (SCAN) {
        for (int i = threadIdx.x; i < nstep; i += RELAX_THREADS) {
            const dfl z = df_from(C.zs[i]);
            ztab[ZTAB * i] = z;
#pragma unroll
            for (int k = 0; k < 3; k++) ztab[ZTAB * i + 1 + k] = df_mul(P.dic[3 * k + 2], z);
        }
        __syncthreads();
    }
    bool active = s < nstroke && nstep > 0;

    int ix = 0, iy = 0;
    if (SCAN && active) {
        ix = s / C.ny;
        iy = s - ix * C.ny;
    }
    // tip (double-float) and its grid coordinate: base cell + fraction
    dfl tip[3], gxy[3];
    int base[3];
    dfl tf[3];
    auto set_height = [&](int iz) {
        dfl g[3];
        if (SCAN) {
            tip[2] = ztab[ZTAB * iz];
#pragma unroll
            for (int k = 0; k < 3; k++) g[k] = df_add(gxy[k], ztab[ZTAB * iz + 1 + k]);
        } else {
            const double *t = S.rTips + ((long long)s * nstep + iz) * 3;
            tip[0] = df_from(t[0]);
            tip[1] = df_from(t[1]);
            tip[2] = df_from(t[2]);
            grid_of(P, tip, g);
        }
        tip_cell(P, g, base, tf);
    };

    dfl d[3] = {P.r0[0], P.r0[1], P.r0[2]};  // first start: r = tip + rPP0
    float3 v = make_float3(0.f, 0.f, 0.f);
    float dt = P.dtmaxf, acoef = P.acoef0f;
    int iz = 0, it = 0, itcount = 0;
    bool fin = P.maxIters <= 0;
    int itsum = 0;
    unsigned long long mine = 0;
    if (active) {
        if (SCAN) {
            tip[0] = df_from(C.xs[ix]);
            tip[1] = df_from(C.ys[iy]);
            const dfl r[3] = {tip[0], tip[1], {0.f, 0.f}};
            grid_of(P, r, gxy);
        }
        set_height(0);
    }

    while (__any_sync(FULL, active)) {
        if (!active) continue;
        dfl u[3], F[3];
        grid_coord_df(P, tf, d, u);
        interp_force_df(P.FE, P.n0, P.n1, P.n2, base, u, F);
        if (fin) {
            // outputs of height iz: position after the last move, grid force there
            const dfl r[3] = {df_add(tip[0], d[0]), df_add(tip[1], d[1]), df_add(tip[2], d[2])};
            if (SCAN) {
                const long long o = (long long)s * nstep + (nstep - 1 - iz);
                if (C.fzs) C.fzs[o] = df_round(F[2]);
                if (C.ppos) {
                    C.ppos[3 * o + 0] = df_round(df_add(r[0], C.offd[0]));
                    C.ppos[3 * o + 1] = df_round(df_add(r[1], C.offd[1]));
                    C.ppos[3 * o + 2] = df_round(df_add(r[2], C.offd[2]));
                }
                if (C.iters) C.iters[o] = itcount;
            } else {
                const long long o = (long long)s * nstep + iz;
                S.rs[3 * o + 0] = df_to(r[0]);
                S.rs[3 * o + 1] = df_to(r[1]);
                S.rs[3 * o + 2] = df_to(r[2]);
                S.fs[3 * o + 0] = df_to(F[0]);
                S.fs[3 * o + 1] = df_to(F[1]);
                S.fs[3 * o + 2] = df_to(F[2]);
                if (S.iters) S.iters[o] = itcount;
            }
            itsum += itcount;
            iz++;
            if (iz == nstep) {
                active = false;
                if (!SCAN && S.itrsum) S.itrsum[s] = itsum;
                if (SCAN && C.df && C.fzs && C.nw > 0) {
                    // np.convolve(fzs, W, 'valid') along ascending z (Fz2df, common.py:421-430)
                    const float *f = C.fzs + (long long)s * nstep;
                    const int nout = nstep - C.nw + 1;
                    float *out = C.df + (long long)s * nout;
                    for (int j = 0; j < nout; j++) {
                        float acc = 0.f;
                        for (int i = 0; i < C.nw; i++) acc = fmaf(f[j + i], C.W[C.nw - 1 - i], acc);
                        out[j] = acc;
                    }
                }
                continue;
            }
            // next height: warm start (relaxTipStroke, ProbeParticle.cpp:643-655)
            set_height(iz);
            if (P.probeStart == 0) {
                d[0] = P.r0[0];
                d[1] = P.r0[1];
                d[2] = P.r0[2];
            } else if (P.probeStart == -1) {  // the probe stays where it was: d = r_old - tip_new
#pragma unroll
                for (int k = 0; k < 3; k++) d[k] = df_add(r[k], df_neg(tip[k]));
            }  // probeStart == 1: d = r - r_tip carries over unchanged
            v = make_float3(0.f, 0.f, 0.f);
            dt = P.dtmaxf;
            acoef = P.acoef0f;
            it = 0;
            fin = P.maxIters <= 0;
            itcount = 0;
            continue;
        }
        const float3 f = pp_force_df(P, F, d);
        const float ff = relax_move_df(P, f, d, v, dt, acoef);
        mine++;
        if (ff < P.convF2f) {
            itcount = it;
            fin = true;
        } else if (++it >= P.maxIters) {
            itcount = P.maxIters;
            fin = true;
        }
    }
    add_iterations(P.iter_total, mine);
}

// ------------------------------------------------------------- AFMulator semantics

struct AfmPrm {
    const float4 *FE;
    int n0, n1, n2;
    float dic[9];  // rows: transpose(inv(cell)) row k times n_k
    float dtmax, damp0;
    float stiff[4], dpos0[4];
    float tA[3], tB[3], tC[3], zstep_w;
    float surf;
    int npix, nz;
    const float4 *points;
    float4 *FEs, *paths;
    int *iters;
    float *X;
    int nw;
    float W[MAX_DF_TAPS];
    unsigned long long *iter_total;
};

__device__ __forceinline__ float dot3(float3 a, const float *b) { return a.x * b[0] + a.y * b[1] + a.z * b[2]; }

__global__ void __launch_bounds__(RELAX_THREADS) relax_afm_kernel(const AfmPrm P) {
    const int p = blockIdx.x * RELAX_THREADS + threadIdx.x;
    bool active = p < P.npix && P.nz > 0;
    const float3 dTip = make_float3(P.tC[0] * P.zstep_w, P.tC[1] * P.zstep_w, P.tC[2] * P.zstep_w);
    // dpos0 rotated to the lab frame (rotMatT)
    const float3 d0 = make_float3(P.tA[0] * P.dpos0[0] + P.tB[0] * P.dpos0[1] + P.tC[0] * P.dpos0[2],
                                  P.tA[1] * P.dpos0[0] + P.tB[1] * P.dpos0[1] + P.tC[1] * P.dpos0[2],
                                  P.tA[2] * P.dpos0[0] + P.tB[2] * P.dpos0[1] + P.tC[2] * P.dpos0[2]);
    float3 tip = make_float3(0.f, 0.f, 0.f), pos = tip;
    if (active) {
        const float4 q = P.points[p];
        tip = make_float3(q.x, q.y, q.z);
        pos = make_float3(tip.x + d0.x, tip.y + d0.y, tip.z + d0.z);
    }
    float dt = P.dtmax, damp = P.damp0;
    const float dtmin = P.dtmax * 0.1f;
    float3 v = make_float3(0.f, 0.f, 0.f);
    int iz = 0, it = 0;
    unsigned long long mine = 0;
    constexpr int NMAX = 128;  // N_RELAX_STEP_MAX (relax.cl:90)

    while (__any_sync(FULL, active)) {
        if (!active) continue;
        float3 g;
        g.x = dot3(pos, P.dic);
        g.y = dot3(pos, P.dic + 3);
        g.z = dot3(pos, P.dic + 6);
        const float4 fe = interp_fe4(P.FE, P.n0, P.n1, P.n2, g);
        float3 f = make_float3(fe.x, fe.y, fe.z);
        const float3 dp = make_float3(pos.x - tip.x, pos.y - tip.y, pos.z - tip.z);
        const float3 dq = make_float3(dot3(dp, P.tA), dot3(dp, P.tB), dot3(dp, P.tC));
        const float r = sqrtf(dq.x * dq.x + dq.y * dq.y + dq.z * dq.z);
        const float rad = P.stiff[3] * (r - P.dpos0[3]) / r;
        const float3 ft = make_float3((dq.x - P.dpos0[0]) * P.stiff[0] + dq.x * rad,
                                      (dq.y - P.dpos0[1]) * P.stiff[1] + dq.y * rad,
                                      (dq.z - P.dpos0[2]) * P.stiff[2] + dq.z * rad);
        f.x += P.tA[0] * ft.x + P.tB[0] * ft.y + P.tC[0] * ft.z + P.tC[0] * P.surf;
        f.y += P.tA[1] * ft.x + P.tB[1] * ft.y + P.tC[1] * ft.z + P.tC[1] * P.surf;
        f.z += P.tA[2] * ft.x + P.tB[2] * ft.y + P.tC[2] * ft.z + P.tC[2] * P.surf;
        // update_FIRE (relax.cl:105-126)
        const float ff = f.x * f.x + f.y * f.y + f.z * f.z;
        const float vv = v.x * v.x + v.y * v.y + v.z * v.z;
        const float vf = v.x * f.x + v.y * f.y + v.z * f.z;
        if (vf < 0.f) {
            v = make_float3(0.f, 0.f, 0.f);
            dt = fmaxf(dtmin, dt * 0.5f);
            damp = P.damp0;
        } else {
            const float cf = damp * sqrtf(vv / (ff + 1e-8f));
            const float cv = 1.f - damp;
            v.x = fmaf(f.x, cf, v.x * cv);
            v.y = fmaf(f.y, cf, v.y * cv);
            v.z = fmaf(f.z, cf, v.z * cv);
            dt = fminf(P.dtmax, dt * 1.1f);
            damp *= 0.99f;
        }
        v.x = fmaf(f.x, dt, v.x);
        v.y = fmaf(f.y, dt, v.y);
        v.z = fmaf(f.z, dt, v.z);
        pos.x = fmaf(v.x, dt, pos.x);
        pos.y = fmaf(v.y, dt, pos.y);
        pos.z = fmaf(v.z, dt, pos.z);
        mine++;
        it++;
        if (ff < 1e-8f || it >= NMAX) {
            const long long o = (long long)p * P.nz + iz;
            if (P.FEs) {
                float4 r4;
                r4.x = fe.x * P.tA[0] + fe.y * P.tA[1] + fe.z * P.tA[2];
                r4.y = fe.x * P.tB[0] + fe.y * P.tB[1] + fe.z * P.tB[2];
                r4.z = fe.x * P.tC[0] + fe.y * P.tC[1] + fe.z * P.tC[2];
                r4.w = fe.w;
                P.FEs[o] = r4;
            }
            if (P.paths) P.paths[o] = make_float4(pos.x, pos.y, pos.z, 0.f);
            if (P.iters) P.iters[o] = (ff < 1e-8f) ? it - 1 : NMAX;
            tip.x += dTip.x;
            tip.y += dTip.y;
            tip.z += dTip.z;
            pos.x += dTip.x;
            pos.y += dTip.y;
            pos.z += dTip.z;
            v = make_float3(0.f, 0.f, 0.f);
            it = 0;
            iz++;
            if (iz == P.nz) {
                active = false;
                if (P.X && P.FEs && P.nw > 0) {
                    // convolveZ (relax.cl:571-608): X[o] = sum_j FEs[o+j].z * W[j]
                    const float4 *fin = P.FEs + (long long)p * P.nz;
                    const int nout = P.nz - P.nw + 1;
                    float *out = P.X + (long long)p * nout;
                    for (int o2 = 0; o2 < nout; o2++) {
                        float acc = 0.f;
                        for (int j = 0; j < P.nw; j++) acc = fmaf(fin[o2 + j].z, P.W[j], acc);
                        out[o2] = acc;
                    }
                }
            }
        }
    }
    add_iterations(P.iter_total, mine);
}

// ---------------------------------------------------------------------- host

static int fill_relax_prm(RelaxPrm &P, const float *FE, const int *n, const double *cell, const double *prm,
                          int probeStart, int relaxAlg, unsigned long long *iter_total) {
    GridGeom g;
    int st = make_geom(n, cell, &g);
    if (st) return st;
    memset(&P, 0, sizeof(P));
    P.FE = reinterpret_cast<const float4 *>(FE);
    P.n0 = n[0];
    P.n1 = n[1];
    P.n2 = n[2];
    for (int k = 0; k < 9; k++) P.dicd[k] = g.dicell[k];
    P.maxIters = (int)prm[0];
    P.convF2 = prm[1];
    P.dtmax = prm[2];
    P.acoef0 = prm[3];
    P.finc = prm[4];
    P.fdec = prm[5];
    P.falpha = prm[6];
    P.lRad = prm[7];
    P.kRad = prm[8];
    for (int k = 0; k < 3; k++) {
        P.rPP0[k] = prm[9 + k];
        P.kSpring[k] = prm[12 + k];
    }
    if (relaxAlg != 0 && relaxAlg != 1) return set_error(PPGPU_ERR_ARG, "relaxAlg %d not in {0,1}", relaxAlg);
    if (probeStart < -1 || probeStart > 1) return set_error(PPGPU_ERR_ARG, "probeStart %d not in {-1,0,1}", probeStart);
    P.relaxAlg = relaxAlg;
    P.probeStart = probeStart;
    P.iter_total = iter_total;
    P.err = device_error_word();
    for (int k = 0; k < 9; k++) P.dic[k] = df_from(P.dicd[k]);
    P.diag = P.dicd[1] == 0.0 && P.dicd[2] == 0.0 && P.dicd[3] == 0.0 && P.dicd[5] == 0.0 && P.dicd[6] == 0.0 &&
             P.dicd[7] == 0.0;
    P.kRadf = df_from(P.kRad);
    P.nl0 = df_from(-P.lRad);
    for (int k = 0; k < 3; k++) {
        P.nr0[k] = df_from(-P.rPP0[k]);
        P.r0[k] = df_from(P.rPP0[k]);
        P.kSf[k] = df_from(P.kSpring[k]);
    }
    P.convF2f = (float)P.convF2;
    P.dtmaxf = (float)P.dtmax;
    P.acoef0f = (float)P.acoef0;
    P.fincf = (float)P.finc;
    P.fdecf = (float)P.fdec;
    P.falphaf = (float)P.falpha;
    return set_ok();
}

}  // namespace ppgpu

using namespace ppgpu;

extern "C" int ppgpu_relax_strokes(const float *FE, const int *n, const double *cell, const double *prm,
                                   int probeStart, int relaxAlg, int nstroke, int nstep, const double *rTips,
                                   double *rs, double *fs, int *iters, int *itrsum,
                                   unsigned long long *iter_total, void *stream) {
    if (!FE || !n || !cell || !prm) return set_error(PPGPU_ERR_ARG, "relax_strokes: null argument");
    if (nstroke < 0 || nstep < 0) return set_error(PPGPU_ERR_ARG, "relax_strokes: negative sizes");
    if (nstroke == 0 || nstep == 0) return set_ok();
    if (!rTips || !rs || !fs) return set_error(PPGPU_ERR_ARG, "relax_strokes: null stroke arrays");
    RelaxPrm P;
    int st = fill_relax_prm(P, FE, n, cell, prm, probeStart, relaxAlg, iter_total);
    if (st) return st;
    StrokeIO S = {nstroke, nstep, rTips, rs, fs, iters, itrsum};
    ScanIO C;
    memset(&C, 0, sizeof(C));
    const unsigned nblk = (unsigned)((nstroke + RELAX_THREADS - 1) / RELAX_THREADS);
    relax_kernel<false><<<nblk, RELAX_THREADS, 0, (cudaStream_t)stream>>>(P, S, C);
    PPGPU_CHECK_LAUNCH("relax_kernel<strokes>");
    return set_ok();
}

extern "C" int ppgpu_relax_scan(const float *FE, const int *n, const double *cell, const double *prm, int nx, int ny,
                                int nz, const double *xs, const double *ys, const double *zs,
                                const double *pos_offset, float *fzs, float *ppos, int *iters, int nw,
                                const double *df_weights, float *df, unsigned long long *iter_total,
                                void *stream) {
    if (!FE || !n || !cell || !prm || !xs || !ys || !zs) return set_error(PPGPU_ERR_ARG, "relax_scan: null argument");
    if (nx < 0 || ny < 0 || nz < 0) return set_error(PPGPU_ERR_ARG, "relax_scan: negative sizes");
    if (df && (nw <= 0 || nw > MAX_DF_TAPS || nw > nz || !df_weights || !fzs))
        return set_error(PPGPU_ERR_ARG, "relax_scan: df needs 1 <= nw <= min(64, nz), weights and fzs");
    if (nx == 0 || ny == 0 || nz == 0) return set_ok();
    RelaxPrm P;
    int st = fill_relax_prm(P, FE, n, cell, prm, 1, 1, iter_total);
    if (st) return st;
    StrokeIO S;
    memset(&S, 0, sizeof(S));
    ScanIO C;
    memset(&C, 0, sizeof(C));
    C.nx = nx;
    C.ny = ny;
    C.nz = nz;
    C.xs = xs;
    C.ys = ys;
    C.zs = zs;
    for (int k = 0; k < 3; k++) {
        C.off[k] = pos_offset ? pos_offset[k] : 0.0;
        C.offd[k] = df_from(C.off[k]);
    }
    C.fzs = fzs;
    C.ppos = ppos;
    C.iters = iters;
    C.df = df;
    C.nw = df ? nw : 0;
    for (int i = 0; i < C.nw; i++) C.W[i] = (float)df_weights[i];
    const long long npix = (long long)nx * ny;
    const unsigned nblk = (unsigned)((npix + RELAX_THREADS - 1) / RELAX_THREADS);
    const size_t smem = (size_t)nz * ZTAB * sizeof(dfl);
    if (smem > 48 * 1024) return set_error(PPGPU_ERR_ARG, "relax_scan: nz = %d heights exceed the table limit (1536)", nz);
    relax_kernel<true><<<nblk, RELAX_THREADS, smem, (cudaStream_t)stream>>>(P, S, C);
    PPGPU_CHECK_LAUNCH("relax_kernel<scan>");
    return set_ok();
}

extern "C" int ppgpu_relax_afm(const float *FE, const int *n, const double *inv_cell, const double *prm, int npix,
                               const float *points, int nz, float *FEs, float *paths, int *iters, int nw,
                               const double *weights, float *X, unsigned long long *iter_total, void *stream) {
    if (!FE || !n || !inv_cell || !prm || (npix > 0 && !points))
        return set_error(PPGPU_ERR_ARG, "relax_afm: null argument");
    if (X && (nw <= 0 || nw > MAX_DF_TAPS || nw > nz || !weights || !FEs))
        return set_error(PPGPU_ERR_ARG, "relax_afm: X needs 1 <= nw <= min(64, nz), weights and FEs");
    if (npix <= 0 || nz <= 0) return set_ok();
    AfmPrm P;
    memset(&P, 0, sizeof(P));
    P.FE = reinterpret_cast<const float4 *>(FE);
    P.n0 = n[0];
    P.n1 = n[1];
    P.n2 = n[2];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) P.dic[3 * r + c] = (float)(inv_cell[3 * r + c] * n[r]);
    P.dtmax = (float)prm[0];
    P.damp0 = (float)prm[1];
    for (int k = 0; k < 4; k++) {
        P.stiff[k] = (float)prm[4 + k];
        P.dpos0[k] = (float)prm[8 + k];
    }
    for (int k = 0; k < 3; k++) {
        P.tA[k] = (float)prm[12 + k];
        P.tB[k] = (float)prm[16 + k];
        P.tC[k] = (float)prm[20 + k];
    }
    P.zstep_w = (float)prm[23];
    P.surf = (float)prm[24];
    P.npix = npix;
    P.nz = nz;
    P.points = reinterpret_cast<const float4 *>(points);
    P.FEs = reinterpret_cast<float4 *>(FEs);
    P.paths = reinterpret_cast<float4 *>(paths);
    P.iters = iters;
    P.X = X;
    P.nw = X ? nw : 0;
    for (int i = 0; i < P.nw; i++) P.W[i] = (float)weights[i];
    P.iter_total = iter_total;
    const unsigned nblk = (unsigned)((npix + RELAX_THREADS - 1) / RELAX_THREADS);
    relax_afm_kernel<<<nblk, RELAX_THREADS, 0, (cudaStream_t)stream>>>(P);
    PPGPU_CHECK_LAUNCH("relax_afm_kernel");
    return set_ok();
}
