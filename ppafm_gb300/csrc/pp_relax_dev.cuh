// pp_relax_dev.cuh -- device side of the relaxation (shared by the single-grid kernels of
// pp_relax.cu and the batched persistent kernel of pp_batch.cu).  The reference functions
// and the precision design are described in pp_relax.cu.
#pragma once

#include <cstring>

#include "pp_common.cuh"
#include "pp_df.cuh"

namespace ppgpu {

// CTA of the single-grid relaxation kernel.  Measured against 64 and 32 threads in the
// pipelined steps (a relaxation beside the next step's force field): the density-overlap step
// 3.18 vs 3.28 / 3.32 ms, the small molecule's unchanged (2.07 ms).
constexpr int RELAX_THREADS = 128;
constexpr int MAX_DF_TAPS = 64;
constexpr unsigned FULL = 0xffffffffu;

// Radial tip spline (TIP::SplineParams, ProbeParticle.cpp:58-62) in device memory: knots
// and, per interval, x0, 1/dx and the coefficients c0..c3 of the cubic Hermite piece in
// u = (x - x0)/dx (spline_hermite.h:45-51), all double-floats.  n == 0: harmonic spring.
struct TipSpline {
    int n;
    const dfl *xs;   // [n]
    const dfl *seg;  // [n - 1][6]
};
// The spline that fill_relax_prm puts into the relaxation parameters (set by
// ppgpu_set_tip_spline; defined in pp_relax.cu).
extern TipSpline g_tip_spline;


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
    TipSpline spl;         // radial tip spline (n 0: the harmonic radial spring)
};

// Radial force of the tip spline at |d| = x (forceRSpline, ProbeParticle.cpp:212-225): the
// interval from the halving search of Spline_Hermite::find_index (spline_hermite.h:159-169),
// kept at most n - 2 (the reference reads past its table beyond the last knot), then the
// cubic in u by Horner's rule.
__device__ __forceinline__ dfl spline_radial_df(const TipSpline &S, dfl x) {
    int i = 0;
    for (int di = S.n; di > 1;) {
        di >>= 1;
        if (df_lt(S.xs[i + di], x)) i += di;
    }
    i = min(i, S.n - 2);
    const dfl *c = S.seg + 6 * i;
    const dfl u = df_mul(df_add(x, df_neg(c[0])), c[1]);
    dfl r = df_add(c[4], df_mul(u, c[5]));
    r = df_add(c[3], df_mul(u, r));
    return df_add(c[2], df_mul(u, r));
}


// ----------------------------------------------------------- interpolation

// Periodic trilinear interpolation of the force (Grid.h:93-111) at the grid coordinate
// base + u (base integer, u double-float): float32 grid values, double-float weights and
// compensated sums, so the only rounding left is that of the stored grid values.
// NC: read-only (non-coherent) gathers; false for a grid written earlier in the same launch.
template <bool NC = true>
__device__ __forceinline__ void interp_force_df(const float4 *FE, int n0, int n1, int n2, const int base[3],
                                                const dfl u[3], dfl F[3]) {
    auto ld = [&](const float4 *q) { return NC ? ldg4(q) : *q; };
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
    const float4 c[8] = {ld(FE + r00 + iz0), ld(FE + r00 + iz1), ld(FE + r01 + iz0), ld(FE + r01 + iz1),
                         ld(FE + r10 + iz0), ld(FE + r10 + iz1), ld(FE + r11 + iz0), ld(FE + r11 + iz1)};
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

// interp_force_df split over a group of TPS lanes (TPS in {1, 2, 4, 8}, groups aligned in the
// warp, sub = lane index in the group, mask = the warp's participating lanes): lane sub gathers
// and weighs corners sub * 8/TPS .. +8/TPS-1, and the partial sums are combined by xor
// shuffles in the same pairing as the one-lane sum ((c0+c1)+(c2+c3))+((c4+c5)+(c6+c7)).
// TwoSum is exact whatever the operand order, so every lane of the group gets the one-lane
// result bit for bit.
template <int TPS, bool NC = true>
__device__ __forceinline__ void interp_force_df_group(const float4 *FE, int n0, int n1, int n2, const int base[3],
                                                      const dfl u[3], dfl F[3], int sub, unsigned mask) {
    if constexpr (TPS == 1) {
        interp_force_df<NC>(FE, n0, n1, n2, base, u, F);
    } else {
        constexpr int CPL = 8 / TPS;  // corners per lane
        auto ld = [&](const float4 *q) { return NC ? ldg4(q) : *q; };
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
        float4 c[CPL];
        dfl w[CPL];
#pragma unroll
        for (int i = 0; i < CPL; i++) {
            const int k = sub * CPL + i;  // corner bits (x, y, z) = (k >> 2, (k >> 1) & 1, k & 1)
            const int bx = k >> 2, by = (k >> 1) & 1, bz = k & 1;
            c[i] = ld(FE + ((long long)(bx ? ix1 : ix0) * n1 + (by ? iy1 : iy0)) * n2 + (bz ? iz1 : iz0));
            w[i] = df_mul(df_mul(bx ? t[0] : m[0], by ? t[1] : m[1]), bz ? t[2] : m[2]);
        }
#pragma unroll
        for (int comp = 0; comp < 3; comp++) {
            dfl p[CPL];
#pragma unroll
            for (int i = 0; i < CPL; i++) {
                const float v = comp == 0 ? c[i].x : (comp == 1 ? c[i].y : c[i].z);
                p[i] = two_prod(w[i].h, v);
                p[i].l = __fmaf_rn(w[i].l, v, p[i].l);
            }
            dfl r;
            if constexpr (CPL == 4)
                r = df_add_raw(df_add_raw(p[0], p[1]), df_add_raw(p[2], p[3]));
            else if constexpr (CPL == 2)
                r = df_add_raw(p[0], p[1]);
            else
                r = p[0];
#pragma unroll
            for (int off = 1; off < TPS; off <<= 1) {
                dfl o;
                o.h = __shfl_xor_sync(mask, r.h, off);
                o.l = __shfl_xor_sync(mask, r.l, off);
                r = df_add_raw(r, o);
            }
            F[comp] = two_sum(r.h, r.l);
        }
    }
}

// Grid coordinate g_k = r . dicell_row_k of a float64 position (Grid.h:46-50).
__device__ __forceinline__ double3 to_grid(const RelaxPrm &P, double x, double y, double z) {
    return make_double3(fma(z, P.dicd[2], fma(y, P.dicd[1], x * P.dicd[0])),
                        fma(z, P.dicd[5], fma(y, P.dicd[4], x * P.dicd[3])),
                        fma(z, P.dicd[8], fma(y, P.dicd[7], x * P.dicd[6])));
}

// Grid coordinate of the displacement d relative to tf (double-float): u_k = tf_k + dic_k . d.
__device__ __forceinline__ void grid_coord_df(const dfl *dic, bool diag, const dfl tf[3], const dfl d[3], dfl u[3]) {
    if (diag) {
#pragma unroll
        for (int k = 0; k < 3; k++) u[k] = df_add(tf[k], df_mul(dic[4 * k], d[k]));
    } else {
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const dfl a = df_add_raw(df_mul(dic[3 * k], d[0]), df_mul(dic[3 * k + 1], d[1]));
            u[k] = df_add(tf[k], df_add(a, df_mul(dic[3 * k + 2], d[2])));
        }
    }
}

// Probe-particle force = grid force + radial spring + lateral spring (getPPforce,
// ProbeParticle.cpp:282-294; forceRSpring, Forces.h:85-89) in double-float, returned as the
// float32 residual: the radial spring is stiff, so l - l0 is a small difference of ~4 A
// lengths, and the force is a small difference of the grid force and the springs.
// SPL: the radial force comes from the tip spline (P.spl) instead of the harmonic spring
// (a template parameter, so the harmonic kernels carry no spline code).
template <bool SPL = false>
__device__ __forceinline__ float3 pp_force_df(const RelaxPrm &P, const dfl F[3], const dfl d[3]) {
    const dfl l2 = df_add(df_add(df_sq(d[0]), df_sq(d[1])), df_sq(d[2]));
    // l = sqrt(l2) and 1/l: approximate float32 root, then one correction from the exact
    // residual l2 - L^2 (error ~ the square of the approximation's)
    const float rs = rsqrt_approx(l2.h);
    const float L = __fmul_rn(l2.h, rs);
    const dfl LL = two_prod(L, L);
    const float res = __fadd_rn(__fsub_rn(__fsub_rn(l2.h, LL.h), LL.l), l2.l);
    const dfl l = fast_two_sum(L, __fmul_rn(res, __fmul_rn(0.5f, rs)));
    dfl s;
    if constexpr (SPL) {
        s = df_div(spline_radial_df(P.spl, l), l);  // radial spline force / l
    } else {
        const dfl x = df_add(l, P.nl0);  // l - l0
        // q = (l - l0) / l: approximate quotient plus the correction from its exact remainder
        const float qh = __fmul_rn(x.h, rs);
        const dfl ql = two_prod(qh, l.h);
        const float rem = __fsub_rn(__fadd_rn(__fsub_rn(__fsub_rn(x.h, ql.h), ql.l), x.l), __fmul_rn(qh, l.l));
        s = df_mul(P.kRadf, two_sum(qh, __fmul_rn(rem, rs)));
    }
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
    // explicitly rounded operations: the same bits in every kernel that inlines this
    const float ff = __fmaf_rn(f.z, f.z, __fmaf_rn(f.y, f.y, __fmul_rn(f.x, f.x)));
    float h;
    if (P.relaxAlg == 1) {
        const float vv = __fmaf_rn(v.z, v.z, __fmaf_rn(v.y, v.y, __fmul_rn(v.x, v.x)));
        const float vf = __fmaf_rn(f.z, v.z, __fmaf_rn(f.y, v.y, __fmul_rn(f.x, v.x)));
        if (vf < 0.f) {
            v = make_float3(0.f, 0.f, 0.f);
            dt = __fmul_rn(dt, P.fdecf);
            acoef = P.acoef0f;
        } else {
            // cf f has length acoef |v|; vv ff below 1e-30 gives cf = 0 instead of an
            // overflow (the reference divides by zero at ff == 0, and cf = 0 at vv == 0)
            const float vf2 = __fmul_rn(vv, ff);  // sqrt(vv/ff) = vv / sqrt(vv ff)
            const float cf = (vf2 > 1e-30f) ? __fmul_rn(__fmul_rn(acoef, vv), rsqrt_approx(vf2)) : 0.f;
            const float cv = __fsub_rn(1.f, acoef);
            v.x = __fmaf_rn(f.x, cf, __fmul_rn(v.x, cv));
            v.y = __fmaf_rn(f.y, cf, __fmul_rn(v.y, cv));
            v.z = __fmaf_rn(f.z, cf, __fmul_rn(v.z, cv));
            dt = fminf(__fmul_rn(dt, P.fincf), P.dtmaxf);
            acoef = __fmul_rn(acoef, P.falphaf);
        }
        h = dt;
    } else {
        const float c = __fsub_rn(1.f, P.acoef0f);
        v.x = __fmul_rn(v.x, c);
        v.y = __fmul_rn(v.y, c);
        v.z = __fmul_rn(v.z, c);
        h = P.dtmaxf;
    }
    v.x = __fmaf_rn(f.x, h, v.x);
    v.y = __fmaf_rn(f.y, h, v.y);
    v.z = __fmaf_rn(f.z, h, v.z);
    d[0] = df_add_f(d[0], __fmul_rn(v.x, h));
    d[1] = df_add_f(d[1], __fmul_rn(v.y, h));
    d[2] = df_add_f(d[2], __fmul_rn(v.z, h));
    return ff;
}

__device__ __forceinline__ void add_iterations(unsigned long long *total, unsigned long long mine) {
    if (!total) return;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(FULL, mine, o);
    if ((threadIdx.x & 31) == 0 && mine) atomicAdd(total, mine);
}

// Tip grid coordinate g = dic . tip split into an integer cell (base) and a fraction (tf).
__device__ __forceinline__ void tip_cell(const dfl g[3], int base[3], dfl tf[3]) {
#pragma unroll
    for (int k = 0; k < 3; k++) tf[k] = split_cell(g[k], base[k]);
}

__device__ __forceinline__ void grid_of(const dfl *dic, bool diag, const dfl r[3], dfl g[3]) {
    if (diag) {
#pragma unroll
        for (int k = 0; k < 3; k++) g[k] = df_mul(dic[4 * k], r[k]);
    } else {
#pragma unroll
        for (int k = 0; k < 3; k++)
            g[k] = df_add(df_add(df_mul(dic[3 * k], r[0]), df_mul(dic[3 * k + 1], r[1])), df_mul(dic[3 * k + 2], r[2]));
    }
}

// Host: relaxation parameters of the C ABI (prm[RELAX_NPARAM]) into RelaxPrm.
static inline int fill_relax_prm(RelaxPrm &P, const float *FE, const int *n, const double *cell, const double *prm,
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
    P.spl = g_tip_spline;
    P.convF2f = (float)P.convF2;
    P.dtmaxf = (float)P.dtmax;
    P.acoef0f = (float)P.acoef0;
    P.fincf = (float)P.finc;
    P.fdecf = (float)P.fdec;
    P.falphaf = (float)P.falpha;
    return set_ok();
}

}  // namespace ppgpu
