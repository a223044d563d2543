/*
 * pp_oracle.c -- CPU restatement of the probe-particle AFM hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the correctness oracle for the
 * CUDA library in ppafm_gb300/csrc.  Only tests/, __graft_entry__.smoke() and
 * the CPU-baseline legs of bench.py may load it, and only as the checker or as
 * the timed CPU baseline -- never as part of the product path.
 *
 * It restates, in plain C99 + OpenMP, the algorithms of the reference ppafm
 * v0.4.0 C++ core (FP64) and of its OpenCL kernels (FP32):
 *
 *   FP64 (CPU path, ppafm/cpp):
 *     oc_grid_setup        GridShape::setCell + Mat3::invert_T_to   (Grid.h:29-36, Mat3.h:275-286)
 *     oc_lj_grid           getLennardJonesFF -> iterateGrid3D_omp<evalCell<addAtom_LJ>>
 *                          (ProbeParticle.cpp:508-513, Grid.h:142-170, ProbeParticle.cpp:262-278,
 *                           Forces.h:120-132)
 *     oc_coulomb_grid      getCoulombFF kinds 0/1/2 (ProbeParticle.cpp:540-554, 192-209,
 *                           Forces.h:237-244)
 *     oc_relax_strokes     relaxTipStrokes_omp / relaxTipStroke / relaxProbe / getPPforce /
 *                           FIREstate::move / interpolate3DvecWrap
 *                          (ProbeParticle.cpp:682-701, 633-676, 297-313, 282-294, 142-174;
 *                           Grid.h:66-69, 93-111; Forces.h:85-89)
 *   FP32 (OpenCL path, ppafm/ocl/cl):
 *     oc_afm_ff_qzs        evalLJC_QZs_noPos (FF.cl:366-423) with getLJ/getCoulomb (FF.cl:128-143)
 *     oc_afm_relax_tilted  relaxStrokesTilted (relax.cl:391-464), update_FIRE (relax.cl:105-126),
 *                          tipForce (relax.cl:37-41).  The texture fetch interpFE (relax.cl:64-73)
 *                          is restated as an explicit FP32 periodic trilinear interpolation.
 *     oc_afm_convolve_z    convolveZ (relax.cl:571-608)
 *
 * The FP64 functions keep the reference's order of floating-point operations so
 * that, compiled with -ffp-contract=off, they agree bit for bit with the reference
 * library built from its own sources.  Everything here is written from the
 * published algorithm; no reference source is included.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---------------------------------------------------------------- constants */

/* Forces.h:12 -- R2SAFE is a float literal promoted to double. */
#define OC_R2SAFE_CPU ((double)1.0e-8f)
/* ProbeParticle.cpp:178-180 */
#define OC_DSTEP 0.1
#define OC_INV_DSTEP 10.0
#define OC_INV_DDSTEP 100.0
/* FF.cl:1-2 */
#define OC_R2SAFE_CL 1e-6f
#define OC_COULOMB_CL 14.399644f
/* relax.cl:90-103 */
#define OC_NRELAX_CL 128
#define OC_F2CONV_CL 1e-8f
#define OC_FTDEC 0.5f
#define OC_FTINC 1.1f
#define OC_FDAMP 0.99f
#define OC_F2SAFE 1e-8f

/* ------------------------------------------------------------- grid shape */

/* Voxel basis (rows = voxel vectors a/na, b/nb, c/nc) and the transposed
 * inverse used to map Cartesian positions to fractional grid coordinates:
 * g_k = r . dicell_row_k.  Follows GridShape::setCell (Grid.h:29-36) and
 * Mat3::invert_T_to (Mat3.h:275-286). */
void oc_grid_setup(const int n[3], const double cell[9], double dcell[9], double dicell[9])
{
    for (int k = 0; k < 3; k++) {
        double inv = 1.0 / n[k];
        for (int j = 0; j < 3; j++) dcell[3 * k + j] = cell[3 * k + j] * inv;
    }
    const double xx = dcell[0], xy = dcell[1], xz = dcell[2];
    const double yx = dcell[3], yy = dcell[4], yz = dcell[5];
    const double zx = dcell[6], zy = dcell[7], zz = dcell[8];
    double cxx = yy * zz - yz * zy;
    double cyx = yz * zx - yx * zz;
    double czx = yx * zy - yy * zx;
    double det = xx * cxx + xy * cyx + xz * czx;
    double idet = 1 / det;
    /* dicell laid out as rows a,b,c: element (row r, col c) at 3*r+c */
    dicell[0] = (yy * zz - yz * zy) * idet; /* xx */
    dicell[3] = (xz * zy - xy * zz) * idet; /* yx */
    dicell[6] = (xy * yz - xz * yy) * idet; /* zx */
    dicell[1] = (yz * zx - yx * zz) * idet; /* xy */
    dicell[4] = (xx * zz - xz * zx) * idet; /* yy */
    dicell[7] = (xz * yx - xx * yz) * idet; /* zy */
    dicell[2] = (yx * zy - yy * zx) * idet; /* xz */
    dicell[5] = (xy * zx - xx * zy) * idet; /* yz */
    dicell[8] = (xx * yy - xy * yx) * idet; /* zz */
}

/* ----------------------------------------------------- pairwise kernels FP64 */

/* Forces.h:120-132: adds the LJ force on a probe displaced by dR from an atom. */
static inline double oc_pair_lj(double dx, double dy, double dz, double c6, double c12,
                                double *fx, double *fy, double *fz)
{
    double ir2 = 1.0 / ((dx * dx + dy * dy + dz * dz) + OC_R2SAFE_CPU);
    double ir6 = ir2 * ir2 * ir2;
    double e6 = c6 * ir6;
    double e12 = c12 * ir6 * ir6;
    double fr = (12 * e12 - 6 * e6) * ir2;
    *fx += dx * fr;
    *fy += dy * fr;
    *fz += dz * fr;
    return e12 - e6;
}

/* Forces.h:237-244: Coulomb with kqq = k_e * Q_probe * Q_atom folded in. */
static inline double oc_pair_coulomb(double dx, double dy, double dz, double kqq,
                                     double *fx, double *fy, double *fz)
{
    double ir2 = 1.0 / ((dx * dx + dy * dy + dz * dz) + OC_R2SAFE_CPU);
    double ir = sqrt(ir2);
    double e = ir * kqq;
    double fr = e * ir2;
    *fx += dx * fr;
    *fy += dy * fr;
    *fz += dz * fr;
    return e;
}

/* ProbeParticle.cpp:192-209: s / pz / dz2 tip multipoles by finite differences. */
static inline double oc_pair_coulomb_kind(double dx, double dy, double dz, double kqq, int kind,
                                          double *fx, double *fy, double *fz)
{
    if (kind == 0) return oc_pair_coulomb(dx, dy, dz, kqq, fx, fy, fz);
    double e = 0, gx = 0, gy = 0, gz = 0;
    if (kind == 1) {
        dz -= OC_DSTEP;
        e += oc_pair_coulomb(dx, dy, dz, -kqq, &gx, &gy, &gz);
        dz += 2 * OC_DSTEP;
        e += oc_pair_coulomb(dx, dy, dz, +kqq, &gx, &gy, &gz);
        *fx += gx * OC_INV_DSTEP;
        *fy += gy * OC_INV_DSTEP;
        *fz += gz * OC_INV_DSTEP;
        return e * OC_INV_DSTEP;
    }
    e += oc_pair_coulomb(dx, dy, dz, -2 * kqq, &gx, &gy, &gz);
    dz -= OC_DSTEP;
    e += oc_pair_coulomb(dx, dy, dz, kqq, &gx, &gy, &gz);
    dz += 2 * OC_DSTEP;
    e += oc_pair_coulomb(dx, dy, dz, kqq, &gx, &gy, &gz);
    *fx += gx * OC_INV_DDSTEP;
    *fy += gy * OC_INV_DDSTEP;
    *fz += gz * OC_INV_DDSTEP;
    return e * OC_INV_DDSTEP;
}

/* ------------------------------------------------------------ grid sampling */

/* Sample a force field on the sub-box [i0, i0+ns) of a full grid of shape n with
 * cell `cell`; grid point (ia,ib,ic) sits at ia*dA + ib*dB + ic*dC (Grid.h:151).
 * kind: -1 = Lennard-Jones with coefs (c6,c12) per atom, 0/1/2 = Coulomb tip kinds
 * with coefs kqq per atom.  Results are ADDED into gridF [ns0,ns1,ns2,3] and gridE
 * [ns0,ns1,ns2] (either may be NULL), C order, like evalCell (ProbeParticle.cpp:262-278). */
void oc_ff_subgrid(const int n[3], const double cell[9], const int i0[3], const int ns[3],
                   int natoms, const double *R, const double *coefs, int kind,
                   double *gridF, double *gridE, int nthreads)
{
    double dcell[9], dicell[9];
    oc_grid_setup(n, cell, dcell, dicell);
    const int ncoef = (kind < 0) ? 2 : 1;
    const long long ntot = (long long)ns[0] * ns[1] * ns[2];
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(static)
    for (long long ip = 0; ip < ntot; ip++) {
        int ic = (int)(ip % ns[2]);
        int ib = (int)((ip / ns[2]) % ns[1]);
        int ia = (int)(ip / ((long long)ns[1] * ns[2]));
        int ga = ia + i0[0], gb = ib + i0[1], gc = ic + i0[2];
        /* pos0 + dCell.a*ia + dCell.b*ib + dCell.c*ic, evaluated left to right */
        double px = ((0.0 + dcell[0] * ga) + dcell[3] * gb) + dcell[6] * gc;
        double py = ((0.0 + dcell[1] * ga) + dcell[4] * gb) + dcell[7] * gc;
        double pz = ((0.0 + dcell[2] * ga) + dcell[5] * gb) + dcell[8] * gc;
        double fx = 0, fy = 0, fz = 0, e = 0;
        const double *c = coefs;
        for (int i = 0; i < natoms; i++) {
            double dx = px - R[3 * i + 0];
            double dy = py - R[3 * i + 1];
            double dz = pz - R[3 * i + 2];
            if (kind < 0)
                e += oc_pair_lj(dx, dy, dz, c[0], c[1], &fx, &fy, &fz);
            else
                e += oc_pair_coulomb_kind(dx, dy, dz, c[0], kind, &fx, &fy, &fz);
            c += ncoef;
        }
        if (gridF) {
            gridF[3 * ip + 0] += fx;
            gridF[3 * ip + 1] += fy;
            gridF[3 * ip + 2] += fz;
        }
        if (gridE) gridE[ip] += e;
    }
}

/* getLennardJonesFF over the whole grid (ProbeParticle.cpp:508-513). */
void oc_lj_grid(const int n[3], const double cell[9], int natoms, const double *R, const double *cLJ,
                double *gridF, double *gridE, int nthreads)
{
    const int z[3] = {0, 0, 0};
    oc_ff_subgrid(n, cell, z, n, natoms, R, cLJ, -1, gridF, gridE, nthreads);
}

/* getCoulombFF over the whole grid (ProbeParticle.cpp:540-554). */
void oc_coulomb_grid(const int n[3], const double cell[9], int natoms, const double *R, const double *kqq,
                     int kind, double *gridF, double *gridE, int nthreads)
{
    const int z[3] = {0, 0, 0};
    oc_ff_subgrid(n, cell, z, n, natoms, R, kqq, kind, gridF, gridE, nthreads);
}

/* ------------------------------------------------------------- relaxation */

typedef struct {
    int n[3];
    double dicell[9];
    const double *gridF; /* [n0,n1,n2,3] */
    /* tip (ProbeParticle.cpp:51-69) */
    double rPP0[3], kSpring[3], lRadial, kRadial;
    /* relaxation (ProbeParticle.cpp:74-114) */
    int maxIters;
    double convF2, dt, damping, finc, fdec, falpha;
    /* radial tip spline (TIP::SplineParams, ProbeParticle.cpp:58-62); spl_n 0: harmonic */
    int spl_n;
    const double *spl_xs, *spl_ydys;
} oc_relax_ctx;

/* Interval search of Spline_Hermite::find_index (spline_hermite.h:159-169): halving steps
 * from n/2 down to 1, advancing while the knot is below x. */
static inline int oc_spline_index(int n, double x, const double *xs)
{
    int i = 0, di = n;
    while (di > 1) {
        di >>= 1;
        int j = i + di;
        if (xs[j] < x) i = j;
    }
    return i;
}

/* Cubic Hermite value (spline_hermite.h:45-51) at u in [0,1] from end values and slopes. */
static inline double oc_hermite(double u, double y0, double y1, double dy0, double dy1)
{
    double y01 = y0 - y1;
    return y0 + u * (dy0 + u * (-3 * y01 - 2 * dy0 - dy1 + u * (2 * y01 + dy0 + dy1)));
}

/* Radial tip force from the spline of |d| (forceRSpline, ProbeParticle.cpp:212-225); the
 * interval index is kept at most n - 2 (the reference reads past its table beyond the last
 * knot). */
static inline double oc_spline_radial(const oc_relax_ctx *C, double x)
{
    int i = oc_spline_index(C->spl_n, x, C->spl_xs);
    if (i > C->spl_n - 2) i = C->spl_n - 2;
    double x0 = C->spl_xs[i], x1 = C->spl_xs[i + 1];
    double dx = x1 - x0;
    double denom = 1 / dx;
    double u = (x - x0) * denom;
    const double *yd = C->spl_ydys + 2 * i;
    return oc_hermite(u, yd[0], yd[2], yd[1] * dx, yd[3] * dx);
}

/* One axis of the periodic index/weight set-up (Grid.h:66-69). */
static inline void oc_wrap_axis(double r, int n, int *im, int *it, double *m, double *t)
{
    if (r >= 0) {
        int i = (int)r;
        *t = r - i;
        *m = 1 - *t;
        *im = i % n;
    } else {
        int j = (int)r;
        *m = j - r;
        *t = 1 - *m;
        *im = j % n + n - 1;
    }
    *it = (*im + 1) % n;
}

/* Periodic trilinear interpolation of a Vec3 grid (Grid.h:93-111). */
static inline void oc_interp(const oc_relax_ctx *C, double gx, double gy, double gz, double out[3])
{
    int imx, itx, imy, ity, imz, itz;
    double mx, tx, my, ty, mz, tz;
    oc_wrap_axis(gx, C->n[0], &imx, &itx, &mx, &tx);
    oc_wrap_axis(gy, C->n[1], &imy, &ity, &my, &ty);
    oc_wrap_axis(gz, C->n[2], &imz, &itz, &mz, &tz);
    const int ny = C->n[1], nz = C->n[2];
#define OC_IDX(a, b, c) ((((long long)(a) * ny + (b)) * nz + (c)) * 3)
    double mxmy = mx * my, mxty = mx * ty, txmy = tx * my, txty = tx * ty;
    const double *G = C->gridF;
    const long long i0 = OC_IDX(imx, imy, imz), i1 = OC_IDX(imx, imy, itz);
    const long long i2 = OC_IDX(imx, ity, imz), i3 = OC_IDX(imx, ity, itz);
    const long long i4 = OC_IDX(itx, ity, imz), i5 = OC_IDX(itx, ity, itz);
    const long long i6 = OC_IDX(itx, imy, imz), i7 = OC_IDX(itx, imy, itz);
#undef OC_IDX
    for (int k = 0; k < 3; k++) {
        double v = G[i0 + k] * (mxmy * mz);
        v += G[i1 + k] * (mxmy * tz);
        v += G[i2 + k] * (mxty * mz);
        v += G[i3 + k] * (mxty * tz);
        v += G[i4 + k] * (txty * mz);
        v += G[i5 + k] * (txty * tz);
        v += G[i6 + k] * (txmy * mz);
        v += G[i7 + k] * (txmy * tz);
        out[k] = v;
    }
}

static inline void oc_to_grid(const oc_relax_ctx *C, const double r[3], double g[3])
{
    for (int k = 0; k < 3; k++)
        g[k] = r[0] * C->dicell[3 * k + 0] + r[1] * C->dicell[3 * k + 1] + r[2] * C->dicell[3 * k + 2];
}

/* Total force on the probe particle (getPPforce, ProbeParticle.cpp:282-294;
 * radial spring forceRSpring, Forces.h:85-89). */
static inline void oc_pp_force(const oc_relax_ctx *C, const double rTip[3], const double r[3], double f[3])
{
    double g[3], d[3];
    oc_to_grid(C, r, g);
    for (int k = 0; k < 3; k++) d[k] = r[k] - rTip[k];
    oc_interp(C, g[0], g[1], g[2], f);
    double l = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    double s = (C->spl_n > 0) ? oc_spline_radial(C, l) / l : C->kRadial * (l - C->lRadial) / l;
    for (int k = 0; k < 3; k++) f[k] += d[k] * s;
    for (int k = 0; k < 3; k++) d[k] -= C->rPP0[k];
    for (int k = 0; k < 3; k++) f[k] += d[k] * C->kSpring[k];
}

/* relaxProbe (ProbeParticle.cpp:297-313) with FIREstate::move (ProbeParticle.cpp:153-172)
 * or the damped leap-frog RELAX::move (ProbeParticle.cpp:84-88).  Returns the iteration
 * index at which |f|^2 < convF2 was first seen, or maxIters. */
static int oc_relax_probe(const oc_relax_ctx *C, int relaxAlg, const double rTip[3], double r[3])
{
    double v[3] = {0, 0, 0};
    double dt = C->dt, acoef = C->damping;
    int iter;
    for (iter = 0; iter < C->maxIters; iter++) {
        double f[3];
        oc_pp_force(C, rTip, r, f);
        if (relaxAlg == 1) {
            double ff = f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
            double vv = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
            double vf = f[0] * v[0] + f[1] * v[1] + f[2] * v[2];
            if (vf < 0) {
                v[0] = v[1] = v[2] = 0.0;
                dt = dt * C->fdec;
                acoef = C->damping;
            } else {
                double cf = acoef * sqrt(vv / ff);
                double cv = 1 - acoef;
                for (int k = 0; k < 3; k++) v[k] *= cv;
                for (int k = 0; k < 3; k++) v[k] += f[k] * cf;
                dt = fmin(dt * C->finc, C->dt);
                acoef = acoef * C->falpha;
            }
            for (int k = 0; k < 3; k++) v[k] += f[k] * dt;
            for (int k = 0; k < 3; k++) r[k] += v[k] * dt;
        } else {
            for (int k = 0; k < 3; k++) v[k] *= 1 - C->damping;
            for (int k = 0; k < 3; k++) v[k] += f[k] * C->dt;
            for (int k = 0; k < 3; k++) r[k] += v[k] * C->dt;
        }
        if (f[0] * f[0] + f[1] * f[1] + f[2] * f[2] < C->convF2) break;
    }
    return iter;
}

/* relaxTipStroke (ProbeParticle.cpp:633-676): returns the iteration sum of the stroke. */
static int oc_relax_stroke(const oc_relax_ctx *C, int probeStart, int relaxAlg, int nstep,
                           const double *rTips, double *rs, double *fs, int *iters_out)
{
    double rTip[3], rp[3];
    for (int k = 0; k < 3; k++) rTip[k] = rTips[k];
    for (int k = 0; k < 3; k++) rp[k] = rTip[k] + C->rPP0[k];
    int itrsum = 0;
    for (int i = 0; i < nstep; i++) {
        const double *tn = rTips + 3 * i;
        if (probeStart == -1) {
            for (int k = 0; k < 3; k++) rTip[k] = tn[k];
        } else if (probeStart == 0) {
            for (int k = 0; k < 3; k++) rTip[k] = tn[k];
            for (int k = 0; k < 3; k++) rp[k] = rTip[k] + C->rPP0[k];
        } else if (probeStart == 1) {
            double drp[3];
            for (int k = 0; k < 3; k++) drp[k] = rp[k] - rTip[k];
            for (int k = 0; k < 3; k++) rTip[k] = tn[k];
            for (int k = 0; k < 3; k++) rp[k] = rTip[k] + drp[k];
        }
        int itr = oc_relax_probe(C, relaxAlg, rTip, rp);
        double g[3], f[3];
        oc_to_grid(C, rp, g);
        oc_interp(C, g[0], g[1], g[2], f);
        for (int k = 0; k < 3; k++) rs[3 * i + k] = rp[k];
        for (int k = 0; k < 3; k++) fs[3 * i + k] = f[k];
        if (iters_out) iters_out[i] = itr;
        itrsum += itr;
    }
    return itrsum;
}

/* relaxTipStrokes_omp (ProbeParticle.cpp:682-701): stroke s occupies elements
 * [s*nstep, (s+1)*nstep) of rTips/rs/fs.  Per-stroke iteration sums go to itrsums
 * (nullable) and per-step iteration counts to iters (nullable, [nstroke*nstep]).
 * params: maxIters, convF2, dt, damping, finc, fdec, falpha, lRadial, kRadial,
 *         rPP0[3] (already made consistent with lRadial), kSpring[3].
 * spl_n knots spl_xs and (value, slope) pairs spl_ydys: the radial tip spline replacing the
 * harmonic radial spring (spl_n 0 or NULL arrays: harmonic). */
void oc_relax_strokes(const int n[3], const double cell[9], const double *gridF,
                      const double *params, int probeStart, int relaxAlg,
                      int nstroke, int nstep, const double *rTips, double *rs, double *fs,
                      int *itrsums, int *iters, int nthreads,
                      int spl_n, const double *spl_xs, const double *spl_ydys)
{
    oc_relax_ctx C;
    C.spl_n = (spl_xs && spl_ydys && spl_n >= 2) ? spl_n : 0;
    C.spl_xs = spl_xs;
    C.spl_ydys = spl_ydys;
    double dcell[9];
    for (int k = 0; k < 3; k++) C.n[k] = n[k];
    oc_grid_setup(n, cell, dcell, C.dicell);
    C.gridF = gridF;
    C.maxIters = (int)params[0];
    C.convF2 = params[1];
    C.dt = params[2];
    C.damping = params[3];
    C.finc = params[4];
    C.fdec = params[5];
    C.falpha = params[6];
    C.lRadial = params[7];
    C.kRadial = params[8];
    for (int k = 0; k < 3; k++) C.rPP0[k] = params[9 + k];
    for (int k = 0; k < 3; k++) C.kSpring[k] = params[12 + k];
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(static)
    for (int s = 0; s < nstroke; s++) {
        long long off = (long long)s * nstep * 3;
        int sum = oc_relax_stroke(&C, probeStart, relaxAlg, nstep, rTips + off, rs + off, fs + off,
                                  iters ? iters + (long long)s * nstep : NULL);
        if (itrsums) itrsums[s] = sum;
    }
}

/* "valid" convolution along the last axis with np.convolve's kernel flip
 * (Fz2df, ppafm/common.py:421-430): out[j] = sum_i F[j+i] * W[nw-1-i]. */
void oc_fz2df(long long ncol, int nz, const double *F, int nw, const double *W, double scale, double *out,
              int nthreads)
{
    int nout = nz - nw + 1;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(static)
    for (long long c = 0; c < ncol; c++) {
        const double *f = F + c * nz;
        for (int j = 0; j < nout; j++) {
            double acc = 0;
            for (int i = 0; i < nw; i++) acc += f[j + i] * W[nw - 1 - i];
            out[c * nout + j] = acc * scale;
        }
    }
}

/* ------------------------------------------------- OpenCL path restated, FP32 */

/* evalLJC_QZs_noPos (FF.cl:366-423): LJ + Coulomb of four tip point charges Qs at
 * z-offsets QZs.  atoms: [na,4] (x,y,z,q); cLJ: [na,2] (c6,c12); origin/dA/dB/dC:
 * grid geometry.  Output FE[nz][ny][nx][4], x fastest (FF.cl:238-242). */
void oc_afm_ff_qzs(const int n[3], const float p0[3], const float dA[3], const float dB[3], const float dC[3],
                   int natoms, const float *atoms, const float *cLJ, const float Qs_in[4], const float QZs[4],
                   float *FE, int nthreads)
{
    const long long ntot = (long long)n[0] * n[1] * n[2];
    float Qs[4];
    for (int k = 0; k < 4; k++) Qs[k] = Qs_in[k] * OC_COULOMB_CL;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(static)
    for (long long iG = 0; iG < ntot; iG++) {
        int ia = (int)(iG % n[0]);
        int ib = (int)((iG / n[0]) % n[1]);
        int ic = (int)(iG / ((long long)n[0] * n[1]));
        float pos[3];
        for (int k = 0; k < 3; k++) pos[k] = p0[k] + dA[k] * ia + dB[k] * ib + dC[k] * ic;
        float fe[4] = {0, 0, 0, 0};
        for (int j = 0; j < natoms; j++) {
            const float *a = atoms + 4 * j;
            float dp[3] = {pos[0] - a[0], pos[1] - a[1], pos[2] - a[2]};
            float ir2 = 1.0f / (dp[0] * dp[0] + dp[1] * dp[1] + dp[2] * dp[2] + OC_R2SAFE_CL);
            float ir6 = ir2 * ir2 * ir2;
            float c6 = cLJ[2 * j], c12 = cLJ[2 * j + 1];
            float E = (c12 * ir6 - c6) * ir6;
            float fr = ((12.0f * c12 * ir6 - 6.0f * c6) * ir6 * ir2);
            fe[0] += fr * dp[0];
            fe[1] += fr * dp[1];
            fe[2] += fr * dp[2];
            fe[3] += E;
            for (int q = 0; q < 4; q++) {
                /* getCoulomb(atom, pos + (0,0,QZ)): dp = (pos + QZ) - atom */
                float d2[3] = {dp[0], dp[1], (pos[2] + QZs[q]) - a[2]};
                float jr2 = 1.0f / (d2[0] * d2[0] + d2[1] * d2[1] + d2[2] * d2[2] + OC_R2SAFE_CL);
                float Eq = a[3] * sqrtf(jr2);
                float fq = Eq * jr2;
                fe[0] += d2[0] * fq * Qs[q];
                fe[1] += d2[1] * fq * Qs[q];
                fe[2] += d2[2] * fq * Qs[q];
                fe[3] += Eq * Qs[q];
            }
        }
        for (int k = 0; k < 4; k++) FE[4 * iG + k] = fe[k];
    }
}

/* periodic trilinear on an x-fastest float4 grid at grid coordinate g */
static inline void oc_afm_interp(const float *FE, const int n[3], float gx, float gy, float gz, float out[4])
{
    float fx = floorf(gx), fy = floorf(gy), fz = floorf(gz);
    float tx = gx - fx, ty = gy - fy, tz = gz - fz;
    long long ix = (long long)fx, iy = (long long)fy, iz = (long long)fz;
    int i0 = (int)(((ix % n[0]) + n[0]) % n[0]), j0 = (int)(((iy % n[1]) + n[1]) % n[1]);
    int k0 = (int)(((iz % n[2]) + n[2]) % n[2]);
    int i1 = (i0 + 1) % n[0], j1 = (j0 + 1) % n[1], k1 = (k0 + 1) % n[2];
#define OC_A(i, j, k) (FE + 4 * (((long long)(k) * n[1] + (j)) * n[0] + (i)))
    for (int c = 0; c < 4; c++) {
        float v00 = OC_A(i0, j0, k0)[c] * (1 - tx) + OC_A(i1, j0, k0)[c] * tx;
        float v10 = OC_A(i0, j1, k0)[c] * (1 - tx) + OC_A(i1, j1, k0)[c] * tx;
        float v01 = OC_A(i0, j0, k1)[c] * (1 - tx) + OC_A(i1, j0, k1)[c] * tx;
        float v11 = OC_A(i0, j1, k1)[c] * (1 - tx) + OC_A(i1, j1, k1)[c] * tx;
        float v0 = v00 * (1 - ty) + v10 * ty;
        float v1 = v01 * (1 - ty) + v11 * ty;
        out[c] = v0 * (1 - tz) + v1 * tz;
    }
#undef OC_A
}

static inline float oc_dot3f(const float *a, const float *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

/* relaxStrokesTilted (relax.cl:391-464).  dinv: rows dinvA,dinvB,dinvC of
 * transpose(inv(cell)) (relax.py:43-47), so dot(pos,dinvA) is the fractional
 * coordinate along A.  tip: rows tipA,tipB,tipC (4 floats each, tipC[3] = -zstep).
 * stiffness (kx,ky,kz,kr), dpos0 (x,y,z,l0), relax (dt, damp, ...), surfFF (4).
 * points [npix,4]; outputs FEs/paths [npix,nz,4]; iters [npix,nz] (nullable). */
void oc_afm_relax_tilted(const float *FE, const int n[3], const float dinv[9], int npix, const float *points,
                         int nz, const float tip[12], const float stiffness[4], const float dpos0[4],
                         const float relax[4], const float surfFF[4], float *FEs, float *paths, int *iters,
                         int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(dynamic, 16)
    for (int ip = 0; ip < npix; ip++) {
        const float *tA = tip, *tB = tip + 4, *tC = tip + 8;
        float dTip[3] = {tC[0] * tC[3], tC[1] * tC[3], tC[2] * tC[3]};
        float d0[3];
        for (int k = 0; k < 3; k++) d0[k] = tA[k] * dpos0[0] + tB[k] * dpos0[1] + tC[k] * dpos0[2];
        float tipPos[3] = {points[4 * ip], points[4 * ip + 1], points[4 * ip + 2]};
        float pos[3] = {tipPos[0] + d0[0], tipPos[1] + d0[1], tipPos[2] + d0[2]};
        float dt = relax[0], damp = relax[1];
        const float dtmax = dt, dtmin = dtmax * 0.1f, damp0 = damp;
        for (int iz = 0; iz < nz; iz++) {
            float fe[4] = {0, 0, 0, 0};
            float v[3] = {0, 0, 0};
            int it;
            for (it = 0; it < OC_NRELAX_CL; it++) {
                float g[3] = {oc_dot3f(pos, dinv) * n[0], oc_dot3f(pos, dinv + 3) * n[1],
                              oc_dot3f(pos, dinv + 6) * n[2]};
                oc_afm_interp(FE, n, g[0], g[1], g[2], fe);
                float f[3] = {fe[0], fe[1], fe[2]};
                float dp[3] = {pos[0] - tipPos[0], pos[1] - tipPos[1], pos[2] - tipPos[2]};
                float dpt[3] = {oc_dot3f(dp, tA), oc_dot3f(dp, tB), oc_dot3f(dp, tC)};
                float r = sqrtf(oc_dot3f(dpt, dpt));
                float ft[3];
                for (int k = 0; k < 3; k++)
                    ft[k] = (dpt[k] - dpos0[k]) * stiffness[k] + dpt[k] * (stiffness[3] * (r - dpos0[3]) / r);
                for (int k = 0; k < 3; k++) f[k] += tA[k] * ft[0] + tB[k] * ft[1] + tC[k] * ft[2];
                for (int k = 0; k < 3; k++) f[k] += tC[k] * surfFF[0];
                float ff = oc_dot3f(f, f), vv = oc_dot3f(v, v), vf = oc_dot3f(v, f);
                if (vf < 0) {
                    v[0] = v[1] = v[2] = 0;
                    dt = fmaxf(dtmin, dt * OC_FTDEC);
                    damp = damp0;
                } else {
                    float cf = damp * sqrtf(vv / (ff + OC_F2SAFE));
                    for (int k = 0; k < 3; k++) v[k] = v[k] * (1 - damp) + f[k] * cf;
                    dt = fminf(dtmax, dt * OC_FTINC);
                    damp *= OC_FDAMP;
                }
                for (int k = 0; k < 3; k++) v[k] += f[k] * dt;
                for (int k = 0; k < 3; k++) pos[k] += v[k] * dt;
                if (ff < OC_F2CONV_CL) break;
            }
            long long ind = (long long)ip * nz + iz;
            FEs[4 * ind + 0] = oc_dot3f(fe, tA);
            FEs[4 * ind + 1] = oc_dot3f(fe, tB);
            FEs[4 * ind + 2] = oc_dot3f(fe, tC);
            FEs[4 * ind + 3] = fe[3];
            paths[4 * ind + 0] = pos[0];
            paths[4 * ind + 1] = pos[1];
            paths[4 * ind + 2] = pos[2];
            paths[4 * ind + 3] = 0;
            if (iters) iters[ind] = it;
            for (int k = 0; k < 3; k++) tipPos[k] += dTip[k];
            for (int k = 0; k < 3; k++) pos[k] += dTip[k];
        }
    }
}

/* convolveZ (relax.cl:571-608): Fout[p][o] = sum_j Fin[p][o+j] * W[j], no flip. */
void oc_afm_convolve_z(int npix, int nzin, int nzout, const float *Fin, const float *W, float *Fout, int nthreads)
{
    int nw = nzin - nzout + 1;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(static)
    for (int p = 0; p < npix; p++) {
        for (int o = 0; o < nzout; o++) {
            float acc[4] = {0, 0, 0, 0};
            for (int j = 0; j < nw; j++)
                for (int c = 0; c < 4; c++) acc[c] += Fin[4 * ((long long)p * nzin + o + j) + c] * W[j];
            for (int c = 0; c < 4; c++) Fout[4 * ((long long)p * nzout + o) + c] = acc[c];
        }
    }
}

int oc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
