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
#include <string>
#include <vector>

#include "pp_common.cuh"
#include "pp_df.cuh"
#include "pp_relax_dev.cuh"

namespace ppgpu {

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

// --------------------------------------------------------- CPU-core semantics

// Scan mode keeps a per-height table in shared memory: (z, g_z0, g_z1, g_z2) as
// double-floats, g_z = dic . (0, 0, z), so a height change needs no float64.
constexpr int ZTAB = 4;

// TPS lanes per stroke (1, 2, 4 or 8): the lanes of a group hold the same state and split
// each trilinear gather (interp_force_df_group, bit-identical to one lane); lane 0 of the
// group writes the outputs.  More lanes per stroke put more warps in flight when a scan has
// few strokes, which is what bounds this kernel.
template <bool SCAN, int TPS, bool SPL>
__global__ void __launch_bounds__(RELAX_THREADS) relax_kernel(const RelaxPrm P, const StrokeIO S, const ScanIO C) {
    extern __shared__ dfl ztab[];
    const int s = (blockIdx.x * RELAX_THREADS + threadIdx.x) / TPS;
    const int sub = (int)(threadIdx.x % TPS);
    const bool lead = sub == 0;
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
            grid_of(P.dic, P.diag, tip, g);
        }
        tip_cell(g, base, tf);
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
            grid_of(P.dic, P.diag, r, gxy);
        }
        set_height(0);
    }

    unsigned am;
    while ((am = __ballot_sync(FULL, active)) != 0u) {
        if (!active) continue;
        dfl u[3], F[3];
        grid_coord_df(P.dic, P.diag, tf, d, u);
        interp_force_df_group<TPS>(P.FE, P.n0, P.n1, P.n2, base, u, F, sub, am);
        if (fin) {
            // outputs of height iz: position after the last move, grid force there
            const dfl r[3] = {df_add(tip[0], d[0]), df_add(tip[1], d[1]), df_add(tip[2], d[2])};
            if (!lead) {
            } else if (SCAN) {
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
                if (!SCAN && S.itrsum && lead) S.itrsum[s] = itsum;
                if (SCAN && C.df && C.fzs && C.nw > 0 && lead) {
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
        const float3 f = pp_force_df<SPL>(P, F, d);
        const float ff = relax_move_df(P, f, d, v, dt, acoef);
        mine += lead ? 1 : 0;
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

constexpr int AFM_RELAX_THREADS = 128;  // as the single-grid kernel: packs beside the next image's force field

__global__ void __launch_bounds__(AFM_RELAX_THREADS) relax_afm_kernel(const AfmPrm P) {
    const int p = blockIdx.x * AFM_RELAX_THREADS + threadIdx.x;
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

TipSpline g_tip_spline = {0, nullptr, nullptr};
static void *g_spline_mem = nullptr;
static std::vector<double> g_spline_xs, g_spline_ydys;  // host copies (for save/restore)

// Uploads the spline tables (see TipSpline); n == 0 clears.  cudaFree of the previous tables
// waits for the kernels that may still read them.
static int upload_tip_spline(int n, const double *xs, const double *ydys) {
    if (n == 0 || !xs || !ydys) {
        if (g_spline_mem) cudaFree(g_spline_mem);
        g_spline_mem = nullptr;
        g_tip_spline = {0, nullptr, nullptr};
        g_spline_xs.clear();
        g_spline_ydys.clear();
        return set_ok();
    }
    if (n < 2) return set_error(PPGPU_ERR_ARG, "tip spline: %d knots (at least 2)", n);
    std::vector<dfl> tab((size_t)n + 6 * (size_t)(n - 1));
    for (int i = 0; i < n; i++) tab[i] = df_from(xs[i]);
    for (int i = 0; i < n - 1; i++) {
        const double x0 = xs[i], dx = xs[i + 1] - x0, denom = 1 / dx;
        const double y0 = ydys[2 * i], y1 = ydys[2 * i + 2], dy0 = ydys[2 * i + 1] * dx, dy1 = ydys[2 * i + 3] * dx;
        const double y01 = y0 - y1;
        const double c[6] = {x0, denom, y0, dy0, -3 * y01 - 2 * dy0 - dy1, 2 * y01 + dy0 + dy1};
        for (int k = 0; k < 6; k++) tab[n + 6 * i + k] = df_from(c[k]);
    }
    void *mem = nullptr;
    cudaError_t e = cudaMalloc(&mem, tab.size() * sizeof(dfl));
    if (e != cudaSuccess) return cuda_fail(e, "tip spline tables");
    e = cudaMemcpy(mem, tab.data(), tab.size() * sizeof(dfl), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(mem);
        return cuda_fail(e, "tip spline upload");
    }
    if (g_spline_mem) cudaFree(g_spline_mem);
    g_spline_mem = mem;
    g_tip_spline = {n, (const dfl *)mem, (const dfl *)mem + n};
    g_spline_xs.assign(xs, xs + n);
    g_spline_ydys.assign(ydys, ydys + 2 * (size_t)n);
    return set_ok();
}

// Runs fn with the tip spline (n, xs, ydys) in place of the current one, then restores it.
int with_tip_spline(int n, const double *xs, const double *ydys, int (*fn)(void *), void *arg) {
    std::vector<double> sx = g_spline_xs, sy = g_spline_ydys;
    const int n0 = (int)sx.size();
    int s = upload_tip_spline(n, xs, ydys);
    if (s) return s;
    s = fn(arg);
    const std::string msg = s ? std::string(ppgpu_last_error()) : std::string();
    const int st = s ? ppgpu_last_status() : 0;
    const int r = upload_tip_spline(n0, n0 ? sx.data() : nullptr, n0 ? sy.data() : nullptr);
    if (s) return set_error(st, "%s", msg.c_str());
    return r;
}

// Lanes per stroke (ppgpu_set_relax_tps).  One lane per stroke is the default: on GB300 the
// scans measured here (16k-26k strokes) ran 15-20 % slower with 4 lanes per stroke, because
// every lane of a group also executes the stroke's FIRE arithmetic, which outweighs the
// latency hidden by the extra warps.
static int g_relax_tps = 1;

static int relax_tps(long long) { return g_relax_tps; }

template <bool SCAN, bool SPL>
static void launch_relax_t(int tps, unsigned nblk, size_t smem, cudaStream_t st, const RelaxPrm &P, const StrokeIO &S,
                           const ScanIO &C) {
    switch (tps) {
    case 8: relax_kernel<SCAN, 8, SPL><<<nblk, RELAX_THREADS, smem, st>>>(P, S, C); break;
    case 4: relax_kernel<SCAN, 4, SPL><<<nblk, RELAX_THREADS, smem, st>>>(P, S, C); break;
    case 2: relax_kernel<SCAN, 2, SPL><<<nblk, RELAX_THREADS, smem, st>>>(P, S, C); break;
    default: relax_kernel<SCAN, 1, SPL><<<nblk, RELAX_THREADS, smem, st>>>(P, S, C); break;
    }
}

template <bool SCAN>
static void launch_relax(int tps, long long nstroke, size_t smem, cudaStream_t st, const RelaxPrm &P, const StrokeIO &S,
                         const ScanIO &C) {
    const unsigned nblk = (unsigned)((nstroke * tps + RELAX_THREADS - 1) / RELAX_THREADS);
    if (P.spl.n > 0)
        launch_relax_t<SCAN, true>(tps, nblk, smem, st, P, S, C);
    else
        launch_relax_t<SCAN, false>(tps, nblk, smem, st, P, S, C);
}

}  // namespace ppgpu

using namespace ppgpu;

extern "C" int ppgpu_set_relax_tps(int tps) {
    if (tps != 0 && tps != 1 && tps != 2 && tps != 4 && tps != 8)
        return set_error(PPGPU_ERR_ARG, "set_relax_tps: %d not in {0 (default), 1, 2, 4, 8}", tps);
    g_relax_tps = tps ? tps : 1;
    return set_ok();
}

extern "C" int ppgpu_set_tip_spline(int n, const double *xs, const double *ydys) {
    if (n < 0) return set_error(PPGPU_ERR_ARG, "set_tip_spline: negative knot count");
    return upload_tip_spline(n, xs, ydys);
}

extern "C" int ppgpu_get_relax_tps(long long nstroke, int *out) {
    if (!out || nstroke < 0) return set_error(PPGPU_ERR_ARG, "get_relax_tps: bad arguments");
    *out = relax_tps(nstroke);
    return set_ok();
}

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
    launch_relax<false>(relax_tps(nstroke), nstroke, 0, (cudaStream_t)stream, P, S, C);
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
    const size_t smem = (size_t)nz * ZTAB * sizeof(dfl);
    if (smem > 48 * 1024) return set_error(PPGPU_ERR_ARG, "relax_scan: nz = %d heights exceed the table limit (1536)", nz);
    launch_relax<true>(relax_tps(npix), npix, smem, (cudaStream_t)stream, P, S, C);
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
    const unsigned nblk = (unsigned)((npix + AFM_RELAX_THREADS - 1) / AFM_RELAX_THREADS);
    relax_afm_kernel<<<nblk, AFM_RELAX_THREADS, 0, (cudaStream_t)stream>>>(P);
    PPGPU_CHECK_LAUNCH("relax_afm_kernel");
    return set_ok();
}
