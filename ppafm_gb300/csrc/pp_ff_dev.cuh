// pp_ff_dev.cuh -- device side of the force-field kernels (shared by the single-grid
// kernels of pp_ff.cu and the batched persistent kernel of pp_batch.cu).
//
// See pp_ff.cu for the design notes; the reference functions are cited there.
#pragma once

#include <cstdint>

#include "pp_common.cuh"

namespace ppgpu {

constexpr int FF_THREADS = 256;   // CTA of the persistent batched kernel (the single-grid kernel
                                  // picks 128 or 256 per call, pp_ff.cu)
constexpr int FF_TILE = 256;       // atoms per shared-memory stage
constexpr int FF_REC = 3;          // float4 per atom record
constexpr float R2CAP = 1e-4f;     // slow-path floor of r^2 (A^2)
constexpr int SPLIT_MAX_CHARGED = 1024;  // LJC: charged atoms summed single-level up to this
constexpr int FF_MAX_P = 8;               // points per thread (z run), at most

enum { M_LJ = 0, M_COUL = 1, M_LJC = 2, M_QZS = 3 };

struct FFParams {
    float4 *FE;
    const float4 *atoms;
    int natoms, ncharged;
    int i0[3], ns[3];
    double dA[3], dB[3], dC[3];
    float eps;
    double eps64;
    float Q, Fmax;
    float Qs[4], QZs[4];  // tip charges (times k_e) and their z offsets: the charges off the
                          // central point (QZ != 0), whose differences the fast kernel sums
    float QZn2[4], QZnsq[4];  // -2 QZ and -QZ^2
    float Qsum;               // all tip charges (times k_e)
    int nq;
    float Qa[4], QZa[4];  // every nonzero tip charge and offset (the plain sums: float64, slow path)
    int nqa;
    int accumulate;
    long long nchunks;
    int nzc;
    int *err;
    float off[3][FF_MAX_P];  // float(dC[c] * i): offsets of a thread's points from its first one
};

// Fills prm.off from prm.dC (host).
inline void ff_set_offsets(FFParams &prm) {
    for (int c = 0; c < 3; c++)
        for (int i = 0; i < FF_MAX_P; i++) prm.off[c][i] = (float)(prm.dC[c] * i);
}

// ------------------------------------------------------------------ TMA helpers

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
// L2 policy for data streamed through once (evicted before the data kept for reuse).
__device__ __forceinline__ uint64_t l2_evict_first() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
// bulk_g2s with an L2 cache policy.
__device__ __forceinline__ void bulk_g2s_hint(void *dst, const void *src, uint32_t bytes, uint64_t *bar, uint64_t pol) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(pol)
        : "memory");
}
// 16-byte global store with an L2 cache policy.
__device__ __forceinline__ void st16_hint(void *p, int4 v, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.v4.b32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(p), "r"(v.x), "r"(v.y), "r"(v.z),
                 "r"(v.w), "l"(pol)
                 : "memory");
}
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Bounded wait (about 2 s of wall time) on an mbarrier phase.
static __device__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (uint32_t i = 0; i < (1u << 26); i++) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((i & 255u) == 255u && global_ns() - t0 > 2000000000ull) break;
    }
    return false;
}

// ------------------------------------------------------------- pair interactions
//
// Atom record (48 B, written by ppgpu_pack_atoms), coordinates relative to the grid origin:
//   r0 = (-x_hi, -y_hi, -x_lo, -y_lo)   r1 = (-z_hi, -z_lo, -6 c6, 12 c12)   r2 = (-c6, c12, kqq, 0)
// The negated coordinates make the hi/lo displacement p - R a pair of packed adds, and the
// LJ force factor 12 c12 ir6 - 6 c6 one fused multiply-add.
//
// Arithmetic is done on pairs of grid points with the packed float32x2 instructions
// (fma.rn.f32x2 & co.), which issue two lanes' worth of FP32 work per instruction.

__device__ __forceinline__ float2 bc(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 rcp2(float2 v) { return make_float2(rcp_approx(v.x), rcp_approx(v.y)); }
__device__ __forceinline__ float2 rsqrt2(float2 v) { return make_float2(rsqrt_approx(v.x), rsqrt_approx(v.y)); }

// Accumulators for P2 pairs of points: force components and energy.
template <int P2>
struct Acc {
    float2 x[P2], y[P2], z[P2], e[P2];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int p = 0; p < P2; p++) x[p] = y[p] = z[p] = e[p] = make_float2(0.f, 0.f);
    }
    __device__ __forceinline__ void fold_from(Acc &a) {
#pragma unroll
        for (int p = 0; p < P2; p++) {
            x[p] = add2(x[p], a.x[p]);
            y[p] = add2(y[p], a.y[p]);
            z[p] = add2(z[p], a.z[p]);
            e[p] = add2(e[p], a.e[p]);
        }
        a.zero();
    }
};

// This thread's P2 pairs of points: hi/lo coordinates of the first point and offsets.
template <int P2>
struct Pts {
    float2 hxy, lxy;
    float hz, lz;
    float2 ox[P2], oy[P2], oz[P2];
};

// Per-atom displacement to the first point and the shared in-plane terms.
struct AtomGeo {
    float2 dxv, dyv, dz0v, dxy2v;
};

template <int P2>
__device__ __forceinline__ AtomGeo atom_geo(const Pts<P2> &q, const float4 &r0, const float4 &r1, float eps) {
    const float2 dxy = add2(add2(q.hxy, make_float2(r0.x, r0.y)), add2(q.lxy, make_float2(r0.z, r0.w)));
    const float dz0 = (q.hz + r1.x) + (q.lz + r1.y);
    AtomGeo g;
    g.dxv = bc(dxy.x);
    g.dyv = bc(dxy.y);
    g.dz0v = bc(dz0);
    g.dxy2v = bc(fmaf(dxy.x, dxy.x, fmaf(dxy.y, dxy.y, eps)));
    return g;
}

// Displacement of pair p and its r^2.
template <bool ORTHO, int P2>
__device__ __forceinline__ void pair_geo(const Pts<P2> &q, const AtomGeo &g, int p, float eps, float2 &dx, float2 &dy,
                                         float2 &dz, float2 &r2) {
    dz = add2(g.dz0v, q.oz[p]);
    if (ORTHO) {
        dx = g.dxv;
        dy = g.dyv;
        r2 = fma2(dz, dz, g.dxy2v);
    } else {
        dx = add2(g.dxv, q.ox[p]);
        dy = add2(g.dyv, q.oy[p]);
        r2 = fma2(dz, dz, fma2(dy, dy, fma2(dx, dx, bc(eps))));
    }
}

// LJ (Forces.h:120-132) of one atom on pair p, from ir2 = 1/r^2.
template <bool WITH_E, int P2>
__device__ __forceinline__ void lj_ir2(float2 ir2, float2 dx, float2 dy, float2 dz, float2 c6n6, float2 c12x12,
                                       float2 c6n, float2 c12, Acc<P2> &a, int p) {
    const float2 ir6 = mul2(mul2(ir2, ir2), ir2);
    const float2 fr = mul2(fma2(c12x12, ir6, c6n6), mul2(ir6, ir2));  // (12 c12 ir6 - 6 c6) ir8
    a.x[p] = fma2(fr, dx, a.x[p]);
    a.y[p] = fma2(fr, dy, a.y[p]);
    a.z[p] = fma2(fr, dz, a.z[p]);
    if (WITH_E) a.e[p] = fma2(fma2(c12, ir6, c6n), ir6, a.e[p]);  // c12 ir12 - c6 ir6
}

// LJ + Coulomb of one charged atom on pair p from ir = 1/r: ir^3 is formed once and serves
// both, ir^6 = (ir^3)^2 for the LJ powers and kqq ir^3 for the Coulomb factor (the energy,
// when wanted, adds kqq ir): 7 multiplies/FMAs before the six accumulations.
template <bool WITH_E, int P2>
__device__ __forceinline__ void ljc_ir(float2 ir, float2 dx, float2 dy, float2 dz, float2 c6n6, float2 c12x12,
                                       float2 c6n, float2 c12, float2 kqq, Acc<P2> &a, Acc<P2> &u, int p) {
    const float2 ir2 = mul2(ir, ir);
    const float2 ir3 = mul2(ir, ir2);
    const float2 ir6 = mul2(ir3, ir3);
    const float2 fr = mul2(fma2(c12x12, ir6, c6n6), mul2(ir6, ir2));  // (12 c12 ir6 - 6 c6) ir8
    a.x[p] = fma2(fr, dx, a.x[p]);
    a.y[p] = fma2(fr, dy, a.y[p]);
    a.z[p] = fma2(fr, dz, a.z[p]);
    if (WITH_E) a.e[p] = fma2(fma2(c12, ir6, c6n), ir6, a.e[p]);
    const float2 fq = mul2(kqq, ir3);
    u.x[p] = fma2(fq, dx, u.x[p]);
    u.y[p] = fma2(fq, dy, u.y[p]);
    u.z[p] = fma2(fq, dz, u.z[p]);
    if (WITH_E) u.e[p] = fma2(kqq, ir, u.e[p]);
}

// Coulomb (Forces.h:237-244) of one atom on pair p, from ir = 1/r.
template <bool WITH_E, int P2>
__device__ __forceinline__ void coul_ir(float2 ir, float2 ir2, float2 dx, float2 dy, float2 dz, float2 kqq,
                                        Acc<P2> &a, int p) {
    const float2 eq = mul2(kqq, ir);
    const float2 fq = mul2(eq, ir2);
    a.x[p] = fma2(fq, dx, a.x[p]);
    a.y[p] = fma2(fq, dy, a.y[p]);
    a.z[p] = fma2(fq, dz, a.z[p]);
    if (WITH_E) a.e[p] = add2(a.e[p], eq);
}

// The AFMulator tip charges (FF.cl:366-423): sum_k Qs_k Coulomb(dz + QZ_k) of one atom.
// Written as Qsum*C(dz) + sum_k Qs_k [C(dz + QZ_k) - C(dz)] with the differences in a
// cancellation-free form, because a neutral multipole tip (e.g. -10, +20, -10 e at
// +-0.1 A) otherwise loses ~(r/QZ)^2 of the float32 significand.
template <bool WITH_E, int P2>
__device__ __forceinline__ void qzs_tip(const FFParams &prm, float q, float2 r2, float2 dx, float2 dy, float2 dz,
                                        float2 dxy2, Acc<P2> &a, int p) {
    const float2 ir0 = rsqrt2(r2);
    const float2 a0 = mul2(r2, ir0);
    const float2 ir03 = mul2(mul2(ir0, ir0), ir0);
    if (prm.Qsum != 0.f) {
        const float2 w = bc(q * prm.Qsum);
        const float2 f = mul2(w, ir03);
        a.x[p] = fma2(f, dx, a.x[p]);
        a.y[p] = fma2(f, dy, a.y[p]);
        a.z[p] = fma2(f, dz, a.z[p]);
        if (WITH_E) a.e[p] = fma2(w, ir0, a.e[p]);
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (k < prm.nq) {
            const float2 dq = add2(dz, bc(prm.QZs[k]));
            const float2 r2q = fma2(dq, dq, dxy2);
            const float2 irq = rsqrt2(r2q);
            const float2 aq = mul2(r2q, irq);
            const float2 num = fma2(bc(prm.QZn2[k]), dz, bc(prm.QZnsq[k]));  // r0^2 - rq^2 = -(2 dz QZ + QZ^2)
            const float2 da = mul2(num, rcp2(add2(a0, aq)));                  // a0 - aq
            const float2 d1 = mul2(da, mul2(ir0, irq));                      // 1/aq - 1/a0
            const float2 irq3 = mul2(mul2(irq, irq), irq);
            const float2 s3 = add2(add2(r2, r2q), mul2(a0, aq));              // a0^2 + a0 aq + aq^2
            const float2 d3 = mul2(mul2(da, s3), mul2(ir03, irq3));           // 1/aq^3 - 1/a0^3
            const float2 w = bc(q * prm.Qs[k]);
            const float2 wd3 = mul2(w, d3);
            a.x[p] = fma2(wd3, dx, a.x[p]);
            a.y[p] = fma2(wd3, dy, a.y[p]);
            a.z[p] = fma2(w, fma2(dz, d3, mul2(bc(prm.QZs[k]), irq3)), a.z[p]);  // (dz+QZ)/aq^3 - dz/a0^3
            if (WITH_E) a.e[p] = fma2(w, d1, a.e[p]);
        }
    }
}

// Overflow-safe |F| <= Fmax clamp preserving direction (io.py:766-778).  A vector whose
// largest component m is below 0.57 Fmax is left as it is without the division and root:
// |F| <= sqrt(3) m < 0.9873 Fmax, so the full test below would not clamp it either (its
// rounded root exceeds sqrt(3) m by a few ulps at most).
__device__ __forceinline__ void clamp_vec(float &x, float &y, float &z, float Fmax) {
    const float m = fmaxf(fabsf(x), fmaxf(fabsf(y), fabsf(z)));
    if (!(m > 0.f) || m < 0.57f * Fmax) return;
    const float s = 1.f / m;
    const float sx = x * s, sy = y * s, sz = z * s;
    const float fr = m * sqrtf(sx * sx + sy * sy + sz * sz);
    if (fr > Fmax) {
        const float k = Fmax / fr;
        x *= k;
        y *= k;
        z *= k;
    }
}

__device__ __forceinline__ bool finite4(const float4 &v) {
    return isfinite(v.x) && isfinite(v.y) && isfinite(v.z) && isfinite(v.w);
}

// Final value of one point from its LJ-or-total sums t and (LJC) electrostatic sums u.
template <int MODE, bool WITH_E>
__device__ __forceinline__ float4 finalize(float tx, float ty, float tz, float te, float ux, float uy, float uz,
                                           float ue, const FFParams &prm) {
    float4 o;
    if (MODE == M_LJC) {
        if (prm.Fmax > 0.f) {
            clamp_vec(tx, ty, tz, prm.Fmax);
            clamp_vec(ux, uy, uz, prm.Fmax);
        }
        o.x = fmaf(prm.Q, ux, tx);
        o.y = fmaf(prm.Q, uy, ty);
        o.z = fmaf(prm.Q, uz, tz);
        o.w = WITH_E ? fmaf(prm.Q, ue, te) : 0.f;
    } else {
        o = make_float4(tx, ty, tz, WITH_E ? te : 0.f);
    }
    return o;
}

// Slow path for one point: all atoms from global memory, scalar, r^2 floored at R2CAP.
template <int MODE, bool WITH_E>
__device__ float4 point_slow(const FFParams &prm, double px, double py, double pz) {
    const float hx = __double2float_rn(px), hy = __double2float_rn(py), hz = __double2float_rn(pz);
    const float lx = __double2float_rn(px - (double)hx), ly = __double2float_rn(py - (double)hy),
                lz = __double2float_rn(pz - (double)hz);
    float t[4] = {0, 0, 0, 0}, u[4] = {0, 0, 0, 0};
    const int nat = (MODE == M_COUL) ? prm.ncharged : prm.natoms;
    for (int j = 0; j < nat; j++) {
        const float4 r0 = prm.atoms[3 * j], r1 = prm.atoms[3 * j + 1], r2r = prm.atoms[3 * j + 2];
        const float dx = (hx + r0.x) + (lx + r0.z);
        const float dy = (hy + r0.y) + (ly + r0.w);
        const float dz = (hz + r1.x) + (lz + r1.y);
        const float dxy2 = fmaf(dx, dx, fmaf(dy, dy, prm.eps));
        const float r2 = fmaxf(fmaf(dz, dz, dxy2), R2CAP);
        const bool charged = j < prm.ncharged;
        if (MODE != M_COUL) {
            const float ir2 = 1.f / r2, ir6 = ir2 * ir2 * ir2;
            const float fr = fmaf(r1.w, ir6, r1.z) * (ir6 * ir2);
            t[0] = fmaf(fr, dx, t[0]);
            t[1] = fmaf(fr, dy, t[1]);
            t[2] = fmaf(fr, dz, t[2]);
            t[3] = fmaf(fmaf(r2r.y, ir6, r2r.x), ir6, t[3]);
        }
        if ((MODE == M_COUL || MODE == M_LJC) && charged) {
            const float ir = rsqrtf(r2);
            const float eq = r2r.z * ir, fq = eq * ir * ir;
            float *a = (MODE == M_LJC) ? u : t;
            a[0] = fmaf(fq, dx, a[0]);
            a[1] = fmaf(fq, dy, a[1]);
            a[2] = fmaf(fq, dz, a[2]);
            a[3] += eq;
        }
        if (MODE == M_QZS && charged) {
            for (int k = 0; k < prm.nqa; k++) {
                const float dq = dz + prm.QZa[k];
                const float rq = fmaxf(fmaf(dq, dq, dxy2), R2CAP);
                const float ir = rsqrtf(rq);
                const float eq = r2r.z * ir * prm.Qa[k], fq = eq * ir * ir;
                t[0] = fmaf(fq, dx, t[0]);
                t[1] = fmaf(fq, dy, t[1]);
                t[2] = fmaf(fq, dq, t[2]);
                t[3] += eq;
            }
        }
    }
    return finalize<MODE, WITH_E>(t[0], t[1], t[2], t[3], u[0], u[1], u[2], u[3], prm);
}

// The force-field kernel.  SPLIT (LJC only): the atom tiles that hold charged atoms are
// summed single-level into the totals and the electrostatic sums are then parked in the
// output slots of this thread's points, so the long neutral-atom phase holds only the
// LJ partial and total sums (used when the charged atoms are at most SPLIT_MAX_CHARGED
// and the output is not accumulated).
//
// ff_block computes the points of block `blk` (NT chunks of P points; NT = the CTA's threads) of the grid
// described by prm.  The shared stages and their mbarriers belong to the calling kernel and
// are initialised once per kernel; T counts the atom tiles this CTA has consumed so far
// (stage = T & 1, mbarrier phase parity = (T >> 1) & 1), so a persistent CTA can run many
// blocks back to back.  Returns false if an atom tile never landed (device error raised).
struct FFShared {
    float4 at[2][FF_TILE * FF_REC];
    uint64_t bar[2];
    int abort_flag;
};

__device__ __forceinline__ void ff_shared_init(FFShared &sh) {
    if (threadIdx.x == 0) {
        mbar_init(&sh.bar[0], 1);
        mbar_init(&sh.bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
}

// ALLQ (SPLIT only): every atom is charged, so there is no neutral phase and the electrostatic
// sums stay in registers instead of waiting in the output slots.
template <int MODE, bool WITH_E, bool ORTHO, int P2, bool SPLIT, int NT = FF_THREADS, bool ALLQ = false>
__device__ __forceinline__ bool ff_block(const FFParams &prm, long long blk, FFShared &sh, uint32_t &T) {
    static_assert(!ALLQ || (MODE == M_LJC && SPLIT), "ALLQ is a form of the split LJ + Coulomb block");
    constexpr int P = 2 * P2;
    auto &s_at = sh.at;
    uint64_t *s_bar = sh.bar;
    int &s_abort = sh.abort_flag;
    const uint32_t T0 = T;

    const int tid = threadIdx.x;
    const long long chunk = blk * NT + tid;
    const bool valid = chunk < prm.nchunks;

    // ---- this thread's points: column (ga, gb), z points gc0 .. gc0+P-1
    int la = 0, lb = 0, lz0 = 0;
    if (valid) {
        const long long col = chunk / prm.nzc;
        lz0 = (int)(chunk - col * prm.nzc) * P;
        la = (int)(col / prm.ns[1]);
        lb = (int)(col - (long long)la * prm.ns[1]);
    }
    const double ga = prm.i0[0] + la, gb = prm.i0[1] + lb, gc = prm.i0[2] + lz0;
    double pd[3];
#pragma unroll
    for (int k = 0; k < 3; k++) pd[k] = ((prm.dA[k] * ga) + prm.dB[k] * gb) + prm.dC[k] * gc;
    Pts<P2> q;
    {
        const float hx = __double2float_rn(pd[0]), hy = __double2float_rn(pd[1]), hz = __double2float_rn(pd[2]);
        q.hxy = make_float2(hx, hy);
        q.lxy = make_float2(__double2float_rn(pd[0] - (double)hx), __double2float_rn(pd[1] - (double)hy));
        q.hz = hz;
        q.lz = __double2float_rn(pd[2] - (double)hz);
#pragma unroll
        for (int p = 0; p < P2; p++) {
            q.ox[p] = make_float2(prm.off[0][2 * p], prm.off[0][2 * p + 1]);
            q.oy[p] = make_float2(prm.off[1][2 * p], prm.off[1][2 * p + 1]);
            q.oz[p] = make_float2(prm.off[2][2 * p], prm.off[2][2 * p + 1]);
        }
    }

    Acc<P2> tot, acc;
    tot.zero();
    acc.zero();
    Acc<(MODE == M_LJC) ? P2 : 1> el;  // LJC electrostatic sums
    el.zero();
    Acc<(MODE == M_LJC && !SPLIT) ? P2 : 1> elacc;
    elacc.zero();

    const int nat = (MODE == M_COUL) ? prm.ncharged : prm.natoms;
    const int ntiles = (nat + FF_TILE - 1) / FF_TILE;
    const float eps = prm.eps;

    T = T0 + ntiles;
    // tile t of this block lives in stage (T0 + t) & 1 and completes phase ((T0 + t) >> 1) & 1
    auto stage = [&](int t) { return (int)((T0 + (uint32_t)t) & 1u); };
    auto parity = [&](int t) { return (uint32_t)(((T0 + (uint32_t)t) >> 1) & 1u); };
    if (tid == 0) {
        s_abort = 0;
        for (int t = 0; t < 2 && t < ntiles; t++) {
            const int nj = min(FF_TILE, nat - t * FF_TILE);
            const uint32_t bytes = (uint32_t)nj * FF_REC * 16u;
            mbar_expect_tx(&s_bar[stage(t)], bytes);
            bulk_g2s(&s_at[stage(t)][0], prm.atoms + (size_t)t * FF_TILE * FF_REC, bytes, &s_bar[stage(t)]);
        }
    }
    __syncthreads();

    // Waits for tile t; false (after a bounded drain) if the copy never landed.
    auto acquire = [&](int t) -> bool {
        if (tid == 0) {
            if (!mbar_wait_bounded(&s_bar[stage(t)], parity(t))) s_abort = 1;
        }
        __syncthreads();
        if (s_abort) {
            if (tid == 0) {
                raise_device_error(prm.err, PPGPU_ERR_DEVICE_TIMEOUT);
                for (int u = t; u < t + 2 && u < ntiles; u++) mbar_wait_bounded(&s_bar[stage(u)], parity(u));
            }
            return false;
        }
        return true;
    };
    // Frees the stage of tile t and starts the copy of tile t + 2 into it.
    auto release = [&](int t) {
        __syncthreads();
        if (tid == 0 && t + 2 < ntiles) {
            const int nj2 = min(FF_TILE, nat - (t + 2) * FF_TILE);
            const uint32_t bytes = (uint32_t)nj2 * FF_REC * 16u;
            mbar_expect_tx(&s_bar[stage(t)], bytes);
            bulk_g2s(&s_at[stage(t)][0], prm.atoms + (size_t)(t + 2) * FF_TILE * FF_REC, bytes, &s_bar[stage(t)]);
        }
    };

    // LJ of atoms [j0, j1) of a tile into accumulator set a (rcp path).
    auto run_lj = [&](const float4 *S, int j0, int j1, Acc<P2> &a) {
        for (int j = j0; j < j1; j++) {
            const float4 r0 = S[3 * j], r1 = S[3 * j + 1];
            float2 c6n = bc(0.f), c12 = bc(0.f);
            if (WITH_E) {
                const float4 r2r = S[3 * j + 2];
                c6n = bc(r2r.x);
                c12 = bc(r2r.y);
            }
            const AtomGeo g = atom_geo<P2>(q, r0, r1, eps);
            const float2 c6n6 = bc(r1.z), c12x12 = bc(r1.w);
#pragma unroll
            for (int p = 0; p < P2; p++) {
                float2 dx, dy, dz, r2;
                pair_geo<ORTHO, P2>(q, g, p, eps, dx, dy, dz, r2);
                lj_ir2<WITH_E, P2>(rcp2(r2), dx, dy, dz, c6n6, c12x12, c6n, c12, a, p);
            }
        }
    };
    // LJ + Coulomb of charged atoms [j0, j1) (rsqrt path) into a (LJ) and u (electrostatic).
    auto run_ljc = [&](const float4 *S, int j0, int j1, Acc<P2> &a, auto &u) {
        for (int j = j0; j < j1; j++) {
            const float4 r0 = S[3 * j], r1 = S[3 * j + 1], r2r = S[3 * j + 2];
            const AtomGeo g = atom_geo<P2>(q, r0, r1, eps);
            const float2 c6n6 = bc(r1.z), c12x12 = bc(r1.w), c6n = bc(r2r.x), c12 = bc(r2r.y), kqq = bc(r2r.z);
#pragma unroll
            for (int p = 0; p < P2; p++) {
                float2 dx, dy, dz, r2;
                pair_geo<ORTHO, P2>(q, g, p, eps, dx, dy, dz, r2);
                ljc_ir<WITH_E, P2>(rsqrt2(r2), dx, dy, dz, c6n6, c12x12, c6n, c12, kqq, a, u, p);
            }
        }
    };

    if constexpr (MODE == M_LJC && SPLIT) {
        const int ta = (prm.ncharged + FF_TILE - 1) / FF_TILE;
        int t = 0;
        for (; t < ta; t++) {  // tiles holding charged atoms: single-level
            if (!acquire(t)) return false;
            const int base = t * FF_TILE, nj = min(FF_TILE, nat - base);
            const int jc = min(nj, prm.ncharged - base);
            const float4 *S = &s_at[stage(t)][0];
            run_ljc(S, 0, jc, tot, el);
            run_lj(S, jc, nj, tot);
            release(t);
        }
        // park the electrostatic sums in this thread's output slots
        if (!ALLQ && valid) {
            const long long colbase = ((long long)la * prm.ns[1] + lb) * prm.ns[2];
#pragma unroll
            for (int p = 0; p < P2; p++) {
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int lz = lz0 + 2 * p + h;
                    if (lz < prm.ns[2]) {
                        const float4 v = h ? make_float4(el.x[p].y, el.y[p].y, el.z[p].y, el.e[p].y)
                                           : make_float4(el.x[p].x, el.y[p].x, el.z[p].x, el.e[p].x);
                        prm.FE[colbase + lz] = v;
                    }
                }
            }
        }
        for (; !ALLQ && t < ntiles; t++) {  // neutral atoms: two-level
            if (!acquire(t)) return false;
            const int nj = min(FF_TILE, nat - t * FF_TILE);
            run_lj(&s_at[stage(t)][0], 0, nj, acc);
            tot.fold_from(acc);
            release(t);
        }
    } else {
        for (int t = 0; t < ntiles; t++) {
            if (!acquire(t)) return false;
            const int base = t * FF_TILE, nj = min(FF_TILE, nat - base);
            const float4 *S = &s_at[stage(t)][0];
            if constexpr (MODE == M_LJ) {
                run_lj(S, 0, nj, acc);
            } else if constexpr (MODE == M_COUL) {
                for (int j = 0; j < nj; j++) {
                    const float4 r0 = S[3 * j], r1 = S[3 * j + 1], r2r = S[3 * j + 2];
                    const AtomGeo g = atom_geo<P2>(q, r0, r1, eps);
                    const float2 kqq = bc(r2r.z);
#pragma unroll
                    for (int p = 0; p < P2; p++) {
                        float2 dx, dy, dz, r2;
                        pair_geo<ORTHO, P2>(q, g, p, eps, dx, dy, dz, r2);
                        const float2 ir = rsqrt2(r2);
                        coul_ir<WITH_E, P2>(ir, mul2(ir, ir), dx, dy, dz, kqq, acc, p);
                    }
                }
            } else if constexpr (MODE == M_LJC) {  // not split: two-level for both sums
                const int jc = max(0, min(nj, prm.ncharged - base));
                run_ljc(S, 0, jc, acc, elacc);
                run_lj(S, jc, nj, acc);
                el.fold_from(elacc);
            } else {  // M_QZS
                const int jc = max(0, min(nj, prm.ncharged - base));
                run_lj(S, 0, nj, acc);
                for (int j = 0; j < jc; j++) {
                    const float4 r0 = S[3 * j], r1 = S[3 * j + 1], r2r = S[3 * j + 2];
                    const AtomGeo g = atom_geo<P2>(q, r0, r1, eps);
#pragma unroll
                    for (int p = 0; p < P2; p++) {
                        float2 dx, dy, dz, r2;
                        pair_geo<ORTHO, P2>(q, g, p, eps, dx, dy, dz, r2);
                        const float2 dxy2 = ORTHO ? g.dxy2v : fma2(dy, dy, fma2(dx, dx, bc(eps)));
                        qzs_tip<WITH_E, P2>(prm, r2r.z, r2, dx, dy, dz, dxy2, acc, p);
                    }
                }
            }
            tot.fold_from(acc);
            release(t);
        }
    }

    if (!valid) return true;
    const long long colbase = ((long long)la * prm.ns[1] + lb) * prm.ns[2];
#pragma unroll
    for (int p = 0; p < P2; p++) {
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int lz = lz0 + 2 * p + h;
            if (lz >= prm.ns[2]) continue;
            float ux = 0.f, uy = 0.f, uz = 0.f, ue = 0.f;
            if constexpr (MODE == M_LJC) {
                if constexpr (SPLIT && ALLQ) {
                    ux = h ? el.x[p].y : el.x[p].x;
                    uy = h ? el.y[p].y : el.y[p].x;
                    uz = h ? el.z[p].y : el.z[p].x;
                    ue = h ? el.e[p].y : el.e[p].x;
                } else if constexpr (SPLIT) {
                    const float4 v = prm.FE[colbase + lz];
                    ux = v.x;
                    uy = v.y;
                    uz = v.z;
                    ue = v.w;
                } else {
                    ux = h ? el.x[p].y : el.x[p].x;
                    uy = h ? el.y[p].y : el.y[p].x;
                    uz = h ? el.z[p].y : el.z[p].x;
                    ue = h ? el.e[p].y : el.e[p].x;
                }
            }
            const float tx = h ? tot.x[p].y : tot.x[p].x, ty = h ? tot.y[p].y : tot.y[p].x;
            const float tz = h ? tot.z[p].y : tot.z[p].x, te = h ? tot.e[p].y : tot.e[p].x;
            float4 o = finalize<MODE, WITH_E>(tx, ty, tz, te, ux, uy, uz, ue, prm);
            if (!finite4(o)) {
                double qd[3];
#pragma unroll
                for (int c = 0; c < 3; c++) qd[c] = ((prm.dA[c] * ga) + prm.dB[c] * gb) + prm.dC[c] * (gc + 2 * p + h);
                o = point_slow<MODE, WITH_E>(prm, qd[0], qd[1], qd[2]);
            }
            float4 *dst = prm.FE + colbase + lz;
            if (prm.accumulate) {
                const float4 old = *dst;
                o.x += old.x;
                o.y += old.y;
                o.z += old.z;
                o.w += old.w;
            }
            *dst = o;
        }
    }
    return true;
}

}  // namespace ppgpu
