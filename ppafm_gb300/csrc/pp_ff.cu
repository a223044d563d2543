// pp_ff.cu -- force-field grid generation on sm_103a.
//
// Computes, for every grid point p, sums over atoms of the Lennard-Jones and
// point-charge Coulomb interactions of the reference core:
//   addAtomLJ      (ppafm/cpp/Forces.h:120-132)
//   addAtomCoulomb (Forces.h:237-244) and the pz / dz2 finite-difference tips
//                  (ppafm/cpp/ProbeParticle.cpp:192-209)
//   evalLJC_QZs_noPos (ppafm/ocl/cl/FF.cl:366-423) for the AFMulator grid
// on the grid of GridShape (ppafm/cpp/Grid.h:29-36, 142-170).
//
// Design (GB300):
//  * Atom records (48 B: hi/lo split coordinates, charge, LJ coefficients) are streamed
//    through shared memory in tiles of FF_TILE atoms by 1-D TMA bulk copies
//    (cp.async.bulk + mbarrier, two stages), so the tile for step t+1 lands while
//    step t is computed.
//  * Each thread owns P consecutive points of one grid column (x,y fixed, z varying),
//    so the in-plane displacement and its square are computed once per atom and
//    shared by the P points.
//  * dR = p - R is formed from float hi/lo pairs of the float64 coordinates, which
//    keeps the displacement accurate to float rounding of |dR| itself instead of the
//    rounding of |p| (that matters for the r^-13 repulsive wall).
//  * Partial sums per atom tile are folded into running totals (two-level summation)
//    to bound the FP32 accumulation error over thousands of atoms.
//  * Points whose float32 result overflows (a grid point within ~5e-3 A of an atom
//    centre) are recomputed by a slow path that floors r^2 at 1e-4 A^2.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <type_traits>
#include <vector>

#include "pp_common.cuh"
#include "pp_ff_dev.cuh"

namespace ppgpu {

template <int MODE, bool WITH_E, bool ORTHO, int P2, bool SPLIT, int NT, bool ALLQ = false>
__global__ void __launch_bounds__(NT, 512 / NT) ff_kernel(const FFParams prm) {
    __shared__ __align__(128) FFShared sh;
    ff_shared_init(sh);
    uint32_t T = 0;
    ff_block<MODE, WITH_E, ORTHO, P2, SPLIT, NT, ALLQ>(prm, (long long)blockIdx.x, sh, T);
}

// ------------------------------------------------------------- float64 kernel
//
// The same sums in float64, one grid point per thread, following the reference's
// arithmetic (Forces.h:120-132, 237-244; ProbeParticle.cpp:192-209).  Used for the pz and
// dz2 tips, whose finite differences (step 0.1 A) cancel ~r^2/h^2 of the float32
// significand, and as the GPU float64 error oracle of the float32 kernels
// (PPGPU_FF_F64).  Atom coordinates are hi + lo (exact to ~1e-13 A); coefficients are
// the float32 values of the records.

__device__ __forceinline__ double coul64(double dx, double dy, double dz, double kqq, double &fx, double &fy,
                                         double &fz) {
    const double ir2 = 1.0 / (((dx * dx + dy * dy) + dz * dz) + 1.0e-8);
    const double ir = sqrt(ir2);
    const double e = ir * kqq;
    const double fr = e * ir2;
    fx += dx * fr;
    fy += dy * fr;
    fz += dz * fr;
    return e;
}

template <int MODE, int KIND>
__global__ void __launch_bounds__(FF_THREADS) ff_f64_kernel(const FFParams prm) {
    __shared__ __align__(16) float4 s_at[FF_TILE * FF_REC];
    const int tid = threadIdx.x;
    const long long pidx = (long long)blockIdx.x * FF_THREADS + tid;
    const long long ntot = (long long)prm.ns[0] * prm.ns[1] * prm.ns[2];
    const bool valid = pidx < ntot;
    const long long q = valid ? pidx : 0;
    const int lz = (int)(q % prm.ns[2]);
    const int lb = (int)((q / prm.ns[2]) % prm.ns[1]);
    const int la = (int)(q / ((long long)prm.ns[1] * prm.ns[2]));
    const double ga = prm.i0[0] + la, gb = prm.i0[1] + lb, gc = prm.i0[2] + lz;
    double p[3];
#pragma unroll
    for (int k = 0; k < 3; k++) p[k] = ((prm.dA[k] * ga) + prm.dB[k] * gb) + prm.dC[k] * gc;
    double F[3] = {0, 0, 0}, E = 0, G[3] = {0, 0, 0}, Ge = 0;
    const int nat = (MODE == M_COUL) ? prm.ncharged : prm.natoms;
    for (int base = 0; base < nat; base += FF_TILE) {
        const int nj = min(FF_TILE, nat - base);
        __syncthreads();
        for (int i = tid; i < nj * FF_REC; i += FF_THREADS) s_at[i] = prm.atoms[(size_t)base * FF_REC + i];
        __syncthreads();
        for (int j = 0; j < nj; j++) {
            const float4 r0 = s_at[3 * j], r1 = s_at[3 * j + 1], r2r = s_at[3 * j + 2];
            const double dx = p[0] + ((double)r0.x + (double)r0.z);
            const double dy = p[1] + ((double)r0.y + (double)r0.w);
            double dz = p[2] + ((double)r1.x + (double)r1.y);
            const double c6 = -(double)r2r.x, c12 = (double)r2r.y, kqqa = (double)r2r.z;
            const bool charged = (base + j) < prm.ncharged;
            if (MODE == M_LJ || MODE == M_LJC || MODE == M_QZS) {
                const double ir2 = 1.0 / (((dx * dx + dy * dy) + dz * dz) + prm.eps64);
                const double ir6 = ir2 * ir2 * ir2;
                const double e6 = c6 * ir6;
                const double e12 = c12 * ir6 * ir6;
                const double fr = (12 * e12 - 6 * e6) * ir2;
                F[0] += dx * fr;
                F[1] += dy * fr;
                F[2] += dz * fr;
                E += e12 - e6;
            }
            if (MODE == M_LJC && charged) Ge += coul64(dx, dy, dz, kqqa, G[0], G[1], G[2]);
            if (MODE == M_QZS && charged) {
                for (int k = 0; k < prm.nqa; k++) {
                    const double dq = dz + (double)prm.QZa[k];
                    const double ir2 = 1.0 / (((dx * dx + dy * dy) + dq * dq) + prm.eps64);
                    const double eq = kqqa * sqrt(ir2) * (double)prm.Qa[k];
                    const double fq = eq * ir2;
                    F[0] += dx * fq;
                    F[1] += dy * fq;
                    F[2] += dq * fq;
                    E += eq;
                }
            }
            if (MODE == M_COUL) {
                const double kqq = kqqa;
                if (KIND == 0) {
                    E += coul64(dx, dy, dz, kqq, F[0], F[1], F[2]);
                } else if (KIND == 1) {
                    double g0 = 0, g1 = 0, g2 = 0, e = 0;
                    dz -= 0.1;
                    e += coul64(dx, dy, dz, -kqq, g0, g1, g2);
                    dz += 2 * 0.1;
                    e += coul64(dx, dy, dz, kqq, g0, g1, g2);
                    F[0] += g0 * 10.0;
                    F[1] += g1 * 10.0;
                    F[2] += g2 * 10.0;
                    E += e * 10.0;
                } else {
                    double g0 = 0, g1 = 0, g2 = 0, e = 0;
                    e += coul64(dx, dy, dz, -2 * kqq, g0, g1, g2);
                    dz -= 0.1;
                    e += coul64(dx, dy, dz, kqq, g0, g1, g2);
                    dz += 2 * 0.1;
                    e += coul64(dx, dy, dz, kqq, g0, g1, g2);
                    F[0] += g0 * 100.0;
                    F[1] += g1 * 100.0;
                    F[2] += g2 * 100.0;
                    E += e * 100.0;
                }
            }
        }
    }
    if (!valid) return;
    if (MODE == M_LJC) {
        auto clamp64 = [&](double *v) {
            const double fr = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
            if (prm.Fmax > 0.f && fr > (double)prm.Fmax) {
                const double k = (double)prm.Fmax / fr;
                v[0] *= k;
                v[1] *= k;
                v[2] *= k;
            }
        };
        clamp64(F);
        clamp64(G);
        for (int k = 0; k < 3; k++) F[k] += (double)prm.Q * G[k];
        E += (double)prm.Q * Ge;
    }
    float4 o = make_float4((float)F[0], (float)F[1], (float)F[2], (float)E);
    float4 *dst = prm.FE + q;
    if (prm.accumulate) {
        const float4 old = *dst;
        o.x += old.x;
        o.y += old.y;
        o.z += old.z;
        o.w += old.w;
    }
    *dst = o;
}

template <int MODE, int KIND>
static int launch_ff64(const FFParams &prm, cudaStream_t st) {
    const long long ntot = (long long)prm.ns[0] * prm.ns[1] * prm.ns[2];
    const long long nblk = (ntot + FF_THREADS - 1) / FF_THREADS;
    if (nblk <= 0) return set_ok();
    if (nblk > 0x7fffffffLL) return set_error(PPGPU_ERR_ARG, "ff grid too large (%lld blocks)", nblk);
    ff_f64_kernel<MODE, KIND><<<(unsigned)nblk, FF_THREADS, 0, st>>>(prm);
    PPGPU_CHECK_LAUNCH("ff_f64_kernel launch");
    return set_ok();
}

static int ff64_dispatch(const FFParams &prm, int mode, int kind, cudaStream_t st) {
    switch (mode) {
        case PPGPU_FF_LJ:
            return launch_ff64<M_LJ, 0>(prm, st);
        case PPGPU_FF_COULOMB:
            if (kind == 0) return launch_ff64<M_COUL, 0>(prm, st);
            if (kind == 1) return launch_ff64<M_COUL, 1>(prm, st);
            return launch_ff64<M_COUL, 2>(prm, st);
        case PPGPU_FF_LJC:
            return launch_ff64<M_LJC, 0>(prm, st);
        default:
            return launch_ff64<M_QZS, 0>(prm, st);
    }
}

// ------------------------------------------------------------------------ host

// Threads per CTA of the single-grid kernel (ppgpu_set_ff_block): 0 = the default, 128.  At
// most 128 registers a thread, so 4 CTAs (16 warps) fit an SM, and the smaller CTAs pack more
// evenly, also beside the blocks of a relaxation running on another stream.  Measured against
// CTAs of 256 threads on small systems (342 atoms, 200^3 points): LJ 1.00 vs 1.03 ms, LJ +
// Coulomb 1.43 vs 1.45 ms alone and 2.11 vs 2.18 ms per step beside the previous step's
// relaxation, the AFMulator's field 4 % faster; on 18540 atoms 2.121 vs 2.166 s.
static int g_ff_block = 0;
constexpr int FF_DEFAULT_THREADS = 128;

template <int MODE, bool WITH_E, int P2, bool SPLIT, int NT>
static void launch_ff_nt(const FFParams &prm, bool ortho, long long nblk, cudaStream_t st) {
    if constexpr (MODE == M_LJC && SPLIT) {
        if (prm.ncharged == prm.natoms) {  // every atom charged: no neutral phase
            if (ortho)
                ff_kernel<MODE, WITH_E, true, P2, SPLIT, NT, true><<<(unsigned)nblk, NT, 0, st>>>(prm);
            else
                ff_kernel<MODE, WITH_E, false, P2, SPLIT, NT, true><<<(unsigned)nblk, NT, 0, st>>>(prm);
            return;
        }
    }
    if (ortho)
        ff_kernel<MODE, WITH_E, true, P2, SPLIT, NT><<<(unsigned)nblk, NT, 0, st>>>(prm);
    else
        ff_kernel<MODE, WITH_E, false, P2, SPLIT, NT><<<(unsigned)nblk, NT, 0, st>>>(prm);
}

template <int MODE, bool WITH_E, int P2, bool SPLIT>
static int launch_ff(FFParams &prm, bool ortho, cudaStream_t st) {
    prm.nzc = (prm.ns[2] + 2 * P2 - 1) / (2 * P2);
    prm.nchunks = (long long)prm.ns[0] * prm.ns[1] * prm.nzc;
    const int nt = g_ff_block ? g_ff_block : FF_DEFAULT_THREADS;
    const long long nblk = (prm.nchunks + nt - 1) / nt;
    if (nblk <= 0) return set_ok();
    if (nblk > 0x7fffffffLL) return set_error(PPGPU_ERR_ARG, "ff grid too large (%lld blocks)", nblk);
    if (nt == 256)
        launch_ff_nt<MODE, WITH_E, P2, SPLIT, 256>(prm, ortho, nblk, st);
    else
        launch_ff_nt<MODE, WITH_E, P2, SPLIT, 128>(prm, ortho, nblk, st);
    PPGPU_CHECK_LAUNCH("ff_kernel launch");
    return set_ok();
}

template <int MODE, int P2, bool SPLIT = false>
static int launch_ff_e(FFParams &prm, bool with_e, bool ortho, cudaStream_t st) {
    return with_e ? launch_ff<MODE, true, P2, SPLIT>(prm, ortho, st) : launch_ff<MODE, false, P2, SPLIT>(prm, ortho, st);
}

static int ff_dispatch(FFParams &prm, int mode, int kind, bool with_e, bool ortho, cudaStream_t st) {
    switch (mode) {
        case PPGPU_FF_LJ:
            return launch_ff_e<M_LJ, 4>(prm, with_e, ortho, st);
        case PPGPU_FF_COULOMB:
            if (kind == 0) return launch_ff_e<M_COUL, 4>(prm, with_e, ortho, st);
            if (kind == 1 || kind == 2) return ff64_dispatch(prm, mode, kind, st);
            return set_error(PPGPU_ERR_ARG, "coulomb kind %d not in {0,1,2}", kind);
        case PPGPU_FF_LJC:
            if (prm.ncharged <= SPLIT_MAX_CHARGED && !prm.accumulate)
                return launch_ff_e<M_LJC, 4, true>(prm, with_e, ortho, st);
            return launch_ff_e<M_LJC, 2, false>(prm, with_e, ortho, st);
        case PPGPU_FF_QZS:
            return launch_ff_e<M_QZS, 4>(prm, with_e, ortho, st);
        default:
            return set_error(PPGPU_ERR_ARG, "unknown force-field mode %d", mode);
    }
}

}  // namespace ppgpu

using namespace ppgpu;

extern "C" int ppgpu_pack_atoms(int natoms, const double *R, const double *cLJ, const double *kqq, float *out,
                                int *ncharged_out) {
    if (natoms < 0 || (natoms > 0 && (!R || !out))) return set_error(PPGPU_ERR_ARG, "pack_atoms: bad arguments");
    std::vector<int> order;
    order.reserve(natoms);
    for (int i = 0; i < natoms; i++)
        if (kqq && kqq[i] != 0.0) order.push_back(i);
    const int nch = (int)order.size();
    for (int i = 0; i < natoms; i++)
        if (!(kqq && kqq[i] != 0.0)) order.push_back(i);
    for (int r = 0; r < natoms; r++) {
        const int i = order[r];
        float *o = out + (size_t)r * PPGPU_ATOM_FLOATS;
        float hi[3], lo[3];
        for (int k = 0; k < 3; k++) {
            const double x = R[3 * i + k];
            hi[k] = (float)x;
            lo[k] = (float)(x - (double)hi[k]);
        }
        const double c6 = cLJ ? cLJ[2 * i] : 0.0, c12 = cLJ ? cLJ[2 * i + 1] : 0.0;
        o[0] = -hi[0];
        o[1] = -hi[1];
        o[2] = -lo[0];
        o[3] = -lo[1];
        o[4] = -hi[2];
        o[5] = -lo[2];
        o[6] = (float)(-6.0 * c6);
        o[7] = (float)(12.0 * c12);
        o[8] = (float)(-c6);
        o[9] = (float)c12;
        o[10] = kqq ? (float)kqq[i] : 0.f;
        o[11] = 0.f;
    }
    if (ncharged_out) *ncharged_out = nch;
    return set_ok();
}

extern "C" int ppgpu_ff_subgrid(float *FE, const int *n, const double *cell, const int *i0, const int *ns,
                                const float *atoms, int natoms, int ncharged, int mode, int coul_kind, double Q,
                                double Fmax, const double *Qs, const double *QZs, int flags, void *stream) {
    if (!FE || !n || !cell || !i0 || !ns) return set_error(PPGPU_ERR_ARG, "ff_grid: null argument");
    if (natoms < 0 || ncharged < 0 || ncharged > natoms) return set_error(PPGPU_ERR_ARG, "ff_grid: bad atom counts");
    if (natoms > 0 && !atoms) return set_error(PPGPU_ERR_ARG, "ff_grid: null atoms");
    if (((uintptr_t)atoms & 15u) != 0 || ((uintptr_t)FE & 15u) != 0)
        return set_error(PPGPU_ERR_ARG, "ff_grid: atoms and FE must be 16-byte aligned");
    for (int k = 0; k < 3; k++) {
        if (n[k] <= 0 || ns[k] < 0 || i0[k] < 0 || i0[k] + ns[k] > n[k])
            return set_error(PPGPU_ERR_ARG, "ff_grid: bad grid/sub-box on axis %d", k);
    }
    if (mode < PPGPU_FF_LJ || mode > PPGPU_FF_QZS) return set_error(PPGPU_ERR_ARG, "unknown force-field mode %d", mode);
    if (mode == PPGPU_FF_COULOMB && (coul_kind < 0 || coul_kind > 2))
        return set_error(PPGPU_ERR_ARG, "coulomb kind %d not in {0,1,2}", coul_kind);
    if (mode == PPGPU_FF_QZS && (!Qs || !QZs)) return set_error(PPGPU_ERR_ARG, "ff_grid: QZS mode needs Qs, QZs");
    GridGeom g;
    int st = make_geom(n, cell, &g);
    if (st) return st;
    FFParams prm;
    memset(&prm, 0, sizeof(prm));
    prm.FE = reinterpret_cast<float4 *>(FE);
    prm.atoms = reinterpret_cast<const float4 *>(atoms);
    prm.natoms = natoms;
    prm.ncharged = ncharged;
    for (int k = 0; k < 3; k++) {
        prm.i0[k] = i0[k];
        prm.ns[k] = ns[k];
        prm.dA[k] = g.dcell[k];
        prm.dB[k] = g.dcell[3 + k];
        prm.dC[k] = g.dcell[6 + k];
    }
    ff_set_offsets(prm);
    // Forces.h:12 (R2SAFE = 1e-8 for the CPU core) and FF.cl:1 (1e-6 for the OpenCL grid).
    prm.eps = (mode == PPGPU_FF_QZS) ? 1e-6f : 1.0e-8f;
    prm.eps64 = (mode == PPGPU_FF_QZS) ? (double)1e-6f : (double)1.0e-8f;
    prm.Q = (float)Q;
    prm.Fmax = (float)Fmax;
    prm.nq = 0;
    prm.nqa = 0;
    prm.Qsum = 0.f;
    if (mode == PPGPU_FF_QZS) {
        // Coulomb constant of FF.cl:2, folded into the tip charges; zero charges dropped.  The
        // kernel sums Qsum C(dz) + sum_k Q_k [C(dz + QZ_k) - C(dz)]: a charge at QZ = 0 only
        // enters Qsum (its difference term is exactly zero, so it is not listed).
        for (int q = 0; q < 4; q++) {
            if (Qs[q] != 0.0) {
                const float qz = (float)QZs[q];
                const float qk = (float)Qs[q] * 14.399644f;
                prm.Qsum += qk;
                prm.Qa[prm.nqa] = qk;
                prm.QZa[prm.nqa] = qz;
                prm.nqa++;
                if (qz == 0.f) continue;
                prm.Qs[prm.nq] = qk;
                prm.QZs[prm.nq] = qz;
                prm.QZn2[prm.nq] = -2.f * qz;
                prm.QZnsq[prm.nq] = -qz * qz;
                prm.nq++;
            }
        }
    }
    prm.accumulate = (flags & PPGPU_FF_ACCUMULATE) ? 1 : 0;
    prm.err = device_error_word();
    const bool with_e = (flags & PPGPU_FF_WITH_E) != 0;
    const bool ortho = (g.dcell[6] == 0.0 && g.dcell[7] == 0.0);
    if ((long long)ns[0] * ns[1] * ns[2] == 0) return set_ok();
    if (mode == PPGPU_FF_COULOMB && ncharged == 0 && !prm.accumulate) {
        // Nothing charged: the grid is exactly zero (plus nothing to add when accumulating).
        PPGPU_CUDA(cudaMemsetAsync(FE, 0, (size_t)ns[0] * ns[1] * ns[2] * 16, (cudaStream_t)stream), "memset FE");
        return set_ok();
    }
    if (flags & PPGPU_FF_F64) return ff64_dispatch(prm, mode, coul_kind, (cudaStream_t)stream);
    return ff_dispatch(prm, mode, coul_kind, with_e, ortho, (cudaStream_t)stream);
}

extern "C" int ppgpu_set_ff_block(int threads) {
    if (threads != 0 && threads != 128 && threads != 256)
        return set_error(PPGPU_ERR_ARG, "set_ff_block: %d not in {0 (by atom count), 128, 256}", threads);
    g_ff_block = threads;
    return set_ok();
}

extern "C" int ppgpu_ff_grid(float *FE, const int *n, const double *cell, const float *atoms, int natoms,
                             int ncharged, int mode, int coul_kind, double Q, double Fmax, const double *Qs,
                             const double *QZs, int flags, void *stream) {
    const int zero[3] = {0, 0, 0};
    if (!n) return set_error(PPGPU_ERR_ARG, "ff_grid: null n");
    return ppgpu_ff_subgrid(FE, n, cell, zero, n, atoms, natoms, ncharged, mode, coul_kind, Q, Fmax, Qs, QZs, flags,
                            stream);
}

// ===================================================================== no-allocation entry
//
// ppgpu_lj_grid_f64_noalloc: the Lennard-Jones grid of getLennardJonesFF, accumulated into a
// caller-owned float64 device grid, for callers that must not allocate device memory at
// call time -- an application whose own allocator reserved the device memory up front, or a
// latency-sensitive loop that cannot afford the device-wide synchronisation of
// cudaMalloc/cudaFree.  All scratch (the packed atom records, a float4 chunk of the grid and
// the kernels' error word) lives in one fixed array below, so the call allocates nothing.
//
// Limits: at most NOALLOC_MAX_ATOMS atoms per call; the grid is processed in chunks of at
// most NOALLOC_CHUNK_PTS points (one z column, n2, must fit in a chunk).  Every GPU on which
// the library's device code is loaded holds the array (5.5 MB) until the process exits; with
// CUDA's default lazy loading that happens at the first call on the device (or at any other
// launch of the library there), and that load itself takes device memory -- callers that
// reserve all device memory make one small call first, or set CUDA_MODULE_LOADING=EAGER.
// All calls share the array and it keeps the last call's contents: calls that overlap on the
// GPU (different streams, or different host threads) race on it.  The calls return as soon
// as their work is queued; a bounded wait that gave up inside them is reported by
// ppgpu_device_status, which reads this array's error word too.

namespace ppgpu {

constexpr int NOALLOC_MAX_ATOMS = 32768;
constexpr long long NOALLOC_CHUNK_PTS = 1LL << 18;
constexpr size_t NOALLOC_REC_BYTES = (size_t)NOALLOC_MAX_ATOMS * FF_REC * 16;        // 1.5 MB
constexpr size_t NOALLOC_CHUNK_BYTES = (size_t)NOALLOC_CHUNK_PTS * 16;                // 4 MB
constexpr size_t NOALLOC_BYTES = NOALLOC_REC_BYTES + NOALLOC_CHUNK_BYTES + 256;      // + error word

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

// Packs LJ atoms (device float64 R [n,3], cLJ [n,2]) into the 48-byte records.
__global__ void pack_lj_records_kernel(float *rec, const double *R, const double *cLJ, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float *o = rec + (size_t)i * 12;
    float hi[3], lo[3];
    for (int k = 0; k < 3; k++) {
        const double x = R[3 * i + k];
        hi[k] = __double2float_rn(x);
        lo[k] = __double2float_rn(x - (double)hi[k]);
    }
    const double c6 = cLJ[2 * i], c12 = cLJ[2 * i + 1];
    o[0] = -hi[0];
    o[1] = -hi[1];
    o[2] = -lo[0];
    o[3] = -lo[1];
    o[4] = -hi[2];
    o[5] = -lo[2];
    o[6] = (float)(-6.0 * c6);
    o[7] = (float)(12.0 * c12);
    o[8] = (float)(-c6);
    o[9] = (float)c12;
    o[10] = 0.f;
    o[11] = 0.f;
}

// Device address of the fixed array, per device.  In host code g_noalloc_scratch names a
// host-side stand-in, not device memory, so the address is looked up with
// cudaGetSymbolAddress once per device with that device current (the lookup loads the
// library's device code on that device if it is not loaded yet; it allocates nothing
// afterwards).  The cache is per process: the library does not survive cudaDeviceReset.
static unsigned char *g_noalloc_addr[64] = {nullptr};
static std::mutex g_noalloc_mu;

static int noalloc_scratch_address(unsigned char **out) {
    int dev = 0;
    PPGPU_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= 64) return set_error(PPGPU_ERR_NO_DEVICE, "device index %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void *p = nullptr;
        PPGPU_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(no-alloc scratch)");
        g_noalloc_addr[dev] = (unsigned char *)p;
    }
    *out = g_noalloc_addr[dev];
    return PPGPU_OK;
}

int *noalloc_error_word_if_loaded() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    return g_noalloc_addr[dev] ? (int *)(g_noalloc_addr[dev] + NOALLOC_REC_BYTES + NOALLOC_CHUNK_BYTES) : nullptr;
}

}  // namespace ppgpu

extern "C" int ppgpu_lj_grid_f64_noalloc(double *gridF, double *gridE, const int *n, const double *cell, int natoms,
                                         const double *Ratoms, const double *cLJs, void *stream) {
    if (!n || !cell) return set_error(PPGPU_ERR_ARG, "lj_grid_f64_noalloc: null n or cell");
    if (!gridF && !gridE) return set_ok();
    if (natoms < 0 || natoms > NOALLOC_MAX_ATOMS)
        return set_error(PPGPU_ERR_ARG, "lj_grid_f64_noalloc: %d atoms; this entry point takes 0..%d", natoms,
                         NOALLOC_MAX_ATOMS);
    if (natoms > 0 && (!Ratoms || !cLJs)) return set_error(PPGPU_ERR_ARG, "lj_grid_f64_noalloc: null atom arrays");
    if (n[2] > NOALLOC_CHUNK_PTS)
        return set_error(PPGPU_ERR_ARG, "lj_grid_f64_noalloc: n2 = %d exceeds the %lld-point chunk", n[2],
                         NOALLOC_CHUNK_PTS);
    GridGeom g;
    int st = make_geom(n, cell, &g);
    if (st) return st;
    unsigned char *base = nullptr;
    if ((st = noalloc_scratch_address(&base))) return st;
    float *rec = (float *)base;
    float *chunk = (float *)(base + NOALLOC_REC_BYTES);
    int *err = (int *)(base + NOALLOC_REC_BYTES + NOALLOC_CHUNK_BYTES);
    cudaStream_t cs = (cudaStream_t)stream;
    // The error word is zero when the library's device code is loaded and is cleared only by
    // ppgpu_device_status, which reports it: a timeout of one call is not lost by the next.
    if (natoms > 0) {
        pack_lj_records_kernel<<<(natoms + 127) / 128, 128, 0, cs>>>(rec, Ratoms, cLJs, natoms);
        PPGPU_CHECK_LAUNCH("pack_lj_records_kernel");
    }
    FFParams prm;
    memset(&prm, 0, sizeof(prm));
    prm.atoms = reinterpret_cast<const float4 *>(rec);
    prm.natoms = natoms;
    prm.ncharged = 0;
    for (int k = 0; k < 3; k++) {
        prm.dA[k] = g.dcell[k];
        prm.dB[k] = g.dcell[3 + k];
        prm.dC[k] = g.dcell[6 + k];
    }
    ff_set_offsets(prm);
    prm.eps = 1.0e-8f;
    prm.eps64 = (double)1.0e-8f;
    prm.err = err;
    const bool with_e = gridE != nullptr;
    const bool ortho = (g.dcell[6] == 0.0 && g.dcell[7] == 0.0);
    // chunks: whole (iy, iz) planes when they fit, otherwise runs of whole z columns
    const long long plane = (long long)n[1] * n[2];
    for (int ia = 0; ia < n[0];) {
        int na_, nb_ = n[1], ib = 0;
        if (plane <= NOALLOC_CHUNK_PTS) {
            na_ = (int)std::min<long long>(n[0] - ia, NOALLOC_CHUNK_PTS / plane);
        } else {
            na_ = 1;
            nb_ = (int)(NOALLOC_CHUNK_PTS / n[2]);
        }
        for (ib = 0; ib < n[1]; ib += nb_) {
            const int nbk = std::min(nb_, n[1] - ib);
            prm.FE = reinterpret_cast<float4 *>(chunk);
            prm.i0[0] = ia;
            prm.i0[1] = ib;
            prm.i0[2] = 0;
            prm.ns[0] = na_;
            prm.ns[1] = nbk;
            prm.ns[2] = n[2];
            prm.accumulate = 0;
            if ((st = ff_dispatch(prm, PPGPU_FF_LJ, 0, with_e, ortho, cs))) return st;
            const long long off = ((long long)ia * n[1] + ib) * n[2];
            const long long m = (long long)na_ * nbk * n[2];
            if ((st = ppgpu_grid_to_f64(gridF ? gridF + 3 * off : nullptr, gridE ? gridE + off : nullptr, chunk, m, 1,
                                        stream)))
                return st;
            if (plane <= NOALLOC_CHUNK_PTS) break;
        }
        ia += na_;
    }
    return set_ok();
}
