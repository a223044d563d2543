// pp_batch.cu -- many systems in one persistent launch (force field + relaxed scan + df).
//
// The reference relaxes one system per call (relaxTipStrokes_omp, ProbeParticle.cpp:682-701,
// driven by HighLevel.perform_relaxation); its batched user, ml/Generator.py:68-144, loops
// over molecules and calls the simulator once per molecule.  Here a batch of systems of
// uneven atom counts, cell and grid sizes runs as one persistent kernel over a packed work
// list:
//
//   phase 1  force-field items: (system, block of grid points).  A CTA takes the next item
//            from a global counter and runs the same TMA-staged LJ + point-charge block as
//            the single-grid kernel (ff_block, pp_ff_dev.cuh), then publishes one more
//            finished block of that system (release).
//   phase 2  relaxation strokes of all systems as one pool, in system order.  Each warp
//            takes chunks of strokes from a global counter; a lane that finishes its stroke
//            takes the next stroke of the warp's chunk, so lanes stay busy until the pool
//            drains (no per-system tail).  A stroke starts once every force-field block of
//            its system is published (acquire; bounded wait).  The relaxation arithmetic is
//            that of relax_kernel (double-float state, float32 FIRE), the Fz -> df
//            convolution runs when a stroke ends.
//
// Relaxation of early systems overlaps the force fields of late ones.  The launch needs no
// host synchronisation and allocates nothing, so the whole step can be captured in a CUDA
// graph.  Tuning knobs (CTAs per SM, pixel-tile shape of the stroke order, strokes per warp
// chunk) are chosen by the autotuner of ppafm_gb300/batch.py.
//
// Restrictions: orthogonal cells (diagonal grid metric, the ORTHO force-field kernel); the
// LJC force field without energy (what the relaxation consumes); at most 1024 charged atoms
// (with images) per system.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "pp_common.cuh"
#include "pp_df.cuh"
#include "pp_ff_dev.cuh"
#include "pp_mlp_dev.cuh"
#include "pp_relax_dev.cuh"

namespace ppgpu {

constexpr int BATCH_THREADS = FF_THREADS;  // 256: one force-field block per CTA item
constexpr int BATCH_MAX_TAPS = 64;

struct BatchJob {  // device copy, one per system
    // force field
    float4 *FE;
    const float4 *atoms;
    int natoms, ncharged;
    int n0, n1, n2;
    double dA[3], dB[3], dC[3];
    float off[3][FF_MAX_P];  // float(dC[c] * i) (FFParams::off)
    long long nchunks;
    int nzc;
    int ff_blocks;
    int publish_need;     // published blocks its strokes wait for: ff_blocks (more: never ready)
    long long ff_block0;  // first item of this system in the force-field list
    // relaxation
    dfl dic[3];              // diagonal grid metric
    int nx, ny, nz;
    int tw, th;              // pixel tile of the stroke order
    int ntx, nty;            // tiles along x and y
    long long stroke0;       // first stroke of this system in the pool
    long long nstrokes;      // ntx*nty*tw*th (tile-padded)
    const dfl *xs, *ys;      // tip x, y (relative to the grid origin)
    const dfl *zs;           // [nz] tip z
    dfl offd[3];
    float *fzs, *ppos, *df;
    int *iters;
};

struct BatchCtr {  // reset before every run
    int ff_next;
    int pad;
    unsigned long long relax_next;
};

struct BatchPrm {
    const BatchJob *jobs;
    const int2 *stab;  // [nstrokes] (system, ix << 16 | iy); system -1 for tile padding
    int njobs;
    long long nff_items;
    long long nstrokes;
    BatchCtr *ctr;
    int *ff_done;  // [njobs] published force-field blocks
    RelaxPrm R;    // springs, FIRE constants (grid fields unused)
    float Q, Fmax;
    int chunk;     // strokes per warp chunk
    int nw;
    float W[BATCH_MAX_TAPS];
    unsigned long long *iter_total;
    int *err;
    unsigned long long wait_ns;  // limit of a stroke's wait for its force field
};

__device__ __forceinline__ int find_job_ff(const BatchPrm &B, long long item) {
    int lo = 0, hi = B.njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (B.jobs[mid].ff_block0 <= item)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}


__device__ __forceinline__ int ld_acquire(const int *p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void red_release_add(int *p, int v) {
    asm volatile("red.release.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}


// Force-field parameters of one system (the LJC mode of ppgpu_ff_grid, no accumulation).
__device__ __forceinline__ FFParams ff_params_of(const BatchJob &J, const BatchPrm &B) {
    FFParams p;
    p.FE = J.FE;
    p.atoms = J.atoms;
    p.natoms = J.natoms;
    p.ncharged = J.ncharged;
    p.i0[0] = p.i0[1] = p.i0[2] = 0;
    p.ns[0] = J.n0;
    p.ns[1] = J.n1;
    p.ns[2] = J.n2;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        p.dA[k] = J.dA[k];
        p.dB[k] = J.dB[k];
        p.dC[k] = J.dC[k];
    }
#pragma unroll
    for (int c = 0; c < 3; c++)
#pragma unroll
        for (int i = 0; i < FF_MAX_P; i++) p.off[c][i] = J.off[c][i];
    p.eps = 1.0e-8f;
    p.eps64 = (double)1.0e-8f;
    p.Q = B.Q;
    p.Fmax = B.Fmax;
    p.nq = 0;
    p.nqa = 0;
    p.Qsum = 0.f;
    p.accumulate = 0;
    p.nchunks = J.nchunks;
    p.nzc = J.nzc;
    p.err = B.err;
    return p;
}

// Per-lane stroke state of the relaxation phase.
struct Stroke {
    int job;  // -1: none
    const float4 *FE;
    int n0, n1, n2;
    dfl dic[3];
    int ix, iy, nz, iz, it, itcount, itsum;
    bool fin, ready;
    unsigned long long wait_t0;
    dfl tip[3];
    int base[3];
    dfl tf[3], d[3];
    float3 v;
    float dt, acoef;
};

__device__ __forceinline__ void stroke_height(Stroke &S, const BatchJob &J) {
    S.tip[2] = J.zs[S.iz];
    const dfl g[3] = {df_mul(S.dic[0], S.tip[0]), df_mul(S.dic[1], S.tip[1]), df_mul(S.dic[2], S.tip[2])};
    tip_cell(g, S.base, S.tf);
}

// Starts global stroke gs; false if it is tile padding outside the scan (no work).
__device__ __forceinline__ bool stroke_start(Stroke &S, const BatchPrm &B, long long gs) {
    const int2 e = B.stab[gs];
    if (e.x < 0) return false;
    const int j = e.x;
    const BatchJob &J = B.jobs[j];
    S.ix = e.y >> 16;
    S.iy = e.y & 0xFFFF;
    if (J.nz <= 0) return false;
    S.job = j;
    S.FE = J.FE;
    S.n0 = J.n0;
    S.n1 = J.n1;
    S.n2 = J.n2;
    S.dic[0] = J.dic[0];
    S.dic[1] = J.dic[1];
    S.dic[2] = J.dic[2];
    S.nz = J.nz;
    S.iz = 0;
    S.it = 0;
    S.itcount = 0;
    S.itsum = 0;
    S.fin = B.R.maxIters <= 0;
    S.ready = false;
    S.wait_t0 = 0;
    S.tip[0] = J.xs[S.ix];
    S.tip[1] = J.ys[S.iy];
    S.d[0] = B.R.r0[0];
    S.d[1] = B.R.r0[1];
    S.d[2] = B.R.r0[2];
    S.v = make_float3(0.f, 0.f, 0.f);
    S.dt = B.R.dtmaxf;
    S.acoef = B.R.acoef0f;
    stroke_height(S, J);
    return true;
}

// One trip of the flattened relaxation loop (the body of relax_kernel<SCAN>).  Returns false
// when the stroke has ended.
__device__ __forceinline__ bool stroke_trip(Stroke &S, const BatchPrm &B, unsigned long long &mine) {
    const RelaxPrm &P = B.R;
    dfl u[3], F[3];
#pragma unroll
    for (int k = 0; k < 3; k++) u[k] = df_add(S.tf[k], df_mul(S.dic[k], S.d[k]));  // diagonal metric
    interp_force_df<false>(S.FE, S.n0, S.n1, S.n2, S.base, u, F);
    if (S.fin) {
        const BatchJob &J = B.jobs[S.job];
        const long long pix = (long long)S.ix * J.ny + S.iy;
        const long long o = pix * S.nz + (S.nz - 1 - S.iz);
        if (J.fzs) J.fzs[o] = df_round(F[2]);
        if (J.ppos) {
#pragma unroll
            for (int k = 0; k < 3; k++) J.ppos[3 * o + k] = df_round(df_add(df_add(S.tip[k], S.d[k]), J.offd[k]));
        }
        if (J.iters) J.iters[o] = S.itcount;
        S.itsum += S.itcount;
        S.iz++;
        if (S.iz == S.nz) {
            if (J.df && J.fzs && B.nw > 0) {
                const float *f = J.fzs + pix * S.nz;
                const int nout = S.nz - B.nw + 1;
                float *out = J.df + pix * nout;
                for (int jj = 0; jj < nout; jj++) {
                    float acc = 0.f;
                    for (int i = 0; i < B.nw; i++) acc = fmaf(f[jj + i], B.W[B.nw - 1 - i], acc);
                    out[jj] = acc;
                }
            }
            return false;
        }
        // next height: the displacement carries over (probeStart 1)
        stroke_height(S, J);
        S.v = make_float3(0.f, 0.f, 0.f);
        S.dt = P.dtmaxf;
        S.acoef = P.acoef0f;
        S.it = 0;
        S.fin = P.maxIters <= 0;
        S.itcount = 0;
        return true;
    }
    const float3 f = pp_force_df(P, F, S.d);
    const float ff = relax_move_df(P, f, S.d, S.v, S.dt, S.acoef);
    mine++;
    if (ff < P.convF2f) {
        S.itcount = S.it;
        S.fin = true;
    } else if (++S.it >= P.maxIters) {
        S.itcount = P.maxIters;
        S.fin = true;
    }
    return true;
}

__device__ __forceinline__ int load_err(const int *err) { return err ? *(volatile const int *)err : 0; }

// Phase 2: the stroke pool.  Lanes without a stroke take the next ones of the warp's chunk;
// the warp takes a new chunk from the global counter when its chunk is used up.
__device__ void relax_phase(const BatchPrm &B) {
    const int lane = threadIdx.x & 31;
    Stroke S;
    S.job = -1;
    bool has = false;
    long long pool_next = 0, pool_end = 0;  // warp-uniform
    bool drained = false;                   // warp-uniform
    unsigned long long mine = 0;
    while (true) {
        unsigned need = __ballot_sync(FULL, !has);
        while (need && !drained) {
            if (pool_next >= pool_end) {
                unsigned long long g = 0;
                if (lane == 0) g = atomicAdd(&B.ctr->relax_next, (unsigned long long)B.chunk);
                g = __shfl_sync(FULL, g, 0);
                if ((long long)g >= B.nstrokes || __any_sync(FULL, load_err(B.err) != 0)) {
                    drained = true;
                    break;
                }
                pool_next = (long long)g;
                pool_end = min(pool_next + (long long)B.chunk, B.nstrokes);
            }
            const int rank = __popc(need & ((1u << lane) - 1u));
            const int take = (int)min((long long)__popc(need), pool_end - pool_next);
            if (((need >> lane) & 1u) && rank < take) has = stroke_start(S, B, pool_next + rank);
            pool_next += take;
            need = __ballot_sync(FULL, !has);
        }
        if (!__any_sync(FULL, has)) break;
        if (has) {
            if (!S.ready) {
                if (ld_acquire(&B.ff_done[S.job]) >= B.jobs[S.job].publish_need) {
                    S.ready = true;
                } else {
                    const unsigned long long t = global_ns();
                    if (S.wait_t0 == 0) {
                        S.wait_t0 = t;
                    } else if (t - S.wait_t0 > B.wait_ns || load_err(B.err) != 0) {
                        raise_device_error(B.err, PPGPU_ERR_DEVICE_TIMEOUT);
                        has = false;  // the stroke is abandoned; the error is reported to the host
                    }
                }
            }
            if (has && S.ready) has = stroke_trip(S, B, mine);
        }
        if (__all_sync(FULL, !(has && S.ready))) __nanosleep(256);  // the warp only waits: back off
    }
    add_iterations(B.iter_total, mine);
}

// Phase 1: force-field items from the global counter until none is left.  An item is
// BATCH_THREADS chunks of a system's grid; a CTA of NT threads takes it in BATCH_THREADS / NT
// parts.  PUBLISH: each finished item is published to its system's strokes (release).
template <int NT, bool PUBLISH>
__device__ __forceinline__ void ff_phase(const BatchPrm &B, FFShared &sh) {
    constexpr int PARTS = BATCH_THREADS / NT;
    static_assert(PARTS * NT == BATCH_THREADS && (PUBLISH ? PARTS == 1 : true), "whole items when published");
    __shared__ long long s_part;
    uint32_t T = 0;
    while (true) {
        if (threadIdx.x == 0) s_part = atomicAdd(&B.ctr->ff_next, 1);
        __syncthreads();
        const long long part = s_part;
        __syncthreads();
        if (part >= B.nff_items * PARTS) break;
        const long long item = part / PARTS;
        const int j = find_job_ff(B, item);
        const BatchJob &J = B.jobs[j];
        const FFParams prm = ff_params_of(J, B);
        const long long blk = (item - J.ff_block0) * PARTS + part % PARTS;
        const bool ok = (J.ncharged == J.natoms) ? ff_block<M_LJC, false, true, 4, true, NT, true>(prm, blk, sh, T)
                                                 : ff_block<M_LJC, false, true, 4, true, NT>(prm, blk, sh, T);
        if constexpr (PUBLISH) {
            __threadfence();
            __syncthreads();
            if (threadIdx.x == 0) red_release_add(&B.ff_done[j], 1);
        }
        if (!ok) break;
    }
}

__global__ void __launch_bounds__(BATCH_THREADS, 2) batch_kernel(const BatchPrm B) {
    __shared__ __align__(128) FFShared sh;
    ff_shared_init(sh);
    ff_phase<BATCH_THREADS, true>(B, sh);
    relax_phase(B);
}

// The force fields alone (the height-synchronous mode computes them before its heights, so
// nothing waits on a published block), one CTA of BATCH_FF_THREADS threads per block (CTA b
// computes part b of the force-field list), BATCH_FF_CTAS_PER_SM of them per SM at up to 128
// registers (more warps per SM than the 256-thread CTAs that share their registers with the
// relaxation).
constexpr int BATCH_FF_THREADS = 128;
constexpr int BATCH_FF_CTAS_PER_SM = 4;
__global__ void __launch_bounds__(BATCH_FF_THREADS, BATCH_FF_CTAS_PER_SM) batch_ff_block_kernel(const BatchPrm B) {
    constexpr int PARTS = BATCH_THREADS / BATCH_FF_THREADS;
    __shared__ __align__(128) FFShared sh;
    ff_shared_init(sh);
    const long long part = blockIdx.x;
    if (part >= B.nff_items * PARTS) return;
    const long long item = part / PARTS;
    const int j = find_job_ff(B, item);
    const BatchJob &J = B.jobs[j];
    const FFParams prm = ff_params_of(J, B);
    const long long blk = (item - J.ff_block0) * PARTS + part % PARTS;
    uint32_t T = 0;
    if (J.ncharged == J.natoms)
        ff_block<M_LJC, false, true, 4, true, BATCH_FF_THREADS, true>(prm, blk, sh, T);
    else
        ff_block<M_LJC, false, true, 4, true, BATCH_FF_THREADS>(prm, blk, sh, T);
}

// ------------------------------------------------------------ height-synchronous mode
//
// The learned warm start needs every stroke of a height at once (its network runs on 128-row
// tiles), so this mode walks the heights in lockstep: for each height iz, the inference
// kernel computes the network's starting displacement of every stroke, then the height kernel
// runs FIRE for every stroke from the better of the two starts (plain: the displacement
// converged at the height above; learned: that plus the proposal) -- better = smaller initial
// force residual, so a bad proposal falls back to the plain start.  The lane that finishes a
// stroke at height iz writes the stroke's network inputs for height iz + 1 at once, while the
// grid cells around the probe are still in L1.  With no network the height kernel starts
// plain and reproduces the flattened kernel's result stroke for stroke.

struct LayerPrm {
    int iz, nz_max;
    dfl *state;                // [nstrokes][3] displacement after the last finished height
    float4 *prop;              // [nstrokes] proposed change of the displacement (NULL: plain)
    unsigned char *xtiles;     // network input tiles of the next height (NULL: no network)
    unsigned char *rec_x;      // training features [samples][MLP_IN] bf16 (NULL: not recorded)
    float4 *rec_t;             // training targets [samples]: OUT_SCALE * (d_converged - d_start_plain)
    int rec_stride;            // strokes gs % rec_stride == 0 are recorded, sample (gs / stride) * nz_max + iz
    unsigned long long *pool;  // this height's stroke counter
    float4 *dd;                // [nstrokes] change of the converged displacement at this height
                               // (written by the height kernel, read by the next feature kernel)
    float accept_f2;           // a proposal is taken when its |F|^2 is at most this
    // long strokes first: strokes that took at least hard_it iterations at the height above
    // are listed (hard_in, *hard_n_in of them) and dispensed before the tile-ordered pool,
    // which skips them (prev_it_in).  This height fills the lists of the next one.
    int hard_it;
    const int *hard_in;
    const unsigned *hard_n_in;
    unsigned long long *hard_ctr;
    int *hard_out;
    unsigned *hard_n_out;
    const unsigned short *prev_it_in;
    unsigned short *prev_it_out;
};

struct DfVec3 {  // a double-float displacement
    dfl c[3];
};

// Tip, grid cell and fraction of global stroke gs at height iz; false for tile padding and for
// heights beyond the system's scan.
struct StrokeAt {
    int job, ix, iy, nz;
    const float4 *FE;  // the system's grid, size and metric (kept in registers)
    int n0, n1, n2;
    dfl dic[3];
    dfl tip[3];
    int base[3];
    dfl tf[3];
};
__device__ __forceinline__ bool stroke_at(const BatchPrm &B, long long gs, int iz, StrokeAt &A) {
    const int2 e = B.stab[gs];
    if (e.x < 0) return false;
    const int j = e.x;
    const BatchJob &J = B.jobs[j];
    A.ix = e.y >> 16;
    A.iy = e.y & 0xFFFF;
    if (iz >= J.nz) return false;
    A.job = j;
    A.nz = J.nz;
    A.FE = J.FE;
    A.n0 = J.n0;
    A.n1 = J.n1;
    A.n2 = J.n2;
    A.dic[0] = J.dic[0];
    A.dic[1] = J.dic[1];
    A.dic[2] = J.dic[2];
    A.tip[0] = J.xs[A.ix];
    A.tip[1] = J.ys[A.iy];
    A.tip[2] = J.zs[iz];
    const dfl g[3] = {df_mul(J.dic[0], A.tip[0]), df_mul(J.dic[1], A.tip[1]), df_mul(J.dic[2], A.tip[2])};
    tip_cell(g, A.base, A.tf);
    return true;
}

__device__ __forceinline__ void load_prev(const BatchPrm &B, const LayerPrm &L, long long gs, dfl d[3]) {
    if (L.iz == 0) {
        d[0] = B.R.r0[0];
        d[1] = B.R.r0[1];
        d[2] = B.R.r0[2];
    } else {
        d[0] = L.state[3 * gs];
        d[1] = L.state[3 * gs + 1];
        d[2] = L.state[3 * gs + 2];
    }
}

// Network inputs of stroke gs at height iz: row gs % 128 of input tile gs / 128 in the
// tensor cores' K-major layout, and the row-major training copy when the stroke is recorded.
constexpr long long XTILE_BYTES = 128LL * MLP_IN * 2;

// What the 3x3x3 stencil row of one stroke needs (the feature layout of pp_mlp_dev.cuh).
struct FeatTask {
    const float4 *FE;
    int n0, n1, n2;
    int gs;     // -1: nothing to write
    int m[3];   // nearest grid node of the start point (unwrapped)
    float e[9];  // features 81..89: 2 s, FEAT_DSCALE (d - rPP0), OUT_SCALE dd
};

// Task of stroke gs at height iz (A = stroke_at(gs, iz)), from the displacement d converged at
// the height above and dd, the change of the converged displacement there.
__device__ __forceinline__ void make_task(const BatchPrm &B, long long gs, const StrokeAt &A, const dfl d[3], float3 dd,
                                          FeatTask &T) {
    T.FE = A.FE;
    T.n0 = A.n0;
    T.n1 = A.n1;
    T.n2 = A.n2;
    T.gs = (int)gs;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const dfl u = df_add(A.tf[k], df_mul(A.dic[k], d[k]));
        int ci;
        const dfl tk = split_cell(u, ci);
        const float t = __fadd_rn(tk.h, tk.l);
        const bool up = t >= 0.5f;  // nearest node
        T.m[k] = ci + A.base[k] + (up ? 1 : 0);
        T.e[k] = 2.f * (up ? t - 1.f : t);
        T.e[3 + k] = FEAT_DSCALE * df_round(df_add(d[k], B.R.nr0[k]));
    }
    T.e[6] = OUT_SCALE * dd.x;
    T.e[7] = OUT_SCALE * dd.y;
    T.e[8] = OUT_SCALE * dd.z;
}

// One warp writes the rows of ntask (1..FEAT_TPC) tasks: FEAT_LPT lanes per task, stencil nodes
// j, j + FEAT_LPT, ... for lane j (all its gathers in flight at once), values staged in the
// warp's row buffers, then one 16-byte store per chunk (the feature layout of pp_mlp_dev.cuh).
constexpr int FEAT_TPC = 8;              // tasks per warp call
constexpr int FEAT_LPT = 32 / FEAT_TPC;  // lanes per task
constexpr int FEAT_NPL = (27 + FEAT_LPT - 1) / FEAT_LPT;  // stencil nodes per lane
__device__ __forceinline__ void warp_features(const FeatTask *tk, int ntask, __nv_bfloat16 (*row)[MLP_IN],
                                              const LayerPrm &L, int iz) {
    const int lane = threadIdx.x & 31, tsk = lane / FEAT_LPT, j = lane % FEAT_LPT;
    const bool act = tsk < ntask && tk[tsk].gs >= 0;
    if (act) {
        const FeatTask &T = tk[tsk];
        float4 q[FEAT_NPL];
#pragma unroll
        for (int r = 0; r < FEAT_NPL; r++) {
            const int node = j + FEAT_LPT * r;
            if (node < 27) {
                const int a = node / 9, b = (node / 3) % 3, c = node % 3;
                const int ix = wrap_index(T.m[0] - 1 + a, T.n0), iy = wrap_index(T.m[1] - 1 + b, T.n1),
                          iz3 = wrap_index(T.m[2] - 1 + c, T.n2);
                q[r] = T.FE[((long long)ix * T.n1 + iy) * T.n2 + iz3];
            }
        }
#pragma unroll
        for (int r = 0; r < FEAT_NPL; r++) {
            const int node = j + FEAT_LPT * r;
            if (node < 27) {
                row[tsk][3 * node] = __float2bfloat16_rn(tanh_fast(FEAT_FSCALE * q[r].x));
                row[tsk][3 * node + 1] = __float2bfloat16_rn(tanh_fast(FEAT_FSCALE * q[r].y));
                row[tsk][3 * node + 2] = __float2bfloat16_rn(tanh_fast(FEAT_FSCALE * q[r].z));
            }
        }
        if (j == FEAT_LPT - 1) {  // a lane with one node fewer
#pragma unroll
            for (int i = 0; i < 9; i++) row[tsk][81 + i] = __float2bfloat16_rn(T.e[i]);
#pragma unroll
            for (int i = 90; i < MLP_IN; i++) row[tsk][i] = __float2bfloat16_rn(0.f);
        }
    }
    __syncwarp();
    // chunk-major: one store instruction writes the same chunk of consecutive rows, which lie
    // 16 bytes apart in the tile layout (full 128-byte lines for aligned groups of 8 strokes)
    constexpr int CH = MLP_IN / 8;  // 16-byte chunks per row
#pragma unroll
    for (int r = 0; r < (FEAT_TPC * CH + 31) / 32; r++) {
        const int qi = lane + 32 * r, ch = qi / FEAT_TPC, t = qi - ch * FEAT_TPC;
        if (ch < CH && t < ntask && tk[t].gs >= 0) {
            const long long gs = tk[t].gs;
            const int4 v = reinterpret_cast<const int4 *>(row[t])[ch];
            if (L.xtiles)  // read once by the inference kernel: keep the force grids in L2 instead
                st16_hint(L.xtiles + (gs >> 7) * XTILE_BYTES + tile_off((int)(gs & 127), 8 * ch, MLP_IN), v, l2_evict_first());
            if (L.rec_x && gs % L.rec_stride == 0)
                reinterpret_cast<int4 *>(L.rec_x + ((gs / L.rec_stride) * L.nz_max + iz) * (MLP_IN * 2))[ch] = v;
        }
    }
    __syncwarp();
}

// Feature kernel: the network inputs of every stroke at height iz (start: the displacement
// converged at the height above, state, and its change there, dd; the rest displacement at
// the first height).  Each warp takes 32 consecutive strokes at a time: every lane builds one
// task, then the warp writes the rows FEAT_TPC at a time (warp_features).
__global__ void __launch_bounds__(256) feature_kernel(const BatchPrm B, const LayerPrm L) {
    __shared__ FeatTask fq[8][32];
    __shared__ __align__(16) __nv_bfloat16 frow[8][FEAT_TPC][MLP_IN];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const long long step = (long long)gridDim.x * 8 * 32;
    for (long long g0 = ((long long)blockIdx.x * 8 + w) * 32; g0 < B.nstrokes; g0 += step) {
        {
            const long long gs = g0 + lane;
            FeatTask &T = fq[w][lane];
            T.gs = -1;
            StrokeAt A;
            if (gs < B.nstrokes && (L.xtiles || gs % L.rec_stride == 0) && stroke_at(B, gs, L.iz, A)) {
                dfl d[3];
                load_prev(B, L, gs, d);
                float3 dd = make_float3(0.f, 0.f, 0.f);
                if (L.iz > 0) {
                    const float4 q = L.dd[gs];
                    dd = make_float3(q.x, q.y, q.z);
                }
                make_task(B, gs, A, d, dd, T);
            }
        }
        __syncwarp();
#pragma unroll 1
        for (int k = 0; k < 32; k += FEAT_TPC) warp_features(&fq[w][k], FEAT_TPC, frow[w], L, L.iz);
    }
}

// Inference kernel: one persistent CTA per SM keeps the weights in shared memory; each of its
// INFER_GROUPS warpgroups runs the network on its own input tiles (fetched by bulk copies into
// its own activation buffer, accumulating in its own 128 TMEM columns), so the SM has that
// many tiles in flight.  The proposal of stroke gs is OUT_SCALE^-1 * y[0..2].
constexpr int INFER_GROUPS = 4;
constexpr int INFER_SMEM = TILE_W1T + TILE_W2T + TILE_W3T + INFER_GROUPS * TILE_ACT;
__global__ void __launch_bounds__(128 * INFER_GROUPS, 1) infer_kernel(const BatchPrm B, const LayerPrm L,
                                                                      const MLPTiles W, const unsigned char *Xtiles) {
    extern __shared__ __align__(128) unsigned char sm[];
    __shared__ uint64_t bar_mma[INFER_GROUPS], bar_copy[INFER_GROUPS];
    __shared__ uint32_t tbase;
    const int tid = threadIdx.x, g = tid >> 7, row = tid & 127;
    unsigned char *sW1t = sm, *sW2t = sW1t + TILE_W1T, *sW3t = sW2t + TILE_W2T;
    unsigned char *act = sW3t + TILE_W3T + g * TILE_ACT;
    copy_tile(sW1t, W.W1t, TILE_W1T);
    copy_tile(sW2t, W.W2t, TILE_W2T);
    copy_tile(sW3t, W.W3t, TILE_W3T);
    if (tid < INFER_GROUPS) {
        tc_mbar_init(&bar_mma[tid]);
        tc_mbar_init(&bar_copy[tid]);
    }
    if (tid < 32) tmem_alloc(&tbase, 128 * INFER_GROUPS);
    cta_handoff();
    const uint32_t tm = tbase + 128u * (uint32_t)g;
    uint32_t ph = 0, phc = 0;
    bool ok = true;
    const long long ntiles = (B.nstrokes + 127) / 128;
    constexpr uint32_t XBYTES = (uint32_t)XTILE_BYTES;
    for (long long tile = (long long)blockIdx.x * INFER_GROUPS + g; tile < ntiles; tile += (long long)gridDim.x * INFER_GROUPS) {
        if (row == 0) {
            fence_async_smem();  // earlier generic writes of act ordered before the async copy
            mbar_expect_tx(&bar_copy[g], XBYTES);
            bulk_g2s_hint(act, Xtiles + tile * XBYTES, XBYTES, &bar_copy[g], l2_evict_first());
        }
        ok &= tc_mbar_wait(&bar_copy[g], phc);
        phc ^= 1u;
        float y[16];
        ok &= mlp_forward(act, sW1t, sW2t, sW3t, W.b1, W.b2, W.b3, tm, &bar_mma[g], ph, y, g);
        const long long gs = tile * 128 + row;
        if (gs < B.nstrokes)
            L.prop[gs] = make_float4(y[0] * (1.f / OUT_SCALE), y[1] * (1.f / OUT_SCALE), y[2] * (1.f / OUT_SCALE), 0.f);
    }
    if (!ok && row == 0) raise_device_error(B.err, PPGPU_ERR_DEVICE_TIMEOUT);
    tc_fence_before();
    __syncthreads();
    if (tid < 32) tmem_dealloc(tbase, 128 * INFER_GROUPS);
}

constexpr float LAYER_ACCEPT_F2 = 1.0f;  // (eV/A)^2: proposals with a larger residual fall back
constexpr int LAYER_HARD_ITERS = 40;     // strokes this long at the height above go first

// ---- float32 FIRE of the learned mode.  A warm-started stroke stops at a different point of
// the |F|^2 < convF2 ball than plain FIRE from the height above, so the double-float
// arithmetic that makes the plain path stop where the reference stops buys nothing there;
// float32 keeps the residual's error (~1e-7 eV/A) far below the criterion (1e-4 eV/A).

// Periodic trilinear interpolation (Grid.h:93-111) at grid coordinate base + u, float32.
__device__ __forceinline__ float3 interp_force_f32(const float4 *FE, int n0, int n1, int n2, const int base[3],
                                                   const float u[3]) {
    int ci[3];
    float t[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const float fl = floorf(u[k]);
        t[k] = u[k] - fl;
        ci[k] = (int)fl + base[k];
    }
    const int ix0 = wrap_index(ci[0], n0), iy0 = wrap_index(ci[1], n1), iz0 = wrap_index(ci[2], n2);
    const int ix1 = (ix0 + 1 == n0) ? 0 : ix0 + 1;
    const int iy1 = (iy0 + 1 == n1) ? 0 : iy0 + 1;
    const int iz1 = (iz0 + 1 == n2) ? 0 : iz0 + 1;
    const long long r00 = ((long long)ix0 * n1 + iy0) * n2, r01 = ((long long)ix0 * n1 + iy1) * n2;
    const long long r10 = ((long long)ix1 * n1 + iy0) * n2, r11 = ((long long)ix1 * n1 + iy1) * n2;
    const float4 c[8] = {FE[r00 + iz0], FE[r00 + iz1], FE[r01 + iz0], FE[r01 + iz1],
                         FE[r10 + iz0], FE[r10 + iz1], FE[r11 + iz0], FE[r11 + iz1]};
    auto lerp = [](float a, float b, float w) { return fmaf(w, b - a, a); };
    auto comp = [&](int k) {
        float v[8];
#pragma unroll
        for (int i = 0; i < 8; i++) v[i] = k == 0 ? c[i].x : (k == 1 ? c[i].y : c[i].z);
        const float a00 = lerp(v[0], v[1], t[2]), a01 = lerp(v[2], v[3], t[2]);
        const float a10 = lerp(v[4], v[5], t[2]), a11 = lerp(v[6], v[7], t[2]);
        return lerp(lerp(a00, a01, t[1]), lerp(a10, a11, t[1]), t[0]);
    };
    return make_float3(comp(0), comp(1), comp(2));
}

// Probe-particle force (getPPforce, ProbeParticle.cpp:282-294; forceRSpring, Forces.h:85-89):
// grid force + radial spring kRad (l - l0)/l d + lateral spring kSpring (d - rPP0).
__device__ __forceinline__ float3 pp_force_f32(const RelaxPrm &P, float3 F, float3 d) {
    const float l2 = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x));
    const float rs = rsqrt_approx(l2);
    const float l = l2 * rs;
    const float sr = P.kRadf.h * ((l + P.nl0.h) * rs);
    return make_float3(fmaf(d.x + P.nr0[0].h, P.kSf[0].h, fmaf(d.x, sr, F.x)),
                       fmaf(d.y + P.nr0[1].h, P.kSf[1].h, fmaf(d.y, sr, F.y)),
                       fmaf(d.z + P.nr0[2].h, P.kSf[2].h, fmaf(d.z, sr, F.z)));
}

// relax_move_df with a float32 displacement.
__device__ __forceinline__ float relax_move_f32(const RelaxPrm &P, float3 f, float3 &d, float3 &v, float &dt,
                                                float &acoef) {
    const float ff = fmaf(f.z, f.z, fmaf(f.y, f.y, f.x * f.x));
    float h;
    if (P.relaxAlg == 1) {
        const float vv = fmaf(v.z, v.z, fmaf(v.y, v.y, v.x * v.x));
        const float vf = fmaf(f.z, v.z, fmaf(f.y, v.y, f.x * v.x));
        if (vf < 0.f) {
            v = make_float3(0.f, 0.f, 0.f);
            dt = dt * P.fdecf;
            acoef = P.acoef0f;
        } else {
            const float vf2 = vv * ff;
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
    d.x = fmaf(v.x, h, d.x);
    d.y = fmaf(v.y, h, d.y);
    d.z = fmaf(v.z, h, d.z);
    return ff;
}

// Height kernel: FIRE at height iz for every stroke of the pool, lanes refilled as in the
// flattened kernel; the strokes listed as long by the height above are dispensed first.
// Writes the height's outputs, the converged displacement (state) and its change (dd).
// LEARNED = false: plain FIRE from the height above in the double-float arithmetic of the
// flattened kernel (the same result stroke for stroke).  LEARNED = true: the start is the
// proposal when its |F|^2 is at most accept_f2 (FIRE's first move made from it in the same
// trip), else the plain start; FIRE in float32.
template <bool LEARNED>
__global__ void __launch_bounds__(BATCH_THREADS, 2) layer_relax_kernel(const BatchPrm B, const LayerPrm L) {
    using Disp = typename std::conditional<LEARNED, float3, DfVec3>::type;
    const int lane = threadIdx.x & 31;
    const RelaxPrm &P = B.R;
    StrokeAt A;
    long long gs = -1;
    bool has = false;
    bool proposal = false;  // learned: this trip evaluates the proposal
    Disp d, d0, dm;
    float3 v = make_float3(0.f, 0.f, 0.f);
    float dt = 0.f, acoef = 0.f;
    int it = 0, itcount = 0;
    bool fin = false;
    long long pool_next = 0, pool_end = 0;
    int src = (L.hard_in && L.hard_n_in) ? 0 : 1;  // 0: the list of long strokes, 1: the pool
    const long long nhard = src == 0 ? (long long)*L.hard_n_in : 0;
    bool drained = false;
    unsigned long long mine = 0;
    const int chunk = B.chunk;
    while (true) {
        unsigned need = __ballot_sync(FULL, !has);
        while (need && !drained) {
            if (pool_next >= pool_end) {
                long long g = 0, lim = 0;
                if (src == 0) {
                    unsigned long long x = 0;
                    if (lane == 0) x = atomicAdd(L.hard_ctr, (unsigned long long)chunk);
                    x = __shfl_sync(FULL, x, 0);
                    if ((long long)x < nhard) {
                        g = (long long)x;
                        lim = nhard;
                    } else {
                        src = 1;
                    }
                }
                if (src == 1) {
                    unsigned long long x = 0;
                    if (lane == 0) x = atomicAdd(L.pool, (unsigned long long)chunk);
                    x = __shfl_sync(FULL, x, 0);
                    g = (long long)x;
                    lim = B.nstrokes;
                }
                if (g >= lim) {
                    drained = true;
                    break;
                }
                pool_next = g;
                pool_end = min(pool_next + (long long)chunk, lim);
            }
            const int rank = __popc(need & ((1u << lane) - 1u));
            const int take = (int)min((long long)__popc(need), pool_end - pool_next);
            if (((need >> lane) & 1u) && rank < take) {
                const long long idx = pool_next + rank;
                gs = (src == 0) ? (long long)L.hard_in[idx] : idx;
                bool ok = stroke_at(B, gs, L.iz, A);
                if (ok && src == 1 && L.prev_it_in && (int)L.prev_it_in[gs] >= L.hard_it) ok = false;  // listed
                if (ok) {
                    dfl p[3];
                    load_prev(B, L, gs, p);
                    if constexpr (LEARNED) {
                        d0 = make_float3(df_round(p[0]), df_round(p[1]), df_round(p[2]));
                        d = d0;
                        proposal = L.prop && P.maxIters > 0;
                        if (proposal) {
                            const float4 q = L.prop[gs];
                            dm = make_float3(d0.x + q.x, d0.y + q.y, d0.z + q.z);
                        }
                    } else {
#pragma unroll
                        for (int k = 0; k < 3; k++) d0.c[k] = d.c[k] = p[k];
                    }
                    v = make_float3(0.f, 0.f, 0.f);
                    dt = P.dtmaxf;
                    acoef = P.acoef0f;
                    it = 0;
                    itcount = 0;
                    fin = P.maxIters <= 0;
                    has = true;
                }
            }
            pool_next += take;
            need = __ballot_sync(FULL, !has);
        }
        if (!__any_sync(FULL, has)) break;
        if (!has) continue;
        // one trip: the force at the current displacement, then either the outputs (fin) or a move
        float3 Fg;       // learned: grid force
        dfl F[3];        // plain: grid force
        if constexpr (LEARNED) {
            const float3 de = proposal ? dm : d;
            const float u[3] = {fmaf(A.dic[0].h, de.x, df_round(A.tf[0])), fmaf(A.dic[1].h, de.y, df_round(A.tf[1])),
                                fmaf(A.dic[2].h, de.z, df_round(A.tf[2]))};
            Fg = interp_force_f32(A.FE, A.n0, A.n1, A.n2, A.base, u);
        } else {
            dfl u[3];
#pragma unroll
            for (int k = 0; k < 3; k++) u[k] = df_add(A.tf[k], df_mul(A.dic[k], d.c[k]));
            interp_force_df<false>(A.FE, A.n0, A.n1, A.n2, A.base, u, F);
        }
        if (fin) {
            const BatchJob &J = B.jobs[A.job];
            const long long pix = (long long)A.ix * J.ny + A.iy;
            const long long o = pix * A.nz + (A.nz - 1 - L.iz);
            dfl dc[3];  // converged displacement
            float3 dd;  // its change from the height above
            if constexpr (LEARNED) {
                dc[0] = {d.x, 0.f};
                dc[1] = {d.y, 0.f};
                dc[2] = {d.z, 0.f};
                dd = make_float3(d.x - d0.x, d.y - d0.y, d.z - d0.z);
                if (J.fzs) J.fzs[o] = Fg.z;
            } else {
#pragma unroll
                for (int k = 0; k < 3; k++) dc[k] = d.c[k];
                dd = make_float3(df_round(df_add(d.c[0], df_neg(d0.c[0]))), df_round(df_add(d.c[1], df_neg(d0.c[1]))),
                                 df_round(df_add(d.c[2], df_neg(d0.c[2]))));
                if (J.fzs) J.fzs[o] = df_round(F[2]);
            }
            if (J.ppos) {
#pragma unroll
                for (int k = 0; k < 3; k++) J.ppos[3 * o + k] = df_round(df_add(df_add(A.tip[k], dc[k]), J.offd[k]));
            }
            if (J.iters) J.iters[o] = itcount;
            L.state[3 * gs] = dc[0];
            L.state[3 * gs + 1] = dc[1];
            L.state[3 * gs + 2] = dc[2];
            if (L.dd) L.dd[gs] = make_float4(dd.x, dd.y, dd.z, 0.f);
            if (L.prev_it_out) L.prev_it_out[gs] = (unsigned short)min(itcount, 65535);
            if (L.hard_out && itcount >= L.hard_it && L.iz + 1 < A.nz) L.hard_out[atomicAdd(L.hard_n_out, 1u)] = (int)gs;
            if (L.rec_t && gs % L.rec_stride == 0) {
                const long long slot = (gs / L.rec_stride) * L.nz_max + L.iz;
                L.rec_t[slot] = make_float4(OUT_SCALE * dd.x, OUT_SCALE * dd.y, OUT_SCALE * dd.z, 0.f);
            }
            has = false;
            continue;
        }
        float ff;
        if constexpr (LEARNED) {
            float3 f = pp_force_f32(P, Fg, proposal ? dm : d);
            if (proposal) {  // taken unless its residual is too large
                proposal = false;
                if (fmaf(f.z, f.z, fmaf(f.y, f.y, f.x * f.x)) > L.accept_f2) continue;  // plain start next trip
                d = dm;
            }
            ff = relax_move_f32(P, f, d, v, dt, acoef);
        } else {
            const float3 f = pp_force_df(P, F, d.c);
            ff = relax_move_df(P, f, d.c, v, dt, acoef);
        }
        mine++;
        if (ff < P.convF2f) {
            itcount = it;
            fin = true;
        } else if (++it >= P.maxIters) {
            itcount = P.maxIters;
            fin = true;
        }
    }
    add_iterations(B.iter_total, mine);
}

// Fz -> df along each stroke after the last height (np.convolve 'valid', Fz2df).
__global__ void batch_df_kernel(const BatchPrm B) {
    for (long long gs = blockIdx.x * (long long)blockDim.x + threadIdx.x; gs < B.nstrokes;
         gs += (long long)gridDim.x * blockDim.x) {
        StrokeAt A;
        if (!stroke_at(B, gs, 0, A)) continue;
        const BatchJob &J = B.jobs[A.job];
        if (!J.df || !J.fzs || B.nw <= 0) continue;
        const long long pix = (long long)A.ix * J.ny + A.iy;
        const float *f = J.fzs + pix * A.nz;
        const int nout = A.nz - B.nw + 1;
        float *out = J.df + pix * nout;
        for (int jj = 0; jj < nout; jj++) {
            float acc = 0.f;
            for (int i = 0; i < B.nw; i++) acc = fmaf(f[jj + i], B.W[B.nw - 1 - i], acc);
            out[jj] = acc;
        }
    }
}

// --------------------------------------------------------------------------- host

struct BatchHandle {
    int dev = 0;
    int njobs = 0;
    int ctas = 0;
    int nz_max = 0;
    BatchPrm prm;
    void *dmem = nullptr;  // job table + coordinate tables + counters
    size_t ctr_bytes = 0;
    void *ctr_base = nullptr;
    // height-synchronous mode (allocated on first use)
    unsigned char *xtiles = nullptr;  // network input tiles of one height (allocation base)
    dfl *state = nullptr;
    float4 *prop = nullptr;
    unsigned long long *pools = nullptr;  // [nz_max] stroke counters, then [nz_max] long-list counters
    unsigned *hard_n = nullptr;           // [nz_max] long strokes listed for each height
    int *hard = nullptr;                  // [2][nstrokes] lists of long strokes (by height parity)
    unsigned short *prev_it = nullptr;    // [2][nstrokes] iterations at the last two heights
    float4 *dd = nullptr;                 // [nstrokes] change of the converged displacement
};

}  // namespace ppgpu

using namespace ppgpu;

extern "C" int ppgpu_batch_create(const ppgpu_batch_job *jobs, int njobs, const double *prm, double Q, double Fmax,
                                  int nw, const double *df_weights, const int *tuning, void **handle) {
    if (!jobs || njobs <= 0 || !prm || !handle) return set_error(PPGPU_ERR_ARG, "batch_create: bad arguments");
    if (nw < 0 || nw > BATCH_MAX_TAPS || (nw > 0 && !df_weights))
        return set_error(PPGPU_ERR_ARG, "batch_create: nw must be in [0, %d] with weights", BATCH_MAX_TAPS);
    int ctas_per_sm = tuning ? tuning[0] : 2, tw = tuning ? tuning[1] : 8, th = tuning ? tuning[2] : 4,
        chunk = tuning ? tuning[3] : 64;
    if (ctas_per_sm < 1 || ctas_per_sm > 2 || tw < 1 || th < 1 || tw * th > 4096 || chunk < 1 || chunk > 4096)
        return set_error(PPGPU_ERR_ARG, "batch_create: bad tuning (ctas/SM 1..2, tile, chunk 1..4096)");
    if (g_tip_spline.n > 0)
        return set_error(PPGPU_ERR_ARG, "batch_create: the batched path uses the harmonic radial spring (clear the tip spline)");
    // relaxation constants (the grid fields of RelaxPrm are unused here)
    BatchPrm B;
    memset(&B, 0, sizeof(B));
    {
        const int n1[3] = {1, 1, 1};
        const double c1[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        int st = fill_relax_prm(B.R, nullptr, n1, c1, prm, 1, 1, nullptr);
        if (st) return st;
    }
    B.Q = (float)Q;
    B.Fmax = (float)Fmax;
    B.chunk = chunk;
    B.nw = nw;
    for (int i = 0; i < nw; i++) B.W[i] = (float)df_weights[i];
    B.njobs = njobs;
    // host job table + coordinate tables
    std::vector<BatchJob> J(njobs);
    std::vector<dfl> tabs;
    std::vector<size_t> xs_off(njobs), ys_off(njobs), z_off(njobs);
    long long ff0 = 0, s0 = 0;
    for (int j = 0; j < njobs; j++) {
        const ppgpu_batch_job &h = jobs[j];
        BatchJob &b = J[j];
        memset(&b, 0, sizeof(b));
        if (!h.FE || (h.natoms > 0 && !h.atoms) || h.natoms < 0 || h.ncharged < 0 || h.ncharged > h.natoms)
            return set_error(PPGPU_ERR_ARG, "batch job %d: bad force-field arguments", j);
        if (h.ncharged > SPLIT_MAX_CHARGED)
            return set_error(PPGPU_ERR_ARG, "batch job %d: %d charged atoms (at most %d)", j, h.ncharged, SPLIT_MAX_CHARGED);
        if (((uintptr_t)h.atoms & 15u) || ((uintptr_t)h.FE & 15u))
            return set_error(PPGPU_ERR_ARG, "batch job %d: FE and atoms must be 16-byte aligned", j);
        const double *c = h.cell;
        if (c[1] != 0.0 || c[2] != 0.0 || c[3] != 0.0 || c[5] != 0.0 || c[6] != 0.0 || c[7] != 0.0)
            return set_error(PPGPU_ERR_ARG, "batch job %d: the batched path needs an orthogonal (diagonal) cell", j);
        if (h.nx < 0 || h.ny < 0 || h.nz < 0 || h.nx > 65535 || h.ny > 65535 ||
            (h.nx * (long long)h.ny * h.nz > 0 && (!h.xs || !h.ys || !h.zs)))
            return set_error(PPGPU_ERR_ARG, "batch job %d: bad scan (at most 65535 pixels per axis)", j);
        if (h.df && (nw <= 0 || nw > h.nz || !h.fzs))
            return set_error(PPGPU_ERR_ARG, "batch job %d: df needs 1 <= nw <= nz and fzs", j);
        GridGeom g;
        int st = make_geom(h.n, h.cell, &g);
        if (st) return st;
        b.FE = reinterpret_cast<float4 *>(h.FE);
        b.atoms = reinterpret_cast<const float4 *>(h.atoms);
        b.natoms = h.natoms;
        b.ncharged = h.ncharged;
        b.n0 = h.n[0];
        b.n1 = h.n[1];
        b.n2 = h.n[2];
        for (int k = 0; k < 3; k++) {
            b.dA[k] = g.dcell[k];
            b.dB[k] = g.dcell[3 + k];
            b.dC[k] = g.dcell[6 + k];
        }
        for (int c = 0; c < 3; c++)
            for (int i = 0; i < FF_MAX_P; i++) b.off[c][i] = (float)(b.dC[c] * i);
        b.nzc = (b.n2 + 7) / 8;  // P = 8 points per thread (P2 = 4)
        b.nchunks = (long long)b.n0 * b.n1 * b.nzc;
        b.ff_blocks = (int)((b.nchunks + BATCH_THREADS - 1) / BATCH_THREADS);
        b.publish_need = b.ff_blocks;
        b.ff_block0 = ff0;
        ff0 += b.ff_blocks;
        for (int k = 0; k < 3; k++) b.dic[k] = df_from(g.dicell[4 * k]);
        b.nx = h.nx;
        b.ny = h.ny;
        b.nz = h.nz;
        b.tw = tw;
        b.th = th;
        b.ntx = (h.nx + tw - 1) / tw;
        b.nty = (h.ny + th - 1) / th;
        b.nstrokes = (long long)b.ntx * b.nty * tw * th;
        if (h.nz == 0) b.nstrokes = 0;
        b.stroke0 = s0;
        s0 += b.nstrokes;
        for (int k = 0; k < 3; k++) b.offd[k] = df_from(h.pos_offset[k]);
        b.fzs = h.fzs;
        b.ppos = h.ppos;
        b.df = h.df;
        b.iters = h.iters;
        xs_off[j] = tabs.size();
        for (int i = 0; i < h.nx; i++) tabs.push_back(df_from(h.xs[i]));
        ys_off[j] = tabs.size();
        for (int i = 0; i < h.ny; i++) tabs.push_back(df_from(h.ys[i]));
        z_off[j] = tabs.size();
        for (int i = 0; i < h.nz; i++) tabs.push_back(df_from(h.zs[i]));
    }
    B.nff_items = ff0;
    B.nstrokes = s0;
    int nz_max = 0;
    for (int j = 0; j < njobs; j++) nz_max = std::max(nz_max, jobs[j].nz);
    BatchHandle *H = new BatchHandle();
    H->nz_max = nz_max;
    cudaGetDevice(&H->dev);
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, H->dev);
    H->ctas = sms * ctas_per_sm;
    H->njobs = njobs;
    // device memory: [jobs][tables][counters: BatchCtr | iter total | ff_done[njobs]]
    // stroke table: the system and pixel of every stroke of the pool (tile order of each system)
    std::vector<int2> stab((size_t)s0);
    for (int j = 0; j < njobs; j++) {
        const BatchJob &b = J[j];
        const int tsz = b.tw * b.th;
        for (long long s = 0; s < b.nstrokes; s++) {
            const long long tile = s / tsz;
            const int r = (int)(s - tile * tsz);
            const int tx = (int)(tile / b.nty), ty = (int)(tile - (long long)tx * b.nty);
            const int ix = tx * b.tw + r / b.th, iy = ty * b.th + r % b.th;
            stab[b.stroke0 + s] = (ix < b.nx && iy < b.ny) ? make_int2(j, (ix << 16) | iy) : make_int2(-1, 0);
        }
    }
    const size_t jobs_b = ((sizeof(BatchJob) * njobs + 255) / 256) * 256;
    const size_t tabs_b = ((sizeof(dfl) * tabs.size() + 255) / 256) * 256;
    const size_t stab_b = ((sizeof(int2) * stab.size() + 255) / 256) * 256;
    H->ctr_bytes = sizeof(BatchCtr) + sizeof(unsigned long long) + sizeof(int) * njobs;
    cudaError_t e = cudaMalloc(&H->dmem, jobs_b + tabs_b + stab_b + H->ctr_bytes);
    if (e != cudaSuccess) {
        delete H;
        return cuda_fail(e, "batch tables");
    }
    char *base = (char *)H->dmem;
    dfl *dtabs = (dfl *)(base + jobs_b);
    for (int j = 0; j < njobs; j++) {
        J[j].xs = dtabs + xs_off[j];
        J[j].ys = dtabs + ys_off[j];
        J[j].zs = dtabs + z_off[j];
    }
    e = cudaMemcpy(base, J.data(), sizeof(BatchJob) * njobs, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !tabs.empty()) e = cudaMemcpy(dtabs, tabs.data(), sizeof(dfl) * tabs.size(), cudaMemcpyHostToDevice);
    int2 *dstab = (int2 *)(base + jobs_b + tabs_b);
    if (e == cudaSuccess && !stab.empty()) e = cudaMemcpy(dstab, stab.data(), sizeof(int2) * stab.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(H->dmem);
        delete H;
        return cuda_fail(e, "batch tables upload");
    }
    H->ctr_base = base + jobs_b + tabs_b + stab_b;
    B.jobs = (const BatchJob *)base;
    B.stab = dstab;
    B.ctr = (BatchCtr *)H->ctr_base;
    B.iter_total = (unsigned long long *)((char *)H->ctr_base + sizeof(BatchCtr));
    B.ff_done = (int *)((char *)H->ctr_base + sizeof(BatchCtr) + sizeof(unsigned long long));
    B.err = device_error_word();
    B.wait_ns = 2000000000ull;
    H->prm = B;
    *handle = H;
    return set_ok();
}

extern "C" int ppgpu_batch_run(void *handle, void *stream) {
    BatchHandle *H = (BatchHandle *)handle;
    if (!H) return set_error(PPGPU_ERR_ARG, "batch_run: null handle");
    cudaStream_t st = (cudaStream_t)stream;
    PPGPU_CUDA(cudaMemsetAsync(H->ctr_base, 0, H->ctr_bytes, st), "batch counters");
    batch_kernel<<<H->ctas, BATCH_THREADS, 0, st>>>(H->prm);
    PPGPU_CHECK_LAUNCH("batch_kernel");
    return set_ok();
}

/* Limit of a stroke's wait for its system's force field (seconds; default 2) and, for tests of
 * failure detection, a system whose force field its strokes treat as never published (held >= 0;
 * -1: none): they give up after the limit, the launch ends, and ppgpu_device_status reports
 * PPGPU_ERR_DEVICE_TIMEOUT.  Synchronous (updates the device table); applies to launches and
 * graphs made after the call. */
extern "C" int ppgpu_batch_set_wait(void *handle, double wait_s, int held) {
    BatchHandle *H = (BatchHandle *)handle;
    if (!H) return set_error(PPGPU_ERR_ARG, "batch_set_wait: null handle");
    if (!(wait_s > 0.0) || wait_s > 60.0) return set_error(PPGPU_ERR_ARG, "batch_set_wait: limit %g s outside (0, 60]", wait_s);
    if (held < -1 || held >= H->njobs) return set_error(PPGPU_ERR_ARG, "batch_set_wait: system %d of %d", held, H->njobs);
    H->prm.wait_ns = (unsigned long long)(wait_s * 1e9);
    std::vector<BatchJob> J(H->njobs);
    PPGPU_CUDA(cudaMemcpy(J.data(), H->prm.jobs, sizeof(BatchJob) * H->njobs, cudaMemcpyDeviceToHost), "batch table read");
    for (int j = 0; j < H->njobs; j++) J[j].publish_need = J[j].ff_blocks + (j == held ? 1 : 0);
    PPGPU_CUDA(cudaMemcpy((void *)H->prm.jobs, J.data(), sizeof(BatchJob) * H->njobs, cudaMemcpyHostToDevice), "batch table write");
    return set_ok();
}

extern "C" int ppgpu_batch_info(void *handle, long long *out4) {
    BatchHandle *H = (BatchHandle *)handle;
    if (!H || !out4) return set_error(PPGPU_ERR_ARG, "batch_info: null argument");
    out4[0] = H->prm.nff_items;
    out4[1] = H->prm.nstrokes;
    out4[2] = H->ctas;
    out4[3] = H->njobs;
    return set_ok();
}

extern "C" int ppgpu_batch_iterations(void *handle, unsigned long long *out, void *stream) {
    BatchHandle *H = (BatchHandle *)handle;
    if (!H || !out) return set_error(PPGPU_ERR_ARG, "batch_iterations: null argument");
    PPGPU_CUDA(cudaMemcpyAsync(out, H->prm.iter_total, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                               (cudaStream_t)stream),
               "batch iterations");
    PPGPU_CUDA(cudaStreamSynchronize((cudaStream_t)stream), "batch iterations");
    return set_ok();
}

extern "C" int ppgpu_batch_destroy(void *handle) {
    BatchHandle *H = (BatchHandle *)handle;
    if (!H) return set_ok();
    cudaFree(H->dmem);
    cudaFree(H->xtiles);
    delete H;
    return set_ok();
}

/* Height-synchronous run (see layer_relax_kernel): force fields, then for each height the
 * proposal kernel (with the network `mlp`, or features only when recording) and the height
 * kernel, then df.  mlp NULL: plain FIRE from the height above (same results as
 * ppgpu_batch_run).  rec_stride > 0: strokes gs % rec_stride == 0 record training pairs,
 * sample (gs / rec_stride) * nz_max + iz: rec_x [.][MLP_IN = 96] bf16 features, rec_t [.][4] f32 targets
 * OUT_SCALE (10/A) * (converged - plain start).  No host synchronisation (graph-capturable). */
extern "C" int ppgpu_batch_run_layered(void *handle, void *mlp, int rec_stride, void *rec_x, void *rec_t, void *stream) {
    BatchHandle *H = (BatchHandle *)handle;
    if (!H) return set_error(PPGPU_ERR_ARG, "batch_run_layered: null handle");
    cudaStream_t st = (cudaStream_t)stream;
    if (rec_stride < 0 || (rec_stride > 0 && (!rec_x || !rec_t)))
        return set_error(PPGPU_ERR_ARG, "batch_run_layered: recording needs rec_x and rec_t");
    const long long ns = H->prm.nstrokes;
    const int nz = H->nz_max;
    const size_t b_ctr = (2 * sizeof(unsigned long long) + sizeof(unsigned)) * (size_t)std::max(nz, 1);
    if (!H->state) {
        const size_t nsx = (size_t)std::max(ns, 1LL);
        const size_t b_state = sizeof(dfl) * 3 * nsx, b_prop = sizeof(float4) * nsx;
        const size_t b_x = (size_t)((ns + 127) / 128) * 128 * MLP_IN * 2;
        const size_t b_hard = sizeof(int) * 2 * nsx, b_it = sizeof(unsigned short) * 2 * nsx, b_dd = sizeof(float4) * nsx;
        void *p = nullptr;
        cudaError_t e = cudaMalloc(&p, b_x + b_state + b_prop + b_ctr + b_hard + b_it + b_dd + 512);
        if (e != cudaSuccess) return cuda_fail(e, "batch layered buffers");
        H->xtiles = (unsigned char *)p;
        H->state = (dfl *)((char *)p + b_x);
        H->prop = (float4 *)((char *)H->state + ((b_state + 15) / 16) * 16);
        H->pools = (unsigned long long *)((char *)H->prop + b_prop);
        H->hard_n = (unsigned *)(H->pools + 2 * std::max(nz, 1));
        H->hard = (int *)((char *)H->pools + ((b_ctr + 15) / 16) * 16);
        H->prev_it = (unsigned short *)(H->hard + 2 * nsx);
        H->dd = (float4 *)((char *)H->prev_it + ((b_it + 255) / 256) * 256);
        // input rows of padding strokes are never written: keep them zero (finite)
        e = cudaMemset(H->xtiles, 0, b_x);
        if (e != cudaSuccess) return cuda_fail(e, "batch layered buffers");
    }
    MLPTiles W;
    memset(&W, 0, sizeof(W));
    if (mlp) {
        void *v[8];
        int rc = ppgpu_mlp_views(mlp, v);
        if (rc) return rc;
        W.W1t = (const unsigned char *)v[0];
        W.W2t = (const unsigned char *)v[1];
        W.W3t = (const unsigned char *)v[2];
        W.W3 = (const unsigned char *)v[3];
        W.W2 = (const unsigned char *)v[4];
        W.b1 = (const float *)v[5];
        W.b2 = (const float *)v[6];
        W.b3 = (const float *)v[7];
    }
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, H->dev);
    // force fields only, one CTA per force-field block (on the 256-molecule learned run 0.7 %
    // faster than a persistent set of CTAs taking blocks from a counter)
    PPGPU_CUDA(cudaMemsetAsync(H->ctr_base, 0, H->ctr_bytes, st), "batch counters");
    {
        constexpr long long parts = BATCH_THREADS / BATCH_FF_THREADS;
        const long long grid = H->prm.nff_items * parts;
        if (grid > 0x7fffffffLL) return set_error(PPGPU_ERR_ARG, "batch_run_layered: %lld force-field blocks", grid);
        if (grid > 0) batch_ff_block_kernel<<<(unsigned)grid, BATCH_FF_THREADS, 0, st>>>(H->prm);
        PPGPU_CHECK_LAUNCH("batch_ff_block_kernel");
    }
    PPGPU_CUDA(cudaMemsetAsync(H->pools, 0, b_ctr, st), "batch layer counters");
    if (mlp) PPGPU_CUDA(cudaFuncSetAttribute(infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, INFER_SMEM), "infer smem");
    const bool propose = mlp || rec_stride > 0;
    for (int iz = 0; iz < nz; iz++) {
        LayerPrm L;
        memset(&L, 0, sizeof(L));
        L.iz = iz;
        L.nz_max = nz;
        L.state = H->state;
        L.prop = mlp ? H->prop : nullptr;
        L.xtiles = mlp ? H->xtiles : nullptr;
        L.rec_x = rec_stride > 0 ? (unsigned char *)rec_x : nullptr;
        L.rec_t = rec_stride > 0 ? (float4 *)rec_t : nullptr;
        L.rec_stride = rec_stride > 0 ? rec_stride : 1;
        L.pool = H->pools + iz;
        L.accept_f2 = LAYER_ACCEPT_F2;
        L.hard_it = LAYER_HARD_ITERS;
        const size_t nsx = (size_t)std::max(ns, 1LL);
        if (iz > 0) {
            L.hard_in = H->hard + (size_t)(iz & 1) * nsx;
            L.hard_n_in = H->hard_n + iz;
            L.prev_it_in = H->prev_it + (size_t)((iz - 1) & 1) * nsx;
        }
        L.hard_ctr = H->pools + nz + iz;
        if (iz + 1 < nz) {
            L.hard_out = H->hard + (size_t)((iz + 1) & 1) * nsx;
            L.hard_n_out = H->hard_n + iz + 1;
        }
        L.prev_it_out = H->prev_it + (size_t)(iz & 1) * nsx;
        L.dd = H->dd;
        if (propose && ns > 0) {
            feature_kernel<<<3 * sms, 256, 0, st>>>(H->prm, L);
            PPGPU_CHECK_LAUNCH("feature_kernel");
            if (mlp) {
                infer_kernel<<<sms, 128 * INFER_GROUPS, INFER_SMEM, st>>>(H->prm, L, W, H->xtiles);
                PPGPU_CHECK_LAUNCH("infer_kernel");
            }
        }
        if (mlp)
            layer_relax_kernel<true><<<H->ctas, BATCH_THREADS, 0, st>>>(H->prm, L);
        else
            layer_relax_kernel<false><<<H->ctas, BATCH_THREADS, 0, st>>>(H->prm, L);
        PPGPU_CHECK_LAUNCH("layer_relax_kernel");
    }
    batch_df_kernel<<<2 * sms, 256, 0, st>>>(H->prm);
    PPGPU_CHECK_LAUNCH("batch_df_kernel");
    return set_ok();
}

/* out2 = (strokes incl. tile padding, largest nz): recorded samples = ceil(strokes/stride) * nz. */
extern "C" int ppgpu_batch_layer_info(void *handle, long long *out2) {
    BatchHandle *H = (BatchHandle *)handle;
    if (!H || !out2) return set_error(PPGPU_ERR_ARG, "batch_layer_info: null argument");
    out2[0] = H->prm.nstrokes;
    out2[1] = H->nz_max;
    return set_ok();
}
