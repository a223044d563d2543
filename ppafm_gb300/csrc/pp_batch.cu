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
#include <vector>

#include "pp_common.cuh"
#include "pp_df.cuh"
#include "pp_ff_dev.cuh"
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
    long long nchunks;
    int nzc;
    int ff_blocks;
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

__device__ __forceinline__ int find_job_stroke(const BatchPrm &B, long long s) {
    int lo = 0, hi = B.njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (B.jobs[mid].stroke0 <= s)
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
    p.eps = 1.0e-8f;
    p.eps64 = (double)1.0e-8f;
    p.Q = B.Q;
    p.Fmax = B.Fmax;
    p.nq = 0;
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
    const int j = find_job_stroke(B, gs);
    const BatchJob &J = B.jobs[j];
    const long long s = gs - J.stroke0;
    const int tsz = J.tw * J.th;
    const long long tile = s / tsz;
    const int r = (int)(s - tile * tsz);
    const int tx = (int)(tile / J.nty), ty = (int)(tile - (long long)tx * J.nty);
    S.ix = tx * J.tw + r / J.th;
    S.iy = ty * J.th + r % J.th;
    if (S.ix >= J.nx || S.iy >= J.ny || J.nz <= 0) return false;
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
    constexpr unsigned long long WAIT_NS = 2000000000ull;
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
                if (ld_acquire(&B.ff_done[S.job]) >= B.jobs[S.job].ff_blocks) {
                    S.ready = true;
                } else {
                    const unsigned long long t = global_ns();
                    if (S.wait_t0 == 0) {
                        S.wait_t0 = t;
                    } else if (t - S.wait_t0 > WAIT_NS || load_err(B.err) != 0) {
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

__global__ void __launch_bounds__(BATCH_THREADS, 2) batch_kernel(const BatchPrm B) {
    __shared__ __align__(128) FFShared sh;
    __shared__ long long s_item;
    ff_shared_init(sh);
    uint32_t T = 0;
    while (true) {
        if (threadIdx.x == 0) s_item = atomicAdd(&B.ctr->ff_next, 1);
        __syncthreads();
        const long long item = s_item;
        __syncthreads();
        if (item >= B.nff_items) break;
        const int j = find_job_ff(B, item);
        const BatchJob &J = B.jobs[j];
        const FFParams prm = ff_params_of(J, B);
        const bool ok = ff_block<M_LJC, false, true, 4, true>(prm, item - J.ff_block0, sh, T);
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) red_release_add(&B.ff_done[j], 1);
        if (!ok) break;
    }
    relax_phase(B);
}

// --------------------------------------------------------------------------- host

struct BatchHandle {
    int dev = 0;
    int njobs = 0;
    int ctas = 0;
    BatchPrm prm;
    void *dmem = nullptr;  // job table + coordinate tables + counters
    size_t ctr_bytes = 0;
    void *ctr_base = nullptr;
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
        if (h.nx < 0 || h.ny < 0 || h.nz < 0 || (h.nx * (long long)h.ny * h.nz > 0 && (!h.xs || !h.ys || !h.zs)))
            return set_error(PPGPU_ERR_ARG, "batch job %d: bad scan", j);
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
        b.nzc = (b.n2 + 7) / 8;  // P = 8 points per thread (P2 = 4)
        b.nchunks = (long long)b.n0 * b.n1 * b.nzc;
        b.ff_blocks = (int)((b.nchunks + BATCH_THREADS - 1) / BATCH_THREADS);
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
    BatchHandle *H = new BatchHandle();
    cudaGetDevice(&H->dev);
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, H->dev);
    H->ctas = sms * ctas_per_sm;
    H->njobs = njobs;
    // device memory: [jobs][tables][counters: BatchCtr | iter total | ff_done[njobs]]
    const size_t jobs_b = ((sizeof(BatchJob) * njobs + 255) / 256) * 256;
    const size_t tabs_b = ((sizeof(dfl) * tabs.size() + 255) / 256) * 256;
    H->ctr_bytes = sizeof(BatchCtr) + sizeof(unsigned long long) + sizeof(int) * njobs;
    cudaError_t e = cudaMalloc(&H->dmem, jobs_b + tabs_b + H->ctr_bytes);
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
    if (e != cudaSuccess) {
        cudaFree(H->dmem);
        delete H;
        return cuda_fail(e, "batch tables upload");
    }
    H->ctr_base = base + jobs_b + tabs_b;
    B.jobs = (const BatchJob *)base;
    B.ctr = (BatchCtr *)H->ctr_base;
    B.iter_total = (unsigned long long *)((char *)H->ctr_base + sizeof(BatchCtr));
    B.ff_done = (int *)((char *)H->ctr_base + sizeof(BatchCtr) + sizeof(unsigned long long));
    B.err = device_error_word();
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
    delete H;
    return set_ok();
}
