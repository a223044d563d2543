// pp_api.cu -- status handling, grid geometry, and the drop-in C symbols of the
// reference core (ppafm/cpp/ProbeParticle.cpp:319-701) over the device kernels.
//
// The drop-in layer keeps the reference's process-global configuration (grid shape,
// cell, borrowed float64 grid pointers, tip and relaxation parameters; ProbeParticle.cpp
// :33-114) and its calling convention: host float64 arrays in, results written back
// into the caller's arrays, force fields ACCUMULATED into the borrowed grid.  Each call
// mirrors its inputs to device memory owned by the library, runs the kernels on a
// library stream and synchronises before returning.
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "pp_common.cuh"

namespace ppgpu {

// ------------------------------------------------------------------ status state

static thread_local int g_status = PPGPU_OK;
static thread_local char g_msg[512] = "ok";

int set_error(int status, const char *fmt, ...) {
    g_status = status;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_msg, sizeof(g_msg), fmt, ap);
    va_end(ap);
    return status;
}

int set_ok() {
    g_status = PPGPU_OK;
    snprintf(g_msg, sizeof(g_msg), "ok");
    return PPGPU_OK;
}

int cuda_fail(cudaError_t e, const char *what) {
    return set_error(PPGPU_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

static std::mutex g_err_mutex;
static int *g_err_words[64] = {nullptr};

int *device_error_word() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lock(g_err_mutex);
    if (!g_err_words[dev]) {
        int *p = nullptr;
        if (cudaMalloc(&p, sizeof(int)) != cudaSuccess) return nullptr;
        if (cudaMemset(p, 0, sizeof(int)) != cudaSuccess) return nullptr;
        g_err_words[dev] = p;
    }
    return g_err_words[dev];
}

int *device_error_word_if_allocated() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lock(g_err_mutex);
    return g_err_words[dev];
}

// GridShape::setCell + Mat3::invert_T_to (Grid.h:29-36, Mat3.h:275-286).
int make_geom(const int *n, const double *cell, GridGeom *g) {
    for (int k = 0; k < 3; k++) {
        if (n[k] <= 0) return set_error(PPGPU_ERR_ARG, "grid size n[%d] = %d must be positive", k, n[k]);
        g->n[k] = n[k];
        const double inv = 1.0 / n[k];
        for (int j = 0; j < 3; j++) g->dcell[3 * k + j] = cell[3 * k + j] * inv;
    }
    const double *d = g->dcell;
    const double xx = d[0], xy = d[1], xz = d[2], yx = d[3], yy = d[4], yz = d[5], zx = d[6], zy = d[7], zz = d[8];
    const double det = xx * (yy * zz - yz * zy) + xy * (yz * zx - yx * zz) + xz * (yx * zy - yy * zx);
    if (!(det != 0.0)) return set_error(PPGPU_ERR_ARG, "grid cell is singular");
    const double id = 1 / det;
    double *m = g->dicell;
    m[0] = (yy * zz - yz * zy) * id;
    m[3] = (xz * zy - xy * zz) * id;
    m[6] = (xy * yz - xz * yy) * id;
    m[1] = (yz * zx - yx * zz) * id;
    m[4] = (xx * zz - xz * zx) * id;
    m[7] = (xz * yx - xx * yz) * id;
    m[2] = (yx * zy - yy * zx) * id;
    m[5] = (xy * zx - xx * zy) * id;
    m[8] = (xx * yy - xy * yx) * id;
    return set_ok();
}

// --------------------------------------------------------------- drop-in state

struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    int ensure(size_t bytes) {
        if (bytes <= cap) return PPGPU_OK;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc (drop-in buffer)");
        cap = bytes;
        return PPGPU_OK;
    }
};

struct HostBuf {
    void *p = nullptr;
    size_t cap = 0;
    int ensure(size_t bytes) {
        if (bytes <= cap) return PPGPU_OK;
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        cudaError_t e = cudaMallocHost(&p, bytes);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMallocHost (staging)");
        cap = bytes;
        return PPGPU_OK;
    }
};

struct Facade {
    int n[3] = {0, 0, 0};
    bool has_n = false;
    double cell[9] = {0};
    bool has_cell = false;
    double *gridF = nullptr;
    double *gridE = nullptr;
    // RELAX / FIRE defaults (ProbeParticle.cpp:76-103)
    int maxIters = 1000;
    double convF2 = 1.0e-8, dt = 0.1, damping = 0.1;
    double finc = 1.1, fdec = 0.5, falpha = 0.99;
    // TIP (zero until setTip, ProbeParticle.cpp:51-55)
    double lRadial = 0, kRadial = 0, rPP0[3] = {0, 0, 0}, kSpring[3] = {0, 0, 0};
    long long last_iters = 0;
    cudaStream_t stream = nullptr;
    DevBuf fe, atoms, strokes, f64stage, counters;
    HostBuf pinned;
};

static Facade g_f;
static std::mutex g_f_mutex;

static int facade_stream(cudaStream_t *st) {
    if (!g_f.stream) {
        cudaError_t e = cudaStreamCreateWithFlags(&g_f.stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamCreate");
    }
    *st = g_f.stream;
    return PPGPU_OK;
}

static long long facade_npts() { return (long long)g_f.n[0] * g_f.n[1] * g_f.n[2]; }

constexpr size_t STAGE_PTS = 1 << 21;  // points per host<->device chunk

// Adds (accumulate) the float4 device grid into the borrowed float64 host grids.
static int facade_accumulate_to_host(const float4 *FEd, cudaStream_t st, bool to_F, bool to_E) {
    const long long npts = facade_npts();
    int s = g_f.pinned.ensure(STAGE_PTS * sizeof(float4));
    if (s) return s;
    float4 *h = (float4 *)g_f.pinned.p;
    for (long long p0 = 0; p0 < npts; p0 += (long long)STAGE_PTS) {
        const long long m = std::min<long long>(STAGE_PTS, npts - p0);
        PPGPU_CUDA(cudaMemcpyAsync(h, FEd + p0, m * sizeof(float4), cudaMemcpyDeviceToHost, st), "D2H force grid");
        PPGPU_CUDA(cudaStreamSynchronize(st), "sync D2H");
        double *F = g_f.gridF + 3 * p0;
        double *E = g_f.gridE ? g_f.gridE + p0 : nullptr;
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < m; i++) {
            if (to_F) {
                F[3 * i] += h[i].x;
                F[3 * i + 1] += h[i].y;
                F[3 * i + 2] += h[i].z;
            }
            if (to_E && E) E[i] += h[i].w;
        }
    }
    return set_ok();
}

// Mirrors the borrowed float64 force grid to the float4 device grid.
static int facade_upload_grid(float4 *FEd, cudaStream_t st) {
    const long long npts = facade_npts();
    int s = g_f.f64stage.ensure(STAGE_PTS * 3 * sizeof(double));
    if (s) return s;
    for (long long p0 = 0; p0 < npts; p0 += (long long)STAGE_PTS) {
        const long long m = std::min<long long>(STAGE_PTS, npts - p0);
        PPGPU_CUDA(cudaMemcpyAsync(g_f.f64stage.p, g_f.gridF + 3 * p0, m * 3 * sizeof(double), cudaMemcpyHostToDevice,
                                   st),
                   "H2D force grid");
        s = ppgpu_grid_from_f64((float *)(FEd + p0), (const double *)g_f.f64stage.p, nullptr, m, st);
        if (s) return s;
    }
    return set_ok();
}

static int facade_ff(int natoms, const double *R, const double *coefs, int mode, int kind) {
    if (!g_f.has_n || !g_f.has_cell) return set_error(PPGPU_ERR_STATE, "setGridN/setGridCell must be called first");
    if (natoms < 0) return set_error(PPGPU_ERR_ARG, "natoms < 0");
    if (!g_f.gridF && !g_f.gridE) return set_ok();  // the reference computes and stores nothing
    if (natoms > 0 && (!R || !coefs)) return set_error(PPGPU_ERR_ARG, "null atom arrays");
    cudaStream_t st;
    int s = facade_stream(&st);
    if (s) return s;
    std::vector<float> rec((size_t)std::max(natoms, 1) * PPGPU_ATOM_FLOATS);
    int nch = 0;
    if (mode == PPGPU_FF_LJ)
        s = ppgpu_pack_atoms(natoms, R, coefs, nullptr, rec.data(), &nch);
    else
        s = ppgpu_pack_atoms(natoms, R, nullptr, coefs, rec.data(), &nch);
    if (s) return s;
    const size_t abytes = rec.size() * sizeof(float);
    if ((s = g_f.atoms.ensure(abytes))) return s;
    PPGPU_CUDA(cudaMemcpyAsync(g_f.atoms.p, rec.data(), abytes, cudaMemcpyHostToDevice, st), "H2D atoms");
    const long long npts = facade_npts();
    if ((s = g_f.fe.ensure((size_t)npts * sizeof(float4)))) return s;
    const int flags = g_f.gridE ? PPGPU_FF_WITH_E : 0;
    s = ppgpu_ff_grid((float *)g_f.fe.p, g_f.n, g_f.cell, (const float *)g_f.atoms.p, natoms, nch, mode, kind, 0.0, 0.0,
                      nullptr, nullptr, flags, st);
    if (s) return s;
    s = facade_accumulate_to_host((const float4 *)g_f.fe.p, st, g_f.gridF != nullptr, g_f.gridE != nullptr);
    if (s) return s;
    return ppgpu_device_status(st);
}

static void facade_params(double *prm) {
    prm[0] = g_f.maxIters;
    prm[1] = g_f.convF2;
    prm[2] = g_f.dt;
    prm[3] = g_f.damping;
    prm[4] = g_f.finc;
    prm[5] = g_f.fdec;
    prm[6] = g_f.falpha;
    prm[7] = g_f.lRadial;
    prm[8] = g_f.kRadial;
    for (int k = 0; k < 3; k++) {
        prm[9 + k] = g_f.rPP0[k];
        prm[12 + k] = g_f.kSpring[k];
    }
}

static int facade_relax_body(int nstroke, int probeStart, int relaxAlg, int nstep, const double *rTips, double *rs,
                             double *fs, int *itrsum_out) {
    if (!g_f.has_n || !g_f.has_cell) return set_error(PPGPU_ERR_STATE, "setGridN/setGridCell must be called first");
    if (!g_f.gridF) return set_error(PPGPU_ERR_STATE, "setFF_Fpointer must be called first");
    if (nstroke < 0 || nstep < 0) return set_error(PPGPU_ERR_ARG, "negative sizes");
    if ((long long)nstroke * nstep == 0) {
        g_f.last_iters = 0;
        if (itrsum_out) *itrsum_out = 0;
        return set_ok();
    }
    if (!rTips || !rs || !fs) return set_error(PPGPU_ERR_ARG, "null stroke arrays");
    cudaStream_t st;
    int s = facade_stream(&st);
    if (s) return s;
    const long long npts = facade_npts();
    if ((s = g_f.fe.ensure((size_t)npts * sizeof(float4)))) return s;
    if ((s = facade_upload_grid((float4 *)g_f.fe.p, st))) return s;
    const size_t nel = (size_t)nstroke * nstep * 3;
    if ((s = g_f.strokes.ensure(nel * 3 * sizeof(double) + (size_t)nstroke * sizeof(int) + 64))) return s;
    double *dT = (double *)g_f.strokes.p;
    double *dR = dT + nel;
    double *dF = dR + nel;
    int *dSum = (int *)(dF + nel);
    if ((s = g_f.counters.ensure(sizeof(unsigned long long)))) return s;
    unsigned long long *dTot = (unsigned long long *)g_f.counters.p;
    PPGPU_CUDA(cudaMemsetAsync(dTot, 0, sizeof(unsigned long long), st), "memset counter");
    PPGPU_CUDA(cudaMemcpyAsync(dT, rTips, nel * sizeof(double), cudaMemcpyHostToDevice, st), "H2D rTips");
    double prm[PPGPU_RELAX_NPARAM];
    facade_params(prm);
    s = ppgpu_relax_strokes((const float *)g_f.fe.p, g_f.n, g_f.cell, prm, probeStart, relaxAlg, nstroke, nstep, dT,
                            dR, dF, nullptr, dSum, dTot, st);
    if (s) return s;
    PPGPU_CUDA(cudaMemcpyAsync(rs, dR, nel * sizeof(double), cudaMemcpyDeviceToHost, st), "D2H rs");
    PPGPU_CUDA(cudaMemcpyAsync(fs, dF, nel * sizeof(double), cudaMemcpyDeviceToHost, st), "D2H fs");
    unsigned long long tot = 0;
    PPGPU_CUDA(cudaMemcpyAsync(&tot, dTot, sizeof(tot), cudaMemcpyDeviceToHost, st), "D2H iterations");
    int sum0 = 0;
    if (itrsum_out) PPGPU_CUDA(cudaMemcpyAsync(&sum0, dSum, sizeof(int), cudaMemcpyDeviceToHost, st), "D2H itrsum");
    if ((s = ppgpu_device_status(st))) return s;
    g_f.last_iters = (long long)tot;
    if (itrsum_out) *itrsum_out = sum0;
    return set_ok();
}

// TIP::SplineParams (ProbeParticle.cpp:58-62): the struct ppafm/core.py passes by pointer.
struct SplineParamsC {
    int rff_n;
    double *rff_xs;
    double *rff_ydys;
};

struct FacadeRelaxArgs {
    int nstroke, probeStart, relaxAlg, nstep;
    const double *rTips;
    double *rs, *fs;
    int *itrsum_out;
};

static int facade_relax_tramp(void *p) {
    FacadeRelaxArgs *a = (FacadeRelaxArgs *)p;
    return facade_relax_body(a->nstroke, a->probeStart, a->relaxAlg, a->nstep, a->rTips, a->rs, a->fs, a->itrsum_out);
}

// relaxTipStroke(s): with a spline, its radial force replaces the harmonic radial spring for
// this call (forceRSpline, ProbeParticle.cpp:212-225).
static int facade_relax(int nstroke, int probeStart, int relaxAlg, int nstep, const double *rTips, double *rs,
                        double *fs, void *spline, int *itrsum_out) {
    if (!spline) return facade_relax_body(nstroke, probeStart, relaxAlg, nstep, rTips, rs, fs, itrsum_out);
    const SplineParamsC *sp = (const SplineParamsC *)spline;
    if (sp->rff_n < 2 || !sp->rff_xs || !sp->rff_ydys) return set_error(PPGPU_ERR_ARG, "tip spline: need at least 2 knots and both arrays");
    FacadeRelaxArgs a = {nstroke, probeStart, relaxAlg, nstep, rTips, rs, fs, itrsum_out};
    return with_tip_spline(sp->rff_n, sp->rff_xs, sp->rff_ydys, facade_relax_tramp, &a);
}

}  // namespace ppgpu

using namespace ppgpu;

// ---------------------------------------------------------------- status API

extern "C" const char *ppgpu_last_error(void) { return g_msg; }
extern "C" int ppgpu_last_status(void) { return g_status; }

// Reads (and clears) the error words that kernels set when a bounded wait gives up: the
// library's per-device word and that of the no-allocation entry point's fixed array.  Words
// that were never allocated or looked up were never written; nothing is allocated here.
extern "C" int ppgpu_device_status(void *stream) {
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "stream synchronize");
    int *words[2] = {device_error_word_if_allocated(), noalloc_error_word_if_loaded()};
    int first = 0;
    for (int *w : words) {
        if (!w) continue;
        int code = 0;
        e = cudaMemcpy(&code, w, sizeof(int), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(e, "read device error word");
        if (code) {
            e = cudaMemset(w, 0, sizeof(int));
            if (e != cudaSuccess) return cuda_fail(e, "clear device error word");
            if (!first) first = code;
        }
    }
    if (first) return set_error(first, "a kernel gave up on a bounded device-side wait (code %d)", first);
    return set_ok();
}

extern "C" int ppgpu_device_info(char *buf, int len) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    cudaDeviceProp p;
    e = cudaGetDeviceProperties(&p, dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceProperties");
    if (buf && len > 0) snprintf(buf, (size_t)len, "sm_%d%d %s sms=%d", p.major, p.minor, p.name, p.multiProcessorCount);
    if (p.major * 10 + p.minor < 100) return set_error(PPGPU_ERR_NO_DEVICE, "device sm_%d%d is not Blackwell", p.major, p.minor);
    return set_ok();
}

// ------------------------------------------------------------ drop-in symbols

extern "C" void setGridN(int *n) {
    std::lock_guard<std::mutex> lock(g_f_mutex);
    if (!n) {
        set_error(PPGPU_ERR_ARG, "setGridN: null");
        return;
    }
    for (int k = 0; k < 3; k++) g_f.n[k] = n[k];
    g_f.has_n = n[0] > 0 && n[1] > 0 && n[2] > 0;
    if (!g_f.has_n)
        set_error(PPGPU_ERR_ARG, "setGridN: sizes must be positive");
    else
        set_ok();
}

extern "C" void setGridCell(double *cell) {
    std::lock_guard<std::mutex> lock(g_f_mutex);
    if (!cell) {
        set_error(PPGPU_ERR_ARG, "setGridCell: null");
        return;
    }
    for (int k = 0; k < 9; k++) g_f.cell[k] = cell[k];
    g_f.has_cell = true;
    set_ok();
}

extern "C" void setFF_Fpointer(double *gridF) {
    std::lock_guard<std::mutex> lock(g_f_mutex);
    g_f.gridF = gridF;
    set_ok();
}
extern "C" void setFF_Epointer(double *gridE) {
    std::lock_guard<std::mutex> lock(g_f_mutex);
    g_f.gridE = gridE;
    set_ok();
}
extern "C" void deleteFF_Fpointer(void) {
    std::lock_guard<std::mutex> lock(g_f_mutex);
    g_f.gridF = nullptr;
}
extern "C" void deleteFF_Epointer(void) {
    std::lock_guard<std::mutex> lock(g_f_mutex);
    g_f.gridE = nullptr;
}

extern "C" void setRelax(int maxIters, double convF2, double dt, double damping) {
    std::lock_guard<std::mutex> lock(g_f_mutex);
    g_f.maxIters = maxIters;
    g_f.convF2 = convF2;
    g_f.dt = dt;  // FIRE::setup: dtmax = dt, acoef0 = damping
    g_f.damping = damping;
    set_ok();
}

extern "C" void setFIRE(double finc, double fdec, double falpha) {
    std::lock_guard<std::mutex> lock(g_f_mutex);
    g_f.finc = finc;
    g_f.fdec = fdec;
    g_f.falpha = falpha;
    set_ok();
}

extern "C" void setTip(double lRad, double kRad, double *rPP0, double *kSpring) {
    std::lock_guard<std::mutex> lock(g_f_mutex);
    g_f.lRadial = lRad;
    g_f.kRadial = kRad;
    for (int k = 0; k < 3; k++) {
        g_f.rPP0[k] = rPP0 ? rPP0[k] : 0.0;
        g_f.kSpring[k] = kSpring ? kSpring[k] : 0.0;
    }
    // TIP::makeConsistent (ProbeParticle.cpp:64-69)
    if (fabs(kRad) > 1e-8)
        g_f.rPP0[2] = -sqrt(lRad * lRad - g_f.rPP0[0] * g_f.rPP0[0] - g_f.rPP0[1] * g_f.rPP0[1]);
    set_ok();
}

extern "C" void getLennardJonesFF(int natoms, double *Ratoms, double *cLJs) {
    std::lock_guard<std::mutex> lock(g_f_mutex);
    facade_ff(natoms, Ratoms, cLJs, PPGPU_FF_LJ, 0);
}

extern "C" void getCoulombFF(int natoms, double *Ratoms, double *kQQs, int kind) {
    std::lock_guard<std::mutex> lock(g_f_mutex);
    if (kind < 0 || kind > 2) {
        set_error(PPGPU_ERR_ARG, "getCoulombFF: kind %d not in {0,1,2}", kind);
        return;
    }
    facade_ff(natoms, Ratoms, kQQs, PPGPU_FF_COULOMB, kind);
}

extern "C" int relaxTipStroke(int probeStart, int relaxAlg, int nstep, double *rTips, double *rs, double *fs,
                              void *splineParams) {
    std::lock_guard<std::mutex> lock(g_f_mutex);
    int sum = 0;
    if (facade_relax(1, probeStart, relaxAlg, nstep, rTips, rs, fs, splineParams, &sum)) return 0;
    return sum;
}

extern "C" int relaxTipStrokes_omp(int nx, int ny, int probeStart, int relaxAlg, int nstep, double *rTips, double *rs,
                                   double *fs, void *splineParams) {
    std::lock_guard<std::mutex> lock(g_f_mutex);
    facade_relax(nx * ny, probeStart, relaxAlg, nstep, rTips, rs, fs, splineParams, nullptr);
    return 0;
}

extern "C" long long ppgpu_last_iterations(void) { return g_f.last_iters; }
