// pp_common.cuh -- shared host/device helpers of libppgpu (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/ppgpu.h"

namespace ppgpu {

// ----------------------------------------------------------------- host status

// Records a status + message as the library's last error; returns the status.
int set_error(int status, const char *fmt, ...);
int set_ok();
// Translates a CUDA error into PPGPU_ERR_CUDA with context.
int cuda_fail(cudaError_t e, const char *what);
// Per-device error word that kernels set when a bounded wait gives up (allocated on first
// use); the _if_allocated form returns it without allocating (nullptr before first use).
int *device_error_word();
int *device_error_word_if_allocated();
// Error word of the no-allocation entry point's fixed array on the current device, or nullptr
// while no call has looked the array up on it (pp_ff.cu); never allocates.
int *noalloc_error_word_if_loaded();
// Runs fn(arg) with the radial tip spline (n knots xs, (value, slope) pairs ydys; n 0: none)
// in place of the current one, then restores it; returns fn's status (pp_relax.cu).
int with_tip_spline(int n, const double *xs, const double *ydys, int (*fn)(void *), void *arg);

#define PPGPU_CUDA(call, what)                           \
    do {                                                 \
        cudaError_t _e = (call);                         \
        if (_e != cudaSuccess) return cuda_fail(_e, what); \
    } while (0)

#define PPGPU_CHECK_LAUNCH(what) PPGPU_CUDA(cudaGetLastError(), what)

// --------------------------------------------------------------- grid geometry

// Voxel basis and its transposed inverse (GridShape::setCell, Grid.h:29-36).
struct GridGeom {
    int n[3];
    double dcell[9];   // rows: a/n0, b/n1, c/n2
    double dicell[9];  // rows: grid coordinate g_k = r . dicell_row_k
};
int make_geom(const int *n, const double *cell, GridGeom *g);

// ----------------------------------------------------------------- device side

// Periodic wrap of an index that is known to be near [0, n).
__device__ __forceinline__ int wrap_index(int i, int n) {
    if (i < 0) {
        i += n;
        if (i < 0) i = ((i % n) + n) % n;
    } else if (i >= n) {
        i -= n;
        if (i >= n) i %= n;
    }
    return i;
}

__device__ __forceinline__ float rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ float rsqrt_approx(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Read-only 16-byte gather.
__device__ __forceinline__ float4 ldg4(const float4 *p) { return __ldg(p); }

// Sets the device error word (first error wins).
__device__ __forceinline__ void raise_device_error(int *err, int code) {
    if (err) atomicCAS(err, 0, code);
}

}  // namespace ppgpu
