/*
 * ppgpu.h -- C ABI of libppgpu.so, the GB300 (sm_103a) probe-particle AFM hot path.
 *
 * Two layers share one library:
 *
 *  1. Drop-in symbols.  The exact names and signatures that the reference's ctypes
 *     layer (ppafm/core.py) binds from ProbeParticle_lib.so, for the in-scope subset.
 *     They keep the reference's process-global state and host (numpy) float64 buffers;
 *     each call mirrors what it needs to the GPU and writes results back into the
 *     caller's arrays.  A ctypes binding written for the reference binds these unchanged.
 *
 *  2. Device API (ppgpu_*).  Plain device pointers, sizes and a CUDA stream (void*,
 *     NULL = legacy default stream).  Every function returns a status code; no function
 *     takes ownership of caller memory.  Force grids are interleaved float4
 *     (Fx, Fy, Fz, E) in C order [n0][n1][n2] (the reference's i3D order, Grid.h:16).
 *
 * Errors: every ppgpu_* call returns PPGPU_OK or an error code, with a message in
 * ppgpu_last_error().  The drop-in symbols return void like the reference; they set the
 * same last-error state (read it with ppgpu_last_error()/ppgpu_last_status()).
 * Device-side waits are bounded: a kernel that gives up sets a device error word that
 * ppgpu_device_status() reads (PPGPU_ERR_DEVICE_TIMEOUT) instead of hanging.
 */
#ifndef PPGPU_H
#define PPGPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status codes */
#define PPGPU_OK 0
#define PPGPU_ERR_ARG 1            /* invalid argument (sizes, null pointers, modes) */
#define PPGPU_ERR_CUDA 2           /* a CUDA runtime / cuFFT call failed */
#define PPGPU_ERR_STATE 3          /* drop-in call before the state it needs was set */
#define PPGPU_ERR_DEVICE_TIMEOUT 4 /* a bounded device-side wait gave up */
#define PPGPU_ERR_NO_DEVICE 5      /* no CUDA device / wrong architecture */

const char *ppgpu_last_error(void);
int ppgpu_last_status(void);
/* Synchronises `stream`, returns PPGPU_OK or the device error recorded by a kernel
 * (and clears it). */
int ppgpu_device_status(void *stream);
/* Library/device description: writes "sm_XY <name>" into buf. */
int ppgpu_device_info(char *buf, int len);

/* =============================================================== 1. drop-in symbols */

/* ProbeParticle.cpp:358  (ppafm/core.py:38) */
void setGridN(int *n);
/* ProbeParticle.cpp:365  (core.py:48) -- cell: 3x3 row vectors a,b,c */
void setGridCell(double *cell);
/* ProbeParticle.cpp:338  (core.py:59) -- borrows the caller's [n0,n1,n2,3] float64 grid */
void setFF_Fpointer(double *gridF);
/* ProbeParticle.cpp:343  (core.py:69) -- borrows the caller's [n0,n1,n2] float64 grid */
void setFF_Epointer(double *gridE);
/* ProbeParticle.cpp:348  (core.py:79) */
void deleteFF_Fpointer(void);
/* ProbeParticle.cpp:353  (core.py:88) */
void deleteFF_Epointer(void);
/* ProbeParticle.cpp:322  (core.py:97; the reference wrapper is broken, the symbol is not) */
void setRelax(int maxIters, double convF2, double dt, double damping);
/* ProbeParticle.cpp:331  (core.py:106) */
void setFIRE(double finc, double fdec, double falpha);
/* ProbeParticle.cpp:371  (core.py:115) -- rPP0 is made consistent with lRad when kRad != 0 */
void setTip(double lRad, double kRad, double *rPP0, double *kSpring);
/* ProbeParticle.cpp:508  (core.py:193) -- gridF (+gridE if set) += LJ field of the atoms */
void getLennardJonesFF(int natoms, double *Ratoms, double *cLJs);
/* ProbeParticle.cpp:540  (core.py:270) -- kind 0 = s, 1 = pz, 2 = dz2 tip */
void getCoulombFF(int natoms, double *Ratoms, double *kQQs, int kind);
/* ProbeParticle.cpp:633  (core.py:312) -- returns the stroke's iteration sum.
 * splineParams: NULL, or a TIP::SplineParams {int rff_n; double *rff_xs; double *rff_ydys;}
 * whose radial force replaces the harmonic radial spring for this call. */
int relaxTipStroke(int probeStart, int relaxAlg, int nstep, double *rTips, double *rs, double *fs,
                   void *splineParams);
/* ProbeParticle.cpp:682  (core.py:322) -- returns 0 like the reference; the total
 * iteration count of the call is available from ppgpu_last_iterations(). */
int relaxTipStrokes_omp(int nx, int ny, int probeStart, int relaxAlg, int nstep, double *rTips, double *rs,
                        double *fs, void *splineParams);
/* Total FIRE iterations of the last relaxTipStroke(s) call (no reference counterpart:
 * the reference discards them, ProbeParticle.cpp:682-701). */
long long ppgpu_last_iterations(void);

/* ================================================================== 2. device API */

/* ---------------------------------------------------------------- atom records
 * Force-field kernels read atoms as packed 48-byte records (12 floats):
 *   [-x_hi, -y_hi, -x_lo, -y_lo] [-z_hi, -z_lo, -6*c6, 12*c12] [-c6, c12, kqq, 0]
 * where x = x_hi + x_lo splits the float64 coordinate (relative to the grid origin)
 * into two floats, kqq is the Coulomb coefficient of the atom (k_e*Q for the CPU-core
 * modes, the bare charge for PPGPU_FF_QZS) and (c6, c12) are the Lennard-Jones
 * coefficients.  The first `ncharged` records are the atoms with kqq != 0.
 * ppgpu_pack_atoms builds this layout on the host. */
#define PPGPU_ATOM_FLOATS 12
int ppgpu_pack_atoms(int natoms, const double *R, const double *cLJ, const double *kqq, float *out,
                     int *ncharged_out);

/* ---------------------------------------------------------------- FF generation
 * mode:
 *   PPGPU_FF_LJ        F += sum_i LJ(p - R_i)                     (getLennardJonesFF)
 *   PPGPU_FF_COULOMB   F += sum_i Coulomb_kind(p - R_i)            (getCoulombFF, coul_kind 0/1/2)
 *   PPGPU_FF_LJC       F  = clamp(F_LJ) + Q * clamp(F_el)          (perform_relaxation's
 *                      FF = FFLJ + Q*FFel after computeLJ / computeELFF_pointCharge clamps,
 *                      HighLevel.py:143-145, 294-296, 374-376; clamp skipped when Fmax <= 0)
 *   PPGPU_FF_QZS       F  = LJ + sum_k Qs[k]*k_e*Coulomb(p + QZs[k] z) (AFMulator point-charge,
 *                      FF.cl:366-423), R2SAFE 1e-6
 * flags: PPGPU_FF_WITH_E (also E in .w; otherwise .w = 0), PPGPU_FF_ACCUMULATE (add into FE),
 *        PPGPU_FF_F64 (float64 sums; result still stored as float4).
 * Grid point (ia,ib,ic) sits at origin + ia*a/n0 + ib*b/n1 + ic*c/n2; atom coordinates
 * in the records are relative to `origin`.  cell: rows a, b, c (float64, host). */
#define PPGPU_FF_LJ 0
#define PPGPU_FF_COULOMB 1
#define PPGPU_FF_LJC 2
#define PPGPU_FF_QZS 3
#define PPGPU_FF_WITH_E 1
#define PPGPU_FF_ACCUMULATE 2
#define PPGPU_FF_F64 4 /* evaluate the sums in float64 (the GPU error oracle); always on for
                          the pz/dz2 Coulomb tips, whose finite differences need it */
int ppgpu_ff_grid(float *FE, const int *n, const double *cell, const float *atoms, int natoms, int ncharged,
                  int mode, int coul_kind, double Q, double Fmax, const double *Qs, const double *QZs, int flags,
                  void *stream);

/* Sub-box variant: fills FE[ns0][ns1][ns2] with the points [i0, i0+ns) of the full grid n. */
int ppgpu_ff_subgrid(float *FE, const int *n, const double *cell, const int *i0, const int *ns,
                     const float *atoms, int natoms, int ncharged, int mode, int coul_kind, double Q,
                     double Fmax, const double *Qs, const double *QZs, int flags, void *stream);

/* ------------------------------------------------------------------- relaxation
 * Tip/relaxation parameters shared by the relax entry points (float64, host):
 *   prm[0]  maxIters        prm[1] convF2    prm[2] dt (= dtmax)  prm[3] damping (= acoef0)
 *   prm[4]  finc            prm[5] fdec      prm[6] falpha
 *   prm[7]  lRadial         prm[8] kRadial   prm[9..11] rPP0 (consistent)  prm[12..14] kSpring
 * (ProbeParticle.cpp:51-114; set by setRelax/setFIRE/setTip.) */
#define PPGPU_RELAX_NPARAM 15

/* relaxTipStrokes_omp semantics on device buffers: stroke s uses rTips[s*nstep .. +nstep)
 * (float64 xyz, relative to the grid origin); writes rs, fs (float64 xyz) and, when
 * non-NULL, iters[s*nstep+i] (int32) and itrsum[s] (int32).  iter_total (nullable, device
 * u64) accumulates all iterations.  probeStart -1/0/1, relaxAlg 0 (damped MD) / 1 (FIRE). */
int ppgpu_relax_strokes(const float *FE, const int *n, const double *cell, const double *prm, int probeStart,
                        int relaxAlg, int nstroke, int nstep, const double *rTips, double *rs, double *fs,
                        int *iters, int *itrsum, unsigned long long *iter_total, void *stream);

/* relaxedScan3D_omp + Fz2df semantics on a regular scan (HighLevel.py:104-124,
 * common.py:421-430): tips at (xs[ix], ys[iy], zs[iz]) with zs descending (the approach
 * order) and coordinates relative to the grid origin; pixel p = ix*ny + iy.
 * Outputs (ascending z, like the reference's reversed arrays; each nullable):
 *   fzs   [nx][ny][nz]   float32   grid Fz at the relaxed position
 *   ppos  [nx][ny][nz][3] float32  relaxed position + pos_offset[3]
 *   iters [nx][ny][nz]   int32
 *   df    [nx][ny][nz-nw+1] float32 = sum_i fzs[j+i]*W[nw-1-i]  (np.convolve 'valid'),
 *         W = df_weights (already scaled by units*f0/k0), nw <= 64; df NULL skips it. */
int ppgpu_relax_scan(const float *FE, const int *n, const double *cell, const double *prm, int nx, int ny, int nz,
                     const double *xs, const double *ys, const double *zs, const double *pos_offset, float *fzs,
                     float *ppos, int *iters, int nw, const double *df_weights, float *df,
                     unsigned long long *iter_total, void *stream);

/* Radial tip spline of the relaxation (TIP::SplineParams + forceRSpline,
 * ProbeParticle.cpp:58-62, 212-225): n knots xs (float64, ascending) and n (value, slope)
 * pairs ydys of the radial force; it replaces the harmonic radial spring in
 * ppgpu_relax_strokes / ppgpu_relax_scan calls made after it is set; n = 0 clears it.  The
 * drop-in relaxTipStroke(s) take the same data as their SplineParams argument (per call).
 * The batched launch refuses to be created while a spline is set. */
int ppgpu_set_tip_spline(int n, const double *xs, const double *ydys);

/* Lanes per stroke of ppgpu_relax_strokes / ppgpu_relax_scan (no reference counterpart):
 * tps 1, 2, 4 or 8 lanes share each stroke's trilinear gathers (same results bit for bit);
 * 0 restores the default, 1.  ppgpu_get_relax_tps returns the value used for nstroke strokes. */
int ppgpu_set_relax_tps(int tps);
/* No counterpart in the reference (a launch-shape knob).  Threads per CTA of the single-grid
 * force-field kernel: 128 or 256, 0 = the default (128). */
int ppgpu_set_ff_block(int threads);
int ppgpu_get_relax_tps(long long nstroke, int *out);

/* AFMulator relaxation (relaxStrokesTilted, relax.cl:391-464, + convolveZ, relax.cl:571-608):
 * prm_afm[0..3] relax_params (dt, damp, -, -), [4..7] stiffness (kx,ky,kz,kr) already divided
 * by -eVA_Nm, [8..11] dpos0 (x,y,z,l0), [12..23] tip rows A,B,C (4 each, C[3] = -zstep),
 * [24..27] surfFF.  inv_cell: rows of transpose(inv(cell)) (fractional coordinates).
 * points: [npix][4] float32 tip start positions relative to the FF origin.
 * Outputs (nullable): FEs/paths [npix][nz][4] float32 (scan order), iters [npix][nz] int32,
 * X [npix][nz-nw+1] float32 = sum_j FEs[o+j].z * W[j] (no flip). */
#define PPGPU_AFM_NPARAM 28
int ppgpu_relax_afm(const float *FE, const int *n, const double *inv_cell, const double *prm_afm, int npix,
                    const float *points, int nz, float *FEs, float *paths, int *iters, int nw,
                    const double *weights, float *X, unsigned long long *iter_total, void *stream);

/* ------------------------------------------------------------------ FFT route
 * A plan handle owns the cuFFT plans and spectrum buffers of one grid shape n (C order
 * [n0][n1][n2], float32 real grids).  lvec: 4x3 float64 (origin, a, b, c). */
#define PPGPU_FFT_F64 1 /* transforms and spectra in float64 (grids stay float32) */
int ppgpu_fft_create(const int *n, int flags, void **handle);
int ppgpu_fft_destroy(void *handle);
/* potential2forces_mem (ppafm/fieldFFT.py:268-319): FE = (ACCUMULATE ? FE : 0)
 * + scale * (Fx, Fy, Fz, E) of the cross-correlation of V with rho (E only with WITH_E). */
int ppgpu_fft_potential2forces(void *handle, const float *V, const float *rho, const double *lvec, double scale,
                               int flags, float *FE, void *stream);
/* getProbeDensity (fieldFFT.py:99-118): normalised Gaussian of width sigma times the
 * multipole coefficients (s, px, py, pz, dz2, dx2, dy2, dxy, dxz, dyz; NULL = pure s). */
int ppgpu_fft_probe_density(void *handle, float *rho, const double *lvec, double sigma, const double *multipole,
                            void *stream);
/* handle_negative_density (ppafm/cli/conv_rho.py:18-22) when fix_negative, then rho^B (:63-64). */
int ppgpu_fft_density_power(void *handle, float *rho, double B, int fix_negative, void *stream);
/* Hartree potential (volts) of a periodic charge density (e/A^3): V_G = 4 pi k_e rho_G / G^2,
 * zero mean.  No counterpart in the reference (it reads potentials from DFT files). */
int ppgpu_fft_poisson(void *handle, const float *rho_charge, const double *lvec, float *V, void *stream);

/* AFMulator Hartree route, cross-correlation (FFTCrossCorrelation.correlate,
 * ppafm/ocl/field.py:800-840): E = IFFT(conj(FFT(rho)) FFT(V)) * scale / N on the plan's grid
 * (scale: the tip density's voxel volume in the reference).  The plan keeps the spectrum of
 * rho; rho NULL reuses it. */
int ppgpu_fft_correlate(void *handle, const float *V, const float *rho, double scale, float *E, void *stream);

/* Sum of normalised 3-D Gaussians on a periodic grid (minimum-image distances): atoms is a
 * DEVICE float64 array [natoms][5] = (x, y, z relative to the origin, sigma, weight).  Builds
 * synthetic electron and tip densities; no counterpart in the reference (it reads densities
 * from DFT files). */
int ppgpu_gaussian_density(float *rho, const int *n, const double *lvec, int natoms, const double *atoms,
                           int accumulate, void *stream);

/* ------------------------------------------------------------ batched systems
 * Many systems (molecules of uneven atom counts, cells and grids) in ONE persistent launch:
 * the LJC force field of each (the PPGPU_FF_LJC mode of ppgpu_ff_grid, no energy, no
 * accumulation), then its relaxed scan with ppgpu_relax_scan semantics and the fused df.
 * Replaces the per-molecule loop of the reference's batched caller (ppafm/ml/Generator.py:
 * 68-144 calling AFMulator once per molecule; relaxTipStrokes_omp, ProbeParticle.cpp:682-701,
 * per system).  Orthogonal cells only; at most 1024 charged atoms (with images) per system.
 * Tip coordinates are HOST arrays (copied at creation); FE, atoms and outputs are device
 * memory.  ppgpu_batch_run allocates nothing and does not synchronise (CUDA-graph safe). */
typedef struct {
    float *FE;            /* device float4 grid [n0][n1][n2], written */
    const float *atoms;   /* device atom records (ppgpu_pack_atoms), charged first */
    int natoms, ncharged;
    int n[3];
    double cell[9];       /* rows a, b, c: diagonal */
    int nx, ny, nz;
    const double *xs, *ys, *zs; /* host; relative to the grid origin; zs in approach order */
    double pos_offset[3];
    float *fzs, *ppos, *df; /* device outputs as in ppgpu_relax_scan (nullable) */
    int *iters;
} ppgpu_batch_job;
/* tuning[4] (NULL = defaults 2, 8, 4, 64): CTAs per SM (1-2), pixel tile width and height of
 * the stroke order, strokes per warp chunk.  prm: PPGPU_RELAX_NPARAM relaxation parameters;
 * Q, Fmax: probe charge and force clamp of the LJC field; df_weights: nw taps (nw 0 = no df). */
int ppgpu_batch_create(const ppgpu_batch_job *jobs, int njobs, const double *prm, double Q, double Fmax, int nw,
                       const double *df_weights, const int *tuning, void **handle);
int ppgpu_batch_run(void *handle, void *stream);
/* out4 = (force-field items, strokes incl. tile padding, CTAs, systems) */
int ppgpu_batch_info(void *handle, long long *out4);
/* FIRE iterations of the last run (synchronises the stream). */
int ppgpu_batch_iterations(void *handle, unsigned long long *out, void *stream);
int ppgpu_batch_destroy(void *handle);
/* No counterpart in the reference (failure detection).  Limit of a stroke's bounded wait for
 * its system's force field (wait_s seconds, default 2) and, for tests, a system whose force
 * field is treated as never published (held >= 0; -1 none): its strokes give up after the
 * limit and ppgpu_device_status reports PPGPU_ERR_DEVICE_TIMEOUT.  Synchronous. */
int ppgpu_batch_set_wait(void *handle, double wait_s, int held);
/* Height-synchronous run with an optional warm-start network (ppgpu_mlp_*; NULL = plain FIRE
 * from the height above): for each height the network proposes every stroke's starting
 * displacement and FIRE starts from the proposal unless its force residual exceeds the plain
 * start's.  rec_stride > 0 records training pairs of strokes gs % rec_stride == 0 at sample
 * (gs / rec_stride) * nz_max + iz: rec_x [.][96] bf16 features, rec_t [.][4] f32 targets.
 * Allocates its state buffers on the first call only; no host synchronisation. */
int ppgpu_batch_run_layered(void *handle, void *mlp, int rec_stride, void *rec_x, void *rec_t, void *stream);
/* out2 = (strokes including tile padding, largest nz). */
int ppgpu_batch_layer_info(void *handle, long long *out2);

/* ------------------------------------------------------------ tensor-core self test
 * D[128][N] (float32) = A[128][K] . B[N][K]^T with bf16 A, B (device, row-major), one tile
 * on the tcgen05 tensor cores (K multiple of 16 up to 128, N multiple of 16 up to 256).
 * No reference counterpart: checks the MMA building block of the warm-start network. */
int ppgpu_tc_selftest(const void *A, const void *B, int K, int N, float *D, void *stream);

/* ------------------------------------------------------------ warm-start network
 * No reference counterpart.  A 96 -> 128 -> 128 -> 16 SiLU MLP (bf16 weights and activations,
 * float32 accumulation) on the tcgen05 tensor cores; float32 master parameters (layout:
 * W1 [96][128] | W2 [128][128] | W3 [128][16] | b1 [128] | b2 [128] | b3 [16]) with Adam.
 * X rows: 96 bf16 (90 features + 6 zeros); T rows: 4 f32 (3 targets); Y rows: 16 f32. */
int ppgpu_mlp_create(unsigned long long seed, void **handle);
int ppgpu_mlp_destroy(void *handle);
int ppgpu_mlp_nparams(void);
int ppgpu_mlp_get(void *handle, int which, float *host); /* 0 params, 1 grads, 2/3 Adam moments */
int ppgpu_mlp_set(void *handle, const float *host);
int ppgpu_mlp_forward(void *handle, const void *X, int n, float *Y, void *stream);
int ppgpu_mlp_backward(void *handle, const void *X, const float *T, const int *idx, int nbatch, void *stream);
int ppgpu_mlp_adam(void *handle, double lr, int step, void *stream);
int ppgpu_mlp_take_loss(void *handle, double *out, void *stream);
int ppgpu_mlp_views(void *handle, void **out8);
/* Loss weights of the three outputs (default 1): loss = mean over samples of sum_o w_o (y_o - t_o)^2. */
int ppgpu_mlp_set_loss_weights(void *handle, const double *w3);

/* -------------------------------------------------------------- grid utilities */
/* Fz -> df along the last axis: out[c][j] = scale * sum_i F[c][j+i] * W[nw-1-i]. */
int ppgpu_fz2df(const float *F, long long ncol, int nz, int nw, const double *W, double scale, float *out,
                void *stream);
/* |F| <= Fmax clamp of a float4 grid, direction preserved (io.py:766-778). */
int ppgpu_clamp_grid(float *FE, long long npts, double Fmax, void *stream);

/* DataGrid.interp_at (ppafm/ocl/field.py:515-572, kernel interp_at, FF.cl:1010-1046): out
 * [nout0][nout1][nout2] float32 = periodic trilinear interpolation of in[nin0][nin1][nin2]
 * (origin origin_in[3], step vectors step_in[3][3] as rows) at origin_out + i a + j b + k c
 * (step_out rows), rotated about rot_center[3] by rot[3][3] (rows; NULL = none). */
int ppgpu_interp_grid(const float *in, const int *nin, const double *origin_in, const double *step_in, float *out,
                      const int *nout, const double *origin_out, const double *step_out, const double *rot,
                      const double *rot_center, void *stream);

/* DataGrid.grad (ppafm/ocl/field.py:454-513, kernel grad, FF.cl:920-961) in C order: FE float4
 * [n0][n1][n2] = scale[0..3] * (dE/dx, dE/dy, dE/dz, E), periodic centred differences with the
 * steps step[3]; accumulate != 0 adds to FE. */
int ppgpu_grad_fd(const float *E, const int *n, const double *step, const double *scale, float *FE, int accumulate,
                  void *stream);
/* ForceField.run_gradPotentialGrid (ppafm/ocl/field.py:1225-1317, kernel gradPotentialGrid,
 * FF.cl:964-1008): field float4 [nout0][nout1][nout2] = (-dV/dx, -dV/dy, -dV/dz, V) at
 * origin_out + i a + j b + k c (step_out rows), centred differences with steps h[3] of the
 * periodic trilinear interpolation of pot[nin0][nin1][nin2] (origin_in, step_in rows). */
int ppgpu_grad_potential_grid(const float *pot, const int *nin, const double *origin_in, const double *step_in,
                              float *field, const int *nout, const double *origin_out, const double *step_out,
                              const double *h, void *stream);
/* The tip charges of ForceField.run_evalLJC_Hartree (ppafm/ocl/field.py:1168-1223, kernel
 * evalLJC_Hartree, FF.cl:860-915): FE float4 [n0][n1][n2] (+)= sum_q Qs[q] * field(p + (0, 0,
 * QZs[q])) at the grid points p = origin + i a + j b + k c (step rows), the float4 field on the
 * same grid interpolated periodically; accumulate != 0 adds to FE (the Lennard-Jones part). */
int ppgpu_tip_charges_field(const float *field, const int *n, const double *origin, const double *step,
                            const double *Qs, const double *QZs, float *FE, int accumulate, void *stream);
/* TipDensity.interp_at (ppafm/ocl/field.py:606-650, kernel interp_tip_at, FF.cl:1049-1093): the
 * origin-centred tip density in[nin0][nin1][nin2] (grid steps step_in[3][3] rows, cell
 * cell_in[3][3] rows) resampled onto out[nout0][nout1][nout2] (steps step_out rows); output
 * indices past the middle are negative positions, points beyond half of the input cell are 0. */
int ppgpu_interp_tip_grid(const float *in, const int *nin, const double *step_in, const double *cell_in, float *out,
                          const int *nout, const double *step_out, void *stream);
/* DataGrid.clamp (ppafm/ocl/field.py:288-340; clamp_hard / clamp_soft, FF.cl:1179-1210):
 * out = in clipped to [minimum, maximum] (soft = 0) or sigmoid-blended into the bounds over
 * width (soft = 1); in == out allowed. */
int ppgpu_scalar_clamp(const float *in, float *out, long long n, double minimum, double maximum, int soft, double width,
                       void *stream);
/* DataGrid.add_mult (ppafm/ocl/field.py:342-376; addMult, FF.cl:1213-1223): out = a + scale*b. */
int ppgpu_scalar_add_mult(const float *a, const float *b, float *out, long long n, double scale, void *stream);
/* DataGrid.power_positive's normalisation sums (ppafm/ocl/field.py:431-452; normalizeSumReduce,
 * FF.cl:1108-1150): device sums[0] = sum of all values, sums[1] = sum of the positive ones
 * (float64). */
int ppgpu_scalar_sums(const float *in, long long n, double *sums, void *stream);
/* DataGrid.power_positive's power (ppafm/ocl/field.py:378-429; power, FF.cl:1095-1106):
 * out = scale * max(0, in)^p; in == out allowed. */
int ppgpu_scalar_power(const float *in, float *out, long long n, double p, double scale, void *stream);
/* FE_out = a*FE_a + b*FE_b (float4 grids; E included). */
int ppgpu_axpby_grid(float *FE_out, const float *FE_a, double a, const float *FE_b, double b, long long npts,
                     void *stream);
/* float64 [npts,3] (+ optional [npts] energy) <-> float4 conversions. */
int ppgpu_grid_from_f64(float *FE, const double *F3, const double *E, long long npts, void *stream);
int ppgpu_grid_to_f64(double *F3, double *E, const float *FE, long long npts, int accumulate, void *stream);

/* ------------------------------------------------------------- no-allocation entry
 * No counterpart in the reference.  The Lennard-Jones grid of getLennardJonesFF with device
 * pointers: gridF [n0,n1,n2,3] and gridE [n0,n1,n2] (float64, either may be NULL) are
 * ACCUMULATED into; Ratoms [natoms,3] (relative to the grid origin) and cLJs [natoms,2]
 * (c6, c12) are float64 device arrays; n and cell are host arrays.  For callers that cannot
 * allocate device memory at call time (an application whose allocator reserved the device
 * memory up front; a latency-sensitive loop that cannot take the device-wide
 * synchronisation of cudaMalloc/cudaFree): it allocates nothing and stages its scratch in a
 * fixed 5.5 MB array.  Limits: natoms <= 32768 and n2 <= 262144 (larger requests return
 * PPGPU_ERR_ARG).
 * Loading: the array is part of the library's device code, which CUDA loads on a device at
 * the first call there (lazy module loading, the default) -- that load takes device memory
 * once, and the device then holds the array until the process exits.  Callers that reserve
 * all device memory make one small call on each device first (or set
 * CUDA_MODULE_LOADING=EAGER).  The first call on a device also looks up the array's device
 * address (cudaGetSymbolAddress, once per device, cached for the process: the library does
 * not survive cudaDeviceReset).
 * All calls share the array and it keeps the last call's contents: calls that overlap on the
 * GPU race.  The call returns once its work is queued on `stream`; a bounded device wait that
 * gave up inside it is reported by ppgpu_device_status(stream), which also allocates
 * nothing. */
int ppgpu_lj_grid_f64_noalloc(double *gridF, double *gridE, const int *n, const double *cell, int natoms,
                              const double *Ratoms, const double *cLJs, void *stream);

/* ------------------------------------------------------------ measurement helper */
/* Runs a dependent-FFMA kernel for `iters` iterations on all SMs and returns the number
 * of FP32 FMAs executed (the caller times it) -- the FP32 roofline denominator. */
int ppgpu_ffma_peak(float *scratch, int iters, long long *fma_count, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* PPGPU_H */
