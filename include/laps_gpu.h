/*
 * laps_gpu.h - C-ABI of the GB300 engine for LAPS's right-hand-side evaluation and RK3
 * time advance.
 *
 * The reference has no library interface: its hot path is a set of argument-less Fortran
 * subroutines sharing module globals, called from the main program `mhd`
 * (src_compressible/mhd.f90).  Each entry point below states which of those subroutines
 * (file:line inside the reference project) it replaces.  A Fortran host binds them through
 * `iso_c_binding` (see fortran/laps_gpu.f90); C, C++ and Python (ctypes) hosts bind them
 * directly.
 *
 * Conventions
 *  - All device memory is owned by the context.  Host arrays are owned by the caller and
 *    are only read or written during the call.
 *  - Real-space arrays use the reference's layout uu(ix,iy,iz,ivar): x fastest, then y,
 *    then z, then the variable (Fortran column-major), float64.
 *  - Every function returns 0 (LAPS_OK) or a negative LAPS_E* code; the text of the last
 *    error is available from laps_last_error().  No C++ exception crosses this boundary.
 *  - One host thread per context.  Each context owns one CUDA stream; calls are
 *    asynchronous on it except where a host array or a scalar result is returned.
 *  - Waits on the device are bounded: a wait that does not finish within the context's
 *    timeout returns LAPS_ETIMEDOUT instead of blocking forever.
 */
#ifndef LAPS_GPU_H
#define LAPS_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------------- codes */
#define LAPS_OK 0
#define LAPS_EINVAL (-1)      /* bad argument or unsupported parameter combination */
#define LAPS_ENOMEM (-2)      /* device allocation failed or above the configured cap */
#define LAPS_ECUDA (-3)       /* CUDA runtime error */
#define LAPS_ETIMEDOUT (-4)   /* a bounded wait on the device expired */
#define LAPS_ESTATE (-5)      /* call out of order (e.g. step before upload) */

/* status bits returned by laps_step / laps_vardt */
#define LAPS_STATUS_NAN 1       /* a NaN was met in the CFL reduction */
#define LAPS_STATUS_DT_FLOOR 2  /* dt < 1e-8: step not taken (src_compressible/mhd.f90:216) */
#define LAPS_STATUS_DEVICE_TIMEOUT 4 /* a bounded device-side wait (tile copy) ran out; results invalid */

/* variants (the reference ships one source tree per variant) */
#define LAPS_VARIANT_3DC 0 /* 3-D compressible, src_compressible/ */
#define LAPS_VARIANT_3DI 1 /* 3-D incompressible, src_incompressible/ */
#define LAPS_VARIANT_2DC 2 /* 2-D compressible, src_compressible/2D/ */

/* arithmetic of the transforms and the right-hand side */
#define LAPS_PREC_FP64 0 /* native IEEE binary64 everywhere */
#define LAPS_PREC_DD 1   /* float-float (two FP32, ~48-bit significand) on the FP32 pipes */
#define LAPS_PREC_FP32 2 /* FP32 transforms and products; state, RK update, CFL, diagnostics in float-float */
#define LAPS_PREC_FP32_F64 3 /* FP32 transforms and products; state, RK update, CFL, diagnostics in FP64 */

/* state layouts for laps_upload_state */
#define LAPS_LAYOUT_PRIMITIVE 0 /* rho, ux, uy, uz, Bx, By, Bz, p (what outNNN.dat holds) */
#define LAPS_LAYOUT_CONSERVED 1 /* rho, rho*ux, rho*uy, rho*uz, Bx, By, Bz, e */

/*
 * Namelist values the hot path reads.  Field names follow the reference's namelists
 * (src_compressible/mhd.f90:30-41); defaults (laps_params_default) are the reference's
 * module initialisers (mhdinit.f90:21-26, dealiasing.f90:10-12, mhd.f90:21, AEBmod.f90:10-12).
 */
typedef struct laps_params {
  int variant;   /* LAPS_VARIANT_* */
  int precision; /* LAPS_PREC_* */
  int nx, ny, nz;
  double Lx, Ly, Lz;
  double adiabatic_index;
  int if_resis, if_resis_exp;
  double resistivity;
  int if_visc, if_visc_exp;
  double viscosity;
  int if_conserve_background;
  int dealias_option; /* 1: spherical 2/3 mask, 2: compact filter, other: none */
  double afx, afy, afz;
  double cfl;
  int if_AEB;
  double radius0, Ur0;
  int if_corotating;
  double corotating_angle;
  int if_Hall;
  double ion_inertial_length;
  double rho0;            /* 3-D incompressible: background density dividing grad(rho u)
                             (src_incompressible/mhdinit.f90:15, default 1) */
  int if_z_radial;        /* 2-D: z is the radial direction of the expanding box
                             (src_compressible/2D/mhd.f90:42) */
  int if_limit_dt_increase; /* 2-D: dt may only decrease (src_compressible/2D/mhd.f90:23) */
  int dstep_calcdt;       /* 2-D: vardt every dstep_calcdt steps (default 20,
                             src_compressible/2D/mhd.f90:20); 3-D variants use 1 */
  int device;             /* CUDA device ordinal */
  int timeout_ms;         /* bound on every device wait (default 600000) */
  long long mem_cap_bytes;/* refuse to allocate more than this (0: no cap) */
  int reserved[8];
} laps_params;

typedef struct laps_ctx laps_ctx;

/* Diagnostics of src_compressible/mhdrms.f90:53-126 and mhd.f90:522-570, plus the
 * engine's own invariants (grid means). */
typedef struct laps_diag {
  double time, dt, radius;
  double uu_ave[8];  /* <rho>, <ux>, <uy>, <uz>, <Bx>, <By>, <Bz>, <p>          */
  double uu_rms[8];  /* <f^2> - <f>^2 for the same eight                         */
  double rho_u2[3];  /* <rho (u_i - <u_i>)^2>                                    */
  double max_divB;   /* max |i k . B_hat| over the spectral grid                 */
  double max_divB_real; /* max |div B| on the grid (src_incompressible/mhd.f90:672-700) */
  double max_divV_real; /* max |div(rho u)| / rho0 on the grid (:701-732)      */
  double e_kin;      /* <rho u^2>/2 */
  double e_mag;      /* <B^2>/2     */
  double h_cross;    /* <u . B>     */
  double h_mag;      /* <A . B>, A_hat = i k x B_hat / k^2 (k != 0) */
} laps_diag;

typedef struct laps_info {
  long long device_bytes; /* device memory held by the context */
  int kx_keep, ky_keep, kz_keep; /* spectral extents the pruned passes touch */
  int kernels_per_step;   /* kernel launches in one fused step */
  int graph;              /* 1 when steps replay a captured CUDA graph */
} laps_info;

/* Fill *p with the reference's defaults. */
int laps_params_default(laps_params* p);

/* Allocate the device state for one run.  Replaces parallel_start / fftw_initialize /
 * grid_initialize / arrays_initialize / AEB_initialize / dealias_initialize
 * (src_compressible/mhd.f90:58-99; fftw.f90:21-39; mhdinit.f90:58-181; AEBmod.f90:16-44;
 * dealiasing.f90:13-67). */
int laps_create(const laps_params* p, laps_ctx** out);

/* Free everything the context holds. */
void laps_destroy(laps_ctx* ctx);

/* Upload the state uu(nx,ny,nz,8) from the host, convert primitive -> conserved when asked,
 * and transform it to Fourier space.  Replaces initial_calc_conserve_variable
 * (mhdinit.f90:1038-1056) + transform_uu_real_to_fourier (fftw.f90:42-71, mhd.f90:121-122). */
int laps_upload_state(laps_ctx* ctx, const double* uu, int layout);

/*
 * Initial-condition parameters: the user-defined namelist values of mhdinit.f90:13-14,48-55
 * (src_compressible; src_incompressible/mhdinit.f90 has the same names).  laps_ic_default
 * fills the reference's module initialisers (T0 = rho0 = B0 = 1, a0 = 0.05,
 * in_out_ratio = 1, nmode* = 16, jet_width = 1, Vjet = 0.3, wave_number_jet = 1, rest 0).
 */
typedef struct laps_ic {
  int ifield; /* background: 0 uniform rho0 / rho0*T0, 1 double current sheet Bx(z), 2 double
                 Harris shear ux(y), 3 uniform B, 4 double current sheet Bx(y) at constant
                 density, 5 jet along x (3-D compressible only) */
  int ipert;  /* perturbation: 0 none, 1 circularly polarised Alfven wave, 6 outward and inward
                 Alfvenic waves, 7 random-phase u, B, rho modes, 8 switchback */
  double T0, rho0, B0, a0;
  double U_fast, U_slow, n_fast, n_slow, press0, shear_width;
  double bx0, by0, bz0, db0, in_out_ratio, dv0, drho0;
  int nmodex, nmodey, nmodez, wave_number_jet;
  double jet_width, Vjet;
  double B0_SB, dB_SB, R0_SB, R1_SB, H_SB, Rm_SB, Rd_SB;
} laps_ic;

/* Fill *ic with the reference's defaults. */
int laps_ic_default(laps_ic* ic);

/* Number of phases laps_init_fields reads for ic (0 for the deterministic cases):
 *   ipert 6: 2 * nmodex * (2 nmodey + 1) * (2 nmodez + 1)  (outward waves, then inward waves)
 *   ipert 7: 3 * (2 nmodex + 1) * (2 nmodey + 1) * (2 nmodez + 1)  (u, B, rho phases)
 * indexed as the reference's phs arrays (mhdinit.f90:523-526,594-597,762-769) without the
 * Fortran 1. */
long long laps_ic_nphases(const laps_ic* ic);

/*
 * Generate the initial state on the device: background_fields_initialize (mhdinit.f90:183-299)
 * + perturbation_initialize for ipert 1, 6, 7, 8 (:302-342,487-688,690-930,931-1019) +
 * initial_calc_conserve_variable (:1038-1056) + transform_uu_real_to_fourier, i.e. what
 * mhd.f90:110-122 does on a fresh start.  The reference draws the phases of ipert 6 and 7
 * with the compiler's random_number; here they are an input (radians, laps_ic_nphases of
 * them; NULL when there are none), so any generator can supply them.  The random-phase
 * modes are placed in the half spectrum and transformed with the state's inverse transform
 * instead of summed point by point; they need |k| < n/2 on every axis (nmodex < nx/2 ...).
 * ipert 2-5 (random 1-D / modulated perturbations) are not built: LAPS_EINVAL.
 * 3-D variants only (the 2-D code has its own initial conditions): LAPS_EINVAL for 2-D.
 */
int laps_init_fields(laps_ctx* ctx, const laps_ic* ic, const double* phases, long long nphases);

/*
 * Angle statistics of the current state, the reference's offline C tool
 * theta_ub_zpm_perp_only (data_process/3D_C/statistics.c:10-356, run per axis by
 * pthread_theta_ub_zpm_perp_only :358-389 on an outNNN.dat): for lags l = 1 .. n_axis/2 grid
 * spacings along `axis` (0 x, 1 y, 2 z), the angle between the components perpendicular to
 * <B>/|<B>| of the increments of u and of B/sqrt(<rho>) ("ub"), and of z+ = u - b and
 * z- = u + b ("zpm").  out receives 4 arrays of n_axis doubles, the contents of the four files
 * the tool writes for the axis: ub method 1, ub method 2, zpm method 1, zpm method 2
 * (method 1: the mean of asin(|a x b| / |a||b|) over points with both parts non-zero;
 * method 2: asin(sum |a x b| / sum |a||b|)); elements 0 and l > n_axis/2 are 0.
 * The means are taken over the state (the reference's mean() starts its sum uninitialised,
 * mathlib.c:9; here it starts at 0).  Float64 on the device.
 */
int laps_angle_statistics(laps_ctx* ctx, int axis, double* out);

/* Set the simulation time and the expanding-box radius: evolve_radius(t)
 * (AEBmod.f90:56-73,87-125), as the restart path does (mhd.f90:101-103). */
int laps_set_time(laps_ctx* ctx, double time);

/* CFL time step with the reference's +-2 % hysteresis against the current dt, then
 * rkt_init: vardt (mhd.f90:328-429, rktmod.f90:15-32).  *dt receives the new dt. */
int laps_vardt(laps_ctx* ctx, double* dt);

/* Advance nsteps full steps.  Each step is vardt; evolve (three RK stages,
 * mhd.f90:298-326); time += dt; evolve_radius(time) (mhd.f90:245-248) - the reference's
 * loop body with its trailing vardt moved to the front.  A step whose dt is below 1e-8 is
 * not taken and sets LAPS_STATUS_DT_FLOOR (mhd.f90:216).  On return *time and *dt hold the
 * values after the last step and *status the OR of the status bits. */
int laps_step(laps_ctx* ctx, int nsteps, double* time, double* dt, int* status);

/* laps_step without the CUDA graph, with a CUDA event recorded on the context's stream
 * after every kernel (no host synchronisation inside the region).  pass_ms[0..5] receive the
 * summed device time of passes A, B, C, D, E (see laps_gb300/csrc/kernels.cuh) and of the
 * small bookkeeping kernels; *total_ms the event time of the whole region.  For profiling;
 * it has no counterpart in the reference. */
int laps_step_profiled(laps_ctx* ctx, int nsteps, double* pass_ms, double* total_ms, int* status);

/* One RK stage irk = 1..3 of evolve with the current dt, for stage-level comparisons
 * (mhd.f90:303-325: calc_flux, transform_flux_real_to_fourier, calc_rhs, rkt, dealias,
 * transform_uu_fourier_to_real, update_uu_prim_from_uu). */
int laps_rk_stage(laps_ctx* ctx, int irk);

/* Inverse-transform the state and copy uu (conserved, nx*ny*nz*8) and uu_prim
 * (ux, uy, uz, p: nx*ny*nz*4) to the host; either pointer may be NULL.  Replaces
 * transform_uu_fourier_to_real + update_uu_prim_from_uu (fftw.f90:73-103,
 * mhdrhs.f90:282-294) as used by output_uu (mhdoutput.f90:72-131). */
int laps_download_state(laps_ctx* ctx, double* uu, double* uu_prim);

/* Copy uu_fourier(nx/2+1,ny,nz,8) (interleaved complex float64) to / from the host. */
int laps_download_spectral(laps_ctx* ctx, double* uf);
int laps_upload_spectral(laps_ctx* ctx, const double* uf);

/* Diagnostics: calc_rms (mhdrms.f90:53-126), calc_max_divB (mhd.f90:522-570), and the
 * kinetic/magnetic energy, cross- and magnetic helicity of the current state. */
int laps_diagnostics(laps_ctx* ctx, laps_diag* d);

/* Shell energy spectra of the current state: e_u[s] = 1/2 sum |u_hat|^2 (velocity
 * u = rho u / rho) and e_b[s] = 1/2 sum |B_hat|^2 over the modes with round(|k|/dk) = s,
 * s < nshell (1..2048), |k| from the unscaled grid wave numbers, dk = 2 pi / max(L); the
 * shells sum to <u^2>/2 and <B^2>/2.  Replaces the reference's post-processing of the
 * output files (data_process/3D_Python/fourier_analysis.py:150-200), which has no shell
 * binning of its own.  Either array may be NULL. */
int laps_spectrum(laps_ctx* ctx, int nshell, double* e_u, double* e_b);

/* Granular entry points in the reference's order, for bisection against its subroutines
 * (unfused: they recompute what laps_step fuses).  Compressible variants for the flux / rhs
 * calls (LAPS_EINVAL for the incompressible one).
 *   laps_calc_flux: calc_flux (mhdrhs.f90:21-124) of the current state, 18 real fields
 *     flux(nx,ny,nz,1:18) in the reference's order, then the expansion term (:157-171) as
 *     field 19 when the expanding box is on.
 *   laps_transform_flux: the same fields forward-transformed (transform_flux_real_to_fourier,
 *     :128-172), (nx/2+1,ny,nz) interleaved complex each.
 *   laps_calc_rhs: fnl(nx/2+1,ny,nz,8) of calc_rhs (:174-279, with the expansion and
 *     explicit-diffusion terms, before rkt); the state is unchanged, the RK register is
 *     overwritten (call between steps).
 *   laps_dealias: dealias (dealiasing.f90:70-113) applied to the state.
 *   laps_transform_uu_k2r / laps_update_prim: transform_uu_fourier_to_real (fftw.f90:73-103)
 *     and update_uu_prim_from_uu (mhdrhs.f90:282-294): uu(nx,ny,nz,8) / uu_prim(nx,ny,nz,4).
 * laps_rk_stage is rkt(irk) with the stage's right-hand side; laps_vardt is vardt. */
int laps_calc_flux(laps_ctx* ctx, double* flux);
int laps_transform_flux(laps_ctx* ctx, double* flux_fourier);
int laps_calc_rhs(laps_ctx* ctx, double* fnl);
int laps_dealias(laps_ctx* ctx);
int laps_transform_uu_k2r(laps_ctx* ctx, double* uu);
int laps_update_prim(laps_ctx* ctx, double* uu_prim);

/* Device-side exchange for a caller that works on the GPU (the learned closure), no
 * counterpart in the reference.  Both wait for the context's stream.
 *   laps_state_real_device: the conserved real state uu(nx,ny,nz,1:8) (as laps_download_state
 *     gives it) into uu_dev, a device buffer of 8*nx*ny*nz doubles.
 *   laps_add_spectral_device: uu_fourier += scale * duf_dev for the 8 fields, duf_dev a device
 *     array in the layout of laps_download_spectral, then the dealias mask or filter. */
int laps_state_real_device(laps_ctx* ctx, double* uu_dev);
int laps_add_spectral_device(laps_ctx* ctx, const double* duf_dev, double scale);

/* The reference's output / restart file outNNN.dat (mhdoutput.f90:72-131, restart.f90:17-63):
 * a Fortran unformatted record with the time as a 4-byte real (12 bytes with its markers),
 * then uu(nx,ny,nz,8) as 8-byte reals in Fortran order.  laps_write_output writes the current
 * state and time (LAPS_LAYOUT_PRIMITIVE: rho, u, B, p as the reference's output_uu does;
 * LAPS_LAYOUT_CONSERVED: the conserved state), copying through page-locked buffers with the
 * device-to-host copies overlapped with the file writes.  laps_read_restart reads such a file
 * (primitive), uploads it and sets the time, which the file holds as a 4-byte real. */
int laps_write_output(laps_ctx* ctx, const char* path, int layout);
int laps_read_restart(laps_ctx* ctx, const char* path, double* time);

/* Ensembles of independent runs.  No counterpart in the reference (one run per mpirun job):
 * a batch owns n member contexts on one device, each created from its own laps_params
 * (grid, variant, precision, eta, nu, d_i, ...), with its own stream, dt, vardt cadence and
 * status.  laps_batch_step advances every member by nsteps of its own steps by replaying one
 * CUDA graph per step that forks to all members' streams and joins back, so members of
 * different sizes run concurrently.  Members are reached through laps_batch_member for
 * upload, set_time, download, diagnostics; laps_step on a member between batch steps is
 * allowed, laps_destroy on a member is not (laps_batch_destroy frees them).
 *   time, dt, status: arrays of n values written after the call (each may be NULL). */
typedef struct laps_batch laps_batch;
int laps_batch_create(const laps_params* members, int n, laps_batch** out);
int laps_batch_size(laps_batch* b);
int laps_batch_member(laps_batch* b, int i, laps_ctx** ctx);
int laps_batch_step(laps_batch* b, int nsteps, double* time, double* dt, int* status);
void laps_batch_destroy(laps_batch* b);
const char* laps_batch_last_error(laps_batch* b); /* NULL: the last laps_batch_create error */

/* Forward transform of nfields real FP64 fields that allocates no device memory, for hosts
 * that cannot call cudaMalloc (their device memory comes from their own pool or framework,
 * or allocation is not allowed after start-up).  It has no counterpart in the reference: it
 * runs the same forward transform as laps_upload_state on buffers the caller owns.
 *   uu: device pointer, uu(nx,ny,nz,nfields) float64;  uf: device pointer,
 *   uu_fourier(nx/2+1,ny,nz,nfields) interleaved complex float64;  stream: a cudaStream_t
 *   (NULL: the default stream).  The call is asynchronous on that stream.
 * The intermediate half spectrum of one field lives in a fixed 32 MiB device array inside
 * the library, which every GPU that loads the library holds until the process exits; grids
 * whose padded half spectrum ((nx/2+1 rounded up to 8) * ny * nz) exceeds 2^21 complex
 * elements - 128^3 fits - are rejected with LAPS_EINVAL.  Every call looks up the array's
 * device address with the caller's device and context current (so a cudaDeviceReset between
 * calls is safe); the first call in a context also loads the library's kernels there, so make
 * that first call before any stream capture.  Every call shares the array, so calls that
 * overlap on the GPU (other streams, other host threads) race.  Errors are reported through
 * laps_last_error(NULL). */
int laps_transform_uu_real_to_fourier_noalloc(const double* uu, double* uf, int nx, int ny, int nz, int nfields,
                                              void* stream);

/* ---------------------------------------------------------------- learned subgrid closure
 * 3x3x3 periodic convolutions in BF16 on the tensor cores (FP32 accumulation), the layers of
 * the subgrid-stress net that closes a coarse incompressible run.  No counterpart in the
 * reference: the closure is an addition, and the plain solver above is its fallback.
 * All pointers are device pointers; calls are asynchronous on `stream` (a cudaStream_t, NULL:
 * the default stream) and allocate nothing.  Errors: laps_last_error(NULL).
 *
 * Activation layout: channels-last BF16 with a one-voxel periodic halo on x: element
 * (z, y, xp, c) at ((z*ny + y)*(nx + 2) + xp)*C + c with xp = x + 1, xp = 0 and nx + 1 holding
 * the values at x = nx - 1 and x = 0; C, the padded channel count, is 16 or 32 (channels past
 * the layer's own count are zero).  nx is a multiple of 128; buffers are 16-byte aligned.
 *
 * laps_conv3_pack: weights w[cout][cin][3][3][3] (float32, the cross-correlation
 *   out[x] = sum_k w[k] in[x + k - 1], k = 0..2 per axis) into the tensor cores' operand
 *   layout, 27 * cin_p * cout_p BF16 values at wpk.  flip = 1 packs the input-gradient layer
 *   instead (channels exchanged, taps mirrored): its forward with act 2 is the backward pass
 *   of the layer with respect to its input.
 * laps_conv3_forward: y = act(conv(x) + bias) over the whole periodic grid, x with cin_p
 *   channels, y (halo written) with cout_p; bias holds cout_p floats, zero past the layer's own
 *   channels (or is NULL).  act 0: linear; act 1: GELU (exact, erf form),
 *   the pre-activation written to zpre when zpre is not NULL; act 2: y = conv(x) * GELU'(gate),
 *   gate a pre-activation with cout_p channels (the backward pass through the previous layer's
 *   activation), bias unused.
 * laps_conv3_wgrad: the weight gradient of a layer, dw[t][co][ci] = sum over the grid of
 *   dz(v, co) * x(v + shift(t), ci) (float32, 27 x cout_p x cin_p, tap t = (kz*3 + ky)*3 + kx,
 *   overwritten), x the layer's input (cin_p channels), dz the gradient at its pre-activation
 *   output (cout_p channels, halo not read); nx a multiple of 64.
 * laps_conv3_status: wait for the stream, then read and clear the convolutions' error word
 *   (*err = 1 when a bounded wait inside a convolution ran out; its output is then invalid). */
int laps_conv3_pack(const float* w, void* wpk, int cin, int cout, int cin_p, int cout_p, int flip, void* stream);
int laps_conv3_forward(const void* x, const void* wpk, const float* bias, void* y, void* zpre, const void* gate,
                       int nx, int ny, int nz, int cin_p, int cout_p, int act, void* stream);
int laps_conv3_wgrad(const void* x, const void* dz, float* dw, int nx, int ny, int nz, int cin_p, int cout_p,
                     void* stream);
int laps_conv3_status(void* stream, int* err);

/* The closure's data on the device (cubic periodic grids of side 2 pi; device pointers;
 * asynchronous on `stream`; no allocation):
 *   laps_closure_filter: box filter of width `ratio` of a fine incompressible state
 *     fine(n,n,n,1:8) (n = nfine, the layout of laps_state_real_device), sampled on the coarse
 *     grid of n/ratio points: coarse(.,.,.,1:8) the filtered state; targets (float32, 12
 *     fields) the subgrid stress tau_ij = <u_i u_j> - <u_i><u_j> - (<b_i b_j> - <b_i><b_j>)
 *     for ij = xx xy xz yy yz zz, the subgrid electromotive force <u x b> - <u> x <b>, and 3
 *     zero fields (the Hall part, not modelled: the training runs have d_i = 0).
 *   laps_closure_pack_input: the net's input from a coarse state (u = rho u / rho and B,
 *     divided by su and sb) in the convolutions' padded layout with 16 channels.
 *   laps_closure_unpack_output: the net's 12 output channels times s into 12 float64 fields.
 *   laps_closure_forcing: from the spectra of those 12 fields (layout of
 *     laps_download_spectral), the closure's right-hand side of the 8 state fields: 0,
 *     the momentum -(i k . tau) projected on k-perpendicular, the induction i k x eps, 0. */
int laps_closure_filter(const double* fine, int nfine, int ratio, double* coarse, float* targets, void* stream);
int laps_closure_pack_input(const double* state, void* x, int n, double su, double sb, void* stream);
int laps_closure_unpack_output(const void* y, double* tau, int n, double s, void* stream);
int laps_closure_forcing(const double* tau_spec, double* force_spec, int n, void* stream);

/* Execution schedules.  No counterpart in the reference: choices of how the engine's kernels
 * are launched that leave every result bit-identical, picked per grid, precision and device by
 * the autotuner (laps_gb300/autotune.py, which times each with laps_step_profiled and caches
 * the fastest).  Bits of laps_set_schedule (default 0):
 *   LAPS_SCHED_PERSISTENT_B   pass B of FP32 lines up to 256 points (3-D) as persistent blocks
 *                             with two buffer sets (the next tile's loads overlap this one's work)
 *   LAPS_SCHED_NO_PREFETCH_E  pass E of FP32 lines without the L2 prefetch of the state and RK
 *                             register rows it updates
 *   LAPS_SCHED_INLINE_MASS    the continuity update in line before pass E instead of on a side
 *                             stream beside pass D
 * A change rebuilds the captured step graph (and an ensemble's, at its next step). */
#define LAPS_SCHED_PERSISTENT_B 1
#define LAPS_SCHED_NO_PREFETCH_E 2
#define LAPS_SCHED_INLINE_MASS 4
#define LAPS_SCHED_ALL 7
int laps_set_schedule(laps_ctx* ctx, int bits);
int laps_get_schedule(laps_ctx* ctx, int* bits);

/* Bounded wait for all queued work of the context. */
int laps_wait(laps_ctx* ctx, int timeout_ms);

/* Device-side time and dt. */
int laps_get_time(laps_ctx* ctx, double* time, double* dt);

int laps_get_info(laps_ctx* ctx, laps_info* info);

/* Text of the last error on this context (or of the last failed laps_create when ctx is NULL). */
const char* laps_last_error(laps_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif /* LAPS_GPU_H */
