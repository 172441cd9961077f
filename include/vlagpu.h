/*
 * vlagpu.h -- C ABI of the GB300 VlaPy time step (libvlagpu.so).
 *
 * The reference (joglekara/VlaPy) is pure Python: its "plugin interface" for
 * the hot path is a set of closures built from the parameter dictionary.
 * Each entry point below replaces one of them and names the reference code it
 * stands in for.  All array arguments of the compute calls are DEVICE
 * pointers owned by the caller (PyTorch tensors in the Python host layer);
 * the plan owns only its constants and scratch.  Every call returns an int
 * status (VG_OK == 0); vg_last_error() gives the message of the last failure
 * on the calling thread.  Calls on one object (plan, batch, sweep,
 * corrector) must come from one host thread at a time and be serialised on
 * one stream; different objects are independent.
 *
 * Layouts (C order, as in the reference): f[nx][nv] with v contiguous,
 * e[nx], driver[nx].  In VG_F64 mode f is float64 and the arithmetic follows
 * the reference's NumPy path; in VG_F32_DELTA_F mode the state is the FP32
 * deviation g = f - f0(v) from a fixed background f0 given at plan creation.
 */
#ifndef VLAGPU_H
#define VLAGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct vg_plan vg_plan;
/* a cudaStream_t, passed opaquely; NULL is the legacy default stream */
typedef void* vg_stream;

enum {
  VG_OK = 0,
  VG_ERR_ARG = 1,          /* bad argument or descriptor */
  VG_ERR_CUDA = 2,         /* a CUDA runtime call failed */
  VG_ERR_UNSUPPORTED = 3,  /* valid in the reference, not implemented here */
  VG_ERR_NUMERIC = 4,      /* NaN/Inf detected in the field */
  VG_ERR_TIMEOUT = 5,      /* a bounded wait ran out */
  VG_ERR_STATE = 6         /* call out of order (e.g. history too small) */
};

/* status bits a plan, batch or sweep raises on the device (vg_*_status) */
enum {
  VG_FLAG_TIMEOUT = 1,    /* a bounded wait of a kernel ran out: its step is not valid */
  VG_FLAG_NONFINITE = 2   /* a field solve produced NaN or Inf: that step and the later ones are not valid */
};

enum { VG_F64 = 0, VG_F32_DELTA_F = 1 };
/* all_params["fokker-planck"]["type"], vlapy/core/collisions.py:292-317 */
enum { VG_COLL_NONE = 0, VG_COLL_LB = 1, VG_COLL_DG = 2 };
/* all_params["vlasov-poisson"]["time"], vlapy/core/vlasov_poisson.py:235-280 */
enum { VG_LEAPFROG = 0, VG_PEFRL = 1, VG_H_SIXTH = 2 };
/* pulse envelopes: VG_ENV_TANH is vlapy/field_driver.py:24-50;
 * VG_ENV_SIN2 is a0*sin(k x - w t)*sin^2(pi t / t_R) on [0, t_R], 0 after. */
enum { VG_ENV_TANH = 0, VG_ENV_SIN2 = 1 };

typedef struct vg_pulse {
  double k0, w0, a0, t_L, t_R, t_wL, t_wR;
  int32_t envelope;
  int32_t reserved;
} vg_pulse;

/* Run descriptor: the derived quantities of stuff_for_time_loop
 * (vlapy/outer_loop.py:125-144).  Array members are HOST pointers copied at
 * vg_plan_create; computing them with NumPy on the host (as the reference
 * does, vlapy/initializers.py:56-89) keeps the grids bit-identical. */
typedef struct vg_run_desc {
  int32_t nx, nv;
  int32_t precision;   /* VG_F64 | VG_F32_DELTA_F */
  int32_t collision;   /* VG_COLL_* ; VG_COLL_NONE when nu == 0 */
  int32_t integrator;  /* VG_LEAPFROG | VG_PEFRL | VG_H_SIXTH */
  int32_t n_pulses;
  double dt, nu, dx, dv;
  double dv_sq;               /* dv ** 2.0 evaluated by the host */
  const double* x;            /* [nx] */
  const double* v;            /* [nv] */
  const double* kx;           /* [nx] */
  const double* kv;           /* [nv] */
  const double* one_over_kx;  /* [nx] */
  const double* v_pow;        /* [5][nv]: v**2.0, v**2, v**3, v**4, v**5 as NumPy evaluates them */
  const vg_pulse* pulses;     /* [n_pulses] */
  const double* f_background; /* [nv] background f0(v) for VG_F32_DELTA_F; NULL for VG_F64 */
} vg_run_desc;

/* Per-step storage of the inner loop (vlapy/outer_loop.py:149-215). DEVICE
 * pointers; any may be NULL to skip that output. */
typedef struct vg_history {
  int32_t nt;          /* steps the arrays hold (first dimension) */
  int32_t store_all;   /* 1: stored_f is float64 [nt][nx][nv]; 0: complex64 [nt][n_slots][nv] */
  int32_t n_modes;     /* x-Fourier modes computed per step when store_all == 0 */
  int32_t n_slots;     /* modes stored per step; n_modes must equal it or be 1 (broadcast) */
  double* fields[8];   /* e, driver, n, j, T, q, fv4, vN: each [nt][nx] */
  double* series[7];   /* mean_n, mean_j, mean_T, mean_e2, mean_de2, mean_f2, mean_flogf: [nt] */
  void* stored_f;
} vg_history;

/* one line of a per-kernel timing record (vg_profile_read, vg_sweep_profile_read) */
typedef struct vg_prof_entry {
  char name[32];
  int64_t launches;
  double total_ms;
  double bytes_per_launch;
} vg_prof_entry;

/* ---- plan lifetime ---------------------------------------------------- */
/* Builds the per-run constants (grids, FFT twiddles, NumPy summation trees)
 * and allocates the plan's scratch with cudaMalloc on the current device.
 * Replaces the closure factories of vlapy/core/step.py:29-113. */
int vg_plan_create(const vg_run_desc* desc, vg_plan** out);
int vg_plan_destroy(vg_plan* plan);
/* Synchronises the device.  *flags: the status bits the plan's kernels raised
 * since it was created (VG_FLAG_NONFINITE: a field solve of vg_run_steps or
 * vg_field_solve wrote NaN or Inf, for instance from a non-finite f).
 * Returns VG_ERR_NUMERIC when that bit is set.  No reference counterpart:
 * NumPy would carry the NaN on without a word. */
int vg_plan_status(vg_plan* plan, int32_t* flags);
const char* vg_last_error(void);
int vg_version(void);

/* ---- sub-operators (the reference's closures) -------------------------- */
/* v-advection f <- Re IFFT_v(exp(-i kv e dt) FFT_v f), in place.
 * Replaces step_edfdv_exponential, vlapy/core/vlasov.py:113-140. */
int vg_edfdv(vg_plan* plan, void* f, const double* e, double dt, vg_stream stream);
/* x-advection f <- Re IFFT_x(exp(-i kx v dt) FFT_x f), in place.
 * Replaces step_vdfdx_exponential, vlapy/core/vlasov.py:83-110. */
int vg_vdfdx(vg_plan* plan, void* f, double dt, vg_stream stream);
/* The alternative v df/dx and e df/dv steppers, FP64 plans only, OUT OF
 * PLACE (f_out must not overlap f_in), as the reference's closures return a
 * new array.  The semi-Lagrangian steps evaluate the not-a-knot cubic spline
 * of each line, extended by one periodic cell at each end, at the departure
 * points (clamped to the extended range), which is what the reference's
 * s = 0 bicubic spline gives there; they agree with it to rounding.  The
 * first semi-Lagrangian call on a plan allocates the plan's spline scratch
 * (cudaMalloc), so make it outside stream capture.
 * vg_vdfdx_sl: f_out(x, v) = spline_x(f(., v))(x - v dt); nx >= 3, nv >= 4.
 *   Replaces update_spatial_adv_sl, vlapy/core/vlasov.py:42-80. */
int vg_vdfdx_sl(vg_plan* plan, const double* f_in, double* f_out, double dt, vg_stream stream);
/* vg_edfdv_sl: f_out(x, v) = spline_v(f(x, .))(v - e(x) dt); nx >= 4, nv >= 3.
 *   Replaces update_velocity_adv_sl, vlapy/core/vlasov.py:168-210. */
int vg_edfdv_sl(vg_plan* plan, const double* f_in, const double* e, double* f_out, double dt,
                vg_stream stream);
/* vg_edfdv_cd2: f_out = f - (e * df/dv) * dt with numpy.gradient's
 * second-order stencils (centred inside, one-sided at the ends), rounded as
 * NumPy rounds them; nv >= 3.
 *   Replaces step_edfdv_center_difference, vlapy/core/vlasov.py:143-165. */
int vg_edfdv_cd2(vg_plan* plan, const double* f_in, const double* e, double* f_out, double dt,
                 vg_stream stream);
/* n(x) = trapz_v f.  Replaces compute_charges, vlapy/core/field.py:27-36. */
int vg_charge_density(vg_plan* plan, const void* f, double* n, vg_stream stream);
/* e = Re IFFT(i/kx FFT(rho)) for a net charge rho[nx] (nx any size).
 * Replaces __fft_solve__, vlapy/core/field.py:39-49. */
int vg_poisson(vg_plan* plan, const double* rho, double* e, vg_stream stream);
/* e = driver + field of (1 - trapz_v f); driver may be NULL (zero).
 * Replaces solve_total_electric_field, vlapy/core/field.py:66-88. */
int vg_field_solve(vg_plan* plan, const void* f, const double* driver, double* e, vg_stream stream);
/* Implicit Fokker-Planck step of the plan's operator, in place.
 * Replaces take_collision_step, vlapy/core/step.py:70-113
 * (matrix makers vlapy/core/collisions.py:26-160, solver :222-265). */
int vg_collision_step(vg_plan* plan, void* f, vg_stream stream);
/* Storage step at index i: stored_f, the eight fields and seven series.
 * Replaces storage_step, vlapy/core/step.py:231-283. */
int vg_storage_step(vg_plan* plan, const void* f, const double* e, const double* de,
                    const vg_history* hist, int32_t i, vg_stream stream);
/* Driver field at time t into out[nx].  Replaces driver_function,
 * vlapy/field_driver.py:24-50. */
int vg_driver(vg_plan* plan, double t, double* out, vg_stream stream);

/* ---- the time step ----------------------------------------------------- */
/* Runs nsteps full steps (VP step, FP step, storage step) for storage
 * indices i0 .. i0+nsteps-1, reading t_i from time_batch[i] and the stored
 * driver de_i from driver_batch[i][:] (both DEVICE arrays of the batch), and
 * evaluating the pulses at the integrator's sub-step times.  f and e are
 * updated in place.  Replaces timestep, vlapy/core/step.py:286-328, looped
 * as in inner_loop, vlapy/outer_loop.py:265-272.  With use_graph != 0 the
 * launch sequence is captured once into a CUDA graph per (pointer set,
 * i0, nsteps) and replayed. */
int vg_run_steps(vg_plan* plan, void* f, double* e, const vg_history* hist,
                 const double* time_batch, const double* driver_batch,
                 int32_t i0, int32_t nsteps, int32_t use_graph, vg_stream stream);

/* ---- field solve without allocation ------------------------------------ */
/* e = driver + Re IFFT(i/kx FFT(1 - trapz_v f)) for f[nx][nv] float64, the
 * same FP64 arithmetic as vg_field_solve, but with no plan and no device
 * allocation of any kind: for callers whose device memory is owned by
 * another allocator (a framework's caching allocator, a fixed pool) or who
 * cannot afford the device-wide synchronisation of cudaMalloc/cudaFree.  All
 * scratch (density, FFT twiddles, summation table, DFT work area) lives in
 * one static device array of about 580 KB that every GPU loading the library
 * keeps until exit.  Limits: 2 <= nx <= 8192, 2 <= nv <= 16384; larger sizes
 * return VG_ERR_ARG.  one_over_kx[nx], driver[nx] (may be NULL) and e[nx] are
 * DEVICE arrays.  The first call on a device (and the first after its context
 * is recreated, e.g. by cudaDeviceReset) fills the array's twiddle table on
 * the caller's stream and waits for that stream: make it during set-up,
 * before any stream capture.  Later calls only launch kernels on the caller's
 * stream (the summation table for nv is written on the device) and copy
 * nothing from the host.  Calls share the array: calls that overlap on the
 * GPU race and must be ordered by the caller.  No counterpart in the
 * reference. */
int vg_field_solve_noalloc(const double* f, int32_t nx, int32_t nv, double dv, const double* one_over_kx,
                           const double* driver, double* e, vg_stream stream);

/* ---- batched FP64 step ------------------------------------------------- */
/* n_runs independent runs of the FP64 time step advanced together: each
 * step is the reference's leapfrog step with exponential advection, the
 * spectral Poisson solve, the implicit collision step of the runs' operator
 * and the per-step moments (vlapy/core/step.py:286-328 applied per run),
 * with every kernel launch covering all runs of one nv (the row operators)
 * or one nx (the x-drift and the Poisson solve).  Each run is described as
 * for vg_plan_create and goes through the same device code as a plan, so it
 * follows the reference's NumPy step as a plan does.  Requirements: FP64,
 * leapfrog, no pulses, one dt for all runs, one collision operator for all
 * runs with nu > 0 (runs with nu = 0 or VG_COLL_NONE skip the collision
 * step, as the reference does), power-of-two nx in [2, 1024], and the runs
 * of one nv contiguous and on the same velocity grid.  No reference
 * counterpart: the reference runs one simulation per process
 * (vlapy/manager.py:35-177). */
typedef struct vg_batch vg_batch;
int vg_batch_create(const vg_run_desc* runs, int32_t n_runs, vg_batch** out);
int vg_batch_destroy(vg_batch* batch);
/* as vg_plan_status, for the batch's field solves */
int vg_batch_status(vg_batch* batch, int32_t* flags);
/* total cells and x points (the e-history row length) */
int vg_batch_sizes(const vg_batch* batch, int64_t* cells, int64_t* x_points);
/* nsteps steps of every run, in place.  f: DEVICE float64, the runs' f[nx][nv]
 * back to back in the order of the descriptors; e: DEVICE float64, the runs'
 * e[nx] back to back.  If e_hist/series_hist are non-NULL, step i of this call
 * is stored at row (hist_row0 + i) of e_hist [rows][x_points] and
 * series_hist [rows][n_runs][7] (mean n, j, T, e^2, driver^2 (0), f^2,
 * f log f), for rows < hist_rows.  use_graph != 0 replays one captured CUDA
 * graph per (buffers, nsteps, rows, stream) on a non-default stream. */
int vg_batch_run_steps(vg_batch* batch, double* f, double* e, int32_t nsteps, double* e_hist, double* series_hist,
                       int32_t hist_rows, int32_t hist_row0, int32_t use_graph, vg_stream stream);
/* per-kernel timing of vg_batch_run_steps (same contract as vg_profile_*) */
int vg_batch_profile_enable(vg_batch* batch, int32_t enable);
int vg_batch_profile_read(vg_batch* batch, vg_prof_entry* out, int32_t max, int32_t* n_out);

/* ---- batched sweep ----------------------------------------------------- */
/* Thousands of independent runs of uneven shape advanced together in the
 * FP32 delta-f mode: every kernel launch of a step covers all runs (work
 * lists of (run, column tile) and (run, row-pair group) items dispatched by
 * shape inside the kernel).  Each run is the reference's leapfrog step with
 * exponential advection, spectral Poisson and, for nu > 0, the chosen
 * collision operator (vlapy/core/step.py:286-328 applied per run), started
 * from f = M(v) (1 + A cos(k x)) on x in [0, 2 pi / k), v in [-vmax, vmax).
 * The sweep owns the run states; per step it stores each run's field e[nx]
 * and its seven series.  No reference counterpart: the reference runs one
 * simulation per process (vlapy/manager.py:35-177). */
typedef struct vg_sweep vg_sweep;
typedef struct vg_sweep_run {
  int32_t nx, nv;    /* powers of two; nx in [8, 256], nv in [64, 2048] */
  double k;          /* fundamental wavenumber (box length 2 pi / k) */
  double amplitude;  /* density perturbation of the initial state */
  double nu;         /* collision frequency; 0 = collisionless */
} vg_sweep_run;
typedef struct vg_sweep_desc {
  int32_t n_runs;
  int32_t collision;  /* VG_COLL_DG or VG_COLL_LB for the runs with nu > 0 */
  double vmax, dt;
  const vg_sweep_run* runs;  /* host [n_runs] */
} vg_sweep_desc;
int vg_sweep_create(const vg_sweep_desc* desc, vg_sweep** out);
int vg_sweep_destroy(vg_sweep* sweep);
/* total phase-space cells and total x points (the e-history row length) */
int vg_sweep_sizes(const vg_sweep* sweep, int64_t* cells, int64_t* x_points);
/* x offset of each run's field in an e-history row (host [n_runs]) */
int vg_sweep_x_offsets(const vg_sweep* sweep, int64_t* out);
/* every run back to its initial state, e = 0, t = 0 */
int vg_sweep_reset(vg_sweep* sweep, vg_stream stream);
/* nsteps leapfrog steps of every run.  If e_hist/series_hist are non-NULL,
 * step i of this call is stored at row (hist_row0 + i) of e_hist
 * [rows][x_points] and series_hist [rows][n_runs][7] (mean n, j, T, e^2,
 * driver^2, f^2, f log f), for rows < hist_rows. */
int vg_sweep_run_steps(vg_sweep* sweep, int32_t nsteps, double* e_hist, double* series_hist,
                       int32_t hist_rows, int32_t hist_row0, int32_t use_graph, vg_stream stream);
/* Caller-created CUDA events (cudaEvent_t, as void*) that each following
 * vg_sweep_run_steps call records on its stream after step k (k < n) has
 * stored its history row, so that another stream can take that row to the
 * host while the later steps run; n = 0 clears them.  The events must stay
 * valid while they are set; graphs captured with them record them too. */
int vg_sweep_set_step_events(vg_sweep* sweep, void* const* events, int32_t n);
/* f = g + f0 of one run as float64 [nx][nv] and its e[nx] (DEVICE pointers) */
int vg_sweep_read_run(vg_sweep* sweep, int32_t run, double* f_out, double* e_out, vg_stream stream);
/* copy every run's FP32 deviation g = f - f0 (runs back to back, [nx][nv]
 * each) and field e (packed like e_hist rows) to / from caller DEVICE
 * buffers; either pointer may be NULL.  set_state also refreshes the FP32
 * copy of e that the first half-kick of the next vg_sweep_run_steps reads.
 * No reference counterpart: they let a caller checkpoint a sweep, or move
 * states between sweeps of different grids (the coarse-grid corrector). */
int vg_sweep_get_state(vg_sweep* sweep, float* g_out, double* e_out, vg_stream stream);
int vg_sweep_set_state(vg_sweep* sweep, const float* g_in, const double* e_in, vg_stream stream);
/* the sweep's own device buffers g [cells] and e [x_points] (valid for its
 * lifetime); a caller may modify g in place between vg_sweep_run_steps
 * calls on the same stream (the corrector does).  Writing e this way would
 * bypass the FP32 copy the kicks read: use vg_sweep_set_state for e. */
int vg_sweep_state_ptr(vg_sweep* sweep, float** g, double** e);
/* Damping rate and frequency of every run from an e history [rows][x_points]
 * (DEVICE) whose row k is time t0 + k dt: the peaks of |FFT_x(e)[1]| in
 * [t_min, t_max], each refined by a parabola in log space, give the rate as
 * the least-squares slope of log peak height against time and the frequency
 * as pi over the mean peak spacing; NaN with fewer than three peaks.
 * rate_out, freq_out: DEVICE [n_runs].  Replaces the host post-processing of
 * vlapy/diagnostics/low_level_helpers.py:69-87 with one launch per sweep (an
 * estimator that is unbiased for undriven runs; rows <= 16384). */
int vg_sweep_damping(vg_sweep* sweep, const double* e_hist, int32_t rows, double t0, double t_min, double t_max,
                     double* rate_out, double* freq_out, vg_stream stream);
/* Synchronises the device; *uses_tma (may be NULL) says whether the x-drift
 * loads its tiles through the tensor-memory accelerator (cp.async.bulk.tensor;
 * every run must start on a whole row of nv floats, and the environment
 * variable VG_SWEEP_NO_TMA, read at vg_sweep_create, must be unset or "0"), and
 * *flags the status bits since creation: VG_FLAG_TIMEOUT for a bounded wait of
 * that kernel that ran out, VG_FLAG_NONFINITE for a field solve that wrote NaN
 * or Inf.  Returns VG_ERR_TIMEOUT, else VG_ERR_NUMERIC, if either is set (the
 * affected steps are not valid). */
int vg_sweep_status(vg_sweep* sweep, int32_t* flags, int32_t* uses_tma);
/* Limit of the TMA x-drift's waits for its tiles, in ns of the global timer
 * (default 2e9).  A wait that runs out sets VG_FLAG_TIMEOUT, lets the copy in
 * flight land (waiting up to the default limit) and ends its CTA, so the step
 * is not valid. */
int vg_sweep_set_wait_limit(vg_sweep* sweep, int64_t ns);
/* Test hook for those waits: while on, the TMA x-drift requests no tiles, so
 * each of its waits runs out after the wait limit, raises VG_FLAG_TIMEOUT and
 * ends its CTA (with no copy in flight to wait for).  The steps are not valid;
 * nothing faults or hangs, and the context stays usable. */
int vg_sweep_inject_lost_tiles(vg_sweep* sweep, int32_t on);
/* per-kernel timing of vg_sweep_run_steps (same contract as vg_profile_*) */
int vg_sweep_profile_enable(vg_sweep* sweep, int32_t enable);
int vg_sweep_profile_read(vg_sweep* sweep, vg_prof_entry* out, int32_t max, int32_t* n_out);

/* ---- measurement ----------------------------------------------------- */
/* Per-kernel device timing of vg_run_steps: while enabled, every kernel of
 * the step sequence is bracketed by CUDA events on the plan's stream and the
 * graph path is bypassed.  vg_profile_read synchronises the stream, then
 * fills up to max entries (kernel name, launches, total milliseconds,
 * algorithmic DRAM bytes per launch) and clears the record.  The FP32 row
 * pass of a call's last leapfrog step, which ends without the next step's
 * leading half kick, is recorded apart ("row_pass_last_f32", and
 * "sweep_row_pass_last" for sweeps), so that "row_pass_f32" and
 * "sweep_row_pass" time the pass of every other step.  No reference
 * counterpart (the reference only logs wall-clock per step,
 * vlapy/manager.py:144-146). */
int vg_profile_enable(vg_plan* plan, int32_t enable);
int vg_profile_read(vg_plan* plan, vg_prof_entry* out, int32_t max, int32_t* n_out);

/* ---- learned coarse-velocity corrector -------------------------------- */
/* No reference counterpart.  A 1-D conv net along v applied to each x row
 * of a coarse run (nv = 128) after a coarse step:
 *   c = P(s * tau * net(d / s, v / vmax, row_feat, d_prev / s)),
 *   g <- m + (d - Pd) + (Pd + c) * min(1, |Pd| / |Pd + c|),
 * m = the mean of the row's group of group_rows consecutive rows (the
 * x-mean of a run when a group is one run's x rows; group_rows = 0: m = 0),
 * d = g - m, d_prev the same of the row before the coarse step, s the RMS
 * of d over the row, tau a global output scale, row_feat one scalar per row
 * (the collision-rate channel), P the orthogonal projection that removes
 * the v-Fourier modes |m| < protect_modes of the 128-point row (those
 * modes, which carry the density and the field, are never corrected), and
 * the min() cap keeps the corrected high part no longer in L2 norm than the
 * coarse step left it.  Four conv1d layers, kernel 5, zero padding 2, 64
 * channels, ReLU after the first three; BF16 tensor cores with FP32
 * accumulation.  Parameters are FP32 in PyTorch conv1d order: W1
 * [64][16][5] (input channels 4..15 unused), b1 [64], W2, b2, W3, b3
 * [64][64][5], [64], W4 [1][64][5], b4 [1] (vg_corr_num_params() = 46593
 * floats).  Loss = mean over cells of (P(net - want))^2 with want =
 * ((target - its group mean) - d) / (s tau). */
typedef struct vg_corrector vg_corrector;
#define VG_CORR_NV 128
/* One batch of rows; all DEVICE pointers, FP32, [rows][128] unless noted. */
typedef struct vg_corr_batch {
  const float* g;         /* state after the coarse step */
  const float* g_prev;    /* state before it; NULL: a zero channel */
  const float* row_feat;  /* [rows]; NULL: a zero channel */
  const float* target;    /* loss, gradients and training only */
  int32_t rows;           /* <= max_rows */
  int32_t group_rows;     /* 0, or a divisor of rows */
} vg_corr_batch;
int vg_corr_num_params(void);
int vg_corr_create(int32_t max_rows, int32_t protect_modes, float vmax, float tau, const float* params_host,
                   vg_corrector** out);
int vg_corr_destroy(vg_corrector* corr);
int vg_corr_set_tau(vg_corrector* corr, float tau);
int vg_corr_get_params(vg_corrector* corr, float* host_out);
/* also clears the optimiser state */
int vg_corr_set_params(vg_corrector* corr, const float* host_in);
/* g_out may alias batch->g (in-place correction).  Engine 0 (default), the
 * tcgen05 tensor cores: apply is one fused persistent kernel per call
 * (weights and activations in shared memory, accumulators in TMEM); the
 * training calls (loss, gradients, train step) run one tcgen05 kernel per
 * layer, forward, data gradient and weight gradient, keeping the activations
 * in HBM for the backward pass.  Every wait is bounded and a wait that ran
 * out raises vg_corr_status.  Engine 1: the same layers on mma.sync. */
int vg_corr_apply(vg_corrector* corr, const vg_corr_batch* batch, float* g_out, vg_stream stream);
int vg_corr_set_engine(vg_corrector* corr, int32_t engine);
/* synchronises; VG_ERR_TIMEOUT (flags != 0) if a bounded wait of a tcgen05
 * kernel ran out since the corrector was created */
int vg_corr_status(vg_corrector* corr, int32_t* flags);
/* loss only (synchronises the stream) */
int vg_corr_loss(vg_corrector* corr, const vg_corr_batch* batch, double* loss_out, vg_stream stream);
/* loss and its gradient w.r.t. all parameters (HOST grad_host, PyTorch
 * order; NULL to keep it on the device); synchronises the stream */
int vg_corr_gradients(vg_corrector* corr, const vg_corr_batch* batch, float* grad_host, double* loss_out,
                      vg_stream stream);
/* one Adam step (beta 0.9, 0.999, eps 1e-8) on the loss of this batch;
 * loss_out may be NULL (then nothing synchronises) */
int vg_corr_train_step(vg_corrector* corr, const vg_corr_batch* batch, float lr, double* loss_out,
                       vg_stream stream);

#ifdef __cplusplus
}
#endif

#endif /* VLAGPU_H */
