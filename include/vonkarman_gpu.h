/*
 * vonkarman_gpu.h -- C ABI of the GB300-native periodic pseudospectral step.
 *
 * Drop-in boundary for the hot path of alejandro-soto-franco/vonkarman.  Every
 * entry point names the reference interface it replaces (file:line in that
 * project).  Plain C types only: status codes, plain pointers and sizes.
 *
 * Data layout.  A spectral component is the reference's ndarray
 * Array3<Complex<f64>> in C order: shape (nx, ny, nz/2+1), iz fastest,
 * interleaved {re, im} doubles (vonkarman-core/src/field.rs:48-50,
 * vonkarman-fft/src/cufft.rs:258,274).  Vector fields are three such arrays.
 * Physical-space arrays are (nx, ny, nz) doubles in C order.
 *
 * Errors.  Every function returns VK_OK (0) or a vk_status code and never
 * aborts; vk_last_error() returns the message of the last failure on that
 * context (or of the last failed vk_create / vk_fft_create when ctx is NULL).
 * The reference panics on CUDA execution errors (vonkarman-fft/src/cufft.rs:262-314);
 * this boundary reports them instead.  A NaN or infinity that enters the
 * solver state (seen by a CFL / max pass, or written by the final stage of a
 * step) makes the next call that synchronises -- vk_time, vk_dt, vk_cfl_dt,
 * vk_tier1 and its field getters, vk_run, vk_step_timed -- return
 * VK_ERR_NONFINITE, the NaN check of the reference's audit
 * (vonkarman-diag/src/audit.rs:175-197); vk_step itself enqueues without a
 * readback.  Setting a new state clears the condition.
 *
 * Threading.  One context per thread; each context owns one CUDA stream and
 * keeps its solver state resident in device memory.  Calls are synchronous
 * with respect to the host unless named *_async.
 */
#ifndef VONKARMAN_GPU_H
#define VONKARMAN_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VK_ABI_VERSION 1

typedef enum vk_status {
  VK_OK = 0,
  VK_ERR_INVALID = 1,      /* bad argument or configuration                    */
  VK_ERR_UNSUPPORTED = 2,  /* valid for the reference, not built here           */
  VK_ERR_CUDA = 3,         /* CUDA runtime error (message in vk_last_error)     */
  VK_ERR_OOM = 4,          /* device allocation failed                          */
  VK_ERR_STATE = 5,        /* call out of order (e.g. step before set_state)    */
  VK_ERR_NONFINITE = 6     /* a NaN/Inf was detected in the state               */
} vk_status;

typedef enum vk_precision {
  VK_PRECISION_FP64 = 0,     /* FP64 throughout (the reference's f64 path)       */
  VK_PRECISION_FP32BULK = 1  /* FFTs, nonlinear term and stages in FP32; ETD
                                coefficients, dt, time and reductions in FP64    */
} vk_precision;

typedef enum vk_etd_variant {
  VK_ETD_REFERENCE = 0,     /* stage formulas of vonkarman-periodic/src/solver.rs:264-378 */
  VK_ETD_COX_MATTHEWS = 1   /* textbook Cox-Matthews / Kassam-Trefethen stages          */
} vk_etd_variant;

typedef enum vk_integrator {
  VK_INTEGRATOR_ETD_RK4 = 0, /* Periodic3D::etd_rk4_step, solver.rs:221-379 */
  VK_INTEGRATOR_RK4 = 1      /* rk4_step, vonkarman-periodic/src/rk4.rs:16-146 */
} vk_integrator;

typedef enum vk_dt_mode {
  VK_DT_CFL = 0,   /* CFL dt every step with the 1% re-tabulation rule (solver.rs:383-396) */
  VK_DT_FIXED = 1  /* dt = dt_fixed (not in the reference)                               */
} vk_dt_mode;

/* Solver configuration.  Mirrors GridSpec (vonkarman-core/src/field.rs:6-14),
 * the physics/integrator parts of ExperimentConfig
 * (vonkarman-bin/src/config.rs:7-116) and the hard-coded CFL safety of
 * Periodic3D::new (solver.rs:89).  Grids are cubic: nx == ny == nz, a power of
 * two in [8, 512]; lx == ly == lz > 0 (vonkarman-bin/src/validate.rs:6-57). */
typedef struct vk_config {
  int32_t nx, ny, nz;
  double lx, ly, lz;
  double nu;
  int32_t precision;    /* vk_precision   */
  int32_t etd_variant;  /* vk_etd_variant */
  int32_t integrator;   /* vk_integrator  */
  int32_t dt_mode;      /* vk_dt_mode     */
  double dt_fixed;      /* used when dt_mode == VK_DT_FIXED */
  double cfl_safety;    /* (0, 1]; the reference uses 0.5 */
  int32_t device;       /* CUDA device ordinal */
  int32_t reserved;
} vk_config;

/* ScalarDiagnostics (vonkarman-diag/src/scalar.rs:6-18), same fields and
 * conventions: enstrophy = <|omega|^2> (no 1/2), dissipation rates
 * -2 nu Omega and -2 nu H2, cfl_number = max|omega| dt / dx. */
typedef struct vk_tier1_out {
  double time;
  uint64_t step;
  double dt;
  double energy;
  double enstrophy;
  double helicity;
  double superhelicity;
  double max_vorticity;
  double energy_dissipation_rate;
  double helicity_dissipation_rate;
  double cfl_number;
} vk_tier1_out;

typedef struct vk_ctx vk_ctx;
typedef struct vk_fft vk_fft;

/* --- library --------------------------------------------------------------- */
int vk_abi_version(void);
/* Message of the last error on ctx; ctx == NULL gives the last error of a
 * failed create call in this thread. */
const char* vk_last_error(const vk_ctx* ctx);
/* Defaults: L = 2 pi, FP64, reference ETD variant, ETD-RK4, CFL dt, safety 0.5. */
void vk_config_default(vk_config* cfg, int32_t n, double nu);

/* --- solver context (replaces Periodic3D, vonkarman-periodic/src/solver.rs:12-618) */
/* Periodic3D::new minus the IC generation (solver.rs:38-108). */
int vk_create(const vk_config* cfg, vk_ctx** out);
int vk_destroy(vk_ctx* ctx);
/* Number of complex entries per spectral component: nx*ny*(nz/2+1). */
int64_t vk_spectral_len(const vk_ctx* ctx);

/* Upload u_hat (3 components) and initialise like Periodic3D::new after its
 * IC transform (solver.rs:69-108): time = 0, step = 0, dt = CFL(u_hat) (or
 * dt_fixed), ETD table built. */
int vk_set_state_host(vk_ctx* ctx, const double* ux, const double* uy, const double* uz);
/* Periodic3D::from_checkpoint (solver.rs:127-159): state, time, step and dt
 * restored; ETD table rebuilt from the stored dt. */
int vk_restore_host(vk_ctx* ctx, const double* ux, const double* uy, const double* uz,
                    double time, uint64_t step_count, double dt);
/* Domain::u_hat / checkpoint_data (domain.rs:71, solver.rs:111-121). */
int vk_get_state_host(vk_ctx* ctx, double* ux, double* uy, double* uz);

/* Domain::step (solver.rs:383-400), nsteps times, enqueued on the context's
 * stream without host synchronisation between steps. */
int vk_step(vk_ctx* ctx, int64_t nsteps);
/* Steps as CUDA graphs (no reference counterpart): with enable != 0 (the
 * default) vk_step, vk_run and the adjoint forward replay each step's ~30
 * kernel launches as one captured graph (one graph per launch sequence,
 * captured the second time that sequence runs); results are those of the
 * eager launches.  Profiling (vk_profile_enable) always launches eagerly. */
int vk_use_graphs(vk_ctx* ctx, int32_t enable);
/* Domain::time / step_count / dt (domain.rs:44-50). */
int vk_time(vk_ctx* ctx, double* out);
int vk_step_count(vk_ctx* ctx, uint64_t* out);
int vk_dt(vk_ctx* ctx, double* out);
/* Domain::cfl_dt (solver.rs:569-577): the CFL estimate of the current state. */
int vk_cfl_dt(vk_ctx* ctx, double* out);

/* ScalarDiagnostics::from_domain (scalar.rs:22-46): Tier-1 of the current state. */
int vk_tier1(vk_ctx* ctx, vk_tier1_out* out);
/* Individual Domain methods (solver.rs:412-567). */
int vk_energy(vk_ctx* ctx, double* out);
int vk_enstrophy(vk_ctx* ctx, double* out);
int vk_helicity(vk_ctx* ctx, double* out);
int vk_superhelicity(vk_ctx* ctx, double* out);
int vk_max_vorticity(vk_ctx* ctx, double* out);

/* Run nsteps steps and record Tier-1 after every `every`-th step into out
 * (capacity max_records); *n_records receives the count.  One host
 * synchronisation at the end (the run loop of vonkarman-bin/src/run.rs:107-132
 * without per-step readbacks). */
int vk_run(vk_ctx* ctx, int64_t nsteps, int64_t every, vk_tier1_out* out, int64_t max_records,
           int64_t* n_records);

/* Diagnostics fused into the step (no reference counterpart; the reference
 * recomputes them from the state, solver.rs:412-535, spectrum.rs:13-60): on
 * every step whose step count is a multiple of tier1_every (spectrum_every)
 * the final stage also accumulates the Tier-1 sums (the shell spectrum) of
 * the new state, and vk_tier1 (vk_spectrum) on that state adds those partials
 * instead of reading the state again.  0 disables; vk_run always fuses the
 * Tier-1 sums of its record steps.  The fused sums equal the separate ones to
 * rounding (same per-mode terms, a different summation order). */
int vk_set_fused_diagnostics(vk_ctx* ctx, int64_t tier1_every, int64_t spectrum_every);

/* energy_spectrum (vonkarman-diag/src/spectrum.rs:13-60): shells[i] = i,
 * spectrum[i] = E(i), n = ceil(sqrt(3) * N/2) + 1 entries. */
int vk_spectrum_len(const vk_ctx* ctx, int32_t* n);
int vk_spectrum(vk_ctx* ctx, double* shells, double* spectrum, int32_t n);

/* compute_nonlinear (vonkarman-periodic/src/nonlinear.rs:15-39) on host arrays:
 * n_hat = P[F(u x omega)] with 3/2 dealiasing; does not touch the solver state. */
int vk_nonlinear_host(vk_ctx* ctx, const double* ux, const double* uy, const double* uz, double* nx_out,
                      double* ny_out, double* nz_out);

/* SpectralOps::apply_viscous (vonkarman-core/src/spectral_ops.rs:154-175) on
 * host arrays: out_c = -(nu |k|^2) u_c, |k|^2 formed as SpectralOps::new does
 * (spectral_ops.rs:26-44); computed on the device in the context's precision,
 * does not touch the solver state. */
int vk_apply_viscous_host(vk_ctx* ctx, double nu, const double* ux, const double* uy, const double* uz,
                          double* out_x, double* out_y, double* out_z);
/* The public fields of SpectralOps (spectral_ops.rs:10-22): kx, ky (n
 * entries, index n/2 mapped to -n/2), kz (n/2+1 entries) and, unless NULL,
 * k_mag_sq ((n, n, n/2+1) doubles, C order), bit-identical to
 * SpectralOps::new (spectral_ops.rs:26-74). */
int vk_wavenumbers(vk_ctx* ctx, double* kx, double* ky, double* kz, double* k_mag_sq);

/* --- discrete adjoint (no reference counterpart: the reference has no
 *     adjoint; the forward map it differentiates is Domain::step with the
 *     reference ETD-RK4 stages, solver.rs:221-400) --------------------------- */
/* Autograd-Function forward: runs nsteps steps (dt_mode must be fixed) from the
 * current state, keeping nsnap level-1 checkpoints (one every
 * ceil(nsteps/nsnap) steps), and returns J = enstrophy of the final state
 * (the reference convention, solver.rs:436-465).  The state advances. */
int vk_adjoint_forward(vk_ctx* ctx, int64_t nsteps, int32_t nsnap, double* J);
/* Checkpoint schedule of the following vk_adjoint_forward / backward pairs.
 * VK_ADJ_TWO_LEVEL (default): the level-1 checkpoints above, each segment
 * recomputed once storing its stage inputs (nsnap + 4 ceil(nsteps/nsnap) + 1
 * states; one recompute pass).  VK_ADJ_BINOMIAL: nsnap state slots (the
 * initial state in one of them) reversed with the binomial treeverse schedule
 * (nsnap + 4 states; each step recomputed at most r times, r the least with
 * C(nsnap - 1 + r, r) >= nsteps), for adjoints the two-level schedule cannot
 * hold in memory.  Both give the same gradient. */
#define VK_ADJ_TWO_LEVEL 0
#define VK_ADJ_BINOMIAL 1
int vk_adjoint_set_schedule(vk_ctx* ctx, int32_t schedule);
/* Autograd-Function backward: dJ/du_0 for the last vk_adjoint_forward, in the
 * L2 inner product of the physical fields (<a,b> = sum w Re(a conj b) / N^6),
 * projected onto real, divergence-free fields with zero Nyquist entries.
 * Two-level schedule: segments are recomputed from their checkpoint storing
 * u, a, b, c of every step (4 ceil(nsteps/nsnap) + 1 states), then reversed;
 * binomial schedule: see vk_adjoint_set_schedule. */
int vk_adjoint_backward(vk_ctx* ctx, double* gx, double* gy, double* gz);
/* Transpose of compute_nonlinear's linearisation at x applied to nbar (raw
 * Euclidean inner product of the stored entries), on host arrays. */
int vk_nonlinear_adjoint_host(vk_ctx* ctx, const double* ux, const double* uy, const double* uz,
                              const double* bx, const double* by, const double* bz, double* ox, double* oy,
                              double* oz);

/* --- measurement (no reference counterpart: the reference has no profiler
 *     hook beyond its total wall time, vonkarman-bin/src/run.rs:73,200) ----- */
/* vk_step with CUDA events recorded on the context's stream around the
 * enqueued steps; *elapsed_ms is the device time between them. */
int vk_step_timed(vk_ctx* ctx, int64_t nsteps, double* elapsed_ms);
/* Per-pass CUDA-event timing of every launch while enabled (see
 * vk_profile_pass_name for the pass ids; VK_NPASS passes). */
#define VK_NPASS 20
int vk_profile_enable(vk_ctx* ctx, int32_t enable);
int vk_profile_read(vk_ctx* ctx, double* ms, int64_t* launches, int32_t n);
const char* vk_profile_pass_name(int32_t id);
/* FP64 (fp64 = 1) or FP32 FMA throughput of the device in GFLOP/s. */
int vk_probe_fma_peak(int32_t device, int32_t fp64, double* gflops);
/* The context's cudaStream_t.  Every operation of the context is ordered on
 * it: a step's ETD table runs on a second stream of the context that forks
 * from and joins back into this one within the step, so work queued on this
 * stream after a step (or a wait on it) sees the whole step. */
int vk_stream(vk_ctx* ctx, void** stream);
/* Record event slot (0..7) on the context's stream; elapsed device time
 * between two recorded slots (waits for slot b). */
int vk_event_mark(vk_ctx* ctx, int32_t slot);
int vk_event_elapsed(vk_ctx* ctx, int32_t a, int32_t b, double* ms);
/* Page-locked host buffers for fast vk_*_host transfers. */
int vk_pinned_alloc(size_t bytes, void** out);
int vk_pinned_free(void* p);

/* --- allocation-free entry point (no counterpart in the reference: its
 *     energy_spectrum, vonkarman-diag/src/spectrum.rs:13-60, works on host
 *     arrays) ------------------------------------------------------------- */
/* Shell spectrum E(k) of a state the caller already holds in device memory,
 * for callers that must not allocate device memory: code recording a CUDA
 * graph, code under a framework's caching allocator that owns all device
 * memory, latency-critical loops that cannot take an allocation's implicit
 * synchronisation.  Nothing is allocated: the scratch is a fixed 896 KiB
 * device array inside the library, held on every GPU that loads it until the
 * process exits, which limits n to 512 (at most 448 shells).
 *   u_hat        three contiguous components (n, n, n/2+1) on the current
 *                device, double2 (precision VK_PRECISION_FP64) or float2
 *                (VK_PRECISION_FP32BULK)
 *   spectrum_out ceil(sqrt(3)*n/2)+1 doubles on the device (spectrum[i] =
 *                E(shell i), conventions of energy_spectrum)
 *   stream       cudaStream_t to enqueue on (NULL = default stream); the call
 *                returns without synchronising.
 * The first call on each device looks up the scratch address
 * (cudaGetSymbolAddress, which also loads the module); make that first call
 * before any stream capture.  The address is looked up again when the
 * device's context changes (after a device reset).  The sums are the
 * Neumaier-compensated column sums of vk_spectrum over 256 partial blocks
 * (vk_spectrum: 8 per SM), so the two agree to rounding, not bitwise.
 * All calls share the one scratch array: calls that overlap on the GPU (other
 * streams, concurrently launched graphs) race and must be serialised by the
 * caller.  Errors: VK_ERR_INVALID / VK_ERR_UNSUPPORTED (n > 512), message in
 * vk_last_error(NULL). */
int vk_spectrum_noalloc(const void* u_hat, int32_t n, double l, int32_t precision, double* spectrum_out,
                        void* stream);

/* --- FFT backend (replaces FftBackend<f64>, vonkarman-fft/src/backend.rs:9-25,
 *     and create_backend, vonkarman-fft/src/select.rs:34-67) ------------------- */
/* Each of nx, ny, nz in {8,16,...,512} or {12,24,...,768}. */
int vk_fft_create(int32_t nx, int32_t ny, int32_t nz, int32_t precision, int32_t device, vk_fft** out);
int vk_fft_destroy(vk_fft* plan);
const char* vk_fft_last_error(const vk_fft* plan);
/* FftBackend::r2c_3d (backend.rs:13): unnormalised forward, host arrays. */
int vk_fft_r2c_host(vk_fft* plan, const double* in, double* out);
/* FftBackend::c2r_3d (backend.rs:18): inverse including 1/(nx ny nz). */
int vk_fft_c2r_host(vk_fft* plan, const double* in, double* out);
/* Device-pointer forms, in the plan's precision (double / float buffers),
 * enqueued on `stream` (a cudaStream_t, NULL = the plan's stream).  r2c does
 * not modify `in`; c2r uses `in` as scratch and overwrites it. */
int vk_fft_r2c_device(vk_fft* plan, const void* in, void* out, void* stream);
int vk_fft_c2r_device(vk_fft* plan, void* in, void* out, void* stream);
/* FftBackend::name / precision_digits (backend.rs:21-24). */
const char* vk_fft_name(const vk_fft* plan);
int vk_fft_precision_digits(const vk_fft* plan);

#ifdef __cplusplus
}
#endif

#endif /* VONKARMAN_GPU_H */
