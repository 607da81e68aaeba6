//! Raw bindings of `libvonkarman_gpu.so`: a line-for-line mirror of
//! `include/vonkarman_gpu.h` (types, constants and every entry point, in the
//! header's order).  The safe wrappers that implement vonkarman's own traits
//! live in the `vonkarman-gpu` crate.
#![allow(non_camel_case_types)]

use std::os::raw::{c_char, c_int, c_void};

pub const VK_ABI_VERSION: c_int = 1;

// vk_status
pub const VK_OK: c_int = 0;
pub const VK_ERR_INVALID: c_int = 1;
pub const VK_ERR_UNSUPPORTED: c_int = 2;
pub const VK_ERR_CUDA: c_int = 3;
pub const VK_ERR_OOM: c_int = 4;
pub const VK_ERR_STATE: c_int = 5;
pub const VK_ERR_NONFINITE: c_int = 6;

// vk_precision
pub const VK_PRECISION_FP64: i32 = 0;
pub const VK_PRECISION_FP32BULK: i32 = 1;
// vk_etd_variant
pub const VK_ETD_REFERENCE: i32 = 0;
pub const VK_ETD_COX_MATTHEWS: i32 = 1;
// vk_integrator
pub const VK_INTEGRATOR_ETD_RK4: i32 = 0;
pub const VK_INTEGRATOR_RK4: i32 = 1;
// vk_dt_mode
pub const VK_DT_CFL: i32 = 0;
pub const VK_DT_FIXED: i32 = 1;
// checkpoint schedules of the adjoint
pub const VK_ADJ_TWO_LEVEL: i32 = 0;
pub const VK_ADJ_BINOMIAL: i32 = 1;
// per-pass timers
pub const VK_NPASS: i32 = 20;

/// Solver configuration (`vk_config`).
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct vk_config {
    pub nx: i32,
    pub ny: i32,
    pub nz: i32,
    pub lx: f64,
    pub ly: f64,
    pub lz: f64,
    pub nu: f64,
    pub precision: i32,
    pub etd_variant: i32,
    pub integrator: i32,
    pub dt_mode: i32,
    pub dt_fixed: f64,
    pub cfl_safety: f64,
    pub device: i32,
    pub reserved: i32,
}

/// `ScalarDiagnostics` (vonkarman-diag/src/scalar.rs:6-18) as `vk_tier1_out`.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct vk_tier1_out {
    pub time: f64,
    pub step: u64,
    pub dt: f64,
    pub energy: f64,
    pub enstrophy: f64,
    pub helicity: f64,
    pub superhelicity: f64,
    pub max_vorticity: f64,
    pub energy_dissipation_rate: f64,
    pub helicity_dissipation_rate: f64,
    pub cfl_number: f64,
}

/// Opaque solver context.
#[repr(C)]
pub struct vk_ctx {
    _private: [u8; 0],
}

/// Opaque FFT plan.
#[repr(C)]
pub struct vk_fft {
    _private: [u8; 0],
}

unsafe extern "C" {
    pub fn vk_abi_version() -> c_int;
    pub fn vk_last_error(ctx: *const vk_ctx) -> *const c_char;
    pub fn vk_config_default(cfg: *mut vk_config, n: i32, nu: f64);
    pub fn vk_create(cfg: *const vk_config, out_: *mut *mut vk_ctx) -> c_int;
    pub fn vk_destroy(ctx: *mut vk_ctx) -> c_int;
    pub fn vk_spectral_len(ctx: *const vk_ctx) -> i64;
    pub fn vk_set_state_host(ctx: *mut vk_ctx, ux: *const f64, uy: *const f64, uz: *const f64) -> c_int;
    pub fn vk_restore_host(ctx: *mut vk_ctx, ux: *const f64, uy: *const f64, uz: *const f64, time: f64, step_count: u64, dt: f64) -> c_int;
    pub fn vk_get_state_host(ctx: *mut vk_ctx, ux: *mut f64, uy: *mut f64, uz: *mut f64) -> c_int;
    pub fn vk_step(ctx: *mut vk_ctx, nsteps: i64) -> c_int;
    pub fn vk_use_graphs(ctx: *mut vk_ctx, enable: i32) -> c_int;
    pub fn vk_time(ctx: *mut vk_ctx, out_: *mut f64) -> c_int;
    pub fn vk_step_count(ctx: *mut vk_ctx, out_: *mut u64) -> c_int;
    pub fn vk_dt(ctx: *mut vk_ctx, out_: *mut f64) -> c_int;
    pub fn vk_cfl_dt(ctx: *mut vk_ctx, out_: *mut f64) -> c_int;
    pub fn vk_tier1(ctx: *mut vk_ctx, out_: *mut vk_tier1_out) -> c_int;
    pub fn vk_energy(ctx: *mut vk_ctx, out_: *mut f64) -> c_int;
    pub fn vk_enstrophy(ctx: *mut vk_ctx, out_: *mut f64) -> c_int;
    pub fn vk_helicity(ctx: *mut vk_ctx, out_: *mut f64) -> c_int;
    pub fn vk_superhelicity(ctx: *mut vk_ctx, out_: *mut f64) -> c_int;
    pub fn vk_max_vorticity(ctx: *mut vk_ctx, out_: *mut f64) -> c_int;
    pub fn vk_run(ctx: *mut vk_ctx, nsteps: i64, every: i64, out_: *mut vk_tier1_out, max_records: i64, n_records: *mut i64) -> c_int;
    pub fn vk_set_fused_diagnostics(ctx: *mut vk_ctx, tier1_every: i64, spectrum_every: i64) -> c_int;
    pub fn vk_spectrum_len(ctx: *const vk_ctx, n: *mut i32) -> c_int;
    pub fn vk_spectrum(ctx: *mut vk_ctx, shells: *mut f64, spectrum: *mut f64, n: i32) -> c_int;
    pub fn vk_nonlinear_host(ctx: *mut vk_ctx, ux: *const f64, uy: *const f64, uz: *const f64, nx_out: *mut f64, ny_out: *mut f64, nz_out: *mut f64) -> c_int;
    pub fn vk_apply_viscous_host(ctx: *mut vk_ctx, nu: f64, ux: *const f64, uy: *const f64, uz: *const f64, out_x: *mut f64, out_y: *mut f64, out_z: *mut f64) -> c_int;
    pub fn vk_wavenumbers(ctx: *mut vk_ctx, kx: *mut f64, ky: *mut f64, kz: *mut f64, k_mag_sq: *mut f64) -> c_int;
    pub fn vk_adjoint_forward(ctx: *mut vk_ctx, nsteps: i64, nsnap: i32, j: *mut f64) -> c_int;
    pub fn vk_adjoint_set_schedule(ctx: *mut vk_ctx, schedule: i32) -> c_int;
    pub fn vk_adjoint_backward(ctx: *mut vk_ctx, gx: *mut f64, gy: *mut f64, gz: *mut f64) -> c_int;
    pub fn vk_nonlinear_adjoint_host(ctx: *mut vk_ctx, ux: *const f64, uy: *const f64, uz: *const f64, bx: *const f64, by: *const f64, bz: *const f64, ox: *mut f64, oy: *mut f64, oz: *mut f64) -> c_int;
    pub fn vk_step_timed(ctx: *mut vk_ctx, nsteps: i64, elapsed_ms: *mut f64) -> c_int;
    pub fn vk_profile_enable(ctx: *mut vk_ctx, enable: i32) -> c_int;
    pub fn vk_profile_read(ctx: *mut vk_ctx, ms: *mut f64, launches: *mut i64, n: i32) -> c_int;
    pub fn vk_profile_pass_name(id: i32) -> *const c_char;
    pub fn vk_probe_fma_peak(device: i32, fp64: i32, gflops: *mut f64) -> c_int;
    pub fn vk_stream(ctx: *mut vk_ctx, stream: *mut *mut c_void) -> c_int;
    pub fn vk_event_mark(ctx: *mut vk_ctx, slot: i32) -> c_int;
    pub fn vk_event_elapsed(ctx: *mut vk_ctx, a: i32, b: i32, ms: *mut f64) -> c_int;
    pub fn vk_pinned_alloc(bytes: usize, out_: *mut *mut c_void) -> c_int;
    pub fn vk_pinned_free(p: *mut c_void) -> c_int;
    pub fn vk_spectrum_noalloc(u_hat: *const c_void, n: i32, l: f64, precision: i32, spectrum_out: *mut f64, stream: *mut c_void) -> c_int;
    pub fn vk_fft_create(nx: i32, ny: i32, nz: i32, precision: i32, device: i32, out_: *mut *mut vk_fft) -> c_int;
    pub fn vk_fft_destroy(plan: *mut vk_fft) -> c_int;
    pub fn vk_fft_last_error(plan: *const vk_fft) -> *const c_char;
    pub fn vk_fft_r2c_host(plan: *mut vk_fft, in_: *const f64, out_: *mut f64) -> c_int;
    pub fn vk_fft_c2r_host(plan: *mut vk_fft, in_: *const f64, out_: *mut f64) -> c_int;
    pub fn vk_fft_r2c_device(plan: *mut vk_fft, in_: *const c_void, out_: *mut c_void, stream: *mut c_void) -> c_int;
    pub fn vk_fft_c2r_device(plan: *mut vk_fft, in_: *mut c_void, out_: *mut c_void, stream: *mut c_void) -> c_int;
    pub fn vk_fft_name(plan: *const vk_fft) -> *const c_char;
    pub fn vk_fft_precision_digits(plan: *const vk_fft) -> c_int;
}
