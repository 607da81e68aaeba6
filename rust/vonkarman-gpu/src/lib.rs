//! vonkarman's own interfaces for the periodic pseudospectral step, backed by
//! the GB300 library through `vonkarman-gpu-sys`:
//!
//! * [`NativeGpuBackend`] implements `FftBackend<f64>`
//!   (vonkarman-fft/src/backend.rs:9-25); [`create_backend_native`] is what a
//!   `BackendMode::Native` arm of `create_backend` (vonkarman-fft/src/select.rs:34-67)
//!   returns.  Unlike `BackendMode::Auto` it never falls back silently.
//! * [`Periodic3DGpu`] implements `Domain<f64>` (vonkarman-core/src/domain.rs:39-81)
//!   with the solver state resident in device memory.
//! * [`EnstrophyGrowth`] is the discrete adjoint as a forward/backward pair
//!   (the autograd-Function pattern, no PyTorch): J(u0) = final enstrophy and
//!   dJ/du0.
//!
//! Errors: construction returns `Result`; the trait methods, whose signatures
//! cannot carry an error, panic with the library's message as the reference's
//! `CufftBackend` does (vonkarman-fft/src/cufft.rs:262-314).

use std::cell::UnsafeCell;
use std::ffi::CStr;

use ndarray::Array3;
use num_complex::Complex;
use vonkarman_core::domain::{Domain, PhysicsParams, Snapshot};
use vonkarman_core::field::{GridSpec, VectorField};
use vonkarman_core::spectral_ops::SpectralOps;
use vonkarman_fft::backend::FftBackend;
use vonkarman_gpu_sys as sys;

type SpecArray = Array3<Complex<f64>>;

fn global_error() -> String {
    unsafe { CStr::from_ptr(sys::vk_last_error(std::ptr::null())) }.to_string_lossy().into_owned()
}

fn as_ptr(a: &SpecArray) -> *const f64 {
    a.as_slice().expect("spectral arrays must be contiguous (standard layout)").as_ptr() as *const f64
}

fn as_mut_ptr(a: &mut SpecArray) -> *mut f64 {
    a.as_slice_mut().expect("spectral arrays must be contiguous (standard layout)").as_mut_ptr() as *mut f64
}

fn zeros_state(grid: &GridSpec) -> [SpecArray; 3] {
    let shape = grid.spectral_shape();
    let z = Complex { re: 0.0, im: 0.0 };
    [Array3::from_elem(shape, z), Array3::from_elem(shape, z), Array3::from_elem(shape, z)]
}

// ---------------------------------------------------------------------------
// FftBackend
// ---------------------------------------------------------------------------

/// `FftBackend<f64>` on the GPU: host arrays in, host arrays out, like
/// `CufftBackend`; the transforms run as the library's pencil passes.
pub struct NativeGpuBackend {
    plan: *mut sys::vk_fft,
    name: String,
}

// One user thread at a time, with synchronous calls (as CufftBackend, cufft.rs:173-175).
unsafe impl Send for NativeGpuBackend {}

impl NativeGpuBackend {
    pub fn new(nx: usize, ny: usize, nz: usize) -> Result<Self, String> {
        let mut plan = std::ptr::null_mut();
        let rc = unsafe {
            sys::vk_fft_create(nx as i32, ny as i32, nz as i32, sys::VK_PRECISION_FP64, 0, &mut plan)
        };
        if rc != sys::VK_OK {
            return Err(global_error());
        }
        let name = unsafe { CStr::from_ptr(sys::vk_fft_name(plan)) }.to_string_lossy().into_owned();
        Ok(Self { plan, name })
    }

    fn error(&self) -> String {
        unsafe { CStr::from_ptr(sys::vk_fft_last_error(self.plan)) }.to_string_lossy().into_owned()
    }
}

impl Drop for NativeGpuBackend {
    fn drop(&mut self) {
        unsafe {
            sys::vk_fft_destroy(self.plan);
        }
    }
}

impl FftBackend<f64> for NativeGpuBackend {
    fn r2c_3d(&self, input: &Array3<f64>, output: &mut SpecArray) {
        let rc = unsafe {
            sys::vk_fft_r2c_host(self.plan, input.as_slice().unwrap().as_ptr(), as_mut_ptr(output))
        };
        assert_eq!(rc, sys::VK_OK, "vk_fft_r2c_host failed: {}", self.error());
    }

    fn c2r_3d(&self, input: &SpecArray, output: &mut Array3<f64>) {
        let rc = unsafe {
            sys::vk_fft_c2r_host(self.plan, as_ptr(input), output.as_slice_mut().unwrap().as_mut_ptr())
        };
        assert_eq!(rc, sys::VK_OK, "vk_fft_c2r_host failed: {}", self.error());
    }

    fn name(&self) -> &str {
        &self.name
    }

    fn precision_digits(&self) -> usize {
        unsafe { sys::vk_fft_precision_digits(self.plan) as usize }
    }
}

/// The `BackendMode::Native` arm of `create_backend`: the GPU backend or a
/// panic naming the cause (no silent fallback).
pub fn create_backend_native(nx: usize, ny: usize, nz: usize) -> Box<dyn FftBackend<f64>> {
    Box::new(NativeGpuBackend::new(nx, ny, nz).unwrap_or_else(|e| panic!("native GPU backend: {e}")))
}

// ---------------------------------------------------------------------------
// Domain
// ---------------------------------------------------------------------------

/// Options beyond `Periodic3D::new(grid, nu, ic, backend)`.
#[derive(Clone, Copy, Debug)]
pub struct GpuOptions {
    pub precision: i32,
    pub etd_variant: i32,
    pub integrator: i32,
    pub dt_mode: i32,
    pub dt_fixed: f64,
    pub cfl_safety: f64,
    pub device: i32,
}

impl Default for GpuOptions {
    fn default() -> Self {
        Self {
            precision: sys::VK_PRECISION_FP64,
            etd_variant: sys::VK_ETD_REFERENCE,
            integrator: sys::VK_INTEGRATOR_ETD_RK4,
            dt_mode: sys::VK_DT_CFL,
            dt_fixed: 0.0,
            cfl_safety: 0.5,
            device: 0,
        }
    }
}

/// `Periodic3D` with its state in device memory.  `u_hat()` returns a host
/// copy refreshed after the state changes.
pub struct Periodic3DGpu {
    ctx: *mut sys::vk_ctx,
    grid: GridSpec,
    params: PhysicsParams,
    fft: NativeGpuBackend,
    ops: SpectralOps<f64>,
    cache: UnsafeCell<[SpecArray; 3]>,
    cache_valid: UnsafeCell<bool>,
}

impl Periodic3DGpu {
    /// `Periodic3D::new` after the IC transform (solver.rs:38-108): `u_hat` is
    /// the spectral initial velocity.
    pub fn new(grid: GridSpec, params: PhysicsParams, u_hat: &[SpecArray; 3], opts: GpuOptions)
               -> Result<Self, String> {
        let mut cfg = sys::vk_config::default();
        unsafe { sys::vk_config_default(&mut cfg, grid.nx as i32, params.nu) };
        cfg.ny = grid.ny as i32;
        cfg.nz = grid.nz as i32;
        cfg.lx = grid.lx;
        cfg.ly = grid.ly;
        cfg.lz = grid.lz;
        cfg.precision = opts.precision;
        cfg.etd_variant = opts.etd_variant;
        cfg.integrator = opts.integrator;
        cfg.dt_mode = opts.dt_mode;
        cfg.dt_fixed = opts.dt_fixed;
        cfg.cfl_safety = opts.cfl_safety;
        cfg.device = opts.device;
        let mut ctx = std::ptr::null_mut();
        if unsafe { sys::vk_create(&cfg, &mut ctx) } != sys::VK_OK {
            return Err(global_error());
        }
        let fft = NativeGpuBackend::new(grid.nx, grid.ny, grid.nz)?;
        let me = Self {
            ctx,
            grid,
            params,
            fft,
            ops: SpectralOps::new(&grid),
            cache: UnsafeCell::new(zeros_state(&grid)),
            cache_valid: UnsafeCell::new(false),
        };
        let rc = unsafe {
            sys::vk_set_state_host(ctx, as_ptr(&u_hat[0]), as_ptr(&u_hat[1]), as_ptr(&u_hat[2]))
        };
        me.check(rc)?;
        Ok(me)
    }

    /// `Periodic3D::from_checkpoint` on this context (solver.rs:127-159).
    pub fn restore(&mut self, u_hat: &[SpecArray; 3], time: f64, step: u64, dt: f64) -> Result<(), String> {
        let rc = unsafe {
            sys::vk_restore_host(self.ctx, as_ptr(&u_hat[0]), as_ptr(&u_hat[1]), as_ptr(&u_hat[2]), time, step, dt)
        };
        self.invalidate();
        self.check(rc)
    }

    /// `n` steps enqueued without a host synchronisation between them.
    pub fn step_n(&mut self, n: i64) -> Result<(), String> {
        let rc = unsafe { sys::vk_step(self.ctx, n) };
        self.invalidate();
        self.check(rc)
    }

    /// Tier-1 (`ScalarDiagnostics::from_domain`, scalar.rs:22-46) in one call.
    pub fn tier1(&self) -> Result<sys::vk_tier1_out, String> {
        let mut t = sys::vk_tier1_out::default();
        self.check(unsafe { sys::vk_tier1(self.ctx, &mut t) })?;
        Ok(t)
    }

    /// `energy_spectrum` (vonkarman-diag/src/spectrum.rs:13-60): (shells, E).
    pub fn energy_spectrum(&self) -> Result<(Vec<f64>, Vec<f64>), String> {
        let mut n = 0i32;
        self.check(unsafe { sys::vk_spectrum_len(self.ctx, &mut n) })?;
        let mut shells = vec![0.0; n as usize];
        let mut spec = vec![0.0; n as usize];
        self.check(unsafe { sys::vk_spectrum(self.ctx, shells.as_mut_ptr(), spec.as_mut_ptr(), n) })?;
        Ok((shells, spec))
    }

    /// `SpectralOps` public fields as the device forms them (bit-identical to
    /// `SpectralOps::new`, spectral_ops.rs:26-74).
    pub fn spectral_ops(&self) -> Result<(Vec<f64>, Vec<f64>, Vec<f64>, Array3<f64>), String> {
        let (nx, ny, nz) = self.grid.spectral_shape();
        let (mut kx, mut ky, mut kz) = (vec![0.0; nx], vec![0.0; ny], vec![0.0; nz]);
        let mut k2 = Array3::from_elem((nx, ny, nz), 0.0);
        let rc = unsafe {
            sys::vk_wavenumbers(self.ctx, kx.as_mut_ptr(), ky.as_mut_ptr(), kz.as_mut_ptr(),
                                k2.as_slice_mut().unwrap().as_mut_ptr())
        };
        self.check(rc)?;
        Ok((kx, ky, kz, k2))
    }

    pub fn ctx(&self) -> *mut sys::vk_ctx {
        self.ctx
    }

    pub fn last_error(&self) -> String {
        unsafe { CStr::from_ptr(sys::vk_last_error(self.ctx)) }.to_string_lossy().into_owned()
    }

    fn check(&self, rc: i32) -> Result<(), String> {
        if rc == sys::VK_OK { Ok(()) } else { Err(self.last_error()) }
    }

    fn invalidate(&self) {
        unsafe { *self.cache_valid.get() = false };
    }

    fn scalar(&self, f: unsafe extern "C" fn(*mut sys::vk_ctx, *mut f64) -> i32, what: &str) -> f64 {
        let mut v = 0.0;
        let rc = unsafe { f(self.ctx, &mut v) };
        assert_eq!(rc, sys::VK_OK, "{what}: {}", self.last_error());
        v
    }
}

impl Drop for Periodic3DGpu {
    fn drop(&mut self) {
        unsafe {
            sys::vk_destroy(self.ctx);
        }
    }
}

impl Domain<f64> for Periodic3DGpu {
    fn step(&mut self) {
        let r = self.step_n(1);
        assert!(r.is_ok(), "vk_step: {}", r.unwrap_err());
    }

    fn time(&self) -> f64 {
        self.scalar(sys::vk_time, "vk_time")
    }

    fn step_count(&self) -> u64 {
        let mut v = 0u64;
        let rc = unsafe { sys::vk_step_count(self.ctx, &mut v) };
        assert_eq!(rc, sys::VK_OK, "vk_step_count: {}", self.last_error());
        v
    }

    fn dt(&self) -> f64 {
        self.scalar(sys::vk_dt, "vk_dt")
    }

    fn energy(&self) -> f64 {
        self.scalar(sys::vk_energy, "vk_energy")
    }

    fn enstrophy(&self) -> f64 {
        self.scalar(sys::vk_enstrophy, "vk_enstrophy")
    }

    fn helicity(&self) -> f64 {
        self.scalar(sys::vk_helicity, "vk_helicity")
    }

    fn superhelicity(&self) -> f64 {
        self.scalar(sys::vk_superhelicity, "vk_superhelicity")
    }

    fn max_vorticity(&self) -> f64 {
        self.scalar(sys::vk_max_vorticity, "vk_max_vorticity")
    }

    fn cfl_dt(&self) -> f64 {
        self.scalar(sys::vk_cfl_dt, "vk_cfl_dt")
    }

    fn u_hat(&self) -> &[SpecArray; 3] {
        // Refresh the host copy after the device state changed.  &self API of
        // the trait: the cache is interior-mutable and the context is used by
        // one thread at a time (the type is not Sync).
        unsafe {
            if !*self.cache_valid.get() {
                let c = &mut *self.cache.get();
                let [x, y, z] = c;
                let rc = sys::vk_get_state_host(self.ctx, as_mut_ptr(x), as_mut_ptr(y), as_mut_ptr(z));
                assert_eq!(rc, sys::VK_OK, "vk_get_state_host: {}", self.last_error());
                *self.cache_valid.get() = true;
            }
            &*self.cache.get()
        }
    }

    fn grid(&self) -> &GridSpec {
        &self.grid
    }

    fn params(&self) -> &PhysicsParams {
        &self.params
    }

    /// As `Periodic3D::snapshot` (solver.rs:589-617): velocity and vorticity
    /// through the native backend's c2r.
    fn snapshot(&self) -> Snapshot<f64> {
        let u_hat = self.u_hat().clone();
        let mut velocity = VectorField::zeros(self.grid);
        for c in 0..3 {
            self.fft.c2r_3d(&u_hat[c], &mut velocity.data[c]);
        }
        let mut omega_hat = zeros_state(&self.grid);
        self.ops.curl(&u_hat, &mut omega_hat);
        let mut vorticity = VectorField::zeros(self.grid);
        for c in 0..3 {
            self.fft.c2r_3d(&omega_hat[c], &mut vorticity.data[c]);
        }
        Snapshot {
            time: self.time(),
            step: self.step_count(),
            dt: self.dt(),
            velocity,
            vorticity,
            u_hat,
            grid: self.grid,
            params: self.params,
        }
    }
}

// ---------------------------------------------------------------------------
// Discrete adjoint as a forward/backward pair
// ---------------------------------------------------------------------------

/// J(u0) = enstrophy after `nsteps` fixed-dt ETD-RK4 steps and dJ/du0.  The
/// checkpoints stay in the context between `forward` and `backward`.  The
/// context must use `VK_DT_FIXED` and the reference ETD variant.
pub struct EnstrophyGrowth<'a> {
    pub dom: &'a mut Periodic3DGpu,
    pub nsteps: i64,
    pub nsnap: i32,
    /// `VK_ADJ_TWO_LEVEL` or `VK_ADJ_BINOMIAL`.
    pub schedule: i32,
    pub dt: f64,
}

impl EnstrophyGrowth<'_> {
    /// Forward: sets u0, runs the steps keeping the schedule's checkpoints,
    /// returns J.  The context's state advances.
    pub fn forward(&mut self, u0: &[SpecArray; 3]) -> Result<f64, String> {
        self.dom.restore(u0, 0.0, 0, self.dt)?;
        self.dom.check(unsafe { sys::vk_adjoint_set_schedule(self.dom.ctx, self.schedule) })?;
        let mut j = 0.0;
        let rc = unsafe { sys::vk_adjoint_forward(self.dom.ctx, self.nsteps, self.nsnap, &mut j) };
        self.dom.invalidate();
        self.dom.check(rc)?;
        Ok(j)
    }

    /// Backward: dJ/du0 of the preceding forward in the L2 inner product of
    /// the physical fields, projected on real, divergence-free, Nyquist-free
    /// fields.
    pub fn backward(&mut self) -> Result<[SpecArray; 3], String> {
        let mut g = zeros_state(&self.dom.grid);
        let [gx, gy, gz] = &mut g;
        let rc = unsafe { sys::vk_adjoint_backward(self.dom.ctx, as_mut_ptr(gx), as_mut_ptr(gy), as_mut_ptr(gz)) };
        self.dom.check(rc)?;
        Ok(g)
    }
}
