//! lbm-cuda: the Rust binding of liblbm_cuda, the GB300 (sm_103a) D2Q9
//! lattice-Boltzmann step that replaces the storage and stepping of
//! chemsim's `src/lbm.rs` (`D2Q9`, `State::step`, the moment accessors).
//!
//! `ffi` is the `extern "C"` block of `include/lbm_cuda.h`, one declaration
//! per entry point with the same parameters.  `CudaD2Q9` and `CudaBatch` are
//! the safe wrappers chemsim's `State` dispatches to (see `chemsim.patch` in
//! this crate for the changes to `src/lbm.rs`, `src/main.rs` and
//! `Cargo.toml`).  A negative status from the library becomes a panic, the
//! way lbm.rs treats a violated invariant (`assert!` / `assert_eq!`,
//! src/lbm.rs:51-52,188,191) under `panic = "abort"` (Cargo.toml:128).

use std::ffi::{CStr, CString};
use std::os::raw::c_int;
use std::path::Path;

pub mod ffi {
    //! Declarations of include/lbm_cuda.h.
    use std::os::raw::{c_char, c_int, c_void};

    #[repr(C)] pub struct LbmLattice { _p: [u8; 0] }
    #[repr(C)] pub struct LbmBatch { _p: [u8; 0] }
    #[repr(C)] pub struct LbmCnn { _p: [u8; 0] }
    #[repr(C)] pub struct LbmDesc {
        pub w: c_int, pub h: c_int, pub tau: f32, pub flags: c_int,
        pub fx: f32, pub fy: f32, pub solid: *const u8,
    }
    #[repr(C)] #[derive(Default, Debug, Clone, Copy)]
    pub struct LbmHealth {
        pub mass: f64, pub momentum_x: f64, pub momentum_y: f64,
        pub min_population: f64, pub min_eq0: f64,
        pub nonfinite_count: i64, pub steps: i64, pub unstable: i32, pub reserved: i32,
    }

    pub const LBM_OK: c_int = 0;
    pub const LBM_ERR_INVALID_ARGUMENT: c_int = -1;
    pub const LBM_ERR_OUT_OF_MEMORY: c_int = -2;
    pub const LBM_ERR_CUDA: c_int = -3;
    pub const LBM_ERR_UNSTABLE: c_int = -4;
    pub const LBM_ERR_TIMEOUT: c_int = -5;
    pub const LBM_ERR_NOT_SUPPORTED: c_int = -6;
    pub const LBM_ERR_STATE: c_int = -7;

    pub const LBM_F32: c_int = 0;
    pub const LBM_F64: c_int = 1;
    pub const LBM_F16DEV: c_int = 2;
    pub const LBM_BF16DEV: c_int = 3;

    pub const LBM_X_ZEROPAD: c_int = 0x00;
    pub const LBM_X_PERIODIC: c_int = 0x01;
    pub const LBM_X_WALL: c_int = 0x02;
    pub const LBM_Y_ZEROPAD: c_int = 0x00;
    pub const LBM_Y_PERIODIC: c_int = 0x04;
    pub const LBM_Y_WALL: c_int = 0x08;
    pub const LBM_SOLID_FULLWAY: c_int = 0x00;
    pub const LBM_SOLID_HALFWAY: c_int = 0x10;
    pub const LBM_FRAME_REF: c_int = 0x00;
    pub const LBM_FRAME_XY: c_int = 0x20;
    pub const LBM_FAST: c_int = 0x40;
    pub const LBM_ROUND_NEAREST: c_int = 0x80;
    pub const LBM_REFERENCE_FLAGS: c_int = 0x00;

    pub const LBM_COLLISION_BGK: c_int = 0;
    pub const LBM_COLLISION_TRT: c_int = 1;

    pub const LBM_RENDER_DENSITY: c_int = 0;
    pub const LBM_RENDER_SPEED: c_int = 1;
    pub const LBM_RENDER_VELOCITY: c_int = 2;
    pub const LBM_RENDER_MOMENTUM: c_int = 3;

    extern "C" {
        pub fn lbm_last_error_string() -> *const c_char;
        pub fn lbm_version() -> c_int;
        pub fn lbm_create(w: c_int, h: c_int, tau: f32, precision: c_int, flags: c_int,
                          out: *mut *mut LbmLattice) -> c_int;
        pub fn lbm_destroy(lat: *mut LbmLattice) -> c_int;
        pub fn lbm_set_discretization(lat: *mut LbmLattice, dx: f32, dt: f32) -> c_int;
        pub fn lbm_set_collision(lat: *mut LbmLattice, kind: c_int, tau: f32, tau_minus: f32) -> c_int;
        pub fn lbm_init_equilibrium(lat: *mut LbmLattice, rho: *const f32, ux: *const f32,
                                    uy: *const f32) -> c_int;
        pub fn lbm_set_populations(lat: *mut LbmLattice, f: *const f32) -> c_int;
        pub fn lbm_get_populations(lat: *mut LbmLattice, f: *mut f32) -> c_int;
        pub fn lbm_set_populations_f64(lat: *mut LbmLattice, f: *const f64) -> c_int;
        pub fn lbm_get_populations_f64(lat: *mut LbmLattice, f: *mut f64) -> c_int;
        pub fn lbm_set_geometry(lat: *mut LbmLattice, solid: *const u8) -> c_int;
        pub fn lbm_set_force(lat: *mut LbmLattice, fx: f32, fy: f32) -> c_int;
        pub fn lbm_step(lat: *mut LbmLattice, nsteps: c_int) -> c_int;
        pub fn lbm_step_moments(lat: *mut LbmLattice, nsteps: c_int) -> c_int;
        pub fn lbm_read_moments(lat: *mut LbmLattice, rho: *mut f32, ux: *mut f32, uy: *mut f32,
                                on_device: c_int) -> c_int;
        pub fn lbm_read_moments_async(lat: *mut LbmLattice, rho: *mut f32, ux: *mut f32,
                                      uy: *mut f32) -> c_int;
        pub fn lbm_step_moments_to(lat: *mut LbmLattice, nsteps: c_int, rho: *mut f32, ux: *mut f32,
                                   uy: *mut f32) -> c_int;
        pub fn lbm_readback_wait(lat: *mut LbmLattice) -> c_int;
        pub fn lbm_check(lat: *mut LbmLattice, out: *mut LbmHealth) -> c_int;
        pub fn lbm_get_time(lat: *mut LbmLattice, time: *mut f32, steps: *mut i64) -> c_int;
        pub fn lbm_set_stream(lat: *mut LbmLattice, stream: *mut c_void) -> c_int;
        pub fn lbm_synchronize(lat: *mut LbmLattice) -> c_int;
        pub fn lbm_device_populations(lat: *mut LbmLattice, base: *mut *mut c_void,
                                      plane_stride: *mut i64, row_pitch: *mut c_int) -> c_int;
        pub fn lbm_set_tile(lat: *mut LbmLattice, cells_per_thread: c_int, rows_per_block: c_int) -> c_int;
        pub fn lbm_check_device_noalloc(populations: *const c_void, precision: c_int, w: c_int, h: c_int,
                                        row_pitch: c_int, plane_stride: i64, dx: f32, dt: f32,
                                        stream: *mut c_void, out: *mut LbmHealth) -> c_int;
        // checkpoint / resume
        pub fn lbm_save(lat: *mut LbmLattice, path: *const c_char) -> c_int;
        pub fn lbm_load(lat: *mut LbmLattice, path: *const c_char) -> c_int;
        // colour map of src/render.rs into an RGBA8 buffer (host, or device when on_device = 1)
        pub fn lbm_render(lat: *mut LbmLattice, mode: c_int, geometry_overlay: c_int, rgba: *mut u8,
                          on_device: c_int) -> c_int;
        pub fn lbm_render_async(lat: *mut LbmLattice, mode: c_int, geometry_overlay: c_int,
                                rgba: *mut u8) -> c_int;
        // batched lattices
        pub fn lbm_batch_create(n: c_int, descs: *const LbmDesc, flags: c_int, out: *mut *mut LbmBatch) -> c_int;
        pub fn lbm_batch_destroy(b: *mut LbmBatch) -> c_int;
        pub fn lbm_batch_size(b: *mut LbmBatch, n: *mut c_int) -> c_int;
        pub fn lbm_batch_lattice(b: *mut LbmBatch, i: c_int, out: *mut *mut LbmLattice) -> c_int;
        pub fn lbm_batch_step(b: *mut LbmBatch, nsteps: c_int) -> c_int;
        pub fn lbm_batch_synchronize(b: *mut LbmBatch) -> c_int;
        pub fn lbm_batch_set_stream(b: *mut LbmBatch, stream: *mut c_void) -> c_int;
        pub fn lbm_batch_set_tile(b: *mut LbmBatch, cells_per_thread: c_int) -> c_int;
        pub fn lbm_batch_tile(b: *mut LbmBatch, cells_per_thread: *mut c_int) -> c_int;
        pub fn lbm_batch_autotune(b: *mut LbmBatch, cache_path: *const c_char, steps_per_trial: c_int) -> c_int;
        // learned coarse-grid correction
        pub fn lbm_cnn_create(h: c_int, w: c_int, max_batch: c_int, seed: u64, out: *mut *mut LbmCnn) -> c_int;
        pub fn lbm_cnn_destroy(net: *mut LbmCnn) -> c_int;
        pub fn lbm_cnn_param_count(net: *mut LbmCnn, n: *mut i64) -> c_int;
        pub fn lbm_cnn_get_params(net: *mut LbmCnn, params: *mut f32) -> c_int;
        pub fn lbm_cnn_set_params(net: *mut LbmCnn, params: *const f32) -> c_int;
        pub fn lbm_cnn_forward(net: *mut LbmCnn, input: *const f32, batch: c_int, out: *mut f32) -> c_int;
        pub fn lbm_cnn_gradients(net: *mut LbmCnn, input: *const f32, target: *const f32, batch: c_int,
                                 loss: *mut f32, grads: *mut f32) -> c_int;
        pub fn lbm_cnn_train_step(net: *mut LbmCnn, input: *const f32, target: *const f32, batch: c_int,
                                  lr: f32, loss: *mut f32) -> c_int;
        pub fn lbm_selftest_wait_timeout(polls: u32, timed_out: *mut c_int) -> c_int;
        pub fn lbm_cnn_load(net: *mut LbmCnn, path: *const c_char) -> c_int;
        pub fn lbm_cnn_save(net: *mut LbmCnn, path: *const c_char) -> c_int;
        pub fn lbm_cnn_set_stream(net: *mut LbmCnn, stream: *mut c_void) -> c_int;
        pub fn lbm_cnn_synchronize(net: *mut LbmCnn) -> c_int;
        pub fn lbm_restrict(fine: *mut LbmLattice, coarse: *mut LbmLattice, factor: c_int) -> c_int;
        pub fn lbm_coarse_features(lat: *mut LbmLattice, s_rho: f32, s_u: f32, image: c_int,
                                   input: *mut f32) -> c_int;
        pub fn lbm_coarse_apply(lat: *mut LbmLattice, corr: *const f32, image: c_int, scale: f32,
                                max_abs: f32) -> c_int;
        pub fn lbm_coarse_target(reference: *mut LbmLattice, cur: *mut LbmLattice, scale: f32, image: c_int,
                                 target: *mut f32) -> c_int;
        pub fn lbm_coarse_run(lat: *mut LbmLattice, net: *mut LbmCnn, nsteps: c_int, k: c_int,
                              s_rho: f32, s_u: f32, scale: f32, max_abs: f32, check_every: c_int,
                              mass_tolerance: f32, fallback_step: *mut i64) -> c_int;
    }
}

use ffi::*;

/// Panics with the library's message when `status` is negative.
pub fn ok(status: c_int) {
    if status != LBM_OK {
        let msg = unsafe { CStr::from_ptr(lbm_last_error_string()) };
        panic!("lbm-cuda status {}: {}", status, msg.to_string_lossy());
    }
}

fn c_path(path: &Path) -> CString {
    CString::new(path.to_string_lossy().as_bytes()).expect("path without NUL bytes")
}

/// Health of a lattice: `State::is_unstable` (src/lbm.rs:815-818) is
/// `unstable`, plus the f64 mass and momentum sums of `Matrix::sum`.
pub type Health = LbmHealth;

/// A device-resident D2Q9 lattice: the storage of `D2Q9`
/// (src/lbm.rs:180-323) and the stepping of `State<D2Q9>`
/// (src/lbm.rs:694-751), one fused kernel launch per time step.
pub struct CudaD2Q9 {
    raw: *mut LbmLattice,
    pub w: usize,
    pub h: usize,
    owned: bool,
}

// A handle is used from one thread at a time (it is not thread-safe), but it
// may move between threads.
unsafe impl Send for CudaD2Q9 {}

impl CudaD2Q9 {
    /// `D2Q9::new` + `State::initial`: a w x h lattice at rest
    /// equilibrium.  `precision` is one of LBM_F32 / LBM_F64 / LBM_F16DEV /
    /// LBM_BF16DEV; `flags` selects boundaries, frame and arithmetic
    /// (LBM_REFERENCE_FLAGS keeps every lbm.rs semantic).
    pub fn new(w: usize, h: usize, tau: f32, precision: c_int, flags: c_int) -> Self {
        let mut raw = std::ptr::null_mut();
        ok(unsafe { lbm_create(w as c_int, h as c_int, tau, precision, flags, &mut raw) });
        CudaD2Q9 { raw, w, h, owned: true }
    }

    /// The raw handle, for entry points without a wrapper.
    pub fn raw(&self) -> *mut LbmLattice {
        self.raw
    }

    fn cells(&self) -> usize {
        self.w * self.h
    }

    /// `Discretization { delta_x, delta_t }` (src/lbm.rs:75-86).
    pub fn set_discretization(&mut self, dx: f32, dt: f32) {
        ok(unsafe { lbm_set_discretization(self.raw, dx, dt) })
    }

    /// `BGK { tau }` or `TRT` (src/lbm.rs:345-451).
    pub fn set_collision(&mut self, kind: c_int, tau: f32, tau_minus: f32) {
        ok(unsafe { lbm_set_collision(self.raw, kind, tau, tau_minus) })
    }

    /// `compute_equilibrium(density, velocity)` (src/lbm.rs:43-71) written
    /// into the lattice; fields row-major y*w+x as `Matrix::new` takes them.
    pub fn init_equilibrium(&mut self, rho: &[f32], ux: &[f32], uy: &[f32]) {
        assert_eq!(rho.len(), self.cells());
        assert_eq!(ux.len(), self.cells());
        assert_eq!(uy.len(), self.cells());
        ok(unsafe { lbm_init_equilibrium(self.raw, rho.as_ptr(), ux.as_ptr(), uy.as_ptr()) })
    }

    /// The nine planes in `D2Q9::directions` order, each row-major y*w+x
    /// (`Matrix::get_underlying` of each population).
    pub fn set_populations(&mut self, f: &[f32]) {
        assert_eq!(f.len(), 9 * self.cells());
        ok(unsafe { lbm_set_populations(self.raw, f.as_ptr()) })
    }

    pub fn populations(&self) -> Vec<f32> {
        let mut f = vec![0f32; 9 * self.cells()];
        ok(unsafe { lbm_get_populations(self.raw, f.as_mut_ptr()) });
        f
    }

    /// `State::geometry` (an `af::Array<bool>`), row-major y*w+x as
    /// `initial_state` and `LBMSim::handle` build it (src/main.rs:77-89,269-312).
    pub fn set_geometry(&mut self, solid: &[bool]) {
        assert_eq!(solid.len(), self.cells());
        let bytes: Vec<u8> = solid.iter().map(|&b| b as u8).collect();
        ok(unsafe { lbm_set_geometry(self.raw, bytes.as_ptr()) })
    }

    pub fn clear_geometry(&mut self) {
        ok(unsafe { lbm_set_geometry(self.raw, std::ptr::null()) })
    }

    pub fn set_force(&mut self, fx: f32, fy: f32) {
        ok(unsafe { lbm_set_force(self.raw, fx, fy) })
    }

    /// n time steps of `State::step` (stream, bounce-back, collide).
    pub fn step(&mut self, n: usize) {
        ok(unsafe { lbm_step(self.raw, n as c_int) })
    }

    /// n time steps whose last one also writes the moments on the device.
    pub fn step_moments(&mut self, n: usize) {
        ok(unsafe { lbm_step_moments(self.raw, n as c_int) })
    }

    /// (density, velocity_x, velocity_y) of `Lattice::density` /
    /// `Lattice::velocity` (src/lbm.rs:117-149), each row-major y*w+x like
    /// `Matrix::get_underlying`.
    pub fn moments(&self) -> (Vec<f32>, Vec<f32>, Vec<f32>) {
        let n = self.cells();
        let (mut r, mut x, mut y) = (vec![0f32; n], vec![0f32; n], vec![0f32; n]);
        ok(unsafe { lbm_read_moments(self.raw, r.as_mut_ptr(), x.as_mut_ptr(), y.as_mut_ptr(), 0) });
        (r, x, y)
    }

    /// The same fields written into device buffers of w*h f32 each (a
    /// renderer that keeps them on the GPU).
    ///
    /// # Safety
    /// The three pointers must be device allocations of at least w*h f32.
    pub unsafe fn moments_to_device(&self, rho: *mut f32, ux: *mut f32, uy: *mut f32) {
        ok(lbm_read_moments(self.raw, rho, ux, uy, 1))
    }

    /// `State::is_unstable` and the conservation sums.
    pub fn health(&self) -> Health {
        let mut h = LbmHealth::default();
        ok(unsafe { lbm_check(self.raw, &mut h) });
        h
    }

    /// `State::time` (f32, accumulated by delta_t per step) and the steps taken.
    pub fn time(&self) -> (f32, i64) {
        let (mut t, mut n) = (0f32, 0i64);
        ok(unsafe { lbm_get_time(self.raw, &mut t, &mut n) });
        (t, n)
    }

    /// One RGBA8 frame of render.rs's colour map (`DisplayMode` order:
    /// density 0, speed 1, velocity 2, momentum density 3).
    pub fn render(&self, mode: c_int, geometry_overlay: bool) -> Vec<u8> {
        let mut rgba = vec![0u8; 4 * self.cells()];
        ok(unsafe { lbm_render(self.raw, mode, geometry_overlay as c_int, rgba.as_mut_ptr(), 0) });
        rgba
    }

    pub fn save(&self, path: &Path) {
        let p = c_path(path);
        ok(unsafe { lbm_save(self.raw, p.as_ptr()) })
    }

    pub fn load(&mut self, path: &Path) {
        let p = c_path(path);
        ok(unsafe { lbm_load(self.raw, p.as_ptr()) })
    }

    pub fn synchronize(&self) {
        ok(unsafe { lbm_synchronize(self.raw) })
    }
}

impl Drop for CudaD2Q9 {
    fn drop(&mut self) {
        if self.owned {
            unsafe {
                lbm_destroy(self.raw);
            }
        }
    }
}

/// Many independent lattices of uneven sizes and relaxation times that step
/// together (no reference counterpart; the batched path of the benchmark).
pub struct CudaBatch {
    raw: *mut LbmBatch,
}

unsafe impl Send for CudaBatch {}

impl CudaBatch {
    /// descs: size, tau, boundary flags, force and optional solid mask of each
    /// member; flags: LBM_FRAME_XY and/or LBM_FAST for all.
    pub fn new(descs: &[LbmDesc], flags: c_int) -> Self {
        let mut raw = std::ptr::null_mut();
        ok(unsafe { lbm_batch_create(descs.len() as c_int, descs.as_ptr(), flags, &mut raw) });
        CudaBatch { raw }
    }

    pub fn len(&self) -> usize {
        let mut n: c_int = 0;
        ok(unsafe { lbm_batch_size(self.raw, &mut n) });
        n as usize
    }

    pub fn is_empty(&self) -> bool {
        self.len() == 0
    }

    /// Member i as a lattice handle owned by the batch.
    pub fn member(&self, i: usize, w: usize, h: usize) -> CudaD2Q9 {
        let mut raw = std::ptr::null_mut();
        ok(unsafe { lbm_batch_lattice(self.raw, i as c_int, &mut raw) });
        CudaD2Q9 { raw, w, h, owned: false }
    }

    pub fn step(&mut self, n: usize) {
        ok(unsafe { lbm_batch_step(self.raw, n as c_int) })
    }

    /// The batch kernel's tile width: 2 or 4 cells per thread.
    pub fn set_tile(&mut self, cells_per_thread: usize) {
        ok(unsafe { lbm_batch_set_tile(self.raw, cells_per_thread as c_int) })
    }

    pub fn tile(&self) -> usize {
        let mut v: c_int = 0;
        ok(unsafe { lbm_batch_tile(self.raw, &mut v) });
        v as usize
    }

    /// Times both tile widths on the members and caches the choice in the
    /// JSON file at `cache`.
    pub fn autotune(&mut self, cache: &Path) {
        let p = c_path(cache);
        ok(unsafe { lbm_batch_autotune(self.raw, p.as_ptr(), 0) })
    }

    pub fn synchronize(&self) {
        ok(unsafe { lbm_batch_synchronize(self.raw) })
    }
}

impl Drop for CudaBatch {
    fn drop(&mut self) {
        unsafe {
            lbm_batch_destroy(self.raw);
        }
    }
}
