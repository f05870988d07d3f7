//! `auto-cuda`: the spectral automata (Lenia, SmoothLife, MNCA) of `auto-core` stepped on one
//! NVIDIA GB300 through the C ABI of `include/lenia_gb300.h`.
//!
//! [`Sim`] keeps the method names of `auto_core::Sim` (crates/auto-core/src/sim.rs:202-595):
//! `new` (Sim::new + automata::build), `step`, `wait` (Gpu::wait), `write_field` / `read_field`
//! for the `state` field, and `tick`.  Failures come back as `Err(String)`, as `Sim::new` returns
//! them (sim.rs:208-219); nothing panics or aborts across the ABI.
//!
//! Not compiled where it was written (no Rust toolchain there).  It declares the entry points this
//! wrapper calls, each with the header's signature; the rest of the header can be declared the same
//! way.

use std::ffi::CStr;
use std::os::raw::{c_char, c_int, c_void};

pub const MAX_KERNELS: usize = 16;

pub const PATH_FP32: i32 = 0;
pub const PATH_TF32: i32 = 1;
pub const PATH_BF16X3: i32 = 2;
pub const PATH_RADIX2: i32 = 3;

pub const SHAPE_LENIA: i32 = 0;
pub const SHAPE_SL_INNER: i32 = 1;
pub const SHAPE_SL_OUTER: i32 = 2;
pub const SHAPE_RING: i32 = 3;

pub const RULE_LENIA: i32 = 0;
pub const RULE_SMOOTHLIFE: i32 = 1;
pub const RULE_MNCA: i32 = 2;

/// `LeniaKernel`: one convolution kernel and its growth parameters.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct LeniaKernel {
    pub shape: i32,
    pub radius: f32,
    pub nshells: i32,
    pub beta: [f32; 3],
    pub ring_lo: f32,
    pub ring_hi: f32,
    pub src: i32,
    pub dst: i32,
    pub mu: f32,
    pub sigma: f32,
    pub weight: f32,
}

/// `LeniaWorldDesc`: one world (grid, channels, kernels, rule, dt).
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct LeniaWorldDesc {
    pub width: u32,
    pub height: u32,
    pub channels: u32,
    pub nkernels: u32,
    pub rule: i32,
    pub dt: f32,
    pub kernels: [LeniaKernel; MAX_KERNELS],
}

impl LeniaWorldDesc {
    /// The reference's `lenia` program (spectral.rs:287-349): R = 13, one shell, mu = 0.15,
    /// sigma = 0.015, dt = 0.1.
    pub fn lenia(width: u32, height: u32) -> Self {
        let mut kernels = [LeniaKernel::default(); MAX_KERNELS];
        kernels[0] = LeniaKernel {
            shape: SHAPE_LENIA,
            radius: 13.0,
            nshells: 1,
            beta: [1.0, 0.0, 0.0],
            mu: 0.15,
            sigma: 0.015,
            weight: 1.0,
            ..Default::default()
        };
        LeniaWorldDesc { width, height, channels: 1, nkernels: 1, rule: RULE_LENIA, dt: 0.1, kernels }
    }
}

#[repr(C)]
pub struct LeniaCtx {
    _private: [u8; 0],
}

unsafe extern "C" {
    fn lenia_last_error(ctx: *const LeniaCtx) -> *const c_char;
    fn lenia_create(worlds: *const LeniaWorldDesc, n: i32, path: i32, out: *mut *mut LeniaCtx) -> c_int;
    fn lenia_destroy(ctx: *mut LeniaCtx) -> c_int;
    fn lenia_write_state(ctx: *mut LeniaCtx, world: i32, host: *const f32, count: usize) -> c_int;
    fn lenia_read_state(ctx: *mut LeniaCtx, world: i32, host: *mut f32, count: usize) -> c_int;
    fn lenia_write_states(ctx: *mut LeniaCtx, host: *const f32, count: usize) -> c_int;
    fn lenia_read_states(ctx: *mut LeniaCtx, host: *mut f32, count: usize) -> c_int;
    fn lenia_write_states_async(ctx: *mut LeniaCtx, host: *const f32, count: usize) -> c_int;
    fn lenia_read_states_async(ctx: *mut LeniaCtx, host: *mut f32, count: usize) -> c_int;
    fn lenia_step(ctx: *mut LeniaCtx, steps: u32) -> c_int;
    fn lenia_sync(ctx: *mut LeniaCtx) -> c_int;
    fn lenia_tick(ctx: *const LeniaCtx, tick: *mut u64) -> c_int;
    fn lenia_seed_patches(ctx: *mut LeniaCtx, world: i32, seed: u32, patches_xywh: *const i32, n: i32) -> c_int;
    fn lenia_seed_tiles(ctx: *mut LeniaCtx, world: i32, seed: u32, pattern: *const f32, pw: i32, ph: i32,
                        spacing: i32) -> c_int;
    fn lenia_cells_per_step(ctx: *const LeniaCtx, cells: *mut u64) -> c_int;
    fn lenia_memory_bytes(ctx: *const LeniaCtx, bytes: *mut u64) -> c_int;
    fn lenia_autotune(ctx: *mut LeniaCtx) -> c_int;
    fn lenia_set_variants(ctx: *mut LeniaCtx, col_variant: i32, row_variant: i32) -> c_int;
    fn lenia_set_chunk_budget(ctx: *mut LeniaCtx, mib: u32) -> c_int;
    fn lenia_set_chunk_lanes(ctx: *mut LeniaCtx, lanes: i32) -> c_int;
    fn lenia_set_persistent(ctx: *mut LeniaCtx, mode: i32) -> c_int;
    fn lenia_step_timed(ctx: *mut LeniaCtx, steps: u32, ms: *mut f32) -> c_int;
    fn lenia_seed_rule(ctx: *mut LeniaCtx, world: i32, seed: u32, kind: i32) -> c_int;
    fn lenia_world_stats(ctx: *mut LeniaCtx, host_out: *mut f32, count: usize) -> c_int;
    fn lenia_step_noalloc(state: *mut f32, width: u32, height: u32, khat: *const f32, mu: f32, sigma: f32, dt: f32,
                          steps: u32, stream: *mut c_void) -> c_int;
}

fn last_error(ctx: *const LeniaCtx) -> String {
    // SAFETY: lenia_last_error never returns NULL and the string lives until the next call.
    unsafe { CStr::from_ptr(lenia_last_error(ctx)).to_string_lossy().into_owned() }
}

fn ok(ctx: *const LeniaCtx, rc: c_int) -> Result<(), String> {
    if rc == 0 { Ok(()) } else { Err(last_error(ctx)) }
}

/// Drop-in for `auto_core::Sim` on the spectral automata: one context owning every device buffer
/// of one or more worlds, which advance together.
pub struct Sim {
    ctx: *mut LeniaCtx,
    cells: Vec<usize>,
}

// A context is used from one thread at a time (`&mut self` to step), like the reference's Sim.
unsafe impl Send for Sim {}

impl Sim {
    /// `Sim::new` (sim.rs:202-282) for `worlds` on step implementation `path` (PATH_*).
    pub fn new(worlds: &[LeniaWorldDesc], path: i32) -> Result<Sim, String> {
        let mut ctx = std::ptr::null_mut();
        let rc = unsafe { lenia_create(worlds.as_ptr(), worlds.len() as i32, path, &mut ctx) };
        ok(std::ptr::null(), rc)?;
        let cells = worlds.iter().map(|w| (w.channels * w.width * w.height) as usize).collect();
        Ok(Sim { ctx, cells })
    }

    /// `Sim::step` (sim.rs:297-309): asynchronous; returns the generations advanced.
    pub fn step(&mut self, steps: u32) -> Result<u64, String> {
        ok(self.ctx, unsafe { lenia_step(self.ctx, steps) })?;
        Ok(steps as u64)
    }

    /// `Gpu::wait` (gpu.rs:131-137).
    pub fn wait(&self) -> Result<(), String> {
        ok(self.ctx, unsafe { lenia_sync(self.ctx) })
    }

    /// `Sim::write_field(gpu, "state", bytes)` for one world: channel-major, row-major f32.
    pub fn write_field(&mut self, world: usize, state: &[f32]) -> Result<(), String> {
        ok(self.ctx, unsafe { lenia_write_state(self.ctx, world as i32, state.as_ptr(), state.len()) })
    }

    /// `Sim::read_field(gpu, "state")` for one world (blocking).
    pub fn read_field(&self, world: usize) -> Result<Vec<f32>, String> {
        let mut v = vec![0f32; self.cells[world]];
        ok(self.ctx, unsafe { lenia_read_state(self.ctx, world as i32, v.as_mut_ptr(), v.len()) })?;
        Ok(v)
    }

    /// Every world's state back to back in world order: one copy for all worlds.
    pub fn write_all(&mut self, states: &[f32]) -> Result<(), String> {
        ok(self.ctx, unsafe { lenia_write_states(self.ctx, states.as_ptr(), states.len()) })
    }

    pub fn read_all(&self) -> Result<Vec<f32>, String> {
        let mut v = vec![0f32; self.cells.iter().sum()];
        ok(self.ctx, unsafe { lenia_read_states(self.ctx, v.as_mut_ptr(), v.len()) })?;
        Ok(v)
    }

    /// Streaming form of `write_all`: returns at once; `states` must stay untouched until `wait`.
    ///
    /// # Safety
    /// The buffer is read by the GPU after this call returns.
    pub unsafe fn write_all_async(&mut self, states: &[f32]) -> Result<(), String> {
        ok(self.ctx, unsafe { lenia_write_states_async(self.ctx, states.as_ptr(), states.len()) })
    }

    /// Streaming form of `read_all`: `out` is filled by the time `wait` returns.
    ///
    /// # Safety
    /// The buffer is written by the GPU after this call returns.
    pub unsafe fn read_all_async(&mut self, out: &mut [f32]) -> Result<(), String> {
        ok(self.ctx, unsafe { lenia_read_states_async(self.ctx, out.as_mut_ptr(), out.len()) })
    }

    /// U[0,1] patches (x, y, w, h) from the PCG hash with `seed` (program.rs:140-147).
    pub fn seed_patches(&mut self, world: usize, seed: u32, patches: &[[i32; 4]]) -> Result<(), String> {
        ok(self.ctx, unsafe {
            lenia_seed_patches(self.ctx, world as i32, seed, patches.as_ptr() as *const i32, patches.len() as i32)
        })
    }

    /// The Lenia tile seeder (spectral.rs:313-335) with the caller's square pattern.
    pub fn seed_tiles(&mut self, world: usize, seed: u32, pattern: &[f32], side: i32, spacing: i32)
                      -> Result<(), String> {
        ok(self.ctx, unsafe { lenia_seed_tiles(self.ctx, world as i32, seed, pattern.as_ptr(), side, side, spacing) })
    }

    /// `Program::cells_per_step` (program.rs:116-119) over every world and channel.
    pub fn cells_per_step(&self) -> u64 {
        let mut c = 0;
        unsafe { lenia_cells_per_step(self.ctx, &mut c) };
        c
    }

    /// `Program::total_bytes` (program.rs:122-129): device bytes this context holds.
    pub fn memory_bytes(&self) -> u64 {
        let mut b = 0;
        unsafe { lenia_memory_bytes(self.ctx, &mut b) };
        b
    }

    /// Time the launch shapes of every size class and keep the fastest.
    pub fn autotune(&mut self) -> Result<(), String> {
        ok(self.ctx, unsafe { lenia_autotune(self.ctx) })
    }

    /// Pin the launch variants of every size class (-1 keeps a pass's current choice).
    pub fn set_variants(&mut self, column: i32, row: i32) -> Result<(), String> {
        ok(self.ctx, unsafe { lenia_set_variants(self.ctx, column, row) })
    }

    /// Chunks of at most `mib` MiB per size class (0: one per class), run on `lanes` (1..4) concurrent
    /// graph branches; results do not depend on either.
    pub fn set_chunks(&mut self, mib: u32, lanes: i32) -> Result<(), String> {
        ok(self.ctx, unsafe { lenia_set_chunk_budget(self.ctx, mib) })?;
        ok(self.ctx, unsafe { lenia_set_chunk_lanes(self.ctx, lanes) })
    }

    /// The persistent step on (`Some(variant)`, or `Some(-1)` for the default variant) or off (`None`).
    pub fn set_persistent(&mut self, variant: Option<i32>) -> Result<(), String> {
        let mode = match variant {
            None => 0,
            Some(v) if v < 0 => 1,
            Some(v) => 2 + v,
        };
        ok(self.ctx, unsafe { lenia_set_persistent(self.ctx, mode) })
    }

    /// `step` then `wait`, returning the device time of those steps in milliseconds.
    pub fn step_timed(&mut self, steps: u32) -> Result<f32, String> {
        let mut ms = 0f32;
        ok(self.ctx, unsafe { lenia_step_timed(self.ctx, steps, &mut ms) })?;
        Ok(ms)
    }

    /// SmoothLife discs (kind 1) or MNCA blocks (kind 2), the reference's seed passes, on the device.
    pub fn seed_rule(&mut self, world: usize, seed: u32, kind: i32) -> Result<(), String> {
        ok(self.ctx, unsafe { lenia_seed_rule(self.ctx, world as i32, seed, kind) })
    }

    /// Per world: mass and toroidal centroid (x, y).
    pub fn world_stats(&mut self) -> Result<Vec<[f32; 3]>, String> {
        let n = self.cells.len();
        let mut v = vec![0f32; 3 * n];
        ok(self.ctx, unsafe { lenia_world_stats(self.ctx, v.as_mut_ptr(), v.len()) })?;
        Ok(v.chunks(3).map(|c| [c[0], c[1], c[2]]).collect())
    }

    /// `Sim::tick`.
    pub fn tick(&self) -> u64 {
        let mut t = 0;
        unsafe { lenia_tick(self.ctx, &mut t) };
        t
    }
}

impl Drop for Sim {
    fn drop(&mut self) {
        unsafe { lenia_destroy(self.ctx) };
    }
}

/// Steps one single-channel, single-kernel Lenia world held in the caller's own device memory,
/// allocating nothing (see `lenia_step_noalloc` in include/lenia_gb300.h).
///
/// # Safety
/// `state` and `khat` are device pointers of the right sizes; `stream` is a cudaStream_t or null.
pub unsafe fn step_noalloc(state: *mut f32, width: u32, height: u32, khat: *const f32, mu: f32, sigma: f32, dt: f32,
                           steps: u32, stream: *mut c_void) -> Result<(), String> {
    ok(std::ptr::null(), unsafe { lenia_step_noalloc(state, width, height, khat, mu, sigma, dt, steps, stream) })
}
