//! `Apic` with the reference's public API (src/apic.rs:397-400, 707-713,
//! 716-776, 779, 2352, 2412, 2429, 1015), stepping on the GPU through the C-ABI
//! of `include/apic_gpu.h`.  The handle owns the device state; the public
//! fields that `src/main.rs` reads are host mirrors refreshed by
//! `sync_to_host` (after every `update` when `mirror` is set, the default, as
//! the GUI needs; a benchmark clears it).  Errors panic, as the reference
//! (built with panic = "abort") does on its own failures.
//!
//! Not compiled in this repository's build: the image has no cargo or rustc.

use std::ffi::{c_char, c_void, CStr};
use ultraviolet::Vec2x8;
use wide::f32x8;

#[repr(C)]
struct ApicWorldProps {
    gravity: f32,
    border_damping: f32,
    cfl: f32,
    solve_error: f32,
}

#[repr(C)]
#[derive(Default)]
struct ApicInfo {
    width: u32,
    height: u32,
    cells: u32,
    cell_size: f32,
    num_chunks: u32,
    num_particles: u32,
    fluid_cells: u32,
    timestamp: u32,
    prev_deltatime: f32,
    mg_levels: u32,
}

#[repr(C)]
struct ApicHandle {
    _private: [u8; 0],
}

// apic_field ids of include/apic_gpu.h
const APIC_F_TRES: i32 = 8;
const APIC_F_DENSITY: i32 = 24;
const APIC_F_SMOOTHED_DENSITY: i32 = 25;
const APIC_F_PRESSURE: i32 = 26;
const APIC_F_FLUID_BITS: i32 = 32;

unsafe extern "C" {
    fn apic_create(w: u32, h: u32, cell: f32, p: *const ApicWorldProps, out: *mut *mut ApicHandle) -> i32;
    fn apic_destroy(h: *mut ApicHandle) -> i32;
    fn apic_update(h: *mut ApicHandle, flags: u32, frame_dt: f32) -> i32;
    fn apic_add_radial_force(h: *mut ApicHandle, x: f32, y: f32, r: f32, s: f32) -> i32;
    fn apic_max_particle_velocity(h: *mut ApicHandle, out: *mut f32) -> i32;
    fn apic_is_fluid(h: *mut ApicHandle, i: i32, j: i32, out: *mut u64) -> i32;
    fn apic_get_info(h: *mut ApicHandle, out: *mut ApicInfo) -> i32;
    fn apic_read_vec2x8(h: *mut ApicHandle, which: i32, dst: *mut f32, floats: u64) -> i32;
    fn apic_read_field(h: *mut ApicHandle, field: i32, dst: *mut c_void, bytes: u64) -> i32;
    fn apic_last_error() -> *const c_char;
    fn apic_update_batch(h: *const *mut ApicHandle, count: u32, flags: u32, frame_dt: f32, status: *mut i32) -> i32;
}

fn ck(rc: i32) {
    if rc != 0 {
        let msg = unsafe { CStr::from_ptr(apic_last_error()) };
        panic!("apic_gpu error {rc}: {}", msg.to_string_lossy());
    }
}

#[derive(Default)]
pub struct DebugOptions {
    pub disable_particle_sort: bool,
}

#[derive(Default, Clone)]
pub struct WorldProperties {
    pub gravity: f32,
    pub border_damping: f32,
    pub cfl: f32,
    pub solve_error: f32,
}

pub struct Apic {
    handle: *mut ApicHandle,
    /// Refresh the host mirrors after every update (the GUI reads them).
    pub mirror: bool,
    pub world_properties: WorldProperties,
    pub width: u32,
    pub height: u32,
    pub cells: u32,
    pub cell_size: f32,
    pub num_chunks: u32,
    pub num_particles: u32,
    pub fluid_cells: u32,
    pub timestamp: u32,
    pub prev_deltatime: f32,
    pub part_positions: Vec<Vec2x8>,
    pub part_velocities: Vec<Vec2x8>,
    pub part_c_u: Vec<Vec2x8>,
    pub part_c_v: Vec<Vec2x8>,
    pub part_time_residual: Vec<f32x8>,
    pub mac_pressure_grid: Vec<f32>,
    pub mac_density: Vec<f32>,
    pub smoothed_density: Vec<f32>,
    /// base_grid.type_fluid of the reference
    pub type_fluid: Vec<u64>,
}

impl Apic {
    pub fn new(width: u32, height: u32, cell_size: f32, world_properties: WorldProperties) -> Apic {
        let p = ApicWorldProps {
            gravity: world_properties.gravity,
            border_damping: world_properties.border_damping,
            cfl: world_properties.cfl,
            solve_error: world_properties.solve_error,
        };
        let mut handle = std::ptr::null_mut();
        ck(unsafe { apic_create(width, height, cell_size, &p, &mut handle) });
        let mut a = Apic {
            handle,
            mirror: true,
            world_properties,
            width,
            height,
            cells: width * height,
            cell_size,
            num_chunks: 0,
            num_particles: 0,
            fluid_cells: 0,
            timestamp: 0,
            prev_deltatime: 0.0,
            part_positions: Vec::new(),
            part_velocities: Vec::new(),
            part_c_u: Vec::new(),
            part_c_v: Vec::new(),
            part_time_residual: Vec::new(),
            mac_pressure_grid: Vec::new(),
            mac_density: Vec::new(),
            smoothed_density: Vec::new(),
            type_fluid: Vec::new(),
        };
        a.sync_to_host();
        a
    }

    pub fn update(&mut self, debug_options: &DebugOptions, frame_deltatime: f32) {
        ck(unsafe { apic_update(self.handle, debug_options.disable_particle_sort as u32, frame_deltatime) });
        if self.mirror {
            self.sync_to_host();
        }
    }

    pub fn add_radial_force(&mut self, x: f32, y: f32, radius: f32, strength: f32) {
        ck(unsafe { apic_add_radial_force(self.handle, x, y, radius, strength) });
    }

    pub fn get_max_particle_velocity(&self) -> f32 {
        let mut v = 0.0f32;
        ck(unsafe { apic_max_particle_velocity(self.handle, &mut v) });
        v
    }

    pub fn is_fluid(&self, i: i32, j: i32) -> u64 {
        let mut v = 0u64;
        ck(unsafe { apic_is_fluid(self.handle, i, j, &mut v) });
        v
    }

    fn read_field<T: Copy + Default>(&self, field: i32, out: &mut Vec<T>, count: usize) {
        out.resize(count, T::default());
        let bytes = (count * std::mem::size_of::<T>()) as u64;
        ck(unsafe { apic_read_field(self.handle, field, out.as_mut_ptr() as *mut c_void, bytes) });
    }

    /// Copy the device state into the public host mirrors.
    pub fn sync_to_host(&mut self) {
        let mut info = ApicInfo::default();
        ck(unsafe { apic_get_info(self.handle, &mut info) });
        self.num_chunks = info.num_chunks;
        self.num_particles = info.num_particles;
        self.fluid_cells = info.fluid_cells;
        self.timestamp = info.timestamp;
        self.prev_deltatime = info.prev_deltatime;
        let chunks = info.num_chunks as usize;
        let floats = chunks as u64 * 16; // Vec2x8: 8 x lanes then 8 y lanes
        for (which, dst) in [&mut self.part_positions, &mut self.part_velocities, &mut self.part_c_u,
                             &mut self.part_c_v].into_iter().enumerate() {
            dst.resize(chunks, Vec2x8::zero());
            ck(unsafe { apic_read_vec2x8(self.handle, which as i32, dst.as_mut_ptr() as *mut f32, floats) });
        }
        let mut tres: Vec<f32> = Vec::new();
        self.read_field(APIC_F_TRES, &mut tres, chunks * 8);
        self.part_time_residual =
            tres.chunks_exact(8).map(|c| f32x8::from(<[f32; 8]>::try_from(c).unwrap())).collect();
        let cells = self.cells as usize;
        let mut buf = Vec::new();
        self.read_field(APIC_F_PRESSURE, &mut buf, cells);
        self.mac_pressure_grid = buf.clone();
        self.read_field(APIC_F_DENSITY, &mut buf, cells);
        self.mac_density = buf.clone();
        self.read_field(APIC_F_SMOOTHED_DENSITY, &mut buf, cells);
        self.smoothed_density = buf;
        let mut bits: Vec<u64> = Vec::new();
        self.read_field(APIC_F_FLUID_BITS, &mut bits, cells.div_ceil(64));
        self.type_fluid = bits;
    }
}

/// One `update` of every scene in `scenes` through `apic_update_batch` (no
/// counterpart in the reference): each scene's result is the one its own
/// `update` gives, bit for bit; the library runs the pressure solves of all
/// scenes as one launch per solve phase where they qualify (its batch tuner
/// chooses), else each scene on its own stream.  Mirrors are refreshed for the
/// scenes that keep `mirror` set.
pub fn update_batch(scenes: &mut [&mut Apic], debug_options: &DebugOptions, frame_deltatime: f32) {
    let hs: Vec<*mut ApicHandle> = scenes.iter().map(|a| a.handle).collect();
    ck(unsafe {
        apic_update_batch(hs.as_ptr(), hs.len() as u32, debug_options.disable_particle_sort as u32, frame_deltatime,
                          std::ptr::null_mut())
    });
    for a in scenes.iter_mut() {
        if a.mirror {
            a.sync_to_host();
        }
    }
}

impl Drop for Apic {
    fn drop(&mut self) {
        unsafe {
            apic_destroy(self.handle);
        }
    }
}
