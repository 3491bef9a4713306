//! `extern "C"` binding of `include/rc.h` (librc.so) for the reference
//! renderer crate.  Every struct is `#[repr(C)]` with the header's field
//! order, and every entry point of the header is declared here with the
//! same parameters; the repository's CPU tests compare both against gcc's
//! view of the header, since this image has no Rust toolchain.
#![allow(non_camel_case_types)]
#![allow(dead_code)]
use std::os::raw::{c_char, c_int, c_void};

pub type rc_status = c_int;
pub const RC_OK: rc_status = 0;
pub const RC_ERR_INVALID_ARG: rc_status = 1;
pub const RC_ERR_OOM: rc_status = 2;
pub const RC_ERR_CUDA: rc_status = 3;
pub const RC_ERR_TIMEOUT: rc_status = 4;
pub const RC_ERR_UNSUPPORTED: rc_status = 5;
pub const RC_ERR_STATE: rc_status = 6;

pub const RC_PRECISION_FP32: i32 = 0;
pub const RC_PRECISION_FP16: i32 = 1;
pub const RC_MEM_HOST: i32 = 0;
pub const RC_MEM_DEVICE: i32 = 1;
pub const RC_VOXEL_OPAQUE: u16 = 0x8000;
pub const RC_NOALLOC_SCRATCH_BYTES: usize = 8 << 20;
pub const RC_MAX_CASCADES: usize = 10;

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct rc_params {
    pub grid: [i32; 3],
    pub num_cascades: i32,
    pub probe_spacing0: i32,
    pub dir_res0: i32,
    pub interval0: i32,
    pub interval_ratio: i32,
    pub precision: i32,
    pub reserved: [i32; 7],
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct rc_voxel {
    pub emission: [u16; 3],
    pub albedo_occ: u16,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct rc_box {
    pub lo: [i32; 3],
    pub hi: [i32; 3],
    pub value: rc_voxel,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct rc_sphere {
    pub centre: [f64; 3],
    pub radius: f64,
    pub velocity: [f64; 3],
    pub value: rc_voxel,
    pub pad: [u32; 2],
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct rc_scene_spec {
    pub grid: [i32; 3],
    pub num_boxes: i32,
    pub box_edge_min: i32,
    pub box_edge_max: i32,
    pub num_spheres: i32,
    pub reserved: i32,
    pub albedo_min: f64,
    pub albedo_max: f64,
    pub radius_min: f64,
    pub radius_max: f64,
    pub emission_min: f64,
    pub emission_max: f64,
    pub speed: f64,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct rc_level_info {
    pub probes: [i32; 3],
    pub spacing: i32,
    pub dir_res: i32,
    pub num_dirs: i32,
    pub interval_lo: i32,
    pub interval_hi: i32,
    pub radiance_elems: i64,
    pub radiance_bytes: i64,
}

/// Opaque engine context (one scene, one GPU).
#[repr(C)]
pub struct rc_context {
    _p: [u8; 0],
}

/// Opaque batch of scenes solved in one persistent launch.
#[repr(C)]
pub struct rc_batch {
    _p: [u8; 0],
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct rc_batch_tiles {
    pub probes_per_item: i32,
    pub dirs_per_item: i32,
    pub blocks_per_item: i32,
    pub walks_per_item: i32,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct rc_shade_material {
    pub ambient: [f32; 4],
    pub diffuse: [f32; 4],
    pub specular: [f32; 4],
    pub shininess: f32,
    pub enable_bit: u32,
    pub color_texture: i32,
    pub normal_texture: i32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct rc_texture {
    pub rgba: *const u8,
    pub width: i32,
    pub height: i32,
    pub srgb: i32,
    pub pad: i32,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct rc_shade_view {
    pub view_proj: [f32; 16],
    pub eye: [f32; 3],
    pub light: [f32; 3],
    pub width: i32,
    pub height: i32,
    pub world_to_grid: [f32; 12],
    pub gi_scale: f32,
    pub pad: i32,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct rc_nrc_params {
    pub first_level: i32,
    pub hash_log2_entries: i32,
    pub base_resolution: i32,
    pub max_resolution: i32,
    pub learning_rate: f32,
    pub beta1: f32,
    pub beta2: f32,
    pub epsilon: f32,
    pub train_fraction_log2: i32,
    pub steps_per_solve: i32,
    pub fallback_threshold: f32,
    pub fallback_tile: i32,
    pub radiance_scale: f32,
    pub plain_level_fraction: f32,
    pub seed: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct rc_nrc_stats {
    pub solves: i64,
    pub steps: i64,
    pub last_loss: f32,
    pub served_levels: i32,
    pub fallback_tiles: i64,
    pub tiles: i64,
    pub served_solves: [i64; RC_MAX_CASCADES],
}

#[link(name = "rc")]
extern "C" {
    // errors
    pub fn rc_status_string(s: rc_status) -> *const c_char;
    pub fn rc_last_error() -> *const c_char;
    pub fn rc_abi_version() -> c_int;

    // host-only helpers
    pub fn rc_params_default(p: *mut rc_params, grid_edge: i32, num_cascades: i32) -> rc_status;
    pub fn rc_params_validate(p: *const rc_params) -> rc_status;
    pub fn rc_level_info_get(p: *const rc_params, level: i32, out: *mut rc_level_info) -> rc_status;
    pub fn rc_fluence_elems(p: *const rc_params) -> i64;
    pub fn rc_scene_generate(spec: *const rc_scene_spec, seed: u64, boxes: *mut rc_box,
                             spheres: *mut rc_sphere) -> rc_status;
    pub fn rc_spheres_advance(spheres: *mut rc_sphere, n: i32, grid: *const i32, frames: i32) -> rc_status;
    pub fn rc_voxelise_host(grid: *const i32, boxes: *const rc_box, nboxes: i32, spheres: *const rc_sphere,
                            nspheres: i32, out: *mut rc_voxel) -> rc_status;
    pub fn rc_directions(n: i32, out_xyz: *mut i32) -> rc_status;
    pub fn rc_solid_angles(n: i32, out: *mut f64) -> rc_status;

    // context
    pub fn rc_create(p: *const rc_params, device: i32, out: *mut *mut rc_context) -> rc_status;
    pub fn rc_destroy(ctx: *mut rc_context) -> rc_status;
    pub fn rc_get_params(ctx: *const rc_context, out: *mut rc_params) -> rc_status;
    pub fn rc_scene_upload(ctx: *mut rc_context, voxels: *const rc_voxel, count: i64, where_: i32) -> rc_status;
    pub fn rc_scene_set_boxes(ctx: *mut rc_context, boxes: *const rc_box, n: i32) -> rc_status;
    pub fn rc_scene_set_mesh(ctx: *mut rc_context, positions: *const f32, nverts: i64, indices: *const u32,
                             ntris: i64, tri_material: *const u16, materials: *const rc_voxel,
                             nmaterials: i32) -> rc_status;
    pub fn rc_scene_set_spheres(ctx: *mut rc_context, spheres: *const rc_sphere, n: i32) -> rc_status;
    pub fn rc_solve(ctx: *mut rc_context, stream: *mut c_void) -> rc_status;
    pub fn rc_synchronize(ctx: *mut rc_context) -> rc_status;
    pub fn rc_get_fluence(ctx: *mut rc_context, out: *mut f32, elems: i64, where_: i32) -> rc_status;
    pub fn rc_get_radiance(ctx: *mut rc_context, level: i32, out: *mut c_void, bytes: i64, where_: i32)
        -> rc_status;
    pub fn rc_fluence_device_ptr(ctx: *mut rc_context, out: *mut *const f32) -> rc_status;
    pub fn rc_get_volume(ctx: *mut rc_context, out: *mut rc_voxel, count: i64, where_: i32) -> rc_status;
    pub fn rc_get_fluence_async(ctx: *mut rc_context, out: *mut f32, elems: i64) -> rc_status;
    pub fn rc_radiance_device_ptr(ctx: *mut rc_context, level: i32, out: *mut *const c_void) -> rc_status;
    pub fn rc_get_stream(ctx: *mut rc_context, out: *mut *mut c_void) -> rc_status;

    // profiling
    pub fn rc_profile_levels(ctx: *mut rc_context, iters: i32, ms_out: *mut f32, count: i32) -> rc_status;
    pub fn rc_set_stage_timing(ctx: *mut rc_context, enable: i32) -> rc_status;
    pub fn rc_get_stage_ms(ctx: *mut rc_context, ms_out: *mut f32, count: i32) -> rc_status;
    pub fn rc_check_status(device: i32, first_failure: *mut u64, failures: *mut u32) -> rc_status;

    // batched form (many scenes, one persistent launch)
    pub fn rc_batch_create(params: *const rc_params, nscenes: i32, device: i32, out: *mut *mut rc_batch)
        -> rc_status;
    pub fn rc_batch_destroy(b: *mut rc_batch) -> rc_status;
    pub fn rc_batch_scene_set(b: *mut rc_batch, scene: i32, boxes: *const rc_box, nboxes: i32,
                              spheres: *const rc_sphere, nspheres: i32) -> rc_status;
    pub fn rc_batch_solve(b: *mut rc_batch, stream: *mut c_void) -> rc_status;
    pub fn rc_batch_synchronize(b: *mut rc_batch) -> rc_status;
    pub fn rc_batch_get_fluence(b: *mut rc_batch, scene: i32, out: *mut f32, elems: i64, where_: i32)
        -> rc_status;
    pub fn rc_batch_get_radiance(b: *mut rc_batch, scene: i32, level: i32, out: *mut c_void, bytes: i64,
                                 where_: i32) -> rc_status;
    pub fn rc_batch_set_spheres(b: *mut rc_batch, scene: i32, spheres: *const rc_sphere, n: i32) -> rc_status;
    pub fn rc_batch_get_fluence_all(b: *mut rc_batch, out: *mut f32, elems: i64, where_: i32) -> rc_status;
    pub fn rc_batch_get_fluence_all_async(b: *mut rc_batch, out: *mut f32, elems: i64) -> rc_status;
    pub fn rc_batch_set_tiles(b: *mut rc_batch, tiles: *const rc_batch_tiles) -> rc_status;
    pub fn rc_batch_get_tiles(b: *const rc_batch, out: *mut rc_batch_tiles) -> rc_status;
    pub fn rc_batch_get_form(b: *const rc_batch, scene_launches: *mut i32) -> rc_status;
    pub fn rc_batch_tune(b: *mut rc_batch, iters: i32, best: *mut rc_batch_tiles, best_ms: *mut f32)
        -> rc_status;

    // headless raster + Blinn-Phong shading
    pub fn rc_shade(ctx: *mut rc_context, view: *const rc_shade_view, vertices: *const f32, nverts: i64,
                    indices: *const u32, ntris: i64, tri_material: *const u16,
                    materials: *const rc_shade_material, nmaterials: i32, textures: *const rc_texture,
                    ntextures: i32, out: *mut f32, where_: i32) -> rc_status;
    pub fn rc_shade_set_mesh(ctx: *mut rc_context, vertices: *const f32, nverts: i64, indices: *const u32,
                             ntris: i64, tri_material: *const u16, materials: *const rc_shade_material,
                             nmaterials: i32, textures: *const rc_texture, ntextures: i32) -> rc_status;
    pub fn rc_shade_draw(ctx: *mut rc_context, view: *const rc_shade_view, out: *mut f32, where_: i32)
        -> rc_status;

    // learned form (neural radiance cache for the far cascades)
    pub fn rc_nrc_params_default(out: *mut rc_nrc_params) -> rc_status;
    pub fn rc_nrc_enable(ctx: *mut rc_context, params: *const rc_nrc_params) -> rc_status;
    pub fn rc_nrc_disable(ctx: *mut rc_context) -> rc_status;
    pub fn rc_nrc_save(ctx: *mut rc_context, out: *mut c_void, bytes: i64, needed: *mut i64) -> rc_status;
    pub fn rc_nrc_load(ctx: *mut rc_context, inp: *const c_void, bytes: i64) -> rc_status;
    pub fn rc_nrc_get_stats(ctx: *mut rc_context, out: *mut rc_nrc_stats) -> rc_status;
    pub fn rc_nrc_query(ctx: *mut rc_context, level: i32, probes: *const i32, dirs: *const i32, n: i64,
                        out: *mut f32) -> rc_status;
    pub fn rc_nrc_tile_gradient(ctx: *mut rc_context, level: i32, probe: i32, d0: i32, n: i32,
                                targets: *const f32, param_grad: *mut f32, pos_grad: *mut f32) -> rc_status;
    pub fn rc_nrc_param_count() -> i32;

    // allocation-free solve into caller-owned device buffers
    pub fn rc_solve_noalloc(p: *const rc_params, voxels: *const rc_voxel, fluence: *mut f32,
                            radiance: *mut c_void, stream: *mut c_void) -> rc_status;
}
