//! Raw bindings of `include/tinytrace_cuda.h`, the C ABI of `libtinytrace_cuda.so`.
//!
//! The library replaces the part of `tinytrace_backend::Context` that the tinytrace rendering
//! hot path uses (buffer and image creation, the BLAS/TLAS builds, the integrate and display
//! dispatches, downloads, timestamps).  Every declaration here mirrors the header one for one;
//! the header cites, beside each entry point, the reference call it replaces.  Structs have the
//! byte layout of the reference's `#[repr(C)]` types, so the arrays of `asset::Scene` and the
//! `Constants` of `Renderer::render_to_target` are passed unchanged; the tests at the end of
//! this file check sizes and field offsets against the values the header asserts.
#![allow(non_camel_case_types)]
#![cfg_attr(not(test), no_std)]

use core::ffi::{c_char, c_void};

pub const TT_ABI_VERSION: i32 = 1;

pub const TT_OK: i32 = 0;
pub const TT_ERR_INVALID_ARGUMENT: i32 = 1;
pub const TT_ERR_OOM: i32 = 2;
pub const TT_ERR_BAD_HANDLE: i32 = 3;
pub const TT_ERR_DEVICE: i32 = 4;
pub const TT_ERR_TIMEOUT: i32 = 5;
pub const TT_ERR_OVERFLOW: i32 = 6;
pub const TT_ERR_UNSUPPORTED: i32 = 7;
pub const TT_ERR_NO_DEVICE: i32 = 8;

pub const TT_LIFETIME_STATIC: u32 = 0;
pub const TT_LIFETIME_SURFACE: u32 = 1;
pub const TT_LIFETIME_SCENE: u32 = 2;
pub const TT_LIFETIME_FRAME: u32 = 3;
pub const TT_LIFETIME_RENDERER: u32 = 4;

pub const TT_LIGHT_SAMPLING_ON_HIT: u32 = 1;
pub const TT_LIGHT_SAMPLING_NEXT_EVENT_ESTIMATION: u32 = 2;

pub const TT_FORMAT_RGBA32F: u32 = 0;
pub const TT_FORMAT_RGBA8_UNORM: u32 = 1;

pub const TT_INTEGRATOR_WAVEFRONT: u64 = 0;
pub const TT_INTEGRATOR_MEGAKERNEL: u64 = 1;
pub const TT_OPTION_INTEGRATOR: u32 = 1;
pub const TT_OPTION_WAVEFRONT_SLOTS: u32 = 2;
pub const TT_OPTION_ACCEL: u32 = 3;
pub const TT_OPTION_STAGE_TIMING: u32 = 4;
pub const TT_OPTION_GRAPHS: u32 = 5;
pub const TT_OPTION_REFILL_LANES: u32 = 6;
pub const TT_OPTION_TRACE_BLOCKS_PER_SM: u32 = 7;
pub const TT_OPTION_RADIANCE_CACHE: u32 = 8;
pub const TT_OPTION_LIGHT_VISIBILITY: u32 = 9;
pub const TT_LIGHT_VISIBILITY_HASH: u64 = 0;
pub const TT_LIGHT_VISIBILITY_TRIANGLE: u64 = 1;
pub const TT_OPTION_LIGHT_SELECTION: u32 = 10;
pub const TT_LIGHT_SELECTION_UNIFORM: u64 = 0;
pub const TT_LIGHT_SELECTION_POWER: u64 = 1;
pub const TT_OPTION_PRIMARY_VISIBILITY: u32 = 11;
pub const TT_PRIMARY_TRAVERSE: u64 = 0;
pub const TT_PRIMARY_RASTER: u64 = 1;
pub const TT_ACCEL_AUTO: u64 = 0;
pub const TT_ACCEL_FLAT: u64 = 1;
pub const TT_ACCEL_TWO_LEVEL: u64 = 2;
pub const TT_ACCEL_FLAT_WIDE: u64 = 3;

pub const TT_SERVER_POLICY_FAIR: u32 = 0;
pub const TT_SERVER_POLICY_SMALLEST_FIRST: u32 = 1;
pub const TT_TRACE_CULL_BACK_FACES: u32 = 1;
pub const TT_TRACE_NOALLOC_MAX_RAYS: u32 = 65536;

pub const TT_TEXTURE_BC1_SRGB: u32 = 1;
pub const TT_TEXTURE_BC5_UNORM: u32 = 2;
pub const TT_TEXTURE_R8_UNORM: u32 = 3;
pub const TT_TEXTURE_R16_FLOAT: u32 = 4;
pub const TT_TEXTURE_MAX_LEVELS: u32 = 16;

pub const TT_STAGE_REGEN: usize = 0;
pub const TT_STAGE_EXTEND: usize = 1;
pub const TT_STAGE_SHADE: usize = 2;
pub const TT_STAGE_SHADOW: usize = 3;
pub const TT_STAGE_REDUCE: usize = 4;
pub const TT_STAGE_MEGAKERNEL: usize = 5;
pub const TT_STAGE_CACHE: usize = 6;
pub const TT_STAGE_CACHE_TRAIN: usize = 7;
pub const TT_STAGE_RESTIR_GBUFFER: usize = 8;
pub const TT_STAGE_RESTIR_INITIAL: usize = 9;
pub const TT_STAGE_RESTIR_TEMPORAL: usize = 10;
pub const TT_STAGE_RESTIR_SPATIAL: usize = 11;
pub const TT_STAGE_RESTIR_SHADE: usize = 12;
pub const TT_STAGE_PRIMARY: usize = 13;
pub const TT_STAGE_COUNT: usize = 16;

pub const TT_CACHE_WEIGHTS: u32 = 16896;
pub const TT_CACHE_GRID_FLOATS: u32 = 16777216;

pub const TT_REQUEST_QUEUED: i32 = 0;
pub const TT_REQUEST_RUNNING: i32 = 1;
pub const TT_REQUEST_DONE: i32 = 2;
pub const TT_REQUEST_FAILED: i32 = 3;

pub type tt_handle = u64;

#[repr(C)]
pub struct tt_context {
    _private: [u8; 0],
}

#[repr(C)]
pub struct tt_server {
    _private: [u8; 0],
}

/// `Constants` of src/lib.rs:234-250 (column-major matrices), 368 bytes.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct tt_constants {
    pub view: [f32; 16],
    pub proj: [f32; 16],
    pub proj_view: [f32; 16],
    pub inverse_view: [f32; 16],
    pub inverse_proj: [f32; 16],
    pub camera_position: [f32; 4],
    pub frame_index: u32,
    pub accumulated_frame_count: u32,
    pub sample_count: u32,
    pub bounce_count: u32,
    pub screen_size: [u32; 2],
    pub tonemap: u32,
    pub light_sampling: u32,
}

/// `MaterialConstants` of src/asset/material.rs:186-231, 192 bytes.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct tt_material_constants {
    pub base_color: [f32; 4],
    pub specular_color: [f32; 4],
    pub transmission_color: [f32; 4],
    pub coat_color: [f32; 4],
    pub fuzz_color: [f32; 4],
    pub emission_color: [f32; 4],
    pub geometry_normal: [f32; 4],
    pub base_weight: f32,
    pub base_metalness: f32,
    pub base_diffuse_roughness: f32,
    pub specular_weight: f32,
    pub specular_roughness: f32,
    pub specular_roughness_anisotropy: f32,
    pub specular_ior: f32,
    pub specular_rotation: f32,
    pub transmission_weight: f32,
    pub transmission_depth: f32,
    pub coat_weight: f32,
    pub coat_roughness: f32,
    pub coat_roughness_anisotropy: f32,
    pub coat_ior: f32,
    pub coat_darkening: f32,
    pub coat_rotation: f32,
    pub fuzz_weight: f32,
    pub fuzz_roughness: f32,
    pub emission_luminance: f32,
    pub geometry_opacity: f32,
}

/// `ProcessedMaterial` of src/asset/material.rs:268-274, 304 bytes (texture index u32::MAX: none).
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct tt_material {
    pub constants: tt_material_constants,
    pub textures: [u32; 27],
    pub padding: u32,
}

/// `ProcessedVertex` of src/asset/mod.rs:44-47: f16 texture coordinates + packed tangent frame.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct tt_vertex {
    pub texture_coordinates: [u16; 2],
    pub tangent_frame: u32,
}

/// `ProcessedMesh` of src/asset/mod.rs:49-64, 32 bytes.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct tt_mesh {
    pub bounding_sphere_center: [f32; 3],
    pub bounding_sphere_radius: f32,
    pub vertex_offset: u32,
    pub vertex_count: u32,
    pub index_offset: u32,
    pub index_count: u32,
}

/// `Instance` of src/scene.rs:236-246, 208 bytes.
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct tt_instance {
    pub transform: [f32; 16],
    pub inverse_transform: [f32; 16],
    pub normal_transform: [f32; 16],
    pub vertex_offset: u32,
    pub index_offset: u32,
    pub material_index: u32,
    pub mesh_index: u32,
}

/// `EmissiveTriangle` of src/asset/mod.rs:68-73, 36 bytes.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct tt_emissive_triangle {
    pub positions: [[i16; 3]; 3],
    pub hash: u16,
    pub texture_coordinates: [[u16; 2]; 3],
    pub instance_index: u32,
}

/// `ProcessedTexture` of src/asset/texture.rs:41-46: mip levels back to back in `data`.
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct tt_texture {
    pub format: u32,
    pub width: u32,
    pub height: u32,
    pub level_count: u32,
    pub data: *const u8,
    pub bytes: u64,
}

/// The arrays of `asset::Scene` (src/asset/mod.rs:77-86) plus the instances and emissive
/// triangles that `Scene::new` flattens from the node tree (src/scene.rs:29-64).
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct tt_scene_desc {
    pub positions: *const i16,
    pub position_count: u64,
    pub indices: *const u32,
    pub index_count: u64,
    pub vertices: *const tt_vertex,
    pub vertex_count: u64,
    pub materials: *const tt_material,
    pub material_count: u32,
    pub mesh_count: u32,
    pub meshes: *const tt_mesh,
    pub instances: *const tt_instance,
    pub instance_count: u32,
    pub emissive_triangle_count: u32,
    pub emissive_triangles: *const tt_emissive_triangle,
    pub textures: *const tt_texture,
    pub texture_count: u32,
    pub reserved: u32,
}

/// `Timings` of src/lib.rs:228-232, in nanoseconds of device time.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct tt_timings {
    pub integrate_ns: u64,
    pub post_process_ns: u64,
    pub scene_build_ns: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct tt_scene_stats {
    pub triangle_count: u64,
    pub instance_count: u64,
    pub emissive_count: u64,
    pub blas_nodes: u64,
    pub tlas_nodes: u64,
    pub blas_levels: u64,
    pub tlas_levels: u64,
    pub device_bytes: u64,
    pub max_stack: u64,
    pub accel: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct tt_stage_timings {
    pub ns: [u64; TT_STAGE_COUNT],
    pub launches: [u64; TT_STAGE_COUNT],
    pub overflow: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct tt_traversal_counters {
    pub rays: u64,
    pub blas_nodes: u64,
    pub tlas_nodes: u64,
    pub triangles: u64,
    pub instances: u64,
    pub hits: u64,
    pub warp_steps: u64,
    pub lane_steps: u64,
}

/// One mesh as `Scene::insert_mesh` receives it (src/asset/mod.rs:20-27), FP32 arrays.
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct tt_mesh_data {
    pub positions: *const f32,
    pub texture_coordinates: *const f32,
    pub indices: *const u32,
    pub normals: *const f32,
    pub tangents: *const f32,
    pub vertex_count: u32,
    pub index_count: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct tt_emissive_source {
    pub positions: *const i16,
    pub vertices: *const tt_vertex,
    pub vertex_count: u64,
    pub indices: *const u32,
    pub index_count: u64,
    pub meshes: *const tt_mesh,
    pub mesh_count: u32,
    pub model_count: u32,
    pub model_mesh: *const u32,
    pub model_instance: *const u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct tt_tune_result {
    pub slots: u32,
    pub refill_lanes: u32,
    pub trace_blocks_per_sm: u32,
    pub renders: u32,
    pub default_ms: f32,
    pub best_ms: f32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct tt_restir_config {
    pub candidates: u32,
    pub temporal_m_cap: f32,
    pub spatial_neighbours: u32,
    pub spatial_radius: f32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct tt_cache_config {
    pub learning_rate: f32,
    pub train_paths_per_frame: u32,
    pub terminate_depth: u32,
    pub seed: u32,
    pub spread_threshold: f32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct tt_cache_status {
    pub steps: u64,
    pub pairs: u64,
    pub last_loss: f32,
    pub pad: f32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct tt_server_config {
    pub hbm_budget_bytes: u64,
    pub max_inflight: u32,
    pub pool_paths: u32,
    pub round_items: u64,
    pub policy: u32,
    pub reserved: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct tt_server_stats {
    pub submitted: u64,
    pub completed: u64,
    pub failed: u64,
    pub queued: u64,
    pub inflight: u64,
    pub bytes_in_flight: u64,
    pub peak_bytes_in_flight: u64,
    pub peak_inflight: u64,
    pub rounds: u64,
    pub round_items: u64,
    pub gpu_busy_ns: u64,
    pub admit_ns: u64,
    pub launch_ns: u64,
    pub copy_out_ns: u64,
    pub wait_ns: u64,
}

#[link(name = "tinytrace_cuda")]
extern "C" {
    // context
    pub fn tt_abi_version() -> i32;
    pub fn tt_last_error() -> *const c_char;
    pub fn tt_context_create(device: i32, out: *mut *mut tt_context) -> i32;
    pub fn tt_context_destroy(ctx: *mut tt_context) -> i32;
    pub fn tt_frame_index(ctx: *mut tt_context, out: *mut u64) -> i32;
    pub fn tt_advance_frame(ctx: *mut tt_context) -> i32;
    pub fn tt_clear_lifetime(ctx: *mut tt_context, lifetime: u32) -> i32;
    pub fn tt_synchronize(ctx: *mut tt_context) -> i32;

    // images
    pub fn tt_image_create(ctx: *mut tt_context, lifetime: u32, width: u32, height: u32, out: *mut tt_handle) -> i32;
    pub fn tt_image_write(ctx: *mut tt_context, image: tt_handle, host: *const f32, bytes: u64) -> i32;
    pub fn tt_image_download(ctx: *mut tt_context, image: tt_handle, host: *mut f32, bytes: u64) -> i32;

    // scene
    pub fn tt_scene_create(ctx: *mut tt_context, desc: *const tt_scene_desc, out: *mut tt_handle) -> i32;
    pub fn tt_scene_stats_get(ctx: *mut tt_context, scene: tt_handle, out: *mut tt_scene_stats) -> i32;
    pub fn tt_scene_update_instances(ctx: *mut tt_context, scene: tt_handle, instances: *const tt_instance,
                                     count: u32) -> i32;
    pub fn tt_mesh_ingest(ctx: *mut tt_context, mesh: *const tt_mesh_data, vertex_offset: u32, index_offset: u32,
                          positions: *mut i16, vertices: *mut tt_vertex, mesh_out: *mut tt_mesh) -> i32;
    pub fn tt_emissive_extract(ctx: *mut tt_context, source: *const tt_emissive_source,
                               out: *mut tt_emissive_triangle, capacity: u64, count: *mut u64) -> i32;
    pub fn tt_scene_bvh_download(ctx: *mut tt_context, scene: tt_handle, blas: *mut c_void, blas_bytes: u64,
                                 tris: *mut c_void, tri_bytes: u64, tlas: *mut c_void, tlas_bytes: u64) -> i32;

    // rendering
    pub fn tt_render(ctx: *mut tt_context, scene: tt_handle, constants: *const tt_constants, target: tt_handle) -> i32;
    pub fn tt_render_counted(ctx: *mut tt_context, scene: tt_handle, constants: *const tt_constants,
                             target: tt_handle, out: *mut tt_traversal_counters) -> i32;
    pub fn tt_tonemap(ctx: *mut tt_context, image: tt_handle, constants: *const tt_constants, format: u32,
                      host_out: *mut c_void, bytes: u64) -> i32;
    pub fn tt_set_option(ctx: *mut tt_context, option: u32, value: u64) -> i32;
    pub fn tt_timings_get(ctx: *mut tt_context, out: *mut tt_timings) -> i32;
    pub fn tt_autotune(ctx: *mut tt_context, scene: tt_handle, constants: *const tt_constants, target: tt_handle,
                       out: *mut tt_tune_result) -> i32;
    pub fn tt_stage_timings_get(ctx: *mut tt_context, out: *mut tt_stage_timings) -> i32;

    // ReSTIR DI
    pub fn tt_restir_configure(ctx: *mut tt_context, config: *const tt_restir_config) -> i32;
    pub fn tt_restir_reset(ctx: *mut tt_context) -> i32;
    pub fn tt_render_restir(ctx: *mut tt_context, scene: tt_handle, constants: *const tt_constants,
                            target: tt_handle) -> i32;
    pub fn tt_restir_download(ctx: *mut tt_context, reservoirs: *mut c_void, bytes: u64) -> i32;

    // learned radiance cache
    pub fn tt_cache_configure(ctx: *mut tt_context, config: *const tt_cache_config) -> i32;
    pub fn tt_cache_query(ctx: *mut tt_context, queries: *const f32, n: u32, radiance: *mut f32) -> i32;
    pub fn tt_cache_train(ctx: *mut tt_context, queries: *const f32, targets: *const f32, n: u32,
                          loss: *mut f32) -> i32;
    pub fn tt_cache_parameters(ctx: *mut tt_context, grid: *mut f32, weights: *mut f32) -> i32;
    pub fn tt_cache_gradients(ctx: *mut tt_context, queries: *const f32, targets: *const f32, n: u32,
                              weight_gradients: *mut f32, grid_gradients: *mut f32, loss: *mut f32) -> i32;
    pub fn tt_cache_status_get(ctx: *mut tt_context, out: *mut tt_cache_status) -> i32;

    // serving
    pub fn tt_server_create(ctx: *mut tt_context, config: *const tt_server_config, out: *mut *mut tt_server) -> i32;
    pub fn tt_server_destroy(server: *mut tt_server) -> i32;
    pub fn tt_server_submit(server: *mut tt_server, scene: tt_handle, constants: *const tt_constants,
                            host_rgba32f: *mut f32, bytes: u64, request_id: *mut u64) -> i32;
    pub fn tt_server_status(server: *mut tt_server, request_id: u64, status: *mut i32, latency_ms: *mut f64) -> i32;
    pub fn tt_server_wait(server: *mut tt_server, request_id: u64, timeout_ms: u32, status: *mut i32) -> i32;
    pub fn tt_server_stats_get(server: *mut tt_server, out: *mut tt_server_stats) -> i32;

    // parity entry points
    pub fn tt_bsdf_eval_batch(ctx: *mut tt_context, material: *const tt_material_constants, samples: *const f32,
                              n: u32, results: *mut f32) -> i32;
    pub fn tt_bsdf_sample_batch(ctx: *mut tt_context, material: *const tt_material_constants, samples: *const f32,
                                n: u32, results: *mut f32) -> i32;
    pub fn tt_trace_batch(ctx: *mut tt_context, scene: tt_handle, rays: *const f32, n: u32, flags: u32,
                          hits: *mut u32) -> i32;
    pub fn tt_trace_batch_noalloc(ctx: *mut tt_context, scene: tt_handle, rays: *const f32, n: u32, flags: u32,
                                  hits: *mut u32) -> i32;
    pub fn tt_math_batch(ctx: *mut tt_context, which: i32, x: *const f32, n: u64, y: *mut f32) -> i32;

    // measurement helpers
    pub fn tt_texture_sample_batch(ctx: *mut tt_context, scene: tt_handle, texture: u32, uvl: *const f32, n: u32,
                                   rgba: *mut f32) -> i32;
    pub fn tt_flush_l2(ctx: *mut tt_context) -> i32;
    pub fn tt_event_record(ctx: *mut tt_context, slot: u32) -> i32;
    pub fn tt_event_elapsed_ms(ctx: *mut tt_context, start_slot: u32, end_slot: u32, ms: *mut f32) -> i32;
    pub fn tt_host_alloc(bytes: u64, out: *mut *mut c_void) -> i32;
    pub fn tt_host_free(ptr: *mut c_void) -> i32;
}

#[cfg(test)]
mod layout {
    use super::*;
    use core::mem::{offset_of, size_of};

    // The values include/tinytrace_cuda.h asserts with TT_LAYOUT_CHECK.
    #[test]
    fn reference_layouts() {
        assert_eq!(size_of::<tt_constants>(), 368);
        assert_eq!(offset_of!(tt_constants, camera_position), 320);
        assert_eq!(offset_of!(tt_constants, frame_index), 336);
        assert_eq!(offset_of!(tt_constants, screen_size), 352);
        assert_eq!(offset_of!(tt_constants, light_sampling), 364);
        assert_eq!(size_of::<tt_material_constants>(), 192);
        assert_eq!(offset_of!(tt_material_constants, base_weight), 112);
        assert_eq!(offset_of!(tt_material_constants, geometry_opacity), 188);
        assert_eq!(size_of::<tt_material>(), 304);
        assert_eq!(offset_of!(tt_material, padding), 300);
        assert_eq!(size_of::<tt_vertex>(), 8);
        assert_eq!(size_of::<tt_mesh>(), 32);
        assert_eq!(size_of::<tt_instance>(), 208);
        assert_eq!(offset_of!(tt_instance, vertex_offset), 192);
        assert_eq!(size_of::<tt_emissive_triangle>(), 36);
        assert_eq!(offset_of!(tt_emissive_triangle, hash), 18);
        assert_eq!(offset_of!(tt_emissive_triangle, instance_index), 32);
        assert_eq!(size_of::<tt_scene_stats>(), 80);
        assert_eq!(size_of::<tt_traversal_counters>(), 64);
    }
}
