/*
 * tinytrace_cuda.h — C ABI of libtinytrace_cuda.so, the GB300 (sm_103a) replacement for the
 * part of tinytrace_backend::Context that the tinytrace rendering hot path uses.
 *
 * The reference renderer (crate `tinytrace`) drives a Vulkan backend; the calls it makes on
 * the hot path are listed beside each entry point as "replaces: <file>:<line>" (paths are
 * relative to the reference project root).  The Rust `Renderer`, `Scene`, `Camera` and
 * `Config` keep their signatures; a thin FFI crate maps them onto these functions.
 *
 * Conventions
 *   - Every function returns a status (TT_OK == 0) except tt_last_error / tt_abi_version.
 *     The message of the last failure on the calling thread is returned by tt_last_error().
 *   - Host arrays are borrowed for the duration of the call only.
 *   - Device resources are owned by the context and named by opaque 64-bit handles
 *     {lifetime:8, epoch:24, index:32}; a handle whose lifetime was cleared since it was
 *     created is rejected with TT_ERR_BAD_HANDLE (the reference panics instead,
 *     crates/tinytrace_backend/src/lib.rs:231-233).
 *   - A context is used by one thread at a time and owns one CUDA stream.
 *   - All structs are plain C with the byte layout of the reference's #[repr(C)] types.
 */
#ifndef TINYTRACE_CUDA_H
#define TINYTRACE_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TT_ABI_VERSION 1

/* status codes */
#define TT_OK 0
#define TT_ERR_INVALID_ARGUMENT 1
#define TT_ERR_OOM 2
#define TT_ERR_BAD_HANDLE 3
#define TT_ERR_DEVICE 4
#define TT_ERR_TIMEOUT 5
#define TT_ERR_OVERFLOW 6
#define TT_ERR_UNSUPPORTED 7
#define TT_ERR_NO_DEVICE 8

/* resource lifetimes: crates/tinytrace_backend/src/lib.rs:61-73 */
#define TT_LIFETIME_STATIC 0
#define TT_LIFETIME_SURFACE 1
#define TT_LIFETIME_SCENE 2
#define TT_LIFETIME_FRAME 3
#define TT_LIFETIME_RENDERER 4

/* light sampling: src/config.rs:3-12, src/includes/constants.glsl:4-6 */
#define TT_LIGHT_SAMPLING_ON_HIT 1
#define TT_LIGHT_SAMPLING_NEXT_EVENT_ESTIMATION 2

/* tonemap output formats (the swapchain write of src/post_process/display.glsl:11 made headless) */
#define TT_FORMAT_RGBA32F 0
#define TT_FORMAT_RGBA8_UNORM 1

/* integrators (tt_set_option TT_OPTION_INTEGRATOR) */
#define TT_INTEGRATOR_WAVEFRONT 0
#define TT_INTEGRATOR_MEGAKERNEL 1
/* context options */
#define TT_OPTION_INTEGRATOR 1      /* TT_INTEGRATOR_*; default wavefront */
#define TT_OPTION_WAVEFRONT_SLOTS 2 /* paths in flight of the wavefront integrator; 0 = default */
#define TT_OPTION_ACCEL 3           /* TT_ACCEL_*: structure built by later tt_scene_create calls */
#define TT_OPTION_STAGE_TIMING 4    /* 1: CUDA events around every integrator launch (tt_stage_timings_get) */
#define TT_OPTION_GRAPHS 5          /* 1 (default): the wavefront loop runs on the device inside one CUDA graph per
                                       render; 0: the host drives it (also used while stage timing is on) */
#define TT_OPTION_REFILL_LANES 6    /* trace warps refill idle lanes below this many busy lanes (1..32; 20) */
#define TT_OPTION_TRACE_BLOCKS_PER_SM 7 /* resident blocks per SM of the trace kernel (0 = all that fit) */
#define TT_OPTION_RADIANCE_CACHE 8  /* 1: wavefront renders end paths in the learned radiance cache and
                                       train it after every frame (tt_cache_configure) */
#define TT_OPTION_LIGHT_VISIBILITY 9 /* TT_LIGHT_VISIBILITY_*: the shadow test of next-event estimation */
/* light visibility (tt_set_option TT_OPTION_LIGHT_VISIBILITY) */
#define TT_LIGHT_VISIBILITY_HASH 0     /* the reference's test (src/integrate/integrate.glsl:180-185): the
                                          hit instance is the light's and (prim + index_offset / 3) % 0xffff
                                          equals the light's 16-bit hash; lights at global triangle index
                                          >= 65535 never pass (parity, default) */
#define TT_LIGHT_VISIBILITY_TRIANGLE 1 /* the hit is the sampled emissive triangle itself (full 32-bit id) */
#define TT_OPTION_LIGHT_SELECTION 10   /* TT_LIGHT_SELECTION_*: how next-event estimation picks a light */
#define TT_LIGHT_SELECTION_UNIFORM 0   /* the reference's uniform pick, random_uint(count) (default) */
#define TT_LIGHT_SELECTION_POWER 1     /* proportional to emitted power (luminance x emission x world area)
                                          through an alias table built at scene creation (Vose's method in
                                          double precision); draws: random_uint(count), then one float for
                                          the alias coin; the density uses the light's own probability */
#define TT_OPTION_PRIMARY_VISIBILITY 11 /* TT_PRIMARY_*: how the wavefront integrator finds camera-ray hits */
#define TT_PRIMARY_TRAVERSE 0  /* camera rays traverse the BVH like every other ray */
#define TT_PRIMARY_RASTER 1    /* flat BVH4 scenes (TT_ACCEL_FLAT): before each sample chunk, every triangle is
                                  bounded on the screen and the chunk's samples in its rectangle are tested
                                  against it with the traversal's ray/triangle test; the smallest (t, instance,
                                  primitive) of each sample is the traversal's closest hit, bit for bit
                                  (default; the other structures traverse) */
/* acceleration structures (tt_set_option TT_OPTION_ACCEL; tt_scene_stats.accel) */
#define TT_ACCEL_AUTO 0      /* flat up to 2^26 instanced triangles, two-level above */
#define TT_ACCEL_FLAT 1      /* one BVH over the world boxes of all (instance, triangle) pairs */
#define TT_ACCEL_TWO_LEVEL 2 /* per-mesh BLAS under a TLAS over instances */
#define TT_ACCEL_FLAT_WIDE 3 /* the flat BVH in a compressed 8-wide format: 80-byte nodes with 8-bit child
                                boxes relative to a per-node origin and power-of-two scales, children in
                                slots by direction octant; rebuilt (not refitted) on instance updates */

/* trace flags */
#define TT_TRACE_CULL_BACK_FACES 1u

typedef struct tt_context tt_context;
typedef uint64_t tt_handle;

/* src/includes/constants.glsl:8-15 == src/lib.rs:234-250 (368 bytes, column-major mat4) */
typedef struct tt_constants {
    float view[16], proj[16], proj_view[16], inverse_view[16], inverse_proj[16];
    float camera_position[4];
    uint32_t frame_index, accumulated_frame_count, sample_count, bounce_count;
    uint32_t screen_size[2];
    uint32_t tonemap;
    uint32_t light_sampling;
} tt_constants;

/* src/material/material.glsl:10-38 == src/asset/material.rs:203-231 (192 bytes) */
typedef struct tt_material_constants {
    float base_color[4], specular_color[4], transmission_color[4], coat_color[4], fuzz_color[4],
        emission_color[4], geometry_normal[4];
    float base_weight, base_metalness, base_diffuse_roughness, specular_weight,
        specular_roughness, specular_roughness_anisotropy, specular_ior, specular_rotation,
        transmission_weight, transmission_depth, coat_weight, coat_roughness,
        coat_roughness_anisotropy, coat_ior, coat_darkening, coat_rotation, fuzz_weight,
        fuzz_roughness, emission_luminance, geometry_opacity;
} tt_material_constants;

/* src/asset/material.rs:268-274 ProcessedMaterial (304 bytes); texture index u32::MAX = none */
typedef struct tt_material {
    tt_material_constants constants;
    uint32_t textures[27];
    uint32_t padding;
} tt_material;

/* src/asset/mod.rs:44-47 ProcessedVertex (8 bytes): f16 uv[2] + packed tangent frame */
typedef struct tt_vertex {
    uint16_t texture_coordinates[2];
    uint32_t tangent_frame;
} tt_vertex;

/* src/asset/mod.rs:49-64 ProcessedMesh (32 bytes) */
typedef struct tt_mesh {
    float bounding_sphere_center[3];
    float bounding_sphere_radius;
    uint32_t vertex_offset, vertex_count, index_offset, index_count;
} tt_mesh;

/* src/scene.rs:236-246 Instance (208 bytes) */
typedef struct tt_instance {
    float transform[16], inverse_transform[16], normal_transform[16];
    uint32_t vertex_offset, index_offset, material_index, mesh_index;
} tt_instance;

/* src/asset/mod.rs:68-73 EmissiveTriangle (36 bytes) */
typedef struct tt_emissive_triangle {
    int16_t positions[3][3];
    uint16_t hash;
    uint16_t texture_coordinates[3][2];
    uint32_t instance_index;
} tt_emissive_triangle;

/* texture formats of ProcessedTexture (src/asset/texture.rs:62-118) */
#define TT_TEXTURE_BC1_SRGB 1  /* ImageFormat::RgbaBc1Srgb: 8-byte BC1 blocks, sRGB colour */
#define TT_TEXTURE_BC5_UNORM 2 /* ImageFormat::RgBc5Unorm: 16-byte blocks, two BC4 channels */
#define TT_TEXTURE_R8_UNORM 3  /* ImageFormat::R8Unorm */
#define TT_TEXTURE_R16_FLOAT 4 /* ImageFormat::R16Float */
#define TT_TEXTURE_MAX_LEVELS 16

/* src/asset/texture.rs:41-46 ProcessedTexture: `data` holds the mip levels back to back, level 0
 * first; level k has (width >> k) x (height >> k) texels, row-major (BC formats: 4 x 4 blocks,
 * row-major, partial blocks at the edges).  Sampled as the scene sampler of src/scene.rs:121-128
 * samples it (trilinear, repeat). */
typedef struct tt_texture {
    uint32_t format, width, height, level_count;
    const uint8_t* data;
    uint64_t bytes;
} tt_texture;

/* The arrays of asset::Scene (src/asset/mod.rs:77-86) plus the flattened instances and
 * emissive triangles that Scene::new derives from the node tree (src/scene.rs:29-64).
 * Materials name textures by their index in `textures` (u32::MAX: none). */
typedef struct tt_scene_desc {
    const int16_t* positions; /* position_count x [i16; 3], snorm16 */
    uint64_t position_count;
    const uint32_t* indices;
    uint64_t index_count;
    const tt_vertex* vertices;
    uint64_t vertex_count;
    const tt_material* materials;
    uint32_t material_count;
    uint32_t mesh_count;
    const tt_mesh* meshes;
    const tt_instance* instances;
    uint32_t instance_count;
    uint32_t emissive_triangle_count;
    const tt_emissive_triangle* emissive_triangles;
    const tt_texture* textures;
    uint32_t texture_count;
    uint32_t reserved;
} tt_scene_desc;

/* Compile-time checks of the byte layouts the ABI shares with the reference's #[repr(C)] types
 * (every C or C++ translation unit that includes this header checks them): sizes and field
 * offsets of Constants (src/lib.rs:234-250), MaterialConstants and ProcessedMaterial
 * (src/asset/material.rs:186-231, 268-274), ProcessedVertex, ProcessedMesh and
 * EmissiveTriangle (src/asset/mod.rs:44-73) and Instance (src/scene.rs:236-246). */
#ifdef __cplusplus
#define TT_LAYOUT_CHECK(cond, what) static_assert(cond, what)
#else
#define TT_LAYOUT_CHECK(cond, what) _Static_assert(cond, what)
#endif
TT_LAYOUT_CHECK(sizeof(tt_constants) == 368, "Constants is 368 bytes");
TT_LAYOUT_CHECK(offsetof(tt_constants, inverse_proj) == 256, "Constants.inverse_proj at 256");
TT_LAYOUT_CHECK(offsetof(tt_constants, camera_position) == 320, "Constants.camera_position at 320");
TT_LAYOUT_CHECK(offsetof(tt_constants, frame_index) == 336, "Constants.frame_index at 336");
TT_LAYOUT_CHECK(offsetof(tt_constants, sample_count) == 344, "Constants.sample_count at 344");
TT_LAYOUT_CHECK(offsetof(tt_constants, screen_size) == 352, "Constants.screen_size at 352");
TT_LAYOUT_CHECK(offsetof(tt_constants, tonemap) == 360, "Constants.tonemap at 360");
TT_LAYOUT_CHECK(offsetof(tt_constants, light_sampling) == 364, "Constants.light_sampling at 364");
TT_LAYOUT_CHECK(sizeof(tt_material_constants) == 192, "MaterialConstants is 192 bytes");
TT_LAYOUT_CHECK(offsetof(tt_material_constants, geometry_normal) == 96, "geometry_normal at 96");
TT_LAYOUT_CHECK(offsetof(tt_material_constants, base_weight) == 112, "base_weight at 112");
TT_LAYOUT_CHECK(offsetof(tt_material_constants, specular_roughness) == 128, "specular_roughness at 128");
TT_LAYOUT_CHECK(offsetof(tt_material_constants, coat_weight) == 152, "coat_weight at 152");
TT_LAYOUT_CHECK(offsetof(tt_material_constants, emission_luminance) == 184, "emission_luminance at 184");
TT_LAYOUT_CHECK(offsetof(tt_material_constants, geometry_opacity) == 188, "geometry_opacity at 188");
TT_LAYOUT_CHECK(sizeof(tt_material) == 304, "ProcessedMaterial is 304 bytes");
TT_LAYOUT_CHECK(offsetof(tt_material, textures) == 192, "ProcessedMaterial.textures at 192");
TT_LAYOUT_CHECK(offsetof(tt_material, padding) == 300, "ProcessedMaterial.padding at 300");
TT_LAYOUT_CHECK(sizeof(tt_vertex) == 8, "ProcessedVertex is 8 bytes");
TT_LAYOUT_CHECK(offsetof(tt_vertex, tangent_frame) == 4, "ProcessedVertex.tangent_frame at 4");
TT_LAYOUT_CHECK(sizeof(tt_mesh) == 32, "ProcessedMesh is 32 bytes");
TT_LAYOUT_CHECK(offsetof(tt_mesh, vertex_offset) == 16, "ProcessedMesh.vertex_offset at 16");
TT_LAYOUT_CHECK(offsetof(tt_mesh, index_count) == 28, "ProcessedMesh.index_count at 28");
TT_LAYOUT_CHECK(sizeof(tt_instance) == 208, "Instance is 208 bytes");
TT_LAYOUT_CHECK(offsetof(tt_instance, normal_transform) == 128, "Instance.normal_transform at 128");
TT_LAYOUT_CHECK(offsetof(tt_instance, vertex_offset) == 192, "Instance.vertex_offset at 192");
TT_LAYOUT_CHECK(offsetof(tt_instance, mesh_index) == 204, "Instance.mesh_index at 204");
TT_LAYOUT_CHECK(sizeof(tt_emissive_triangle) == 36, "EmissiveTriangle is 36 bytes");
TT_LAYOUT_CHECK(offsetof(tt_emissive_triangle, hash) == 18, "EmissiveTriangle.hash at 18");
TT_LAYOUT_CHECK(offsetof(tt_emissive_triangle, texture_coordinates) == 20, "EmissiveTriangle.uv at 20");
TT_LAYOUT_CHECK(offsetof(tt_emissive_triangle, instance_index) == 32, "EmissiveTriangle.instance_index at 32");

/* src/lib.rs:228-232 Timings, in nanoseconds of device time */
typedef struct tt_timings {
    uint64_t integrate_ns;
    uint64_t post_process_ns;
    uint64_t scene_build_ns;
} tt_timings;

/* Scene statistics.  triangle_count counts the triangle records of the structure: the mesh
 * triangles (two-level) or the instanced triangles (flat).  For a flat scene the tlas fields
 * describe the flat BVH and the blas fields are zero. */
typedef struct tt_scene_stats {
    uint64_t triangle_count, instance_count, emissive_count;
    uint64_t blas_nodes, tlas_nodes, blas_levels, tlas_levels;
    uint64_t device_bytes;
    uint64_t max_stack;
    uint64_t accel; /* TT_ACCEL_FLAT or TT_ACCEL_TWO_LEVEL */
} tt_scene_stats;

/* Device time per integrator stage of the last render (tt_render or tt_render_restir), summed
 * over its launches (with TT_OPTION_STAGE_TIMING on).  Extends the integrate/post-process timestamps of
 * src/lib.rs:149-193 (backend timing.rs:62-68) to the wavefront stages. */
#define TT_STAGE_REGEN 0
#define TT_STAGE_EXTEND 1  /* closest-hit trace of extension rays */
#define TT_STAGE_SHADE 2
#define TT_STAGE_SHADOW 3  /* closest-hit trace of shadow rays */
#define TT_STAGE_REDUCE 4
#define TT_STAGE_MEGAKERNEL 5
#define TT_STAGE_CACHE 6   /* radiance-cache queries of paths ending in the cache */
#define TT_STAGE_CACHE_TRAIN 7      /* radiance-cache training after a cached frame (pairs + Adam steps) */
#define TT_STAGE_RESTIR_GBUFFER 8   /* ReSTIR DI passes of tt_render_restir */
#define TT_STAGE_RESTIR_INITIAL 9
#define TT_STAGE_RESTIR_TEMPORAL 10
#define TT_STAGE_RESTIR_SPATIAL 11
#define TT_STAGE_RESTIR_SHADE 12
#define TT_STAGE_PRIMARY 13         /* rasterised primary visibility (TT_PRIMARY_RASTER): bounds and keys */
#define TT_STAGE_COUNT 16
typedef struct tt_stage_timings {
    uint64_t ns[TT_STAGE_COUNT];
    uint64_t launches[TT_STAGE_COUNT];
    uint64_t overflow; /* 1: more launches than the 4096 recorded per render */
} tt_stage_timings;

/* Traversal counters from the instrumented render (roofline accounting). */
typedef struct tt_traversal_counters {
    uint64_t rays, blas_nodes, tlas_nodes, triangles, instances, hits;
    uint64_t warp_steps, lane_steps; /* wavefront traversal: warp steps and the active lanes summed over them */
} tt_traversal_counters;

/* ---------------------------------------------------------------- context */
int32_t tt_abi_version(void);
const char* tt_last_error(void);
/* replaces: crates/tinytrace_backend/src/lib.rs:171-213 Context::new(None) */
int32_t tt_context_create(int32_t device, tt_context** out);
int32_t tt_context_destroy(tt_context* ctx);
/* replaces: crates/tinytrace_backend/src/lib.rs:268-270 Context::frame_index */
int32_t tt_frame_index(tt_context* ctx, uint64_t* out);
/* replaces the frame advance of crates/tinytrace_backend/src/lib.rs:393-410 Context::present
 * (headless: there is no swapchain to present) */
int32_t tt_advance_frame(tt_context* ctx);
/* replaces: crates/tinytrace_backend/src/lib.rs:253-255 clear_resources_with_lifetime */
int32_t tt_clear_lifetime(tt_context* ctx, uint32_t lifetime);
/* replaces: crates/tinytrace_backend/src/lib.rs:293-300 wait_until_idle */
int32_t tt_synchronize(tt_context* ctx);

/* ---------------------------------------------------------------- images */
/* replaces: src/lib.rs:213-226 create_render_target (create_image, Rgba32Float) */
int32_t tt_image_create(tt_context* ctx, uint32_t lifetime, uint32_t width, uint32_t height,
                        tt_handle* out);
/* replaces: crates/tinytrace_backend/src/copy.rs:102-163 write_images (RGBA32F, tightly packed) */
int32_t tt_image_write(tt_context* ctx, tt_handle image, const float* host, uint64_t bytes);
/* replaces: crates/tinytrace_backend/src/copy.rs:183-264 download (RGBA32F, tightly packed) */
int32_t tt_image_download(tt_context* ctx, tt_handle image, float* host, uint64_t bytes);

/* ---------------------------------------------------------------- scene */
/* replaces: src/scene.rs:28-186 Scene::new — buffer creation and upload
 * (crates/tinytrace_backend/src/copy.rs:62-100) and the BLAS/TLAS builds
 * (crates/tinytrace_backend/src/resource.rs:728-880, 891-1085), which become a GPU LBVH. */
int32_t tt_scene_create(tt_context* ctx, const tt_scene_desc* desc, tt_handle* out);
int32_t tt_scene_stats_get(tt_context* ctx, tt_handle scene, tt_scene_stats* out);
/* Moves instances (the TLAS update of the reference: TlasBuildMode::Update,
 * crates/tinytrace_backend/src/resource.rs:993-1003): new transforms, inverse and normal
 * transforms for all `count` instances of the scene (mesh, material and offsets unchanged).
 * The world-space structure (flat BVH or TLAS) keeps its topology and refits its boxes, so
 * closest hits stay exact; traversal slows as instances move far from where it was built. */
int32_t tt_scene_update_instances(tt_context* ctx, tt_handle scene, const tt_instance* instances, uint32_t count);
/* ---------------------------------------------------------------- mesh ingest */
/* One mesh as Scene::insert_mesh receives it (src/asset/mod.rs:20-27 Mesh), FP32 host arrays.
 * texture_coordinates (vertex_count x 2), indices (index_count), normals (vertex_count x 3)
 * and tangents (vertex_count x 4) may be NULL: zeros, 0..vertex_count-1, normals generated
 * from the triangles (src/asset/mod.rs:226-242), tangents generated. */
typedef struct tt_mesh_data {
    const float* positions;
    const float* texture_coordinates;
    const uint32_t* indices;
    const float* normals;
    const float* tangents;
    uint32_t vertex_count, index_count;
} tt_mesh_data;

/* replaces: src/asset/mod.rs:89-161 Scene::insert_mesh (host loop) with the per-vertex work on
 * the device: writes vertex_count snorm16 positions (x, y, z) relative to the bounding sphere
 * (src/asset/mod.rs:308-321) to `positions`, vertex_count packed vertices (f16 texture
 * coordinates, TangentFrame of src/asset/normal.rs:17-36) to `vertices`, and the mesh record
 * with the given offsets to `mesh`.  Generated tangents are cross(up, n) / |.| with w = +1
 * (up = +y unless |n.y| >= 0.999, then +x) in place of the reference's mikktspace tangents.
 * TT_ERR_INVALID_ARGUMENT for an index >= vertex_count or a degenerate or non-finite bounding
 * sphere (the reference panics on both). */
int32_t tt_mesh_ingest(tt_context* ctx, const tt_mesh_data* mesh, uint32_t vertex_offset, uint32_t index_offset,
                       int16_t* positions, tt_vertex* vertices, tt_mesh* mesh_out);

/* The scene arrays and the (mesh, instance) pairs of the emissive models, in scene order. */
typedef struct tt_emissive_source {
    const int16_t* positions; /* vertex_count x 3 (all meshes) */
    const tt_vertex* vertices;
    uint64_t vertex_count;
    const uint32_t* indices;
    uint64_t index_count;
    const tt_mesh* meshes;
    uint32_t mesh_count;
    uint32_t model_count;
    const uint32_t* model_mesh;     /* model_count mesh indices */
    const uint32_t* model_instance; /* model_count instance indices */
} tt_emissive_source;

/* replaces: src/asset/mod.rs:163-193 Scene::emissive_triangles_in_model over every emissive
 * model (src/scene.rs:29-64 collects them): the triangles of the models in order, each with
 * its quantised positions, texture coordinates, hash (index_offset / 3 + offset % 65535) as
 * u16 and instance index.  `capacity` triangles fit in `out`; `*count` receives the number
 * written.  TT_ERR_INVALID_ARGUMENT for a mesh, index or vertex out of range,
 * TT_ERR_OVERFLOW when `capacity` is too small. */
int32_t tt_emissive_extract(tt_context* ctx, const tt_emissive_source* source, tt_emissive_triangle* out,
                            uint64_t capacity, uint64_t* count);

/* BVH arrays for node-for-node comparison: blas nodes (128 B each), triangle records
 * (48 B each), tlas nodes (128 B each; the flat BVH of a flat scene, 80 B each in the
 * compressed wide format).  Sizes in bytes must match tt_scene_stats. */
int32_t tt_scene_bvh_download(tt_context* ctx, tt_handle scene, void* blas, uint64_t blas_bytes,
                              void* tris, uint64_t tri_bytes, void* tlas, uint64_t tlas_bytes);

/* ---------------------------------------------------------------- rendering */
/* replaces: src/integrate/mod.rs:39-61 Integrator::integrate (dispatch of integrate.glsl)
 * with the timestamps of src/lib.rs:149,157 */
int32_t tt_render(tt_context* ctx, tt_handle scene, const tt_constants* constants,
                  tt_handle target);
/* Same render with traversal counters (an instrumented kernel; slower). */
int32_t tt_render_counted(tt_context* ctx, tt_handle scene, const tt_constants* constants,
                          tt_handle target, tt_traversal_counters* out);
/* replaces: src/post_process/mod.rs:42-57 PostProcess::run (display.glsl) writing a host
 * buffer instead of a swapchain image; format TT_FORMAT_*. */
int32_t tt_tonemap(tt_context* ctx, tt_handle image, const tt_constants* constants,
                   uint32_t format, void* host_out, uint64_t bytes);
/* Integrator choice and tuning (no counterpart in the reference: it has one megakernel).
 * Both integrators produce bit-identical images. */
int32_t tt_set_option(tt_context* ctx, uint32_t option, uint64_t value);
/* replaces: src/lib.rs:167-178 Renderer::timings */
int32_t tt_timings_get(tt_context* ctx, tt_timings* out);
/* Autotuner (no reference counterpart: the reference's ray-query pipeline has no tunables).
 * Times renders of `constants` (give it a few samples per pixel) into `target` while it
 * varies, one after the other, the wavefront pool size, the trace kernel's refill threshold
 * and its resident blocks per SM, keeps the fastest of each, and leaves those options set on
 * the context.  The last render's image stays in `target`. */
typedef struct tt_tune_result {
    uint32_t slots, refill_lanes, trace_blocks_per_sm, renders;
    float default_ms, best_ms;
} tt_tune_result;
int32_t tt_autotune(tt_context* ctx, tt_handle scene, const tt_constants* constants, tt_handle target,
                    tt_tune_result* out);
/* ---------------------------------------------------------------- ReSTIR DI
 * Direct lighting at the primary hit by spatiotemporal reservoir resampling over the emissive
 * triangles (Bitterli et al. 2020): an addition with no reference counterpart (the reference
 * samples one light per vertex, src/includes/scene.glsl:114-136).  One sample per pixel per
 * frame; the context keeps the previous frame's G-buffer, reservoirs and camera for temporal
 * reuse; the frame accumulation rule of tt_render applies to the target. */
typedef struct tt_restir_config {
    uint32_t candidates;         /* initial light candidates per pixel (32) */
    float temporal_m_cap;        /* previous-frame M capped at this many times `candidates` (20) */
    uint32_t spatial_neighbours; /* neighbours merged per pixel (5) */
    float spatial_radius;        /* neighbour disk radius in pixels (30) */
} tt_restir_config;
int32_t tt_restir_configure(tt_context* ctx, const tt_restir_config* config);
/* Forgets the previous frame (the next frame does no temporal reuse). */
int32_t tt_restir_reset(tt_context* ctx);
/* Candidates follow TT_OPTION_LIGHT_SELECTION (uniform, or by emitted power).  Textured
 * materials are sampled at the primary hit with its ray-differential mip level and
 * at light points with mip level 4, as the path tracer samples them. */
int32_t tt_render_restir(tt_context* ctx, tt_handle scene, const tt_constants* constants, tt_handle target);
/* Final reservoirs of the last ReSTIR frame, width * height * 32 bytes (row-major pixels:
 * light index u32, r1, r2, w_sum, M, W, 0, 0). */
int32_t tt_restir_download(tt_context* ctx, void* reservoirs, uint64_t bytes);

/* ---------------------------------------------------------------- learned radiance cache
 * An addition without reference counterpart: a hash-grid-encoded MLP predicting outgoing
 * radiance from (position in the scene's unit cube, outgoing direction, shading normal,
 * roughness), trained online on radiance the path tracer produces (Mueller et al. 2021/2022).
 * Grid: 16 levels x 2^19 entries x 2 features; MLP: 64 inputs, 4 hidden layers of 64 ReLU
 * units, 3 outputs; queries are 12 floats: pos xyz, dir xyz, normal xyz, roughness, 0, 0. */
#define TT_CACHE_WEIGHTS 16896u          /* 4 x 64 x 64 hidden weights + 8 x 64 output rows (3 used) */
#define TT_CACHE_GRID_FLOATS 16777216u   /* 16 levels x 2^19 entries x 2 features */
/* Defaults of a context that was never configured: {1e-2, 65536, 1, 1, 0.01}. */
typedef struct tt_cache_config {
    float learning_rate;            /* Adam step size */
    uint32_t train_paths_per_frame; /* paths traced to full depth to produce training radiance */
    uint32_t terminate_depth;       /* other paths end in the cache at this vertex, or, with a spread
                                       threshold, at the first vertex from this depth on whose path
                                       spread exceeds it */
    uint32_t seed;                  /* parameter initialisation */
    float spread_threshold;         /* 0: end at terminate_depth; c > 0: the path-spread rule of neural
                                       radiance caching (Mueller et al. 2021): end where
                                       sum_i sqrt(d_i^2 / (p_i |cos_i|)) > c * sqrt(d_1^2 / (4 pi |cos_1|)) */
} tt_cache_config;
/* (Re)initialises the cache with `config`; tt_set_option(TT_OPTION_RADIANCE_CACHE, 1) makes
 * tt_render use it. */
int32_t tt_cache_configure(tt_context* ctx, const tt_cache_config* config);
int32_t tt_cache_query(tt_context* ctx, const float* queries, uint32_t n, float* radiance);
/* One Adam step on the mean relative L2 loss of n (query, target radiance) pairs; returns the
 * summed loss before the step. */
int32_t tt_cache_train(tt_context* ctx, const float* queries, const float* targets, uint32_t n, float* loss);
/* The gradients one tt_cache_train step would apply, without applying them (parameters and Adam
 * state unchanged): weight_gradients (TT_CACHE_WEIGHTS floats) and grid_gradients
 * (TT_CACHE_GRID_FLOATS floats, may be null) of the mean relative L2 loss of the n pairs, and
 * the summed loss.  For checking the tensor-core backward pass against a reference. */
int32_t tt_cache_gradients(tt_context* ctx, const float* queries, const float* targets, uint32_t n,
                           float* weight_gradients, float* grid_gradients, float* loss);
/* FP32 parameters: grid (TT_CACHE_GRID_FLOATS, may be null) and weights (TT_CACHE_WEIGHTS). */
int32_t tt_cache_parameters(tt_context* ctx, float* grid, float* weights);
typedef struct tt_cache_status {
    uint64_t steps;      /* Adam steps taken */
    uint64_t pairs;      /* training pairs built from the last cached frame */
    float last_loss;     /* mean relative L2 loss of the last step */
    float pad;
} tt_cache_status;
int32_t tt_cache_status_get(tt_context* ctx, tt_cache_status* out);

/* ---------------------------------------------------------------- serving
 * Continuous-batching render server (no reference counterpart: the reference renders one frame
 * at a time on the caller's thread).  Scenes are created on the server's context beforehand and
 * stay resident; while a server lives, the caller neither clears the scene lifetime nor uses the
 * context from another thread.  Submitted requests (scene + constants) queue in arrival order.
 * A scheduler thread renders the admitted requests together in rounds: each round takes the
 * next sample chunk of every admitted request (round_items work items in total, shared evenly)
 * and traces them through one shared wavefront path pool and one set of persistent kernels
 * (one CUDA graph launch per round).  Between rounds it retires finished requests, copying their
 * images into the callers' buffers while the next round renders, and admits queued requests
 * (in arrival order, or smallest first: TT_SERVER_POLICY_*) while the batch has room and the
 * request's device memory fits in the HBM budget next to the requests already admitted.  A
 * request's image is the same, bit for bit, alone or among others. */
typedef struct tt_server tt_server;
typedef struct tt_server_config {
    uint64_t hbm_budget_bytes; /* device memory admitted requests may hold (0 = 150 GB); the
                                  shared pool (236 bytes per path slot) is allocated once, apart */
    uint32_t max_inflight;     /* requests rendered together (0 = 16, at most 64) */
    uint32_t pool_paths;       /* path slots of the shared wavefront pool (0 = 2^21, at most 2^24) */
    uint64_t round_items;      /* (pixel, sample) work items per round across the batch (0 = 2^26) */
    uint32_t policy;           /* TT_SERVER_POLICY_* */
    uint32_t reserved;         /* 0 */
} tt_server_config;
/* FAIR: queued requests are admitted in arrival order and every request of the batch gets an
 * equal share of each round's work items.  SMALLEST_FIRST: the queued request with the fewest
 * samples is admitted first; each round serves the oldest admitted request with up to a quarter
 * of its work items (so that large requests keep progressing) and then the requests with the
 * least remaining work (full chunks until the round's work items are spent; the rest wait). */
#define TT_SERVER_POLICY_FAIR 0u
#define TT_SERVER_POLICY_SMALLEST_FIRST 1u
typedef struct tt_server_stats {
    uint64_t submitted, completed, failed, queued, inflight;
    uint64_t bytes_in_flight, peak_bytes_in_flight, peak_inflight;
    /* rounds rendered, their work items, their device time (CUDA events around each round), and
     * the scheduler thread's time admitting, launching, copying images out and waiting for rounds */
    uint64_t rounds, round_items, gpu_busy_ns, admit_ns, launch_ns, copy_out_ns, wait_ns;
} tt_server_stats;
#define TT_REQUEST_QUEUED 0
#define TT_REQUEST_RUNNING 1
#define TT_REQUEST_DONE 2
#define TT_REQUEST_FAILED 3
int32_t tt_server_create(tt_context* ctx, const tt_server_config* config, tt_server** out);
/* Finishes the queued and in-flight requests, then stops the scheduler. */
int32_t tt_server_destroy(tt_server* server);
/* host_rgba32f: width * height * 16 bytes, written when the request completes; it must stay
 * valid until then.  constants.sample_count and bounce_count must be at least 1, bounce_count
 * below 65536, and the image at most 4096 x 4096 pixels. */
int32_t tt_server_submit(tt_server* server, tt_handle scene, const tt_constants* constants, float* host_rgba32f,
                         uint64_t bytes, uint64_t* request_id);
/* Status (TT_REQUEST_*) and, once done, submit-to-completion latency in milliseconds. */
int32_t tt_server_status(tt_server* server, uint64_t request_id, int32_t* status, double* latency_ms);
/* Blocks until the request is done or failed, or timeout_ms passes (then TT_ERR_TIMEOUT). */
int32_t tt_server_wait(tt_server* server, uint64_t request_id, uint32_t timeout_ms, int32_t* status);
int32_t tt_server_stats_get(tt_server* server, tt_server_stats* out);

/* Per-stage device time of the last render (synchronises the context's stream). */
int32_t tt_stage_timings_get(tt_context* ctx, tt_stage_timings* out);

/* ---------------------------------------------------------------- parity entry points */
/* replaces: src/material/test.rs:112-151 BdsfSampler::sample.  samples: n x 8 floats
 * (wi xyz, generator state bits, wo xyz, 0); results: n x 8 floats (bsdf rgb, pdf,
 * generator state after bsdf_prepare, probability of the diffuse, metal, specular lobes). */
int32_t tt_bsdf_eval_batch(tt_context* ctx, const tt_material_constants* material,
                           const float* samples, uint32_t n, float* results);
/* bsdf_prepare + bsdf_sample (src/material/bsdf.glsl:115-120,163-203).  samples: n x 4
 * (wi xyz, state bits); results: n x 12 (bsdf rgb, pdf, wo xyz, lobe, state bits, 0, 0, 0). */
int32_t tt_bsdf_sample_batch(tt_context* ctx, const tt_material_constants* material,
                             const float* samples, uint32_t n, float* results);
/* Closest-hit ray queries (src/integrate/integrate.glsl:112-127, 168-185).  rays: n x 8
 * floats (origin xyz, tmin, direction xyz, tmax); hits: n x 8 words (hit, t, u, v bits,
 * instance, primitive, 0, 0).  flags: TT_TRACE_*. */
int32_t tt_trace_batch(tt_context* ctx, tt_handle scene, const float* rays, uint32_t n,
                       uint32_t flags, uint32_t* hits);
/* Allocation-free variant of tt_trace_batch; it has no counterpart in the reference.
 * It is for callers that cannot allocate device memory when they issue ray queries: an
 * application that owns the whole device-memory budget through its own pool, or a real-time
 * frame loop in which an allocation's implicit device synchronisation would stall the frame.
 * Rays, hits and the traversal error word are staged in one static device array of the
 * library, sized for TT_TRACE_NOALLOC_MAX_RAYS rays (4 MiB + 256 bytes, held by every GPU
 * that loads the library until the process exits).  Arguments and results are those of
 * tt_trace_batch; n above TT_TRACE_NOALLOC_MAX_RAYS is rejected with TT_ERR_INVALID_ARGUMENT
 * before any GPU work.  The first call on a device looks the array's device address up
 * (cudaGetSymbolAddress) with that device current; make that first call before any stream
 * capture.  The address is kept until the process exits: after a device reset
 * (cudaDeviceReset) the entry point must not be called on that device again.  Every call
 * shares the array and leaves its contents behind (the error word is cleared at the start of
 * each call); calls whose GPU work overlaps (two contexts of one device) race on it.  The call
 * synchronises the context stream before it returns, and reports an error word left pending
 * by an earlier asynchronous call on the context as tt_trace_batch does. */
#define TT_TRACE_NOALLOC_MAX_RAYS 65536u
int32_t tt_trace_batch_noalloc(tt_context* ctx, tt_handle scene, const float* rays, uint32_t n,
                               uint32_t flags, uint32_t* hits);
/* Device elementary functions (0 sin, 1 cos, 2 exp, 3 log, 4 acos) for accuracy tests. */
int32_t tt_math_batch(tt_context* ctx, int32_t which, const float* x, uint64_t n, float* y);

/* ---------------------------------------------------------------- measurement helpers */
/* textureLod of texture `texture` of a scene at n (u, v, lod) float triples -> n RGBA floats
 * (the sampling the shading kernels perform; for parity tests of the decoders and filter). */
int32_t tt_texture_sample_batch(tt_context* ctx, tt_handle scene, uint32_t texture, const float* uvl, uint32_t n,
                                float* rgba);
/* Write a buffer larger than L2 on the context stream. */
int32_t tt_flush_l2(tt_context* ctx);
/* Record event `slot` (0..15) on the context stream / elapsed ms between two slots. */
int32_t tt_event_record(tt_context* ctx, uint32_t slot);
int32_t tt_event_elapsed_ms(tt_context* ctx, uint32_t start_slot, uint32_t end_slot, float* ms);
/* Pinned host memory for end-to-end copies (cudaMallocHost / cudaFreeHost). */
int32_t tt_host_alloc(uint64_t bytes, void** out);
int32_t tt_host_free(void* ptr);

#ifdef __cplusplus
}
#endif

#endif /* TINYTRACE_CUDA_H */
