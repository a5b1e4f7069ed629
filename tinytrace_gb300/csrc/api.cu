// C ABI of libtinytrace_cuda.so (declared in include/tinytrace_cuda.h): contexts, handle
// pools with lifetimes and epochs, scene upload + LBVH build, rendering, tonemapping and the
// parity entry points.  Every entry point converts failures into a status code and a
// thread-local message; nothing throws or aborts across the ABI.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "tt_internal.h"
#include "tt_cache.cuh"
#include "tt_kernels.h"
#include "tt_texture.cuh"

namespace tt {

thread_local std::string g_last_error;

void fail(int32_t code, const std::string& message) { throw Error{code, message}; }
void check_cuda(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return;
    int32_t code = e == cudaErrorMemoryAllocation ? TT_ERR_OOM
                   : e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver ? TT_ERR_NO_DEVICE
                                                                                 : TT_ERR_DEVICE;
    fail(code, std::string(what) + ": " + cudaGetErrorString(e));
}

DeviceBuffer& DeviceBuffer::operator=(DeviceBuffer&& o) noexcept {
    if (this != &o) {
        if (ptr) cudaFree(ptr);
        ptr = o.ptr;
        bytes = o.bytes;
        o.ptr = nullptr;
        o.bytes = 0;
    }
    return *this;
}
DeviceBuffer::~DeviceBuffer() {
    if (ptr) cudaFree(ptr);
}
void DeviceBuffer::alloc(size_t n) {
    if (ptr) {
        cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    size_t b = n == 0 ? 16 : n;
    check_cuda(cudaMalloc(&ptr, b), "cudaMalloc");
    bytes = n;
}

namespace {

constexpr uint32_t KIND_IMAGE = 1, KIND_SCENE = 2;
constexpr int LIFETIMES = 5;
constexpr int EVENT_SLOTS = 16;
constexpr size_t L2_FLUSH_BYTES = 512ull << 20;
#ifndef TT_LEAF_MAX
#define TT_LEAF_MAX 2
#endif
constexpr int BLAS_LEAF_MAX = TT_LEAF_MAX;  // triangles per leaf
constexpr uint64_t FLAT_AUTO_MAX_TRIANGLES = 1ull << 26;

struct ImageRes {
    DeviceBuffer buf;
    uint32_t width = 0, height = 0;
};

struct SceneRes {
    DeviceBuffer positions, indices, vertices, materials, meshes, instances, emissive, inst_xform, inst_bucket, light_prim;
    DeviceBuffer tex_table, tex_data, srgb, light_alias, light_rec;
    BvhResult bvh;
    DevScene dev{};
    tt_scene_stats stats{};
    std::vector<tt_instance> host_instances;  // for tt_scene_update_instances' checks
    std::vector<tt_emissive_triangle> host_emissive;  // to rebuild the light alias table on updates
    std::vector<tt_material> host_materials;
    std::vector<tt_mesh> host_meshes;  // to rebuild the compressed wide structure on instance updates
    uint32_t material_count = 0;
};

// Slot pool and queues of the wavefront integrator, grown on demand and kept across frames.
struct WavefrontBuffers {
    DeviceBuffer org, dir, thr, acc, pa1, pa0, pe, hit, hslot, active, shadow, counters, samples, running, ndc_mip;
    uint32_t slots = 0;
    uint64_t sample_items = 0;
    uint32_t pixels = 0;
};

// Rasterised primary visibility (primary.cu): per-record rectangles and pair counts, per-instance
// bounds and the closest-hit keys of one sample chunk, grown on demand.
struct PrimaryState {
    DeviceBuffer key, rect, edge, count, live_pos, live_rec, live_first, inst, flags;  // flags: total, ok, live_n, next
    uint64_t key_items = 0, records = 0, instances = 0;
};

// ReSTIR DI state kept between frames: two G-buffers and two final reservoir arrays
// (current and previous frame), the initial and temporal reservoirs, the previous camera.
struct RestirState {
    DeviceBuffer gbuf[2], final_res[2], initial, temporal, gtex, glob, queue, queue_count;
    uint64_t pixels = 0;
    uint32_t cur = 0;
    RestirHistory history{};
    tt_restir_config config{32u, 20.0f, 5u, 30.0f};
};

// Learned radiance cache: device parameters, the configuration and the integrator's buffers
// (queued queries, training records and pairs).
struct CacheState {
    DeviceBuffer grid, grid_m, grid_v, grid_grad, w, w_m, w_v, w_grad, w16, loss, grid16;
    DeviceBuffer cq, cq_slot, cq_out, rec, train_final, tq, tt, tcount, spread;
    uint64_t cq_cap = 0, rec_cap = 0, final_cap = 0;
    bool enabled = false;
    float last_loss = 0.0f;
    uint32_t last_pairs = 0;
    tt_cache_config config{1e-2f, 65536u, 1u, 1u, 0.01f};
    uint32_t step = 0;
    bool ready = false;
    CacheDevice dev() const {
        return CacheDevice{grid.as<float>(), grid_m.as<float>(), grid_v.as<float>(), grid_grad.as<float>(),
                           w.as<float>(), w_m.as<float>(), w_v.as<float>(), w_grad.as<float>(), w16.as<__half>(),
                           loss.as<float>(), grid16.as<__half>()};
    }
};

struct Pool {
    uint32_t epoch = 1;
    std::vector<std::unique_ptr<ImageRes>> images;
    std::vector<std::unique_ptr<SceneRes>> scenes;
};

}  // namespace
}  // namespace tt

struct tt_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    tt::Pool pools[tt::LIFETIMES];
    uint64_t frame_index = 0;
    cudaEvent_t ev_integrate[2] = {nullptr, nullptr};
    cudaEvent_t ev_post[2] = {nullptr, nullptr};
    cudaEvent_t user_events[tt::EVENT_SLOTS] = {};
    bool integrate_timed = false, post_timed = false;
    float scene_build_ms = 0.0f;
    tt::DeviceBuffer err_word, counters, l2_flush;
    uint32_t* err_host = nullptr;  // pinned
    bool err_pending = false;
    uint32_t integrator = TT_INTEGRATOR_WAVEFRONT;
    uint32_t wavefront_slots = 0;  // 0 = default
    uint32_t accel = TT_ACCEL_AUTO;
    tt::WavefrontBuffers wf;
    bool stage_timing = false;
    bool graphs = true;
    uint32_t light_visibility = TT_LIGHT_VISIBILITY_HASH;  // TT_OPTION_LIGHT_VISIBILITY
    uint32_t light_selection = TT_LIGHT_SELECTION_UNIFORM; // TT_OPTION_LIGHT_SELECTION
    uint32_t primary = TT_PRIMARY_RASTER;                   // TT_OPTION_PRIMARY_VISIBILITY
    tt::PrimaryState prim;
    uint32_t refill_lanes = 20;       // TT_OPTION_REFILL_LANES
    uint32_t trace_blocks_per_sm = 0; // TT_OPTION_TRACE_BLOCKS_PER_SM (0 = as many as fit)
    int occupancy_sms = 0, occupancy_blocks = 0;
    cudaStream_t capture[2] = {nullptr, nullptr};  // capture streams of the graph-driven loop
    std::vector<cudaEvent_t> stage_events;  // 2 * StageTimer::MAX_LAUNCHES, created on first use
    tt::StageTimer stage_timer;
    tt::RestirState restir;
    tt::CacheState cache;
};

namespace tt {
// Traversal stack entries (32-bit words) a structure can need: BVH4 nodes push at most 3 entries
// per level (+1 for the instance marker of the two-level structure's transition); the wide format
// pushes at most a node group and a triangle group (two words each) per level.
uint64_t structure_stack_need(const BvhResult& b) {
    if (b.flat && b.wide) return 4ull * b.flat_levels + 2ull;
    if (b.flat) return 3ull * b.flat_levels + 1ull;
    return 3ull * (b.blas_levels + b.tlas_levels) + 1ull;
}
void raise_device_error(uint32_t e) {
    if (e & ERR_STACK_OVERFLOW) fail(TT_ERR_OVERFLOW, "traversal stack overflow");
    if (e & ERR_ITERATION_LIMIT) fail(TT_ERR_TIMEOUT, "traversal iteration limit reached");
    if (e & ERR_TENSOR_WAIT) fail(TT_ERR_TIMEOUT, "radiance-cache tensor-core wait limit reached");
    if (e & ERR_PRIMARY_MISMATCH) fail(TT_ERR_DEVICE, "a rasterised camera-ray hit failed its ray/triangle test");
    if (e) fail(TT_ERR_DEVICE, "unknown device error bits " + std::to_string(e));
}
namespace {

uint64_t make_handle(uint32_t lifetime, uint32_t kind, uint32_t epoch, uint32_t index) {
    return ((uint64_t)(lifetime & 0xfu) << 60) | ((uint64_t)(kind & 0xfu) << 56) |
           ((uint64_t)(epoch & 0xffffffu) << 32) | index;
}

template <class T>
T* lookup(tt_context* ctx, tt_handle h, uint32_t kind) {
    uint32_t lifetime = (uint32_t)(h >> 60) & 0xfu;
    uint32_t k = (uint32_t)(h >> 56) & 0xfu;
    uint32_t epoch = (uint32_t)(h >> 32) & 0xffffffu;
    uint32_t index = (uint32_t)h;
    if (lifetime >= (uint32_t)LIFETIMES || k != kind) fail(TT_ERR_BAD_HANDLE, "handle of the wrong kind");
    Pool& p = ctx->pools[lifetime];
    if ((p.epoch & 0xffffffu) != epoch) fail(TT_ERR_BAD_HANDLE, "stale handle: its lifetime was cleared");
    if constexpr (std::is_same<T, ImageRes>::value) {
        if (index >= p.images.size() || !p.images[index]) fail(TT_ERR_BAD_HANDLE, "unknown image handle");
        return p.images[index].get();
    } else {
        if (index >= p.scenes.size() || !p.scenes[index]) fail(TT_ERR_BAD_HANDLE, "unknown scene handle");
        return p.scenes[index].get();
    }
}

void require(bool cond, const char* msg) {
    if (!cond) fail(TT_ERR_INVALID_ARGUMENT, msg);
}

void use_device(tt_context* ctx) { check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice"); }

// Reads back the device error word after the stream drained.
void check_device_errors(tt_context* ctx) {
    if (!ctx->err_pending) return;
    ctx->err_pending = false;
    raise_device_error(*ctx->err_host);
}
void sync(tt_context* ctx) {
    check_cuda(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    check_device_errors(ctx);
}
void arm_error_word(tt_context* ctx) {
    check_cuda(cudaMemsetAsync(ctx->err_word.ptr, 0, 4, ctx->stream), "memset");
}
void fetch_error_word(tt_context* ctx) {
    check_cuda(cudaMemcpyAsync(ctx->err_host, ctx->err_word.ptr, 4, cudaMemcpyDeviceToHost, ctx->stream),
               "error word");
    ctx->err_pending = true;
}

template <class T>
void upload(DeviceBuffer& b, const T* host, uint64_t count, cudaStream_t st) {
    b.alloc(count * sizeof(T));
    if (count) check_cuda(cudaMemcpyAsync(b.ptr, host, count * sizeof(T), cudaMemcpyHostToDevice, st), "upload");
}

// Which shading code a material runs: the OpenPBR lobes that can carry weight, NEE eligibility
// (integrate.glsl:293-295) and emission.  Hits on materials with equal signatures share one
// shading queue of the wavefront integrator.  (A signature built from lobe_set_of alone merged
// the textured Cornell box's Lambertian walls, specular weight 0, with its textured specular
// materials, whose texture loads then diverged inside warps: shade 21.7 -> 39.0 ms per frame.)
uint32_t shading_signature(const tt_material_constants& m) {
    uint32_t sig = 0u;
    if (m.fuzz_weight > 0.0f) sig |= 1u;
    if (m.coat_weight > 0.0f) sig |= 2u;
    if (m.base_metalness > 0.0f) sig |= 4u;
    if (m.base_metalness < 1.0f && m.specular_weight > 0.0f) sig |= 8u;
    if (m.base_metalness < 1.0f && m.transmission_weight > 0.0f) sig |= 16u;
    if (m.base_metalness < 1.0f && m.transmission_weight < 1.0f) sig |= 32u;
    if (m.specular_roughness > 0.15f) sig |= 64u;
    if (m.emission_luminance > 0.0f) sig |= 128u;
    return sig;
}

// Shading-queue bucket per instance: the HIT_BUCKETS - 1 signatures covering the most
// instanced triangles get their own bucket, all others share the last one.  `lobes` receives
// byte b = the union of lobe_set_of over bucket b's materials (the shade kernel's variant).
std::vector<uint8_t> instance_buckets(const tt_scene_desc* d, uint32_t& lobes) {
    std::map<uint32_t, uint64_t> weight;
    std::vector<uint32_t> sig(d->instance_count);
    for (uint32_t i = 0; i < d->instance_count; ++i) {
        const tt_instance& in = d->instances[i];
        sig[i] = shading_signature(d->materials[in.material_index].constants);
        weight[sig[i]] += d->meshes[in.mesh_index].index_count / 3u + 1u;
    }
    std::vector<std::pair<uint64_t, uint32_t>> order;
    for (auto& kv : weight) order.push_back({kv.second, kv.first});
    std::sort(order.begin(), order.end(), [](auto& a, auto& b) { return a.first != b.first ? a.first > b.first : a.second < b.second; });
    std::map<uint32_t, uint8_t> bucket;
    for (size_t k = 0; k < order.size(); ++k) bucket[order[k].second] = (uint8_t)std::min<size_t>(k, HIT_BUCKETS - 1);
    std::vector<uint8_t> out(std::max<uint32_t>(d->instance_count, 1), 0);
    lobes = 0u;
    for (uint32_t i = 0; i < d->instance_count; ++i) {
        out[i] = bucket[sig[i]];
        lobes |= lobe_set_of(d->materials[d->instances[i].material_index].constants) << (8u * out[i]);
    }
    return out;
}

// Primitive index of each emissive triangle inside its instance's mesh (the triangle whose
// snorm16 positions it copies; Scene::new lists a model's triangles in order,
// src/asset/mod.rs:163-193, so the running index is tried first).  0xffffffff: no match.
std::vector<uint32_t> light_primitives(const tt_scene_desc* d) {
    std::vector<uint32_t> out(std::max<uint64_t>(d->emissive_triangle_count, 1), 0xffffffffu);
    std::vector<uint32_t> next(d->instance_count, 0);
    for (uint32_t e = 0; e < d->emissive_triangle_count; ++e) {
        const tt_emissive_triangle& t = d->emissive_triangles[e];
        const tt_instance& in = d->instances[t.instance_index];
        const tt_mesh& me = d->meshes[in.mesh_index];
        uint32_t tris = me.index_count / 3u;
        auto same = [&](uint32_t p) {
            for (int k = 0; k < 3; ++k) {
                const int16_t* v = d->positions + 3ull * (me.vertex_offset + d->indices[me.index_offset + 3u * p + k]);
                if (v[0] != t.positions[k][0] || v[1] != t.positions[k][1] || v[2] != t.positions[k][2]) return false;
            }
            return true;
        };
        uint32_t guess = next[t.instance_index];
        if (guess < tris && same(guess)) {
            out[e] = guess;
        } else {
            for (uint32_t p = 0; p < tris; ++p)
                if (same(p)) {
                    out[e] = p;
                    break;
                }
        }
        if (out[e] != 0xffffffffu) next[t.instance_index] = out[e] + 1u;
    }
    return out;
}

// Alias table of the emissive triangles by emitted power (TT_LIGHT_SELECTION_POWER): power =
// emission_luminance x luminance(emission_color) x world-space area in double precision (area
// alone when the emission is textured), Vose's alias method with index-ordered work stacks;
// entries (keep probability, alias, pdf = power / total, 0).  All powers zero: uniform.
static float bits_float(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
std::vector<float4> light_alias_table(const tt_scene_desc* d) {
    uint32_t n = d->emissive_triangle_count;
    std::vector<float4> out(std::max<uint32_t>(n, 1u), make_float4(1.0f, 0.0f, 0.0f, 0.0f));
    if (n == 0) return out;
    std::vector<double> power(n);
    double total = 0.0;
    for (uint32_t e = 0; e < n; ++e) {
        const tt_emissive_triangle& t = d->emissive_triangles[e];
        const tt_instance& in = d->instances[t.instance_index];
        const tt_material& m = d->materials[in.material_index];
        double p[3][3];
        for (int k = 0; k < 3; ++k) {
            double v[3] = {t.positions[k][0] / 32767.0, t.positions[k][1] / 32767.0, t.positions[k][2] / 32767.0};
            for (int r = 0; r < 3; ++r)
                p[k][r] = in.transform[r] * v[0] + in.transform[4 + r] * v[1] + in.transform[8 + r] * v[2] +
                          in.transform[12 + r];
        }
        double e1[3] = {p[1][0] - p[0][0], p[1][1] - p[0][1], p[1][2] - p[0][2]};
        double e2[3] = {p[2][0] - p[0][0], p[2][1] - p[0][1], p[2][2] - p[0][2]};
        double c[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        double area = 0.5 * std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        bool textured = m.textures[5] != 0xffffffffu || m.textures[25] != 0xffffffffu;
        const tt_material_constants& mc = m.constants;
        double lum = 0.2126 * mc.emission_color[0] + 0.7152 * mc.emission_color[1] + 0.0722 * mc.emission_color[2];
        double pw = textured ? area : (double)mc.emission_luminance * lum * area;
        power[e] = std::isfinite(pw) && pw > 0.0 ? pw : 0.0;
        total += power[e];
    }
    if (!(total > 0.0)) {
        for (uint32_t e = 0; e < n; ++e) out[e] = make_float4(1.0f, bits_float(e), (float)(1.0 / n), 0.0f);
        return out;
    }
    std::vector<double> scaled(n);
    std::vector<uint32_t> small, large;
    for (uint32_t e = 0; e < n; ++e) {
        scaled[e] = power[e] / total * (double)n;
        (scaled[e] < 1.0 ? small : large).push_back(e);
    }
    std::vector<uint32_t> alias(n);
    std::vector<double> keep(n, 1.0);
    for (uint32_t e = 0; e < n; ++e) alias[e] = e;
    while (!small.empty() && !large.empty()) {
        uint32_t s = small.back(), g = large.back();
        small.pop_back();
        large.pop_back();
        keep[s] = scaled[s];
        alias[s] = g;
        scaled[g] = (scaled[g] + scaled[s]) - 1.0;
        (scaled[g] < 1.0 ? small : large).push_back(g);
    }
    for (uint32_t e = 0; e < n; ++e)
        out[e] = make_float4((float)keep[e], bits_float(alias[e]), (float)(power[e] / total), 0.0f);
    return out;
}

// Host-side validation: every index the kernels will follow must be in range.
void validate_scene(const tt_scene_desc* d) {
    require(d != nullptr, "scene desc is null");
    require(d->position_count == 0 || d->positions, "positions pointer is null");
    require(d->index_count == 0 || d->indices, "indices pointer is null");
    require(d->vertex_count == 0 || d->vertices, "vertices pointer is null");
    require(d->material_count == 0 || d->materials, "materials pointer is null");
    require(d->mesh_count == 0 || d->meshes, "meshes pointer is null");
    require(d->instance_count == 0 || d->instances, "instances pointer is null");
    require(d->emissive_triangle_count == 0 || d->emissive_triangles, "emissive pointer is null");
    require(d->position_count < (1ull << 32) && d->index_count < (1ull << 32) && d->vertex_count < (1ull << 32),
            "arrays above 2^32 entries are not supported");
    uint64_t verts = std::min(d->position_count, d->vertex_count);
    uint64_t tris = 0;
    for (uint32_t m = 0; m < d->mesh_count; ++m) {
        const tt_mesh& me = d->meshes[m];
        uint64_t end = (uint64_t)me.index_offset + me.index_count;
        require(end <= d->index_count, "mesh index range exceeds the index buffer");
        uint32_t used = me.index_count / 3u * 3u;
        for (uint32_t k = 0; k < used; ++k)
            require((uint64_t)d->indices[me.index_offset + k] + me.vertex_offset < verts,
                    "mesh index points outside the vertex arrays");
        tris += me.index_count / 3u;
    }
    require(tris < (1ull << 27), "more than 2^27 triangles in one scene");
    require(d->instance_count < (1ull << 27), "more than 2^27 instances in one scene");
    for (uint32_t i = 0; i < d->instance_count; ++i) {
        const tt_instance& in = d->instances[i];
        require(in.mesh_index < d->mesh_count, "instance mesh_index out of range");
        require(in.material_index < d->material_count, "instance material_index out of range");
        const tt_mesh& me = d->meshes[in.mesh_index];
        require(in.index_offset == me.index_offset && in.vertex_offset == me.vertex_offset,
                "instance offsets must equal its mesh's offsets (src/scene.rs:52-53)");
        for (int k = 0; k < 16; ++k)
            require(std::isfinite(in.transform[k]) && std::isfinite(in.inverse_transform[k]) &&
                        std::isfinite(in.normal_transform[k]),
                    "instance matrices must be finite");
    }
    for (uint32_t e = 0; e < d->emissive_triangle_count; ++e)
        require(d->emissive_triangles[e].instance_index < d->instance_count,
                "emissive triangle instance_index out of range");
    require(d->texture_count == 0 || d->textures, "textures pointer is null");
    for (uint32_t t = 0; t < d->texture_count; ++t) {
        const tt_texture& tx = d->textures[t];
        require(tx.format >= TT_TEXTURE_BC1_SRGB && tx.format <= TT_TEXTURE_R16_FLOAT, "unknown texture format");
        require(tx.width >= 1 && tx.height >= 1 && tx.width <= 65536 && tx.height <= 65536, "bad texture extent");
        require(tx.level_count >= 1 && tx.level_count <= TT_TEXTURE_MAX_LEVELS, "bad texture level count");
        require((tx.width >> (tx.level_count - 1)) >= 1 && (tx.height >> (tx.level_count - 1)) >= 1,
                "texture level count exceeds its mip chain");
        uint64_t bytes = 0;
        for (uint32_t l = 0; l < tx.level_count; ++l) bytes += texture_level_bytes(tx.format, tx.width >> l, tx.height >> l);
        require(tx.bytes == bytes, "texture byte count does not match its levels");
        require(bytes == 0 || tx.data, "texture data pointer is null");
    }
    for (uint32_t m = 0; m < d->material_count; ++m)
        for (int t = 0; t < 27; ++t) {
            uint32_t index = d->materials[m].textures[t];
            require(index == 0xffffffffu || index < d->texture_count, "material texture index out of range");
        }
}

// The texture table and level data on the device (levels 16-byte aligned), the sRGB table,
// and the materials with their set texture slots recorded in the padding word.
void upload_textures(const tt_scene_desc* d, SceneRes* s, cudaStream_t st) {
    std::vector<DevTexture> table(d->texture_count);
    uint64_t total = 0;
    for (uint32_t t = 0; t < d->texture_count; ++t) {
        const tt_texture& tx = d->textures[t];
        DevTexture& dt = table[t];
        dt = DevTexture{};
        dt.format = tx.format;
        dt.levels = tx.level_count;
        dt.width = tx.width;
        dt.height = tx.height;
        for (uint32_t l = 0; l < tx.level_count; ++l) {
            dt.offset[l] = total;
            total += (texture_level_bytes(tx.format, tx.width >> l, tx.height >> l) + 15u) / 16u * 16u;
        }
    }
    std::vector<uint8_t> data(total);
    for (uint32_t t = 0; t < d->texture_count; ++t) {
        const tt_texture& tx = d->textures[t];
        uint64_t at = 0;
        for (uint32_t l = 0; l < tx.level_count; ++l) {
            uint64_t n = texture_level_bytes(tx.format, tx.width >> l, tx.height >> l);
            std::memcpy(data.data() + table[t].offset[l], tx.data + at, n);
            at += n;
        }
    }
    upload(s->tex_table, table.data(), table.size(), st);
    upload(s->tex_data, data.data(), data.size(), st);
    std::vector<float> srgb(256);
    for (int i = 0; i < 256; ++i) {  // sRGB EOTF
        double c = i / 255.0;
        srgb[i] = (float)(c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4));
    }
    upload(s->srgb, srgb.data(), srgb.size(), st);
    std::vector<tt_material> mats(d->materials, d->materials + d->material_count);
    bool textured = false;
    for (tt_material& m : mats) {
        uint32_t mask = 0;
        for (int t = 0; t < 27; ++t)
            if (m.textures[t] != 0xffffffffu) mask |= 1u << t;
        m.padding = mask;
        textured = textured || (mask & (LOAD_SLOTS | EMISSION_SLOTS)) != 0u;
    }
    upload(s->materials, mats.data(), mats.size(), st);
    check_cuda(cudaStreamSynchronize(st), "texture upload");  // the host staging vectors go out of scope
    s->dev.textures = s->tex_table.as<DevTexture>();
    s->dev.tex_data = s->tex_data.as<uint8_t>();
    s->dev.srgb = s->srgb.as<float>();
    s->dev.textured = textured ? 1u : 0u;
}

template <class F>
int32_t guarded(F&& f) {
    try {
        f();
        return TT_OK;
    } catch (const Error& e) {
        g_last_error = e.message;
        return e.code;
    } catch (const std::bad_alloc&) {
        g_last_error = "host allocation failed";
        return TT_ERR_OOM;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return TT_ERR_DEVICE;
    } catch (...) {
        g_last_error = "unknown failure";
        return TT_ERR_DEVICE;
    }
}

}  // namespace
}  // namespace tt

using namespace tt;

constexpr uint32_t WAVEFRONT_DEFAULT_SLOTS = 1u << 21;
constexpr uint32_t WAVEFRONT_MAX_CHUNK_SPP = 64;

// Sizes (growing only) the wavefront pool for this frame and returns its device pointers.
static WfParams wavefront_buffers(tt_context* ctx, const tt_constants& c) {
    WavefrontBuffers& b = ctx->wf;
    uint64_t WH = (uint64_t)c.screen_size[0] * c.screen_size[1];
    uint32_t chunk_spp = std::min<uint32_t>(c.sample_count, WAVEFRONT_MAX_CHUNK_SPP);
    uint64_t items = WH * chunk_spp;
    uint32_t want = ctx->wavefront_slots ? ctx->wavefront_slots : WAVEFRONT_DEFAULT_SLOTS;
    uint32_t slots = (uint32_t)std::min<uint64_t>(want, std::max<uint64_t>(items, 1));
    slots = (slots + 127u) / 128u * 128u;
    if (slots > b.slots) {
        b.org.alloc(16ull * slots);
        b.dir.alloc(16ull * slots);
        b.thr.alloc(16ull * slots);
        b.acc.alloc(16ull * slots);
        b.pa1.alloc(16ull * slots);
        b.pa0.alloc(16ull * slots);
        b.pe.alloc(16ull * slots);
        b.hit.alloc(16ull * HIT_BUCKETS * slots);
        b.hslot.alloc(4ull * HIT_BUCKETS * slots);
        b.active.alloc(4ull * slots);
        b.shadow.alloc(32ull * slots);
        b.ndc_mip.alloc(8ull * slots);
        b.slots = slots;
    }
    if (!b.counters.ptr) b.counters.alloc(64);
    if (items > b.sample_items) {
        b.samples.alloc(16ull * items);
        b.sample_items = items;
    }
    if (WH > b.pixels) {
        b.running.alloc(16ull * WH);
        b.pixels = (uint32_t)WH;
    }
    WfParams w{};
    w.org = b.org.as<float4>();
    w.dir = b.dir.as<float4>();
    w.thr = b.thr.as<float4>();
    w.acc = b.acc.as<float4>();
    w.pa1 = b.pa1.as<float4>();
    w.pa0 = b.pa0.as<float4>();
    w.pe = b.pe.as<float4>();
    w.hit = b.hit.as<uint4>();
    w.hslot = b.hslot.as<uint32_t>();
    w.active = b.active.as<uint32_t>();
    w.shadow = b.shadow.as<float4>();
    w.counters = b.counters.as<uint32_t>();
    w.samples = b.samples.as<float4>();
    w.running = b.running.as<float4>();
    w.ndc_mip = b.ndc_mip.as<float2>();
    w.P = slots;
    w.chunk_spp = chunk_spp;
    w.refill = ctx->refill_lanes;
    if (ctx->occupancy_sms == 0) trace_occupancy(&ctx->occupancy_sms, &ctx->occupancy_blocks);
    int per_sm = ctx->trace_blocks_per_sm ? std::min<int>(ctx->trace_blocks_per_sm, ctx->occupancy_blocks)
                                          : ctx->occupancy_blocks;
    w.trace_blocks = (uint32_t)std::max(1, ctx->occupancy_sms * per_sm);
    return w;
}

// Rasterised primary visibility buffers for a frame of `c` on scene `sc` (grown on demand).
static void primary_buffers(tt_context* ctx, const tt_constants& c, const DevScene& sc, uint32_t chunk_spp,
                            PrimaryParams& v) {
    PrimaryState& S = ctx->prim;
    uint64_t items = (uint64_t)c.screen_size[0] * c.screen_size[1] * chunk_spp;
    if (items > S.key_items) {
        S.key.alloc(8ull * items);
        S.key_items = items;
    }
    if ((uint64_t)sc.tri_count + 1 > S.records) {
        S.rect.alloc(16ull * sc.tri_count);
        S.edge.alloc(48ull * sc.tri_count);
        S.count.alloc(4ull * (sc.tri_count + 1ull));
        S.live_pos.alloc(4ull * (sc.tri_count + 1ull));
        S.live_rec.alloc(4ull * sc.tri_count);
        S.live_first.alloc(4ull * (sc.tri_count + 1ull));
        S.records = (uint64_t)sc.tri_count + 1;
    }
    if (sc.instance_count > S.instances) {
        S.inst.alloc(sizeof(PrimaryInstance) * (uint64_t)sc.instance_count);
        S.instances = sc.instance_count;
    }
    if (!S.flags.ptr) S.flags.alloc(32);
    v.key = S.key.as<unsigned long long>();
    v.rect = S.rect.as<float4>();
    v.edge = S.edge.as<float4>();
    v.count = S.count.as<uint32_t>();
    v.live_pos = S.live_pos.as<uint32_t>();
    v.live_rec = S.live_rec.as<uint32_t>();
    v.live_first = S.live_first.as<uint32_t>();
    v.total = S.flags.as<unsigned long long>();
    v.ok = reinterpret_cast<uint32_t*>(S.flags.as<unsigned char>() + 8);
    v.live_n = reinterpret_cast<uint32_t*>(S.flags.as<unsigned char>() + 12);
    v.next = reinterpret_cast<uint32_t*>(S.flags.as<unsigned char>() + 16);
    v.inst = S.inst.as<PrimaryInstance>();
    v.records = sc.tri_count;
    v.sms = std::max(1, ctx->occupancy_sms);
}

namespace tt {
void set_last_error(const std::string& message) { g_last_error = message; }
DevScene scene_view(tt_context* ctx, tt_handle scene) {
    require(ctx, "null context");
    DevScene d = lookup<SceneRes>(ctx, scene, KIND_SCENE)->dev;
    d.light_exact = ctx->light_visibility == TT_LIGHT_VISIBILITY_TRIANGLE ? 1u : 0u;
    d.light_power = ctx->light_selection == TT_LIGHT_SELECTION_POWER ? 1u : 0u;
    return d;
}
int context_device(tt_context* ctx) { return ctx->device; }
bool context_primary_raster(tt_context* ctx) { return ctx->primary == TT_PRIMARY_RASTER; }
}  // namespace tt

static void cache_ready(tt_context* ctx) {
    CacheState& C = ctx->cache;
    if (C.ready) return;
    C.grid.alloc(4 * CACHE_GRID_PARAMS);
    C.grid16.alloc(2 * CACHE_GRID_PARAMS);
    C.grid_m.alloc(4 * CACHE_GRID_PARAMS);
    C.grid_v.alloc(4 * CACHE_GRID_PARAMS);
    C.grid_grad.alloc(4 * CACHE_GRID_PARAMS);
    C.w.alloc(4 * CACHE_PARAMS);
    C.w_m.alloc(4 * CACHE_PARAMS);
    C.w_v.alloc(4 * CACHE_PARAMS);
    C.w_grad.alloc(4 * CACHE_PARAMS);
    C.w16.alloc(2 * CACHE_PARAMS);
    C.loss.alloc(16);
    cache_set_level_scales();
    cache_init(C.dev(), C.config.seed, ctx->stream);
    C.step = 0;
    C.ready = true;
}

// Radiance-cache buffers of one frame: queued queries (one per path slot), training records
// (train_paths_per_frame paths x (bounce_count + 1) vertices) and the pairs built from them.
static void cache_frame_buffers(tt_context* ctx, const tt_constants& c, const DevScene& sc, WfParams& w) {
    cache_ready(ctx);
    CacheState& C = ctx->cache;
    if (w.P > C.cq_cap) {
        C.cq.alloc(48ull * w.P);
        C.cq_slot.alloc(4ull * w.P);
        C.cq_out.alloc(12ull * w.P);
        C.spread.alloc(16ull * w.P);
        C.cq_cap = w.P;
    }
    uint64_t items = (uint64_t)c.screen_size[0] * c.screen_size[1] * c.sample_count;
    uint32_t paths = std::max<uint32_t>(C.config.train_paths_per_frame, 1u);
    uint64_t stride = std::max<uint64_t>(items / paths, 1);
    require(stride <= 0xffffffffull, "too many samples per training path");
    uint64_t final_n = items / stride + 1;
    uint64_t rec_n = final_n * (c.bounce_count + 1ull);
    if (final_n > C.final_cap) {
        C.train_final.alloc(16ull * final_n);
        C.final_cap = final_n;
    }
    if (rec_n > C.rec_cap) {
        C.rec.alloc(sizeof(TrainRecord) * rec_n);
        C.tq.alloc(48ull * rec_n);
        C.tt.alloc(12ull * rec_n);
        C.rec_cap = rec_n;
    }
    if (!C.tcount.ptr) C.tcount.alloc(16);
    w.cache_on = 1u;
    w.cache_depth = C.config.terminate_depth;
    w.spread_c = C.config.spread_threshold;
    w.spread = C.spread.as<float4>();
    w.train_stride = (uint32_t)stride;
    w.rec_cap = (uint32_t)std::min<uint64_t>(C.rec_cap, 0xffffffffull);
    w.cache_bound = sc.tlas_bound > 0.0f ? sc.tlas_bound : 1.0f;
    w.cq = C.cq.as<CacheQuery>();
    w.cq_slot = C.cq_slot.as<uint32_t>();
    w.cq_out = C.cq_out.as<float>();
    w.rec = C.rec.as<TrainRecord>();
    w.train_final = C.train_final.as<float4>();
    w.cache_grid = C.grid16.as<__half>();
    w.cache_w16 = C.w16.as<__half>();
}

// After a cached frame: training pairs from the frame's training paths, then up to four Adam
// steps of at most 16,384 pairs each.
static void cache_train_after_frame(tt_context* ctx, const WfParams& w) {
    CacheState& C = ctx->cache;
    cudaStream_t st = ctx->stream;
    cache_targets(w.rec, w.counters + CTRL_RECORDS, w.rec_cap, w.train_final, C.tq.as<CacheQuery>(), C.tt.as<float>(),
                  C.tcount.as<uint32_t>(), st);
    uint32_t pairs = 0;
    check_cuda(cudaMemcpyAsync(&pairs, C.tcount.ptr, 4, cudaMemcpyDeviceToHost, st), "pairs");
    check_cuda(cudaStreamSynchronize(st), "sync");
    C.last_pairs = pairs;
    constexpr uint32_t BATCH = 16384;
    for (uint32_t k = 0; k < 4 && k * BATCH < pairs; ++k) {
        uint32_t n = std::min(BATCH, pairs - k * BATCH);
        cache_train_step(C.dev(), C.tq.as<CacheQuery>() + (uint64_t)k * BATCH, C.tt.as<float>() + 3ull * k * BATCH, n,
                         C.config.learning_rate, ++C.step, ctx->err_word.as<uint32_t>(), st);
    }
}

// The context's per-launch timer for the next render when TT_OPTION_STAGE_TIMING is on (its
// events are created on first use), else null; either way the previous render's record is
// dropped (count -1: the last render was not timed per stage).
static StageTimer* begin_stage_timing(tt_context* ctx) {
    StageTimer* timer = nullptr;
    if (ctx->stage_timing) {
        if (ctx->stage_events.empty()) {
            ctx->stage_events.resize(2 * StageTimer::MAX_LAUNCHES);
            for (auto& ev : ctx->stage_events) check_cuda(cudaEventCreate(&ev), "event");
        }
        timer = &ctx->stage_timer;
        timer->events = ctx->stage_events.data();
        timer->count = 0;
        timer->overflow = false;
        timer->open = false;
    }
    ctx->stage_timer.count = timer ? 0 : -1;
    return timer;
}

static void render_impl(tt_context* ctx, tt_handle scene, const tt_constants* c, tt_handle target, bool counted,
                        tt_traversal_counters* out) {
    require(ctx && c, "null argument");
    use_device(ctx);
    SceneRes* s = lookup<SceneRes>(ctx, scene, KIND_SCENE);
    ImageRes* img = lookup<ImageRes>(ctx, target, KIND_IMAGE);
    require(c->screen_size[0] == img->width && c->screen_size[1] == img->height,
            "constants.screen_size must equal the target extent");
    RenderParams p;
    p.sc = s->dev;
    p.sc.light_exact = ctx->light_visibility == TT_LIGHT_VISIBILITY_TRIANGLE ? 1u : 0u;
    p.sc.light_power = ctx->light_selection == TT_LIGHT_SELECTION_POWER ? 1u : 0u;
    p.c = *c;
    p.target = img->buf.as<float4>();
    p.err = ctx->err_word.as<uint32_t>();
    p.counters = ctx->counters.as<unsigned long long>();
    arm_error_word(ctx);
    if (counted) check_cuda(cudaMemsetAsync(ctx->counters.ptr, 0, 64, ctx->stream), "memset");
    bool wavefront = ctx->integrator == TT_INTEGRATOR_WAVEFRONT && c->sample_count > 0 && c->bounce_count > 0;
    WfParams w{};
    if (wavefront) w = wavefront_buffers(ctx, *c);
    if (!s->dev.textured) w.ndc_mip = nullptr;
    bool cached = wavefront && ctx->cache.enabled && !counted;
    if (cached) cache_frame_buffers(ctx, *c, s->dev, w);
    // camera rays from rasterised keys: flat BVH4 scenes with a regular camera (instrumented
    // renders too, so that their counters describe the same work)
    PrimaryParams pv{};
    const PrimaryParams* prim = nullptr;
    if (wavefront && ctx->primary == TT_PRIMARY_RASTER && s->dev.tri_record && s->dev.tri_count > 0 &&
        primary_camera(*c, pv)) {
        primary_buffers(ctx, *c, s->dev, w.chunk_spp, pv);
        w.vis = pv.key;
        w.vis_ok = pv.ok;
        prim = &pv;
    }
    StageTimer* timer = begin_stage_timing(ctx);
    check_cuda(cudaEventRecord(ctx->ev_integrate[0], ctx->stream), "event");
    if (prim) {
        stage_begin(timer, TT_STAGE_PRIMARY, ctx->stream);
        primary_setup(p, pv, ctx->stream);
        stage_end(timer, ctx->stream);
    }
    if (wavefront && ctx->graphs && !timer) {
        for (auto& cs : ctx->capture)
            if (!cs) check_cuda(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "capture stream");
        render_wavefront_graph(p, w, counted, ctx->stream, ctx->capture[0], ctx->capture[1], prim);
    } else if (wavefront) {
        render_wavefront(p, w, ctx->err_host + 1, counted, ctx->stream, timer, prim);
    } else {
        stage_begin(timer, TT_STAGE_MEGAKERNEL, ctx->stream);
        launch_integrate(p, counted, ctx->stream);
        stage_end(timer, ctx->stream);
    }
    check_cuda(cudaGetLastError(), "integrate launch");
    check_cuda(cudaEventRecord(ctx->ev_integrate[1], ctx->stream), "event");
    ctx->integrate_timed = true;
    if (cached) {
        stage_begin(timer, TT_STAGE_CACHE_TRAIN, ctx->stream);
        cache_train_after_frame(ctx, w);
        stage_end(timer, ctx->stream);
    }
    fetch_error_word(ctx);
    if (counted) {
        unsigned long long h[8];
        check_cuda(cudaMemcpyAsync(h, ctx->counters.ptr, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream), "copy");
        sync(ctx);
        out->rays = h[0];
        out->blas_nodes = h[1];
        out->tlas_nodes = h[2];
        out->triangles = h[3];
        out->instances = h[4];
        out->hits = h[5];
        out->warp_steps = h[6];
        out->lane_steps = h[7];
    }
}

// Copies host data into stream-ordered device scratch, runs `launch`, copies results back.
template <class L>
static void batch(tt_context* ctx, const void* in, uint64_t in_bytes, const void* extra, uint64_t extra_bytes,
                  void* out, uint64_t out_bytes, L&& launch) {
    use_device(ctx);
    cudaStream_t st = ctx->stream;
    void *din = nullptr, *dex = nullptr, *dout = nullptr;
    check_cuda(cudaMallocAsync(&din, in_bytes ? in_bytes : 16, st), "cudaMallocAsync");
    check_cuda(cudaMallocAsync(&dout, out_bytes ? out_bytes : 16, st), "cudaMallocAsync");
    if (extra_bytes) check_cuda(cudaMallocAsync(&dex, extra_bytes, st), "cudaMallocAsync");
    if (in_bytes) check_cuda(cudaMemcpyAsync(din, in, in_bytes, cudaMemcpyHostToDevice, st), "upload");
    if (extra_bytes) check_cuda(cudaMemcpyAsync(dex, extra, extra_bytes, cudaMemcpyHostToDevice, st), "upload");
    launch(din, dex, dout);
    check_cuda(cudaGetLastError(), "batch launch");
    if (out_bytes) check_cuda(cudaMemcpyAsync(out, dout, out_bytes, cudaMemcpyDeviceToHost, st), "download");
    cudaFreeAsync(din, st);
    cudaFreeAsync(dout, st);
    if (dex) cudaFreeAsync(dex, st);
    sync(ctx);
}

extern "C" {

int32_t tt_abi_version(void) { return TT_ABI_VERSION; }
const char* tt_last_error(void) { return g_last_error.c_str(); }

int32_t tt_context_create(int32_t device, tt_context** out) {
    return guarded([&] {
        require(out != nullptr, "out is null");
        int count = 0;
        cudaError_t e = cudaGetDeviceCount(&count);
        if (e != cudaSuccess || count == 0) fail(TT_ERR_NO_DEVICE, "no CUDA device available");
        require(device >= 0 && device < count, "device index out of range");
        std::unique_ptr<tt_context> ctx(new tt_context());
        ctx->device = device;
        use_device(ctx.get());
        check_cuda(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking), "stream");
        for (auto& ev : ctx->ev_integrate) check_cuda(cudaEventCreate(&ev), "event");
        for (auto& ev : ctx->ev_post) check_cuda(cudaEventCreate(&ev), "event");
        for (auto& ev : ctx->user_events) check_cuda(cudaEventCreate(&ev), "event");
        ctx->err_word.alloc(16);
        ctx->counters.alloc(8 * 8);
        check_cuda(cudaMallocHost(&ctx->err_host, 16), "cudaMallocHost");
        *ctx->err_host = 0;
        *out = ctx.release();
    });
}

int32_t tt_context_destroy(tt_context* ctx) {
    return guarded([&] {
        if (!ctx) return;
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
        for (auto& p : ctx->pools) {
            p.images.clear();
            p.scenes.clear();
        }
        ctx->err_word = DeviceBuffer();
        ctx->counters = DeviceBuffer();
        ctx->l2_flush = DeviceBuffer();
        for (auto& ev : ctx->ev_integrate) cudaEventDestroy(ev);
        for (auto& ev : ctx->ev_post) cudaEventDestroy(ev);
        for (auto& ev : ctx->user_events) cudaEventDestroy(ev);
        for (auto& ev : ctx->stage_events) cudaEventDestroy(ev);
        for (auto& cs : ctx->capture)
            if (cs) cudaStreamDestroy(cs);
        if (ctx->err_host) cudaFreeHost(ctx->err_host);
        cudaStreamDestroy(ctx->stream);
        delete ctx;
    });
}

int32_t tt_frame_index(tt_context* ctx, uint64_t* out) {
    return guarded([&] {
        require(ctx && out, "null argument");
        *out = ctx->frame_index;
    });
}

int32_t tt_advance_frame(tt_context* ctx) {
    return guarded([&] {
        require(ctx, "null context");
        ctx->frame_index++;
    });
}

int32_t tt_clear_lifetime(tt_context* ctx, uint32_t lifetime) {
    return guarded([&] {
        require(ctx, "null context");
        require(lifetime < (uint32_t)LIFETIMES, "unknown lifetime");
        use_device(ctx);
        sync(ctx);
        Pool& p = ctx->pools[lifetime];
        p.images.clear();
        p.scenes.clear();
        p.epoch++;
    });
}

int32_t tt_synchronize(tt_context* ctx) {
    return guarded([&] {
        require(ctx, "null context");
        use_device(ctx);
        sync(ctx);
    });
}

int32_t tt_image_create(tt_context* ctx, uint32_t lifetime, uint32_t width, uint32_t height, tt_handle* out) {
    return guarded([&] {
        require(ctx && out, "null argument");
        require(lifetime < (uint32_t)LIFETIMES, "unknown lifetime");
        require(width > 0 && height > 0 && width <= 65536 && height <= 65536, "bad image extent");
        use_device(ctx);
        auto img = std::make_unique<ImageRes>();
        img->width = width;
        img->height = height;
        img->buf.alloc((uint64_t)width * height * 16ull);
        check_cuda(cudaMemsetAsync(img->buf.ptr, 0, img->buf.bytes, ctx->stream), "memset");
        Pool& p = ctx->pools[lifetime];
        p.images.push_back(std::move(img));
        *out = make_handle(lifetime, KIND_IMAGE, p.epoch, (uint32_t)(p.images.size() - 1));
    });
}

int32_t tt_image_write(tt_context* ctx, tt_handle image, const float* host, uint64_t bytes) {
    return guarded([&] {
        require(ctx && host, "null argument");
        use_device(ctx);
        ImageRes* img = lookup<ImageRes>(ctx, image, KIND_IMAGE);
        require(bytes == img->buf.bytes, "byte count must equal width * height * 16");
        check_cuda(cudaMemcpyAsync(img->buf.ptr, host, bytes, cudaMemcpyHostToDevice, ctx->stream), "write");
        sync(ctx);
    });
}

int32_t tt_image_download(tt_context* ctx, tt_handle image, float* host, uint64_t bytes) {
    return guarded([&] {
        require(ctx && host, "null argument");
        use_device(ctx);
        ImageRes* img = lookup<ImageRes>(ctx, image, KIND_IMAGE);
        require(bytes == img->buf.bytes, "byte count must equal width * height * 16");
        check_cuda(cudaMemcpyAsync(host, img->buf.ptr, bytes, cudaMemcpyDeviceToHost, ctx->stream), "download");
        sync(ctx);
    });
}

int32_t tt_scene_create(tt_context* ctx, const tt_scene_desc* d, tt_handle* out) {
    return guarded([&] {
        require(ctx && out, "null argument");
        validate_scene(d);
        use_device(ctx);
        cudaStream_t st = ctx->stream;
        auto s = std::make_unique<SceneRes>();
        cudaEvent_t e0, e1;
        check_cuda(cudaEventCreate(&e0), "event");
        check_cuda(cudaEventCreate(&e1), "event");
        check_cuda(cudaEventRecord(e0, st), "event");
        upload(s->positions, d->positions, d->position_count * 3ull, st);
        upload(s->indices, d->indices, d->index_count, st);
        upload(s->vertices, d->vertices, d->vertex_count, st);
        upload_textures(d, s.get(), st);
        upload(s->meshes, d->meshes, d->mesh_count, st);
        upload(s->instances, d->instances, d->instance_count, st);
        s->host_instances.assign(d->instances, d->instances + d->instance_count);
        s->host_emissive.assign(d->emissive_triangles, d->emissive_triangles + d->emissive_triangle_count);
        s->host_materials.assign(d->materials, d->materials + d->material_count);
        s->material_count = d->material_count;
        upload(s->emissive, d->emissive_triangles, d->emissive_triangle_count, st);
        std::vector<uint32_t> lprim = light_primitives(d);
        upload(s->light_prim, lprim.data(), lprim.size(), st);
        std::vector<float4> alias = light_alias_table(d);
        upload(s->light_alias, alias.data(), alias.size(), st);
        std::vector<float4> xf(4ull * d->instance_count);
        for (uint32_t i = 0; i < d->instance_count; ++i) {
            const float* m = d->instances[i].inverse_transform;
            for (int r = 0; r < 3; ++r) xf[4ull * i + r] = make_float4(m[r], m[4 + r], m[8 + r], m[12 + r]);
            uint32_t w[4] = {d->instances[i].mesh_index, d->instances[i].material_index,
                             d->instances[i].index_offset, d->instances[i].vertex_offset};
            float4 v;
            std::memcpy(&v, w, 16);
            xf[4ull * i + 3] = v;
        }
        upload(s->inst_xform, xf.data(), xf.size(), st);
        uint32_t bucket_lobes = 0u;
        std::vector<uint8_t> buckets = instance_buckets(d, bucket_lobes);
        upload(s->inst_bucket, buckets.data(), buckets.size(), st);
        BuildInput bi{s->positions.as<int16_t>(), s->indices.as<uint32_t>(), d->meshes, d->mesh_count,
                      d->instances, d->instance_count};
        uint64_t instanced = 0;
        for (uint32_t i = 0; i < d->instance_count; ++i) instanced += d->meshes[d->instances[i].mesh_index].index_count / 3u;
        bool wide = ctx->accel == TT_ACCEL_FLAT_WIDE;
        bool flat = wide || ctx->accel == TT_ACCEL_FLAT ||
                    (ctx->accel == TT_ACCEL_AUTO && instanced <= FLAT_AUTO_MAX_TRIANGLES);
        if (flat && instanced >= (1ull << 27))
            fail(TT_ERR_OVERFLOW, "more than 2^27 instanced triangles for the flat BVH");
        s->host_meshes.assign(d->meshes, d->meshes + d->mesh_count);
        build_scene_bvh(bi, st, BLAS_LEAF_MAX, flat, wide, s->bvh);
        check_cuda(cudaEventRecord(e1, st), "event");
        check_cuda(cudaEventSynchronize(e1), "event");
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        ctx->scene_build_ms = ms;
        uint64_t need_stack = structure_stack_need(s->bvh);
        if (need_stack > (uint64_t)TRAVERSAL_STACK)
            fail(TT_ERR_OVERFLOW, "scene BVH is too deep for the traversal stack (" +
                                      std::to_string(need_stack) + " entries needed)");
        DevScene& ds = s->dev;
        ds.stack_need = (uint32_t)need_stack;
        ds.positions = s->positions.as<int16_t>();
        ds.indices = s->indices.as<uint32_t>();
        ds.vertices = s->vertices.as<tt_vertex>();
        ds.materials = s->materials.as<tt_material>();
        ds.instances = s->instances.as<tt_instance>();
        ds.meshes = s->meshes.as<tt_mesh>();
        ds.light_prim = s->light_prim.as<uint32_t>();
        ds.light_alias = s->light_alias.as<float4>();
        ds.emissive = s->emissive.as<tt_emissive_triangle>();
        ds.inst_xform = s->inst_xform.as<float4>();
        ds.inst_bucket = s->inst_bucket.as<uint8_t>();
        ds.bucket_lobes = bucket_lobes;
        ds.emissive_count = d->emissive_triangle_count;
        ds.instance_count = d->instance_count;
        s->light_rec.alloc(16ull * LIGHT_RECORD * std::max<uint32_t>(d->emissive_triangle_count, 1u));
        ds.light_rec = s->light_rec.as<float4>();
        launch_light_records(ds, s->light_rec.as<float4>(), d->emissive_triangle_count, st);
        tt_scene_stats& stt = s->stats;
        stt.instance_count = d->instance_count;
        stt.emissive_count = d->emissive_triangle_count;
        if (flat) {
            ds.blas = nullptr;
            ds.tris = s->bvh.flat_tris.as<float4>();
            ds.tlas = s->bvh.flat_nodes_buf.as<uint4>();
            ds.has_tlas = s->bvh.flat_nodes > 0 ? 1u : 0u;
            ds.tlas_bound = s->bvh.flat_bound;
            ds.flat = 1u;
            ds.wide = wide ? 1u : 0u;
            ds.tri_base = wide ? nullptr : s->bvh.flat_tri_base.as<uint32_t>();
            ds.tri_record = wide ? nullptr : s->bvh.flat_tri_record.as<uint32_t>();
            ds.tri_count = wide ? 0u : (uint32_t)s->bvh.flat_tri_count;
            stt.triangle_count = s->bvh.flat_tri_count;
            stt.tlas_nodes = s->bvh.flat_nodes;
            stt.tlas_levels = s->bvh.flat_levels;
            stt.accel = wide ? TT_ACCEL_FLAT_WIDE : TT_ACCEL_FLAT;
        } else {
            ds.blas = s->bvh.blas.as<uint4>();
            ds.tris = s->bvh.tris.as<float4>();
            ds.tlas = s->bvh.tlas.as<uint4>();
            ds.has_tlas = s->bvh.tlas_nodes > 0 ? 1u : 0u;
            ds.tlas_bound = s->bvh.tlas_bound;
            ds.flat = 0u;
            ds.wide = 0u;
            stt.triangle_count = s->bvh.tri_count;
            stt.blas_nodes = s->bvh.blas_nodes;
            stt.tlas_nodes = s->bvh.tlas_nodes;
            stt.blas_levels = s->bvh.blas_levels;
            stt.tlas_levels = s->bvh.tlas_levels;
            stt.accel = TT_ACCEL_TWO_LEVEL;
        }
        stt.device_bytes = s->positions.bytes + s->indices.bytes + s->vertices.bytes + s->materials.bytes + s->meshes.bytes +
                           s->instances.bytes + s->emissive.bytes + s->inst_xform.bytes + s->inst_bucket.bytes + s->bvh.blas.bytes +
                           s->bvh.tris.bytes + s->bvh.tlas.bytes + s->bvh.flat_nodes_buf.bytes +
                           s->bvh.flat_tris.bytes + s->light_rec.bytes;
        stt.max_stack = need_stack;
        Pool& p = ctx->pools[TT_LIFETIME_SCENE];
        p.scenes.push_back(std::move(s));
        *out = make_handle(TT_LIFETIME_SCENE, KIND_SCENE, p.epoch, (uint32_t)(p.scenes.size() - 1));
    });
}

int32_t tt_scene_update_instances(tt_context* ctx, tt_handle scene, const tt_instance* instances, uint32_t count) {
    return guarded([&] {
        require(ctx && (count == 0 || instances), "null argument");
        use_device(ctx);
        SceneRes* s = lookup<SceneRes>(ctx, scene, KIND_SCENE);
        require(count == s->host_instances.size(), "instance count must equal the scene's");
        for (uint32_t i = 0; i < count; ++i) {
            const tt_instance &a = instances[i], &b = s->host_instances[i];
            require(a.mesh_index == b.mesh_index && a.index_offset == b.index_offset &&
                        a.vertex_offset == b.vertex_offset && a.material_index == b.material_index,
                    "an update may change transforms only (mesh, material and offsets stay)");
            for (int k = 0; k < 16; ++k)
                require(std::isfinite(a.transform[k]) && std::isfinite(a.inverse_transform[k]) &&
                            std::isfinite(a.normal_transform[k]),
                        "instance matrices must be finite");
        }
        cudaStream_t st = ctx->stream;
        if (count) {
            check_cuda(cudaMemcpyAsync(s->instances.ptr, instances, sizeof(tt_instance) * count, cudaMemcpyHostToDevice, st),
                       "instances");
            std::vector<float4> xf(4ull * count);
            for (uint32_t i = 0; i < count; ++i) {
                const float* m = instances[i].inverse_transform;
                for (int r = 0; r < 3; ++r) xf[4ull * i + r] = make_float4(m[r], m[4 + r], m[8 + r], m[12 + r]);
                uint32_t w[4] = {instances[i].mesh_index, instances[i].material_index, instances[i].index_offset,
                                 instances[i].vertex_offset};
                std::memcpy(&xf[4ull * i + 3], w, 16);
            }
            check_cuda(cudaMemcpyAsync(s->inst_xform.ptr, xf.data(), 16ull * xf.size(), cudaMemcpyHostToDevice, st),
                       "instance rows");
            launch_light_records(s->dev, s->light_rec.as<float4>(), s->dev.emissive_count, st);
            if (s->bvh.wide) {
                // quantised child boxes cannot be refitted in place: the wide structure is rebuilt
                // (same build as tt_scene_create, over the moved instances)
                BvhResult nb;
                BuildInput bi{s->positions.as<int16_t>(), s->indices.as<uint32_t>(), s->host_meshes.data(),
                              (uint32_t)s->host_meshes.size(), instances, count};
                build_scene_bvh(bi, st, BLAS_LEAF_MAX, true, true, nb);
                uint64_t need = structure_stack_need(nb);
                if (need > (uint64_t)TRAVERSAL_STACK)
                    fail(TT_ERR_OVERFLOW, "updated BVH is too deep for the traversal stack (" + std::to_string(need) +
                                              " entries needed); the scene keeps its previous structure");
                s->bvh = std::move(nb);
                s->dev.tris = s->bvh.flat_tris.as<float4>();
                s->dev.tlas = s->bvh.flat_nodes_buf.as<uint4>();
                s->dev.stack_need = (uint32_t)need;
                s->stats.tlas_nodes = s->bvh.flat_nodes;
                s->stats.tlas_levels = s->bvh.flat_levels;
                s->stats.max_stack = need;
            } else {
                refit_scene_bvh(s->instances.as<tt_instance>(), st, s->bvh);  // synchronises the stream
            }
            s->dev.tlas_bound = s->bvh.flat ? s->bvh.flat_bound : s->bvh.tlas_bound;
            s->host_instances.assign(instances, instances + count);
            // emitted powers follow the new world-space areas
            tt_scene_desc ld{};
            ld.instances = s->host_instances.data();
            ld.instance_count = count;
            ld.materials = s->host_materials.data();
            ld.material_count = (uint32_t)s->host_materials.size();
            ld.emissive_triangles = s->host_emissive.data();
            ld.emissive_triangle_count = (uint32_t)s->host_emissive.size();
            std::vector<float4> alias = light_alias_table(&ld);
            check_cuda(cudaMemcpyAsync(s->light_alias.ptr, alias.data(), 16ull * alias.size(), cudaMemcpyHostToDevice, st),
                       "light alias table");
            check_cuda(cudaStreamSynchronize(st), "light alias table");
        }
    });
}

int32_t tt_scene_stats_get(tt_context* ctx, tt_handle scene, tt_scene_stats* out) {
    return guarded([&] {
        require(ctx && out, "null argument");
        *out = lookup<SceneRes>(ctx, scene, KIND_SCENE)->stats;
    });
}

int32_t tt_mesh_ingest(tt_context* ctx, const tt_mesh_data* mesh, uint32_t vertex_offset, uint32_t index_offset,
                       int16_t* positions, tt_vertex* vertices, tt_mesh* mesh_out) {
    return guarded([&] {
        require(ctx && mesh && mesh_out, "null argument");
        require(mesh->vertex_count == 0 || (mesh->positions && positions && vertices), "null array");
        require(mesh->index_count == 0 || mesh->indices, "null indices");
        use_device(ctx);
        mesh_ingest(*mesh, vertex_offset, index_offset, positions, vertices, mesh_out, ctx->stream);
    });
}

int32_t tt_emissive_extract(tt_context* ctx, const tt_emissive_source* source, tt_emissive_triangle* out,
                            uint64_t capacity, uint64_t* count) {
    return guarded([&] {
        require(ctx && source && count, "null argument");
        const tt_emissive_source& s = *source;
        require(s.model_count == 0 || (s.model_mesh && s.model_instance && s.meshes), "null model arrays");
        require((s.vertex_count == 0 || (s.positions && s.vertices)) && (s.index_count == 0 || s.indices),
                "null scene arrays");
        std::vector<uint64_t> first;
        uint64_t total = emissive_count(s, first);
        *count = total;
        if (total > capacity) fail(TT_ERR_OVERFLOW, "emissive output capacity too small");
        require(total == 0 || out, "null output");
        use_device(ctx);
        emissive_extract(s, out, ctx->stream);
    });
}

int32_t tt_scene_bvh_download(tt_context* ctx, tt_handle scene, void* blas, uint64_t blas_bytes, void* tris,
                              uint64_t tri_bytes, void* tlas, uint64_t tlas_bytes) {
    return guarded([&] {
        require(ctx, "null context");
        use_device(ctx);
        SceneRes* s = lookup<SceneRes>(ctx, scene, KIND_SCENE);
        const tt_scene_stats& stt = s->stats;
        uint64_t node_bytes = s->bvh.wide ? 80ull : 128ull;
        require(blas_bytes == stt.blas_nodes * 128ull && tri_bytes == stt.triangle_count * 48ull &&
                    tlas_bytes == stt.tlas_nodes * node_bytes,
                "byte counts must match tt_scene_stats");
        bool flat = s->bvh.flat;
        const void* src_tris = flat ? s->bvh.flat_tris.ptr : s->bvh.tris.ptr;
        const void* src_tlas = flat ? s->bvh.flat_nodes_buf.ptr : s->bvh.tlas.ptr;
        if (blas && blas_bytes)
            check_cuda(cudaMemcpyAsync(blas, s->bvh.blas.ptr, blas_bytes, cudaMemcpyDeviceToHost, ctx->stream), "copy");
        if (tris && tri_bytes)
            check_cuda(cudaMemcpyAsync(tris, src_tris, tri_bytes, cudaMemcpyDeviceToHost, ctx->stream), "copy");
        if (tlas && tlas_bytes)
            check_cuda(cudaMemcpyAsync(tlas, src_tlas, tlas_bytes, cudaMemcpyDeviceToHost, ctx->stream), "copy");
        sync(ctx);
    });
}

int32_t tt_render(tt_context* ctx, tt_handle scene, const tt_constants* constants, tt_handle target) {
    return guarded([&] { render_impl(ctx, scene, constants, target, false, nullptr); });
}

int32_t tt_render_counted(tt_context* ctx, tt_handle scene, const tt_constants* constants, tt_handle target,
                          tt_traversal_counters* out) {
    return guarded([&] {
        require(out != nullptr, "null counters");
        render_impl(ctx, scene, constants, target, true, out);
    });
}

int32_t tt_tonemap(tt_context* ctx, tt_handle image, const tt_constants* constants, uint32_t format,
                   void* host_out, uint64_t bytes) {
    return guarded([&] {
        require(ctx && constants && host_out, "null argument");
        require(format == TT_FORMAT_RGBA32F || format == TT_FORMAT_RGBA8_UNORM, "unknown format");
        use_device(ctx);
        ImageRes* img = lookup<ImageRes>(ctx, image, KIND_IMAGE);
        uint64_t n = (uint64_t)img->width * img->height;
        uint64_t need = n * (format == TT_FORMAT_RGBA32F ? 16ull : 4ull);
        require(bytes == need, "byte count does not match the image and format");
        void* d = nullptr;
        check_cuda(cudaMallocAsync(&d, need, ctx->stream), "cudaMallocAsync");
        check_cuda(cudaEventRecord(ctx->ev_post[0], ctx->stream), "event");
        launch_tonemap(img->buf.as<float4>(), n, constants->tonemap, format, d, ctx->stream);
        check_cuda(cudaGetLastError(), "tonemap launch");
        check_cuda(cudaEventRecord(ctx->ev_post[1], ctx->stream), "event");
        ctx->post_timed = true;
        check_cuda(cudaMemcpyAsync(host_out, d, need, cudaMemcpyDeviceToHost, ctx->stream), "download");
        check_cuda(cudaFreeAsync(d, ctx->stream), "cudaFreeAsync");
        sync(ctx);
    });
}

int32_t tt_set_option(tt_context* ctx, uint32_t option, uint64_t value) {
    return guarded([&] {
        require(ctx, "null context");
        if (option == TT_OPTION_INTEGRATOR) {
            require(value == TT_INTEGRATOR_WAVEFRONT || value == TT_INTEGRATOR_MEGAKERNEL, "unknown integrator");
            ctx->integrator = (uint32_t)value;
        } else if (option == TT_OPTION_WAVEFRONT_SLOTS) {
            require(value <= (1ull << 26), "wavefront slot count above 2^26");
            ctx->wavefront_slots = (uint32_t)value;
        } else if (option == TT_OPTION_REFILL_LANES) {
            require(value >= 1 && value <= 32, "refill lanes must be in 1..32");
            ctx->refill_lanes = (uint32_t)value;
        } else if (option == TT_OPTION_TRACE_BLOCKS_PER_SM) {
            require(value <= 64, "trace blocks per SM above 64");
            ctx->trace_blocks_per_sm = (uint32_t)value;
        } else if (option == TT_OPTION_LIGHT_VISIBILITY) {
            require(value == TT_LIGHT_VISIBILITY_HASH || value == TT_LIGHT_VISIBILITY_TRIANGLE,
                    "unknown light visibility");
            ctx->light_visibility = (uint32_t)value;
        } else if (option == TT_OPTION_LIGHT_SELECTION) {
            require(value == TT_LIGHT_SELECTION_UNIFORM || value == TT_LIGHT_SELECTION_POWER, "unknown light selection");
            ctx->light_selection = (uint32_t)value;
        } else if (option == TT_OPTION_PRIMARY_VISIBILITY) {
            require(value == TT_PRIMARY_TRAVERSE || value == TT_PRIMARY_RASTER, "unknown primary visibility");
            ctx->primary = (uint32_t)value;
        } else if (option == TT_OPTION_RADIANCE_CACHE) {
            require(value <= 1, "radiance cache is 0 or 1");
            ctx->cache.enabled = value != 0;
        } else if (option == TT_OPTION_GRAPHS) {
            require(value <= 1, "graphs is 0 or 1");
            ctx->graphs = value != 0;
        } else if (option == TT_OPTION_STAGE_TIMING) {
            require(value <= 1, "stage timing is 0 or 1");
            ctx->stage_timing = value != 0;
        } else if (option == TT_OPTION_ACCEL) {
            require(value == TT_ACCEL_AUTO || value == TT_ACCEL_FLAT || value == TT_ACCEL_TWO_LEVEL ||
                        value == TT_ACCEL_FLAT_WIDE,
                    "unknown acceleration structure");
            ctx->accel = (uint32_t)value;
        } else {
            fail(TT_ERR_INVALID_ARGUMENT, "unknown option");
        }
    });
}

int32_t tt_autotune(tt_context* ctx, tt_handle scene, const tt_constants* constants, tt_handle target,
                    tt_tune_result* out) {
    return guarded([&] {
        require(ctx && constants && out, "null argument");
        use_device(ctx);
        require(ctx->integrator == TT_INTEGRATOR_WAVEFRONT, "the autotuner tunes the wavefront integrator");
        bool timing = ctx->stage_timing;
        ctx->stage_timing = false;
        *out = tt_tune_result{};
        // integrate time of one render (the fastest of two, after a warm-up render)
        auto measure = [&]() -> float {
            float best = INFINITY;
            for (int k = 0; k < 3; ++k) {
                render_impl(ctx, scene, constants, target, false, nullptr);
                sync(ctx);
                float ms = 0.0f;
                check_cuda(cudaEventElapsedTime(&ms, ctx->ev_integrate[0], ctx->ev_integrate[1]), "elapsed");
                if (k > 0) best = std::min(best, ms);
                out->renders++;
            }
            return best;
        };
        if (ctx->occupancy_sms == 0) trace_occupancy(&ctx->occupancy_sms, &ctx->occupancy_blocks);
        out->default_ms = measure();
        float best = out->default_ms;
        auto tune = [&](uint32_t& option, std::vector<uint32_t> candidates) {
            uint32_t keep = option;
            for (uint32_t v : candidates) {
                if (v == keep) continue;
                option = v;
                float ms = measure();
                if (ms < best) {
                    best = ms;
                    keep = v;
                }
            }
            option = keep;
        };
        uint64_t items = (uint64_t)constants->screen_size[0] * constants->screen_size[1] *
                         std::min<uint32_t>(constants->sample_count, WAVEFRONT_MAX_CHUNK_SPP);
        std::vector<uint32_t> slots;
        for (uint32_t s = 1u << 18; s <= (1u << 25); s <<= 1)
            if (s <= std::max<uint64_t>(items, 1u << 18)) slots.push_back(s);
        if (ctx->wavefront_slots == 0) ctx->wavefront_slots = WAVEFRONT_DEFAULT_SLOTS;
        tune(ctx->wavefront_slots, slots);
        tune(ctx->refill_lanes, {8u, 12u, 16u, 20u, 24u, 28u});
        std::vector<uint32_t> blocks;
        for (int b = ctx->occupancy_blocks; b >= 1 && b >= ctx->occupancy_blocks - 2; --b) blocks.push_back((uint32_t)b);
        if (ctx->trace_blocks_per_sm == 0) ctx->trace_blocks_per_sm = (uint32_t)ctx->occupancy_blocks;
        tune(ctx->trace_blocks_per_sm, blocks);
        render_impl(ctx, scene, constants, target, false, nullptr);  // leave the tuned image in the target
        out->renders++;
        ctx->stage_timing = timing;
        out->slots = ctx->wavefront_slots;
        out->refill_lanes = ctx->refill_lanes;
        out->trace_blocks_per_sm = ctx->trace_blocks_per_sm;
        out->best_ms = best;
    });
}

int32_t tt_restir_configure(tt_context* ctx, const tt_restir_config* config) {
    return guarded([&] {
        require(ctx && config, "null argument");
        require(config->candidates >= 1 && config->candidates <= 1024, "candidates must be in 1..1024");
        require(config->temporal_m_cap >= 0.0f && std::isfinite(config->temporal_m_cap), "bad temporal M cap");
        require(config->spatial_neighbours <= 64, "at most 64 spatial neighbours");
        require(config->spatial_radius >= 0.0f && config->spatial_radius <= 4096.0f, "bad spatial radius");
        ctx->restir.config = *config;
    });
}

int32_t tt_restir_reset(tt_context* ctx) {
    return guarded([&] {
        require(ctx, "null context");
        ctx->restir.history.valid = 0u;
    });
}

int32_t tt_render_restir(tt_context* ctx, tt_handle scene, const tt_constants* constants, tt_handle target) {
    return guarded([&] {
        require(ctx && constants, "null argument");
        use_device(ctx);
        SceneRes* s = lookup<SceneRes>(ctx, scene, KIND_SCENE);
        ImageRes* img = lookup<ImageRes>(ctx, target, KIND_IMAGE);
        require(constants->screen_size[0] == img->width && constants->screen_size[1] == img->height,
                "constants.screen_size must equal the target extent");
        RestirState& R = ctx->restir;
        uint64_t WH = (uint64_t)img->width * img->height;
        if (WH != R.pixels) {
            for (auto& b : R.gbuf) b.alloc(64ull * WH);
            for (auto& b : R.final_res) b.alloc(32ull * WH);
            R.initial.alloc(32ull * WH);
            R.temporal.alloc(32ull * WH);
            R.glob.alloc(16ull * LOBE_RECORD * WH);
            R.queue.alloc(4ull * HIT_BUCKETS * WH);
            R.queue_count.alloc(4ull * HIT_BUCKETS);
            R.pixels = WH;
            R.history.valid = 0u;
        }
        RenderParams p;
        p.sc = s->dev;
        p.sc.light_power = ctx->light_selection == TT_LIGHT_SELECTION_POWER ? 1u : 0u;
        p.c = *constants;
        p.target = img->buf.as<float4>();
        p.err = ctx->err_word.as<uint32_t>();
        p.counters = ctx->counters.as<unsigned long long>();
        RestirParams rp;
        rp.gtex = nullptr;
        if (s->dev.textured) {
            if (R.gtex.bytes < 16ull * WH) R.gtex.alloc(16ull * WH);
            rp.gtex = R.gtex.as<float4>();
        }
        rp.gbuf = R.gbuf[R.cur].as<Surface>();
        rp.glob = R.glob.as<float4>();
        rp.prev_gbuf = R.gbuf[R.cur ^ 1u].as<Surface>();
        rp.initial = R.initial.as<Reservoir>();
        rp.queue = R.queue.as<uint32_t>();
        rp.queue_count = R.queue_count.as<uint32_t>();
        rp.temporal = R.temporal.as<Reservoir>();
        rp.final_out = R.final_res[R.cur].as<Reservoir>();
        rp.prev = R.final_res[R.cur ^ 1u].as<Reservoir>();
        rp.history = R.history;
        rp.candidates = R.config.candidates;
        rp.neighbours = R.config.spatial_neighbours;
        rp.m_cap = R.config.temporal_m_cap * (float)R.config.candidates;
        rp.radius = R.config.spatial_radius;
        // the camera rays' hits from rasterised keys (one sample per pixel: the path tracer's
        // first sample) on flat BVH4 scenes
        PrimaryParams pv{};
        bool raster = ctx->primary == TT_PRIMARY_RASTER && s->dev.tri_record && s->dev.tri_count > 0 &&
                      primary_camera(*constants, pv);
        if (raster) {
            if (ctx->occupancy_sms == 0) trace_occupancy(&ctx->occupancy_sms, &ctx->occupancy_blocks);
            primary_buffers(ctx, *constants, s->dev, 1u, pv);
        }
        rp.vis = raster ? pv.key : nullptr;
        rp.vis_ok = raster ? pv.ok : nullptr;
        arm_error_word(ctx);
        StageTimer* timer = begin_stage_timing(ctx);
        check_cuda(cudaEventRecord(ctx->ev_integrate[0], ctx->stream), "event");
        if (raster) {
            WfParams chunk{};  // sample 0 of the frame: chunk_sample0 = 0, one sample
            chunk.chunk_spp = 1u;
            stage_begin(timer, TT_STAGE_PRIMARY, ctx->stream);
            primary_setup(p, pv, ctx->stream);
            primary_chunk(p, pv, chunk, ctx->stream);
            stage_end(timer, ctx->stream);
        }
        render_restir(p, rp, ctx->stream, timer);
        check_cuda(cudaGetLastError(), "restir launch");
        check_cuda(cudaEventRecord(ctx->ev_integrate[1], ctx->stream), "event");
        ctx->integrate_timed = true;
        fetch_error_word(ctx);
        std::memcpy(R.history.camera_position, constants->camera_position, sizeof(R.history.camera_position));
        std::memcpy(R.history.view, constants->view, sizeof(R.history.view));
        std::memcpy(R.history.inverse_proj, constants->inverse_proj, sizeof(R.history.inverse_proj));
        R.history.valid = 1u;
        R.cur ^= 1u;
    });
}

int32_t tt_restir_download(tt_context* ctx, void* reservoirs, uint64_t bytes) {
    return guarded([&] {
        require(ctx && reservoirs, "null argument");
        use_device(ctx);
        RestirState& R = ctx->restir;
        require(R.pixels > 0 && bytes == 32ull * R.pixels, "byte count must equal width * height * 32");
        check_cuda(cudaMemcpyAsync(reservoirs, R.final_res[R.cur ^ 1u].ptr, bytes, cudaMemcpyDeviceToHost, ctx->stream),
                   "download");
        sync(ctx);
    });
}


int32_t tt_cache_configure(tt_context* ctx, const tt_cache_config* config) {
    return guarded([&] {
        require(ctx && config, "null argument");
        require(config->learning_rate > 0.0f && std::isfinite(config->learning_rate), "bad learning rate");
        require(config->terminate_depth >= 1, "terminate_depth must be at least 1");
        require(config->spread_threshold >= 0.0f && std::isfinite(config->spread_threshold), "bad spread threshold");
        use_device(ctx);
        ctx->cache.config = *config;
        ctx->cache.ready = false;
        cache_ready(ctx);
        sync(ctx);
    });
}

int32_t tt_cache_query(tt_context* ctx, const float* queries, uint32_t n, float* radiance) {
    return guarded([&] {
        require(ctx && (n == 0 || (queries && radiance)), "null argument");
        use_device(ctx);
        cache_ready(ctx);
        CacheDevice d = ctx->cache.dev();
        arm_error_word(ctx);
        batch(ctx, queries, 48ull * n, nullptr, 0, radiance, 12ull * n, [&](void* din, void*, void* dout) {
            cache_infer(d, static_cast<const CacheQuery*>(din), n, static_cast<float*>(dout),
                        ctx->err_word.as<uint32_t>(), ctx->stream);
        });
        fetch_error_word(ctx);
        sync(ctx);
    });
}

int32_t tt_cache_train(tt_context* ctx, const float* queries, const float* targets, uint32_t n, float* loss) {
    return guarded([&] {
        require(ctx && (n == 0 || (queries && targets)), "null argument");
        use_device(ctx);
        cache_ready(ctx);
        CacheState& C = ctx->cache;
        CacheDevice d = C.dev();
        uint32_t step = ++C.step;
        arm_error_word(ctx);
        batch(ctx, queries, 48ull * n, targets, 12ull * n, nullptr, 0, [&](void* din, void* dex, void*) {
            cache_train_step(d, static_cast<const CacheQuery*>(din), static_cast<const float*>(dex), n,
                             C.config.learning_rate, step, ctx->err_word.as<uint32_t>(), ctx->stream);
        });
        fetch_error_word(ctx);
        sync(ctx);
        if (loss) check_cuda(cudaMemcpy(loss, C.loss.ptr, 4, cudaMemcpyDeviceToHost), "loss");
    });
}

int32_t tt_cache_gradients(tt_context* ctx, const float* queries, const float* targets, uint32_t n,
                           float* weight_gradients, float* grid_gradients, float* loss) {
    return guarded([&] {
        require(ctx && weight_gradients && (n == 0 || (queries && targets)), "null argument");
        use_device(ctx);
        cache_ready(ctx);
        CacheState& C = ctx->cache;
        CacheDevice d = C.dev();
        arm_error_word(ctx);
        cache_clear_gradients(d, ctx->stream);
        check_cuda(cudaMemsetAsync(C.loss.ptr, 0, 4, ctx->stream), "memset");
        batch(ctx, queries, 48ull * n, targets, 12ull * n, nullptr, 0, [&](void* din, void* dex, void*) {
            cache_gradients(d, static_cast<const CacheQuery*>(din), static_cast<const float*>(dex), n,
                            ctx->err_word.as<uint32_t>(), ctx->stream);
        });
        fetch_error_word(ctx);
        check_cuda(cudaMemcpyAsync(weight_gradients, C.w_grad.ptr, 4 * CACHE_PARAMS, cudaMemcpyDeviceToHost,
                                   ctx->stream), "weight gradients");
        if (grid_gradients)
            check_cuda(cudaMemcpyAsync(grid_gradients, C.grid_grad.ptr, 4 * CACHE_GRID_PARAMS, cudaMemcpyDeviceToHost,
                                       ctx->stream), "grid gradients");
        float summed = 0.0f;
        check_cuda(cudaMemcpyAsync(&summed, C.loss.ptr, 4, cudaMemcpyDeviceToHost, ctx->stream), "loss");
        cache_clear_gradients(d, ctx->stream);  // the next training step starts from zero gradients
        sync(ctx);
        if (loss) *loss = summed;
    });
}

int32_t tt_cache_status_get(tt_context* ctx, tt_cache_status* out) {
    return guarded([&] {
        require(ctx && out, "null argument");
        use_device(ctx);
        sync(ctx);
        CacheState& C = ctx->cache;
        *out = tt_cache_status{};
        out->steps = C.step;
        out->pairs = C.last_pairs;
        if (C.ready && C.step > 0) {
            float sum = 0.0f;
            check_cuda(cudaMemcpy(&sum, C.loss.ptr, 4, cudaMemcpyDeviceToHost), "loss");
            uint32_t n = std::min<uint32_t>(16384u, std::max<uint32_t>(C.last_pairs, 1u));
            out->last_loss = sum / (3.0f * (float)n);
        }
    });
}

int32_t tt_cache_parameters(tt_context* ctx, float* grid, float* weights) {
    return guarded([&] {
        require(ctx && weights, "null argument");
        use_device(ctx);
        cache_ready(ctx);
        CacheState& C = ctx->cache;
        if (grid)
            check_cuda(cudaMemcpyAsync(grid, C.grid.ptr, 4 * CACHE_GRID_PARAMS, cudaMemcpyDeviceToHost, ctx->stream),
                       "grid");
        check_cuda(cudaMemcpyAsync(weights, C.w.ptr, 4 * CACHE_PARAMS, cudaMemcpyDeviceToHost, ctx->stream), "weights");
        sync(ctx);
    });
}

int32_t tt_stage_timings_get(tt_context* ctx, tt_stage_timings* out) {
    return guarded([&] {
        require(ctx && out, "null argument");
        use_device(ctx);
        sync(ctx);
        *out = tt_stage_timings{};
        const StageTimer& t = ctx->stage_timer;
        require(t.count >= 0, "the last render ran without TT_OPTION_STAGE_TIMING");
        for (int i = 0; i < t.count; ++i) {
            float ms = 0.0f;
            check_cuda(cudaEventElapsedTime(&ms, ctx->stage_events[2 * i], ctx->stage_events[2 * i + 1]), "elapsed");
            out->ns[t.stage[i]] += (uint64_t)((double)ms * 1.0e6);
            out->launches[t.stage[i]] += 1;
        }
        out->overflow = t.overflow ? 1u : 0u;
    });
}

int32_t tt_timings_get(tt_context* ctx, tt_timings* out) {
    return guarded([&] {
        require(ctx && out, "null argument");
        use_device(ctx);
        sync(ctx);
        float a = 0.0f, b = 0.0f;
        if (ctx->integrate_timed) check_cuda(cudaEventElapsedTime(&a, ctx->ev_integrate[0], ctx->ev_integrate[1]), "elapsed");
        if (ctx->post_timed) check_cuda(cudaEventElapsedTime(&b, ctx->ev_post[0], ctx->ev_post[1]), "elapsed");
        out->integrate_ns = (uint64_t)((double)a * 1.0e6);
        out->post_process_ns = (uint64_t)((double)b * 1.0e6);
        out->scene_build_ns = (uint64_t)((double)ctx->scene_build_ms * 1.0e6);
    });
}

int32_t tt_bsdf_eval_batch(tt_context* ctx, const tt_material_constants* material, const float* samples,
                           uint32_t n, float* results) {
    return guarded([&] {
        require(ctx && material && (n == 0 || (samples && results)), "null argument");
        batch(ctx, samples, 32ull * n, material, sizeof(tt_material_constants), results, 32ull * n,
              [&](void* din, void* dex, void* dout) {
                  launch_bsdf_eval(static_cast<const tt_material_constants*>(dex), static_cast<const float4*>(din), n,
                                   static_cast<float4*>(dout), ctx->stream);
              });
    });
}

int32_t tt_bsdf_sample_batch(tt_context* ctx, const tt_material_constants* material, const float* samples,
                             uint32_t n, float* results) {
    return guarded([&] {
        require(ctx && material && (n == 0 || (samples && results)), "null argument");
        batch(ctx, samples, 16ull * n, material, sizeof(tt_material_constants), results, 48ull * n,
              [&](void* din, void* dex, void* dout) {
                  launch_bsdf_sample(static_cast<const tt_material_constants*>(dex), static_cast<const float4*>(din),
                                     n, static_cast<float4*>(dout), ctx->stream);
              });
    });
}

int32_t tt_trace_batch(tt_context* ctx, tt_handle scene, const float* rays, uint32_t n, uint32_t flags,
                       uint32_t* hits) {
    return guarded([&] {
        require(ctx && (n == 0 || (rays && hits)), "null argument");
        SceneRes* s = lookup<SceneRes>(ctx, scene, KIND_SCENE);
        arm_error_word(ctx);
        batch(ctx, rays, 32ull * n, nullptr, 0, hits, 32ull * n, [&](void* din, void*, void* dout) {
            launch_trace(s->dev, static_cast<const float4*>(din), n, flags, static_cast<uint4*>(dout),
                         ctx->err_word.as<uint32_t>(), ctx->stream);
            fetch_error_word(ctx);
        });
    });
}

int32_t tt_trace_batch_noalloc(tt_context* ctx, tt_handle scene, const float* rays, uint32_t n, uint32_t flags,
                               uint32_t* hits) {
    return guarded([&] {
        require(ctx && (n == 0 || (rays && hits)), "null argument");
        use_device(ctx);
        SceneRes* s = lookup<SceneRes>(ctx, scene, KIND_SCENE);
        trace_batch_noalloc(ctx->device, s->dev, rays, n, flags, hits, ctx->stream);
        // the stream is synchronised: an error word still pending from an earlier asynchronous
        // call on this context is reported here, as tt_trace_batch reports it
        check_device_errors(ctx);
    });
}

int32_t tt_math_batch(tt_context* ctx, int32_t which, const float* x, uint64_t n, float* y) {
    return guarded([&] {
        require(ctx && (n == 0 || (x && y)), "null argument");
        require(which >= 0 && which <= 4, "unknown function");
        batch(ctx, x, 4ull * n, nullptr, 0, y, 4ull * n, [&](void* din, void*, void* dout) {
            launch_math(which, static_cast<const float*>(din), n, static_cast<float*>(dout), ctx->stream);
        });
    });
}

int32_t tt_texture_sample_batch(tt_context* ctx, tt_handle scene, uint32_t texture, const float* uvl, uint32_t n,
                                float* rgba) {
    return guarded([&] {
        require(ctx && (n == 0 || (uvl && rgba)), "null argument");
        use_device(ctx);
        SceneRes* s = lookup<SceneRes>(ctx, scene, KIND_SCENE);
        require(texture < s->tex_table.bytes / sizeof(DevTexture), "texture index out of range");
        DevScene sc = s->dev;
        batch(ctx, uvl, 12ull * n, nullptr, 0, rgba, 16ull * n, [&](void* din, void*, void* dout) {
            launch_texture_sample(sc, texture, static_cast<const float*>(din), n, static_cast<float4*>(dout),
                                  ctx->stream);
        });
    });
}

int32_t tt_flush_l2(tt_context* ctx) {
    return guarded([&] {
        require(ctx, "null context");
        use_device(ctx);
        if (!ctx->l2_flush.ptr) ctx->l2_flush.alloc(L2_FLUSH_BYTES);
        check_cuda(cudaMemsetAsync(ctx->l2_flush.ptr, (int)(ctx->frame_index & 0xff), L2_FLUSH_BYTES, ctx->stream),
                   "flush");
    });
}

int32_t tt_event_record(tt_context* ctx, uint32_t slot) {
    return guarded([&] {
        require(ctx && slot < (uint32_t)EVENT_SLOTS, "bad argument");
        use_device(ctx);
        check_cuda(cudaEventRecord(ctx->user_events[slot], ctx->stream), "event");
    });
}

int32_t tt_event_elapsed_ms(tt_context* ctx, uint32_t a, uint32_t b, float* ms) {
    return guarded([&] {
        require(ctx && ms && a < (uint32_t)EVENT_SLOTS && b < (uint32_t)EVENT_SLOTS, "bad argument");
        use_device(ctx);
        check_cuda(cudaEventSynchronize(ctx->user_events[b]), "event sync");
        check_cuda(cudaEventElapsedTime(ms, ctx->user_events[a], ctx->user_events[b]), "elapsed");
    });
}

int32_t tt_host_alloc(uint64_t bytes, void** out) {
    return guarded([&] {
        require(out != nullptr, "null argument");
        check_cuda(cudaMallocHost(out, bytes ? bytes : 16), "cudaMallocHost");
    });
}

int32_t tt_host_free(void* p) {
    return guarded([&] {
        if (p) check_cuda(cudaFreeHost(p), "cudaFreeHost");
    });
}

}  // extern "C"
