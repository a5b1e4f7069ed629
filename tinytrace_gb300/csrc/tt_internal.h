// Host-side internals shared by the translation units of libtinytrace_cuda.so.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/tinytrace_cuda.h"

namespace tt {

// Status carrying a message; thrown inside the library and converted to a return code at
// the C ABI boundary.
struct Error {
    int32_t code;
    std::string message;
};
[[noreturn]] void fail(int32_t code, const std::string& message);
void check_cuda(cudaError_t e, const char* what);
// Maps the bits of a device error word (ERR_* of tt_bvh.cuh) to a thrown status; returns when
// no bit is set.  Every path that reads an error word back reports it through this function.
void raise_device_error(uint32_t error_bits);

// A device allocation owned by a resource.
struct DeviceBuffer {
    void* ptr = nullptr;
    size_t bytes = 0;
    DeviceBuffer() = default;
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    DeviceBuffer(DeviceBuffer&& o) noexcept : ptr(o.ptr), bytes(o.bytes) { o.ptr = nullptr; o.bytes = 0; }
    DeviceBuffer& operator=(DeviceBuffer&& o) noexcept;
    ~DeviceBuffer();
    void alloc(size_t n);
    template <class T>
    T* as() const { return static_cast<T*>(ptr); }
};

// Result of the LBVH build for one scene.
struct BvhResult {
    DeviceBuffer blas;   // 128-byte BVH4 nodes
    DeviceBuffer tris;   // 48-byte triangle records (BLAS leaf order)
    DeviceBuffer tlas;   // 128-byte BVH4 nodes
    uint64_t blas_nodes = 0, tlas_nodes = 0, tri_count = 0;
    uint32_t blas_levels = 0, tlas_levels = 0;
    float tlas_bound = 0.0f;  // max |coordinate| of the instance world boxes
    std::vector<uint64_t> tlas_level_start, flat_level_start;  // first node of each level (+ end)
    // single-level BVH over the world boxes of every (instance, triangle) pair; `wide`: its nodes
    // are in the compressed 8-wide format (80-byte nodes, records in the wide order)
    bool flat = false;
    bool wide = false;
    DeviceBuffer flat_nodes_buf;  // 128-byte BVH4 nodes (80-byte wide nodes when `wide`)
    DeviceBuffer flat_tris;       // 48-byte records: object-space vertices, primitive, instance
    uint64_t flat_nodes = 0, flat_tri_count = 0;
    uint32_t flat_levels = 0;
    float flat_bound = 0.0f;      // max |coordinate| of the triangle world boxes
    // flat BVH4 only: first scene triangle index of each instance (instance_count + 1 entries)
    // and the record of each scene triangle index (flat_tri_count entries)
    DeviceBuffer flat_tri_base, flat_tri_record;
};

struct BuildInput {
    const int16_t* positions;     // device
    const uint32_t* indices;      // device
    const tt_mesh* meshes_host;   // host
    uint32_t mesh_count;
    const tt_instance* instances_host;  // host
    uint32_t instance_count;
};

// Thread-local message behind tt_last_error.
void set_last_error(const std::string& message);

// Builds, on `stream`, either the two-level structure (BLAS with one root per mesh, node index
// == mesh index, and TLAS with root 0) or, when `flat`, one BVH over the world boxes of all
// (instance, triangle) pairs (root 0), in BVH4 nodes or, when `wide`, in the compressed 8-wide
// format.
void build_scene_bvh(const BuildInput& in, cudaStream_t stream, int leaf_max, bool flat, bool wide, BvhResult& out);

// Refits the world-space structure (the flat BVH, or the TLAS) to new instance transforms
// (device array `d_instances`), keeping its topology; updates the slab-margin bound.
void refit_scene_bvh(const tt_instance* d_instances, cudaStream_t stream, BvhResult& b);

// Bytes of one texture level of w x h texels (BC formats in 4 x 4 blocks).
inline uint64_t texture_level_bytes(uint32_t format, uint32_t w, uint32_t h) {
    uint64_t blocks = (uint64_t)((w + 3u) / 4u) * ((h + 3u) / 4u);
    switch (format) {
        case TT_TEXTURE_BC1_SRGB: return 8ull * blocks;
        case TT_TEXTURE_BC5_UNORM: return 16ull * blocks;
        case TT_TEXTURE_R8_UNORM: return (uint64_t)w * h;
        default: return 2ull * w * h;  // TT_TEXTURE_R16_FLOAT
    }
}

// In-place exclusive prefix sum of n device u32 values on `stream`.
void exclusive_scan_u32(uint32_t* data, uint64_t n, cudaStream_t stream);

// Scene::insert_mesh (src/asset/mod.rs:89-161) with the per-vertex work on the device: host
// arrays in, snorm16 positions, packed vertices and the mesh record out.
void mesh_ingest(const tt_mesh_data& mesh, uint32_t vertex_offset, uint32_t index_offset, int16_t* out_positions,
                 tt_vertex* out_vertices, tt_mesh* out_mesh, cudaStream_t st);

// Scene::emissive_triangles_in_model (src/asset/mod.rs:163-193) for a list of models.
// emissive_count checks the models' meshes and index ranges and returns the triangle total
// (`first`: the exclusive prefix of the models' triangle counts).
uint64_t emissive_count(const tt_emissive_source& src, std::vector<uint64_t>& first);
void emissive_extract(const tt_emissive_source& src, tt_emissive_triangle* out, cudaStream_t st);

}  // namespace tt
