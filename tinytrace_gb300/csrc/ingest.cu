// Mesh ingest on the GPU: Scene::insert_mesh of the reference (src/asset/mod.rs:89-161,
// normal.rs:17-62, math/mod.rs:3-41) and Scene::emissive_triangles_in_model
// (src/asset/mod.rs:163-193) for large meshes.
//
// The bounding-sphere centre is the reference's running mean (src/asset/mod.rs:308-321), a
// sequential float recurrence, so it is computed on the host where the positions already are.
// Everything per vertex or per triangle runs on the device:
//   radius      max |p - centre| (non-negative float bits ordered as u32, atomicMax);
//   positions   snorm16 of (p - centre) / radius (round half away from zero, truncate);
//   normals     when absent: per vertex, the sum of the incident triangles'
//               cross(p1 - p0, p2 - p0) in triangle order (the corners of every vertex are
//               listed with a count / scan / fill pass and sorted), then v * (1 / |v|);
//   tangents    when absent: cross(up, n) / |.| with w = +1 (up = +y unless |n.y| >= 0.999);
//   frames      TangentFrame::new: 10+10-bit octahedral normal, 11-bit angle of the tangent
//               around the decoded normal (tatan2), bitangent sign bit;
//   texture coordinates to f16, round to nearest even.
// All float operations are written out in the reference's order and compiled without
// contraction, so the CPU restatement reproduces every bit.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "tt_common.cuh"
#include "tt_internal.h"

namespace tt {
namespace {

unsigned grid_of(uint64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

__global__ void radius_kernel(const float* p, uint32_t n, f3 c, uint32_t* out_bits) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    f3 d = f3{p[3ull * i], p[3ull * i + 1], p[3ull * i + 2]} - c;
    float len = sqrtf(dot(d, d));
    // lengths are >= 0 (or NaN, whose bits order above every finite length)
    atomicMax(out_bits, __float_as_uint(len));
}

// src/math/mod.rs:31-37
__device__ __forceinline__ int quantize_snorm16(float v) {
    float round = v >= 0.0f ? 0.5f : -0.5f;
    v = v >= -1.0f ? v : -1.0f;
    v = v <= 1.0f ? v : 1.0f;
    return (int)(v * 32767.0f + round);
}

__global__ void quantize_kernel(const float* p, uint32_t n, f3 c, const uint32_t* radius_bits, int16_t* out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float r = __uint_as_float(*radius_bits);
    out[3ull * i] = (int16_t)quantize_snorm16((p[3ull * i] - c.x) / r);
    out[3ull * i + 1] = (int16_t)quantize_snorm16((p[3ull * i + 1] - c.y) / r);
    out[3ull * i + 2] = (int16_t)quantize_snorm16((p[3ull * i + 2] - c.z) / r);
}

// Corner k (triangle k / 3) counted at its vertex; an index out of range raises the flag.
__global__ void corner_count_kernel(const uint32_t* idx, uint32_t corners, uint32_t n, uint32_t* count,
                                    uint32_t* bad) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= corners) return;
    uint32_t v = idx[k];
    if (v >= n) {
        atomicOr(bad, 1u);
        return;
    }
    atomicAdd(count + v, 1u);
}
__global__ void corner_fill_kernel(const uint32_t* idx, uint32_t corners, const uint32_t* start, uint32_t* fill,
                                   uint32_t* list) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= corners) return;
    uint32_t v = idx[k];  // checked by corner_count_kernel
    list[start[v] + atomicAdd(fill + v, 1u)] = k;
}

// generate_normals (src/asset/mod.rs:226-242) for one vertex: its corners sorted into
// triangle order, the triangles' cross products summed in that order, then normalised.
__global__ void normals_kernel(const float* p, const uint32_t* idx, uint32_t n, const uint32_t* start,
                               const uint32_t* count, uint32_t* list, float* normals) {
    uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    uint32_t* l = list + start[v];
    uint32_t k = count[v];
    for (uint32_t a = 1; a < k; ++a) {  // insertion sort: a vertex has few corners
        uint32_t x = l[a];
        uint32_t b = a;
        while (b > 0 && l[b - 1] > x) {
            l[b] = l[b - 1];
            --b;
        }
        l[b] = x;
    }
    f3 s = f3{0.0f, 0.0f, 0.0f};
    for (uint32_t a = 0; a < k; ++a) {
        uint32_t t = l[a] / 3u;
        uint32_t i0 = idx[3 * t], i1 = idx[3 * t + 1], i2 = idx[3 * t + 2];
        f3 p0 = f3{p[3ull * i0], p[3ull * i0 + 1], p[3ull * i0 + 2]};
        f3 p1 = f3{p[3ull * i1], p[3ull * i1 + 1], p[3ull * i1 + 2]};
        f3 p2 = f3{p[3ull * i2], p[3ull * i2 + 1], p[3ull * i2 + 2]};
        s = s + cross(p1 - p0, p2 - p0);
    }
    f3 nr = normalize(s);
    normals[3ull * v] = nr.x;
    normals[3ull * v + 1] = nr.y;
    normals[3ull * v + 2] = nr.z;
}

// src/math/mod.rs:24-29
__device__ __forceinline__ uint32_t quantize_unorm(float v, int bits) {
    float scale = (float)((1 << bits) - 1);
    v = v >= 0.0f ? v : 0.0f;
    v = v <= 1.0f ? v : 1.0f;
    return (uint32_t)(int)(v * scale + 0.5f);
}
// f32::signum: +1 for +0, -1 for -0
__device__ __forceinline__ float signum(float v) { return signbit(v) ? -1.0f : 1.0f; }

// TangentFrame::new (src/asset/normal.rs:17-36) with encode_octahedron / decode_octahedron
// (src/math/mod.rs:3-22), orthonormal (normal.rs:55-62) and angle_around_normal (normal.rs:41-52).
__device__ uint32_t tangent_frame(f3 n, f3 t, float w) {
    float l1 = fabsf(n.x) + fabsf(n.y) + fabsf(n.z);
    f3 m = n / l1;
    float ox, oy;
    if (m.z < 0.0f) {
        ox = (1.0f - fabsf(m.y)) * signum(m.x) * 0.5f + 0.5f;
        oy = (1.0f - fabsf(m.x)) * signum(m.y) * 0.5f + 0.5f;
    } else {
        ox = m.x * 0.5f + 0.5f;
        oy = m.y * 0.5f + 0.5f;
    }
    uint32_t u = quantize_unorm(ox, 10), v = quantize_unorm(oy, 10);
    float dx = (float)u / 1023.0f * 2.0f - 1.0f, dy = (float)v / 1023.0f * 2.0f - 1.0f;
    f3 d = f3{dx, dy, 1.0f - fabsf(dx) - fabsf(dy)};
    float tz = fminf(fmaxf(-d.z, 0.0f), 1.0f);
    d.x += d.x >= 0.0f ? -tz : tz;
    d.y += d.y >= 0.0f ? -tz : tz;
    d = normalize(d);
    f3 o = fabsf(d.x) > fabsf(d.z) ? normalize(f3{-d.y, d.x, 0.0f}) : normalize(f3{0.0f, -d.z, d.y});
    float angle = tatan2(dot(n, cross(o, t)), dot(o, t));
    if (angle < 0.0f) angle = angle + 2.0f * PI;
    uint32_t a = quantize_unorm(angle / TAU, 11);
    return (w >= 0.0f ? 1u : 0u) << 31 | a << 20 | v << 10 | u;
}

__global__ void frames_kernel(const float* normals, const float* tangents, const float* uv, uint32_t n,
                              tt_vertex* out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    f3 nr = f3{normals[3ull * i], normals[3ull * i + 1], normals[3ull * i + 2]};
    f3 t;
    float w;
    if (tangents) {
        t = f3{tangents[4ull * i], tangents[4ull * i + 1], tangents[4ull * i + 2]};
        w = tangents[4ull * i + 3];
    } else {
        f3 up = fabsf(nr.y) < 0.999f ? f3{0.0f, 1.0f, 0.0f} : f3{1.0f, 0.0f, 0.0f};
        t = normalize(cross(up, nr));
        w = 1.0f;
    }
    tt_vertex vx;
    vx.texture_coordinates[0] = __half_as_ushort(__float2half_rn(uv ? uv[2ull * i] : 0.0f));
    vx.texture_coordinates[1] = __half_as_ushort(__float2half_rn(uv ? uv[2ull * i + 1] : 0.0f));
    vx.tangent_frame = tangent_frame(nr, t, w);
    out[i] = vx;
}

// One thread per emitted triangle; `first` holds the exclusive prefix of the models'
// triangle counts (model_count + 1 entries).
__global__ void emissive_kernel(const int16_t* positions, const tt_vertex* vertices, uint64_t vertex_count,
                                const uint32_t* indices, const tt_mesh* meshes, const uint32_t* model_mesh,
                                const uint32_t* model_instance, const uint64_t* first, uint32_t model_count,
                                tt_emissive_triangle* out, uint32_t* bad) {
    uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= first[model_count]) return;
    uint32_t lo = 0, hi = model_count;  // the model with first[lo] <= t < first[lo + 1]
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) / 2;
        if (first[mid] <= t) lo = mid;
        else hi = mid;
    }
    const tt_mesh me = meshes[model_mesh[lo]];  // mesh indices and index ranges checked on the host
    uint32_t offset = (uint32_t)(t - first[lo]);
    tt_emissive_triangle e;
    for (int c = 0; c < 3; ++c) {
        uint64_t v = (uint64_t)me.vertex_offset + indices[(uint64_t)me.index_offset + 3ull * offset + c];
        if (v >= vertex_count) {
            atomicOr(bad, 1u);
            v = 0;
        }
        e.positions[c][0] = positions[3 * v];
        e.positions[c][1] = positions[3 * v + 1];
        e.positions[c][2] = positions[3 * v + 2];
        e.texture_coordinates[c][0] = vertices[v].texture_coordinates[0];
        e.texture_coordinates[c][1] = vertices[v].texture_coordinates[1];
    }
    e.hash = (uint16_t)(me.index_offset / 3u + offset % 65535u);
    e.instance_index = model_instance[lo];
    out[t] = e;
}

}  // namespace

void mesh_ingest(const tt_mesh_data& mesh, uint32_t vertex_offset, uint32_t index_offset, int16_t* out_positions,
                 tt_vertex* out_vertices, tt_mesh* out_mesh, cudaStream_t st) {
    const uint32_t n = mesh.vertex_count;
    const float* positions = mesh.positions;
    // the reference's running mean (src/asset/mod.rs:308-317), in its order
    f3 c = f3{0.0f, 0.0f, 0.0f};
    for (uint32_t i = 0; i < n; ++i) {
        float k = (float)(i + 1u);
        c.x = c.x + (positions[3ull * i] - c.x) / k;
        c.y = c.y + (positions[3ull * i + 1] - c.y) / k;
        c.z = c.z + (positions[3ull * i + 2] - c.z) / k;
    }
    std::vector<uint32_t> sequence;
    const uint32_t* indices = mesh.indices;
    uint32_t m = mesh.index_count;
    if (!indices) {
        sequence.resize(n);
        for (uint32_t i = 0; i < n; ++i) sequence[i] = i;
        indices = sequence.data();
        m = n;
    }
    if (!mesh.normals && m % 3u != 0u) fail(TT_ERR_INVALID_ARGUMENT, "index count is not a multiple of 3");

    DeviceBuffer d_pos, d_idx, d_nrm, d_tan, d_uv, d_q, d_vtx, d_word;
    d_word.alloc(8);  // [0] radius bits, [1] bad-index flag
    check_cuda(cudaMemsetAsync(d_word.ptr, 0, 8, st), "memset");
    uint32_t* radius_bits = d_word.as<uint32_t>();
    uint32_t* bad = radius_bits + 1;
    if (n) {
        d_pos.alloc(12ull * n);
        check_cuda(cudaMemcpyAsync(d_pos.ptr, positions, 12ull * n, cudaMemcpyHostToDevice, st), "positions");
        radius_kernel<<<grid_of(n, 256), 256, 0, st>>>(d_pos.as<float>(), n, c, radius_bits);
        d_q.alloc(6ull * n);
        quantize_kernel<<<grid_of(n, 256), 256, 0, st>>>(d_pos.as<float>(), n, c, radius_bits, d_q.as<int16_t>());
        d_nrm.alloc(12ull * n);
    }
    if (mesh.normals && n) {
        check_cuda(cudaMemcpyAsync(d_nrm.ptr, mesh.normals, 12ull * n, cudaMemcpyHostToDevice, st), "normals");
    } else if (n) {
        DeviceBuffer count, start, fill, list;
        count.alloc(4ull * n);
        fill.alloc(4ull * n);
        start.alloc(4ull * n);
        check_cuda(cudaMemsetAsync(count.ptr, 0, 4ull * n, st), "memset");
        check_cuda(cudaMemsetAsync(fill.ptr, 0, 4ull * n, st), "memset");
        if (m) {
            d_idx.alloc(4ull * m);
            list.alloc(4ull * m);
            check_cuda(cudaMemcpyAsync(d_idx.ptr, indices, 4ull * m, cudaMemcpyHostToDevice, st), "indices");
            corner_count_kernel<<<grid_of(m, 256), 256, 0, st>>>(d_idx.as<uint32_t>(), m, n, count.as<uint32_t>(),
                                                                 bad);
        }
        uint32_t flag = 0;
        check_cuda(cudaMemcpyAsync(&flag, bad, 4, cudaMemcpyDeviceToHost, st), "flag");
        check_cuda(cudaStreamSynchronize(st), "ingest");
        if (flag) fail(TT_ERR_INVALID_ARGUMENT, "mesh index out of range");
        check_cuda(cudaMemcpyAsync(start.ptr, count.ptr, 4ull * n, cudaMemcpyDeviceToDevice, st), "counts");
        exclusive_scan_u32(start.as<uint32_t>(), n, st);
        if (m)
            corner_fill_kernel<<<grid_of(m, 256), 256, 0, st>>>(d_idx.as<uint32_t>(), m, start.as<uint32_t>(),
                                                                fill.as<uint32_t>(), list.as<uint32_t>());
        normals_kernel<<<grid_of(n, 256), 256, 0, st>>>(d_pos.as<float>(), d_idx.as<uint32_t>(), n,
                                                        start.as<uint32_t>(), count.as<uint32_t>(),
                                                        list.as<uint32_t>(), d_nrm.as<float>());
        check_cuda(cudaStreamSynchronize(st), "ingest normals");  // before the local buffers are freed
    }
    if (mesh.tangents && n) {
        d_tan.alloc(16ull * n);
        check_cuda(cudaMemcpyAsync(d_tan.ptr, mesh.tangents, 16ull * n, cudaMemcpyHostToDevice, st), "tangents");
    }
    if (mesh.texture_coordinates && n) {
        d_uv.alloc(8ull * n);
        check_cuda(cudaMemcpyAsync(d_uv.ptr, mesh.texture_coordinates, 8ull * n, cudaMemcpyHostToDevice, st), "uv");
    }
    if (n) {
        d_vtx.alloc(8ull * n);
        frames_kernel<<<grid_of(n, 256), 256, 0, st>>>(d_nrm.as<float>(), mesh.tangents ? d_tan.as<float>() : nullptr,
                                                       mesh.texture_coordinates ? d_uv.as<float>() : nullptr, n,
                                                       d_vtx.as<tt_vertex>());
        check_cuda(cudaMemcpyAsync(out_positions, d_q.ptr, 6ull * n, cudaMemcpyDeviceToHost, st), "positions");
        check_cuda(cudaMemcpyAsync(out_vertices, d_vtx.ptr, 8ull * n, cudaMemcpyDeviceToHost, st), "vertices");
    }
    uint32_t words[2] = {0u, 0u};
    check_cuda(cudaMemcpyAsync(words, d_word.ptr, 8, cudaMemcpyDeviceToHost, st), "radius");
    check_cuda(cudaStreamSynchronize(st), "ingest");
    check_cuda(cudaGetLastError(), "ingest kernels");
    float radius;
    std::memcpy(&radius, &words[0], 4);
    if (n && !(std::isfinite(c.x) && std::isfinite(c.y) && std::isfinite(c.z) && std::isfinite(radius) &&
               radius > 0.0f))
        fail(TT_ERR_INVALID_ARGUMENT, "degenerate or non-finite bounding sphere");
    out_mesh->bounding_sphere_center[0] = c.x;
    out_mesh->bounding_sphere_center[1] = c.y;
    out_mesh->bounding_sphere_center[2] = c.z;
    out_mesh->bounding_sphere_radius = radius;
    out_mesh->vertex_offset = vertex_offset;
    out_mesh->vertex_count = n;
    out_mesh->index_offset = index_offset;
    out_mesh->index_count = m;
}

uint64_t emissive_count(const tt_emissive_source& s, std::vector<uint64_t>& first) {
    first.assign(s.model_count + 1ull, 0);
    for (uint32_t k = 0; k < s.model_count; ++k) {
        if (s.model_mesh[k] >= s.mesh_count) fail(TT_ERR_INVALID_ARGUMENT, "model mesh index out of range");
        const tt_mesh& me = s.meshes[s.model_mesh[k]];
        if ((uint64_t)me.index_offset + me.index_count > s.index_count)
            fail(TT_ERR_INVALID_ARGUMENT, "mesh index range out of range");
        first[k + 1] = first[k] + me.index_count / 3u;
    }
    if (first[s.model_count] && s.vertex_count == 0) fail(TT_ERR_INVALID_ARGUMENT, "emissive source without vertices");
    return first[s.model_count];
}

void emissive_extract(const tt_emissive_source& s, tt_emissive_triangle* out, cudaStream_t st) {
    std::vector<uint64_t> first;
    uint64_t total = emissive_count(s, first);
    if (total == 0) return;
    DeviceBuffer d_pos, d_vtx, d_idx, d_mesh, d_mm, d_mi, d_first, d_out, d_bad;
    d_pos.alloc(6ull * s.vertex_count);
    d_vtx.alloc(8ull * s.vertex_count);
    d_idx.alloc(4ull * s.index_count);
    d_mesh.alloc(sizeof(tt_mesh) * s.mesh_count);
    d_mm.alloc(4ull * s.model_count);
    d_mi.alloc(4ull * s.model_count);
    d_first.alloc(8ull * first.size());
    d_out.alloc(sizeof(tt_emissive_triangle) * total);
    d_bad.alloc(4);
    check_cuda(cudaMemsetAsync(d_bad.ptr, 0, 4, st), "memset");
    check_cuda(cudaMemcpyAsync(d_pos.ptr, s.positions, 6ull * s.vertex_count, cudaMemcpyHostToDevice, st), "h2d");
    check_cuda(cudaMemcpyAsync(d_vtx.ptr, s.vertices, 8ull * s.vertex_count, cudaMemcpyHostToDevice, st), "h2d");
    check_cuda(cudaMemcpyAsync(d_idx.ptr, s.indices, 4ull * s.index_count, cudaMemcpyHostToDevice, st), "h2d");
    check_cuda(cudaMemcpyAsync(d_mesh.ptr, s.meshes, sizeof(tt_mesh) * s.mesh_count, cudaMemcpyHostToDevice, st),
               "h2d");
    check_cuda(cudaMemcpyAsync(d_mm.ptr, s.model_mesh, 4ull * s.model_count, cudaMemcpyHostToDevice, st), "h2d");
    check_cuda(cudaMemcpyAsync(d_mi.ptr, s.model_instance, 4ull * s.model_count, cudaMemcpyHostToDevice, st), "h2d");
    check_cuda(cudaMemcpyAsync(d_first.ptr, first.data(), 8ull * first.size(), cudaMemcpyHostToDevice, st), "h2d");
    emissive_kernel<<<grid_of(total, 256), 256, 0, st>>>(
        d_pos.as<int16_t>(), d_vtx.as<tt_vertex>(), s.vertex_count, d_idx.as<uint32_t>(), d_mesh.as<tt_mesh>(),
        d_mm.as<uint32_t>(), d_mi.as<uint32_t>(), d_first.as<uint64_t>(), s.model_count,
        d_out.as<tt_emissive_triangle>(), d_bad.as<uint32_t>());
    uint32_t bad = 0;
    check_cuda(cudaMemcpyAsync(&bad, d_bad.ptr, 4, cudaMemcpyDeviceToHost, st), "flag");
    check_cuda(cudaMemcpyAsync(out, d_out.ptr, sizeof(tt_emissive_triangle) * total, cudaMemcpyDeviceToHost, st),
               "d2h");
    check_cuda(cudaStreamSynchronize(st), "emissive extract");
    check_cuda(cudaGetLastError(), "emissive kernel");
    if (bad) fail(TT_ERR_INVALID_ARGUMENT, "emissive triangle vertex out of range");
}

}  // namespace tt
