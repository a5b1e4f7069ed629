// TEST INFRASTRUCTURE — the CPU oracle for the tinytrace rendering hot path.
// Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg may load this code.
// It is the checker, never the product.
//
// Scene::insert_mesh (src/asset/mod.rs:89-161) and Scene::emissive_triangles_in_model
// (src/asset/mod.rs:163-193) restated sequentially, as the reference runs them on the CPU:
//   * bounding_sphere (src/asset/mod.rs:308-321): running mean mean + (p - mean) / (i + 1) in
//     f32, radius the largest |p - centre|;
//   * quantize_snorm / quantize_unorm / encode_octahedron / decode_octahedron
//     (src/math/mod.rs:3-37);
//   * generate_normals (src/asset/mod.rs:226-242): face normals added to their three vertices
//     triangle by triangle, then normalize (v * (1 / |v|));
//   * TangentFrame::new (src/asset/normal.rs:17-62) with atan2 replaced by tatan2 (the same
//     function the CUDA kernel evaluates);
//   * generated tangents: cross(up, n) normalised with w = +1, up = +y unless |n.y| >= 0.999,
//     then +x (the reference runs mikktspace, src/asset/mod.rs:244-265; that crate is not
//     available here and the CUDA path documents the same substitute);
//   * f16 texture coordinates rounded to nearest even (half::f16::from_f32).
#pragma once

#include <cmath>
#include <cstdint>
#include <vector>

#include "ref_math.h"

namespace ref {

inline int quantize_snorm(float v, int bits) {
    float scale = (float)((1 << (bits - 1)) - 1);
    float round = v >= 0.0f ? 0.5f : -0.5f;
    v = v >= -1.0f ? v : -1.0f;
    v = v <= 1.0f ? v : 1.0f;
    return (int)(v * scale + round);
}

inline uint32_t quantize_unorm(float v, int bits) {
    float scale = (float)((1 << bits) - 1);
    v = v >= 0.0f ? v : 0.0f;
    v = v <= 1.0f ? v : 1.0f;
    return (uint32_t)(int)(v * scale + 0.5f);
}

inline float signum(float v) { return std::signbit(v) ? -1.0f : 1.0f; }

inline v2 encode_octahedron(v3 n) {
    n = n / (std::fabs(n.x) + std::fabs(n.y) + std::fabs(n.z));
    if (n.z < 0.0f) {
        float wx = (1.0f - std::fabs(n.y)) * signum(n.x);
        float wy = (1.0f - std::fabs(n.x)) * signum(n.y);
        return v2{wx * 0.5f + 0.5f, wy * 0.5f + 0.5f};
    }
    return v2{n.x * 0.5f + 0.5f, n.y * 0.5f + 0.5f};
}

inline v3 decode_octahedron(v2 o) {
    float x = o.x * 2.0f - 1.0f, y = o.y * 2.0f - 1.0f;
    v3 n = v3{x, y, 1.0f - std::fabs(x) - std::fabs(y)};
    float t = clampf(-n.z, 0.0f, 1.0f);
    n.x += n.x >= 0.0f ? -t : t;
    n.y += n.y >= 0.0f ? -t : t;
    return normalize(n);
}

inline v3 orthonormal(v3 n) {
    if (std::fabs(n.x) > std::fabs(n.z)) return normalize(v3{-n.y, n.x, 0.0f});
    return normalize(v3{0.0f, -n.z, n.y});
}

inline uint32_t tangent_frame(v3 normal, v3 tangent, float w) {
    v2 o = encode_octahedron(normal);
    uint32_t u = quantize_unorm(o.x, 10), v = quantize_unorm(o.y, 10);
    v3 a = orthonormal(decode_octahedron(v2{(float)u / 1023.0f, (float)v / 1023.0f}));
    float angle = tatan2(dot(normal, cross(a, tangent)), dot(a, tangent));
    if (angle < 0.0f) angle = angle + 2.0f * PI_1;
    uint32_t q = quantize_unorm(angle / (2.0f * PI_1), 11);
    return (w >= 0.0f ? 1u : 0u) << 31 | q << 20 | v << 10 | u;
}

struct IngestVertex {
    uint16_t uv[2];
    uint32_t frame;
};

// Returns 0, or 1 for an index out of range / an index count that is not a multiple of 3
// while normals are generated / a degenerate or non-finite bounding sphere.
inline int mesh_ingest(const float* positions, const float* uv, const uint32_t* indices, const float* normals,
                       const float* tangents, uint32_t n, uint32_t m, int16_t* out_positions,
                       IngestVertex* out_vertices, float* sphere) {
    auto P = [&](uint32_t i) { return v3{positions[3ull * i], positions[3ull * i + 1], positions[3ull * i + 2]}; };
    v3 c = v3{0.0f, 0.0f, 0.0f};
    for (uint32_t i = 0; i < n; ++i) c = c + (P(i) - c) / (float)(i + 1u);
    float r = 0.0f;
    for (uint32_t i = 0; i < n; ++i) {
        float len = length(P(i) - c);
        if (len > r || len != len) r = len;
    }
    sphere[0] = c.x;
    sphere[1] = c.y;
    sphere[2] = c.z;
    sphere[3] = r;
    if (n && !(std::isfinite(c.x) && std::isfinite(c.y) && std::isfinite(c.z) && std::isfinite(r) && r > 0.0f))
        return 1;
    for (uint32_t i = 0; i < n; ++i) {
        v3 q = (P(i) - c) / r;
        out_positions[3ull * i] = (int16_t)quantize_snorm(q.x, 16);
        out_positions[3ull * i + 1] = (int16_t)quantize_snorm(q.y, 16);
        out_positions[3ull * i + 2] = (int16_t)quantize_snorm(q.z, 16);
    }
    std::vector<uint32_t> seq;
    if (!indices) {
        seq.resize(n);
        for (uint32_t i = 0; i < n; ++i) seq[i] = i;
        indices = seq.data();
        m = n;
    }
    std::vector<v3> nrm(n, v3{0.0f, 0.0f, 0.0f});
    if (normals) {
        for (uint32_t i = 0; i < n; ++i) nrm[i] = v3{normals[3ull * i], normals[3ull * i + 1], normals[3ull * i + 2]};
    } else {
        if (m % 3u) return 1;
        for (uint32_t k = 0; k < m; ++k)
            if (indices[k] >= n) return 1;
        for (uint32_t t = 0; t < m / 3u; ++t) {
            uint32_t i0 = indices[3 * t], i1 = indices[3 * t + 1], i2 = indices[3 * t + 2];
            v3 f = cross(P(i1) - P(i0), P(i2) - P(i0));
            nrm[i0] = nrm[i0] + f;
            nrm[i1] = nrm[i1] + f;
            nrm[i2] = nrm[i2] + f;
        }
        for (uint32_t i = 0; i < n; ++i) nrm[i] = normalize(nrm[i]);
    }
    for (uint32_t i = 0; i < n; ++i) {
        v3 t;
        float w;
        if (tangents) {
            t = v3{tangents[4ull * i], tangents[4ull * i + 1], tangents[4ull * i + 2]};
            w = tangents[4ull * i + 3];
        } else {
            v3 up = std::fabs(nrm[i].y) < 0.999f ? v3{0.0f, 1.0f, 0.0f} : v3{1.0f, 0.0f, 0.0f};
            t = normalize(cross(up, nrm[i]));
            w = 1.0f;
        }
        out_vertices[i].uv[0] = float_to_half(uv ? uv[2ull * i] : 0.0f);
        out_vertices[i].uv[1] = float_to_half(uv ? uv[2ull * i + 1] : 0.0f);
        out_vertices[i].frame = tangent_frame(nrm[i], t, w);
    }
    return 0;
}

}  // namespace ref
