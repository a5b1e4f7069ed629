// TEST INFRASTRUCTURE — the CPU oracle for the tinytrace rendering hot path (the checker,
// never the product; only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg
// may load it).
//
// Byte layouts of the reference's GPU scene, the RNG, tangent-frame decoding and uniform
// emissive-triangle sampling, restated from the reference GLSL/Rust.
#pragma once

#include <cstdint>

#include "ref_math.h"

namespace ref {

// src/material/material.glsl:10-38 / src/asset/material.rs:203-231 (192 bytes).
struct MaterialConstants {
    v4 base_color, specular_color, transmission_color, coat_color, fuzz_color, emission_color,
        geometry_normal;
    float base_weight, base_metalness, base_diffuse_roughness, specular_weight,
        specular_roughness, specular_roughness_anisotropy, specular_ior, specular_rotation,
        transmission_weight, transmission_depth, coat_weight, coat_roughness,
        coat_roughness_anisotropy, coat_ior, coat_darkening, coat_rotation, fuzz_weight,
        fuzz_roughness, emission_luminance, geometry_opacity;
};
static_assert(sizeof(MaterialConstants) == 192, "MaterialConstants is 192 bytes");

// src/asset/material.rs:268-274 (ProcessedMaterial, 304 bytes).
struct Material {
    MaterialConstants constants;
    uint32_t textures[27];
    uint32_t padding;
};
static_assert(sizeof(Material) == 304, "Material is 304 bytes");

// src/scene.rs:236-246, src/includes/scene.glsl:71-74 (208 bytes). Matrices column-major.
struct Instance {
    float transform[16], inverse_transform[16], normal_transform[16];
    uint32_t vertex_offset, index_offset, material_index, mesh_index;
};
static_assert(sizeof(Instance) == 208, "Instance is 208 bytes");

// src/asset/mod.rs:44-47, src/includes/scene.glsl:18-21 (8 bytes).
struct Vertex {
    uint16_t uv[2];  // f16
    uint32_t tangent_frame;
};

// src/asset/mod.rs:68-73, src/includes/scene.glsl:11-16 (36 bytes).
struct EmissiveTriangle {
    int16_t positions[3][3];
    uint16_t hash;
    uint16_t uv[3][2];  // f16
    uint32_t instance_index;
};
static_assert(sizeof(EmissiveTriangle) == 36, "EmissiveTriangle is 36 bytes");

// src/asset/mod.rs:49-64 (ProcessedMesh, 32 bytes).
struct Mesh {
    float center[3];
    float radius;
    uint32_t vertex_offset, vertex_count, index_offset, index_count;
};

// src/includes/constants.glsl:8-15, src/lib.rs:234-250 (368 bytes).
struct Constants {
    float view[16], proj[16], proj_view[16], inverse_view[16], inverse_proj[16];
    v4 camera_position;
    uint32_t frame_index, accumulated_frame_count, sample_count, bounce_count;
    uint32_t screen_size[2];
    uint32_t tonemap, light_sampling;
};
static_assert(sizeof(Constants) == 368, "Constants is 368 bytes");

constexpr uint32_t LIGHT_SAMPLING_NONE = 1;
constexpr uint32_t LIGHT_SAMPLING_NEXT_EVENT_ESTIMATION = 2;
constexpr uint32_t INVALID_INDEX = 4294967295u;

// column-major 4x4 * (v, w): result.r = m[0][r]*v.x + m[1][r]*v.y + m[2][r]*v.z + m[3][r]*w
inline v4 mat4_mul(const float* m, v4 v) {
    v4 r;
    r.x = m[0] * v.x + m[4] * v.y + m[8] * v.z + m[12] * v.w;
    r.y = m[1] * v.x + m[5] * v.y + m[9] * v.z + m[13] * v.w;
    r.z = m[2] * v.x + m[6] * v.y + m[10] * v.z + m[14] * v.w;
    r.w = m[3] * v.x + m[7] * v.y + m[11] * v.z + m[15] * v.w;
    return r;
}
// mat4x3(m) * vec4(p, 1.0)
inline v3 mat43_point(const float* m, v3 p) {
    return v3{m[0] * p.x + m[4] * p.y + m[8] * p.z + m[12] * 1.0f,
              m[1] * p.x + m[5] * p.y + m[9] * p.z + m[13] * 1.0f,
              m[2] * p.x + m[6] * p.y + m[10] * p.z + m[14] * 1.0f};
}
// mat3(m) * v
inline v3 mat3_vec(const float* m, v3 v) {
    return v3{m[0] * v.x + m[4] * v.y + m[8] * v.z, m[1] * v.x + m[5] * v.y + m[9] * v.z,
              m[2] * v.x + m[6] * v.y + m[10] * v.z};
}

// ---------------------------------------------------------------- RNG (random.glsl:4-50)
inline uint32_t jenkins_hash(uint32_t x) {
    x += x << 10;
    x ^= x >> 6;
    x += x << 3;
    x ^= x >> 11;
    x += x << 15;
    return x;
}
struct Generator {
    uint32_t state;
};
inline Generator init_generator_from_index(uint32_t index, uint32_t frame) {
    return Generator{jenkins_hash(index ^ jenkins_hash(frame))};
}
inline Generator init_generator_from_pixel(uint32_t px, uint32_t py, uint32_t width,
                                           uint32_t frame) {
    return init_generator_from_index(px + py * width, frame);
}
inline float uint_to_unit_float(uint32_t v) { return bitsf(0x3f800000u | (v >> 9)) - 1.0f; }
inline uint32_t xor_shift(uint32_t& s) {
    s ^= s << 13;
    s ^= s >> 17;
    s ^= s << 5;
    return s;
}
inline float random_float(Generator& g) { return uint_to_unit_float(xor_shift(g.state)); }
inline uint32_t random_uint(Generator& g, uint32_t end) { return xor_shift(g.state) % end; }
// GLSL evaluates constructor arguments left to right.
inline v2 random_vec2(Generator& g) {
    float a = random_float(g);
    float b = random_float(g);
    return v2{a, b};
}

// ---------------------------------------------------------------- sample.glsl:7-30
inline v3 sample_triangle(v2 r) {
    r.x = r.x / 2.0f;
    r.y = r.y / 2.0f;
    float offset = r.y - r.x;
    if (offset > 0.0f) r.y += offset;
    else r.x -= offset;
    return v3{r.x, r.y, 1.0f - r.x - r.y};
}
constexpr float PI = 3.1415926535897932f;
constexpr float TAU = 6.283185307179586f;
constexpr float INVERSE_PI = 1.0f / PI;
inline v3 cosine_hemisphere_sample(v2 r) {
    float rr = std::sqrt(r.x);
    float theta = 2.0f * PI * r.y;
    float s, c;
    tsincos(theta, &s, &c);
    float x = rr * c, y = rr * s;
    float z = std::sqrt(fmx(0.0f, 1.0f - x * x - y * y));
    return v3{x, y, z};
}
inline float cosine_hemisphere_density(float n_dot_s) {
    if (n_dot_s <= 1e-6f) return 1e-6f / PI;
    return n_dot_s / PI;
}

// ---------------------------------------------------------------- octahedron.glsl:16-24
inline v3 octahedron_decode(v2 o) {
    v2 s = v2{o.x * 2.0f - 1.0f, o.y * 2.0f - 1.0f};
    v3 n = v3{s.x, s.y, 1.0f - std::fabs(s.x) - std::fabs(s.y)};
    float t = clampf(-n.z, 0.0f, 1.0f);
    n.x += n.x >= 0.0f ? -t : t;
    n.y += n.y >= 0.0f ? -t : t;
    return normalize(n);
}

// ---------------------------------------------------------------- scene.glsl:29-64
inline v3 deterministic_orthonormal_vector(v3 n) {
    if (std::fabs(n.x) > std::fabs(n.z)) return v3{-n.y, n.x, 0.0f};
    return v3{0.0f, -n.z, n.y};
}
inline float dequantize_unorm(uint32_t bits, uint32_t value) {
    return (float)value / (float)((1u << bits) - 1u);
}
inline float dequantize_snorm16(int16_t value) { return (float)(int)value / 32767.0f; }
inline v3 dequantize_snorm3(const int16_t* v) {
    return v3{dequantize_snorm16(v[0]), dequantize_snorm16(v[1]), dequantize_snorm16(v[2])};
}
struct TangentFrame {
    v3 normal, tangent;
    float bitangent_sign;
};
inline TangentFrame decode_tangent_frame(uint32_t enc) {
    TangentFrame tf;
    v2 uv = v2{dequantize_unorm(10, enc & 0x3ffu), dequantize_unorm(10, (enc >> 10) & 0x3ffu)};
    tf.normal = octahedron_decode(uv);
    v3 ortho = deterministic_orthonormal_vector(tf.normal);
    float angle = dequantize_unorm(11, (enc >> 20) & 0x7ffu) * TAU;
    float s, c;
    tsincos(angle, &s, &c);
    tf.tangent = ortho * c + cross(tf.normal, ortho) * s;
    tf.bitangent_sign = (enc >> 31) == 1u ? 1.0f : -1.0f;
    return tf;
}

// ---------------------------------------------------------------- math.glsl:18-64
struct Basis {
    v3 normal, tangent, bitangent;
};
inline v3 transform_to_basis(const Basis& b, v3 d) {
    return normalize(d.x * b.tangent + d.y * b.bitangent + d.z * b.normal);
}
inline v3 transform_from_basis(const Basis& b, v3 d) {
    return normalize(v3{dot(d, b.tangent), dot(d, b.bitangent), dot(d, b.normal)});
}
inline v3 gram_schmidt(v3 n, v3 t) { return normalize(t - n * dot(n, t)); }

inline v3 interp3(v3 b, v3 a0, v3 a1, v3 a2) { return b.x * a0 + b.y * a1 + b.z * a2; }
inline v2 interp2(v3 b, v2 a0, v2 a1, v2 a2) {
    return v2{b.x * a0.x + b.y * a1.x + b.z * a2.x, b.x * a0.y + b.y * a1.y + b.z * a2.y};
}
inline v2 uv_of(const uint16_t* h) { return v2{half_to_float(h[0]), half_to_float(h[1])}; }

// Alias-table entry of one emissive triangle (power-proportional light selection).
struct LightAlias {
    float keep;
    uint32_t alias;
    float pdf;
};

struct SceneView {
    const int16_t* positions;  // [i16;3]
    const uint32_t* indices;
    const Vertex* vertices;
    const Material* materials;
    const Instance* instances;
    const EmissiveTriangle* emissive;
    uint32_t emissive_count;
    const LightAlias* light_alias;  // non-null: pick lights by power
};

// ---------------------------------------------------------------- scene.glsl:107-136
struct DirectLightSample {
    v3 barycentric, position, normal;
    v2 uv;
    uint32_t instance, hash;
    float area, light_probability;
    uint32_t index;  // the emissive triangle drawn
};
inline DirectLightSample sample_random_light(const SceneView& sc, Generator& g) {
    uint32_t index = random_uint(g, sc.emissive_count);
    float light_probability = 1.0f / (float)sc.emissive_count;
    if (sc.light_alias) {  // keep `index` with its probability, else its alias
        float coin = random_float(g);
        if (!(coin < sc.light_alias[index].keep)) index = sc.light_alias[index].alias;
        light_probability = sc.light_alias[index].pdf;
    }
    const EmissiveTriangle& tri = sc.emissive[index];
    v3 bary = sample_triangle(random_vec2(g));
    const float* m = sc.instances[tri.instance_index].transform;
    v3 p0 = mat43_point(m, dequantize_snorm3(tri.positions[0]));
    v3 p1 = mat43_point(m, dequantize_snorm3(tri.positions[1]));
    v3 p2 = mat43_point(m, dequantize_snorm3(tri.positions[2]));
    DirectLightSample s;
    s.area = fmx(0.00001f, 0.5f * length(cross(p1 - p0, p2 - p0)));
    s.normal = normalize(cross(p1 - p0, p2 - p0));
    s.position = interp3(bary, p0, p1, p2);
    s.uv = interp2(bary, uv_of(tri.uv[0]), uv_of(tri.uv[1]), uv_of(tri.uv[2]));
    s.barycentric = bary;
    s.instance = tri.instance_index;
    s.hash = (uint32_t)tri.hash;
    s.light_probability = light_probability;
    s.index = index;
    return s;
}

}  // namespace ref
