// TEST INFRASTRUCTURE — the CPU oracle for the tinytrace rendering hot path (the checker,
// never the product; only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg
// may load it).
//
// Textured materials of src/integrate/integrate.glsl:91-106, 134-154, 219-266: the mip level
// of the primary hit from its texture-coordinate differentials, and textureLod through the
// scene sampler (src/scene.rs:121-128: linear filtering between texels and between mip
// levels, repeat addressing; an explicit LOD, so no anisotropy) for the formats of
// src/asset/texture.rs: BC1 sRGB, BC5 unorm, R8 unorm, R16 float.
//
// The texel values and the filter follow these definitions (the Vulkan sampler does not fix
// palette rounding or weight precision, so they are stated here and the CUDA path follows
// the same ones):
//   BC1  5:6:5 endpoints expanded by bit replication; c0 > c1 (as u16): c2 = (2 c0 + c1 + 1) / 3,
//        c3 = (c0 + 2 c1 + 1) / 3 per 8-bit channel (integer division), otherwise
//        c2 = (c0 + c1 + 1) / 2 and c3 = transparent black; channels to linear through the sRGB
//        curve tabulated for the 256 byte values (in double, rounded to float).
//   BC4  (each BC5 channel) index 0 -> e0 / 255, 1 -> e1 / 255; e0 > e1: k -> ((8 - k) e0 + (k - 1) e1)
//        / 1785; otherwise k = 2..5 -> ((6 - k) e0 + (k - 1) e1) / 1275, 6 -> 0, 7 -> 1.
//   LOD  min(max(lod, 0), levels - 1) with NaN -> 0; the two levels around it blended
//        (1 - f) a + f b when the fraction f is positive.
//   texel  u - floor(u) (0 when not finite) scaled by the level width minus 0.5; floor and
//        fraction; columns wrapped modulo the width; bilinear weights summed in the order
//        (1-a)(1-b) t00, a(1-b) t10, (1-a) b t01, a b t11.
#pragma once

#include <cmath>
#include <cstdint>
#include <vector>

#include "ref_bsdf.h"
#include "ref_scene.h"

namespace ref {

constexpr uint32_t TEX_BC1_SRGB = 1, TEX_BC5_UNORM = 2, TEX_R8_UNORM = 3, TEX_R16_FLOAT = 4;

struct TextureDesc {  // tt_texture
    uint32_t format, width, height, level_count;
    const uint8_t* data;
    uint64_t bytes;
};

struct Texture {
    uint32_t format = 0, width = 0, height = 0;
    std::vector<std::vector<uint8_t>> levels;
};

inline uint64_t texture_level_bytes(uint32_t format, uint32_t w, uint32_t h) {
    uint64_t blocks = (uint64_t)((w + 3) / 4) * ((h + 3) / 4);
    if (format == TEX_BC1_SRGB) return 8 * blocks;
    if (format == TEX_BC5_UNORM) return 16 * blocks;
    if (format == TEX_R8_UNORM) return (uint64_t)w * h;
    return 2ull * w * h;
}

inline const std::vector<float>& srgb_table() {
    static const std::vector<float> t = [] {
        std::vector<float> v(256);
        for (int i = 0; i < 256; ++i) {
            double c = i / 255.0;
            v[i] = (float)(c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4));
        }
        return v;
    }();
    return t;
}

inline uint32_t expand5(uint32_t v) { return (v << 3) | (v >> 2); }
inline uint32_t expand6(uint32_t v) { return (v << 2) | (v >> 4); }

inline float bc4_texel(const uint8_t* b, uint32_t t) {
    uint32_t e0 = b[0], e1 = b[1];
    uint64_t bits = 0;
    for (int k = 0; k < 6; ++k) bits |= (uint64_t)b[2 + k] << (8 * k);
    uint32_t k = (uint32_t)(bits >> (3 * t)) & 7u;
    if (k == 0) return (float)e0 / 255.0f;
    if (k == 1) return (float)e1 / 255.0f;
    if (e0 > e1) return (float)((8 - k) * e0 + (k - 1) * e1) / 1785.0f;
    if (k == 6) return 0.0f;
    if (k == 7) return 1.0f;
    return (float)((6 - k) * e0 + (k - 1) * e1) / 1275.0f;
}

inline v4 texel(const Texture& tx, uint32_t level, uint32_t x, uint32_t y) {
    uint32_t w = tx.width >> level;
    const uint8_t* d = tx.levels[level].data();
    uint32_t bw = (w + 3) / 4;
    uint32_t t = (y % 4) * 4 + (x % 4);
    switch (tx.format) {
        case TEX_BC1_SRGB: {
            const uint8_t* b = d + 8ull * ((uint64_t)(y / 4) * bw + x / 4);
            uint32_t c0 = b[0] | (uint32_t)b[1] << 8, c1 = b[2] | (uint32_t)b[3] << 8;
            uint32_t idx = b[4] | (uint32_t)b[5] << 8 | (uint32_t)b[6] << 16 | (uint32_t)b[7] << 24;
            uint32_t sel = (idx >> (2 * t)) & 3u;
            uint32_t a[3] = {expand5(c0 >> 11), expand6((c0 >> 5) & 63), expand5(c0 & 31)};
            uint32_t e[3] = {expand5(c1 >> 11), expand6((c1 >> 5) & 63), expand5(c1 & 31)};
            uint32_t r[3];
            for (int ch = 0; ch < 3; ++ch) {
                if (sel == 0) r[ch] = a[ch];
                else if (sel == 1) r[ch] = e[ch];
                else if (c0 > c1) r[ch] = sel == 2 ? (2 * a[ch] + e[ch] + 1) / 3 : (a[ch] + 2 * e[ch] + 1) / 3;
                else r[ch] = sel == 2 ? (a[ch] + e[ch] + 1) / 2 : 0;
            }
            const std::vector<float>& s = srgb_table();
            return v4{s[r[0]], s[r[1]], s[r[2]], (c0 <= c1 && sel == 3) ? 0.0f : 1.0f};
        }
        case TEX_BC5_UNORM: {
            const uint8_t* b = d + 16ull * ((uint64_t)(y / 4) * bw + x / 4);
            return v4{bc4_texel(b, t), bc4_texel(b + 8, t), 0.0f, 1.0f};
        }
        case TEX_R8_UNORM:
            return v4{(float)d[(uint64_t)y * w + x] / 255.0f, 0.0f, 0.0f, 1.0f};
        default: {
            uint16_t h = (uint16_t)(d[2ull * ((uint64_t)y * w + x)] | d[2ull * ((uint64_t)y * w + x) + 1] << 8);
            return v4{half_to_float(h), 0.0f, 0.0f, 1.0f};
        }
    }
}

inline int wrap_index(int i, int n) {
    int r = i % n;
    return r < 0 ? r + n : r;
}
inline float wrap_coordinate(float u) {
    float f = u - std::floor(u);
    return std::isfinite(f) ? f : 0.0f;
}
inline v4 add4(v4 a, v4 b) { return v4{a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
inline v4 mul4(v4 a, float s) { return v4{a.x * s, a.y * s, a.z * s, a.w * s}; }

inline v4 sample_level(const Texture& tx, uint32_t level, v2 uv) {
    uint32_t w = tx.width >> level, h = tx.height >> level;
    float x = wrap_coordinate(uv.x) * (float)w - 0.5f;
    float y = wrap_coordinate(uv.y) * (float)h - 0.5f;
    float xf = std::floor(x), yf = std::floor(y);
    float a = x - xf, b = y - yf;
    int xi = (int)xf, yi = (int)yf;
    uint32_t x0 = wrap_index(xi, (int)w), x1 = wrap_index(xi + 1, (int)w);
    uint32_t y0 = wrap_index(yi, (int)h), y1 = wrap_index(yi + 1, (int)h);
    float ia = 1.0f - a, ib = 1.0f - b;
    v4 r = mul4(texel(tx, level, x0, y0), ia * ib);
    r = add4(r, mul4(texel(tx, level, x1, y0), a * ib));
    r = add4(r, mul4(texel(tx, level, x0, y1), ia * b));
    r = add4(r, mul4(texel(tx, level, x1, y1), a * b));
    return r;
}

// textureLod
inline v4 sample_texture(const Texture& tx, v2 uv, float lod) {
    float q = (float)(tx.levels.size() - 1);
    float d = fmn(fmx(lod, 0.0f), q);
    float lf = std::floor(d);
    uint32_t l0 = (uint32_t)lf;
    float f = d - lf;
    v4 r = sample_level(tx, l0, uv);
    if (f > 0.0f) r = add4(mul4(r, 1.0f - f), mul4(sample_level(tx, l0 + 1, uv), f));
    return r;
}

// MaterialTextures slots (src/material/material.glsl:40-68)
enum : int {
    T_BASE_COLOR = 0, T_SPECULAR_COLOR, T_TRANSMISSION_COLOR, T_COAT_COLOR, T_FUZZ_COLOR, T_EMISSION_COLOR,
    T_GEOMETRY_NORMAL, T_BASE_WEIGHT, T_BASE_METALNESS, T_BASE_DIFFUSE_ROUGHNESS, T_SPECULAR_WEIGHT,
    T_SPECULAR_ROUGHNESS, T_SPECULAR_ROUGHNESS_ANISOTROPY, T_SPECULAR_IOR, T_SPECULAR_ROTATION,
    T_TRANSMISSION_WEIGHT, T_TRANSMISSION_DEPTH, T_COAT_WEIGHT, T_COAT_ROUGHNESS, T_COAT_ROUGHNESS_ANISOTROPY,
    T_COAT_IOR, T_COAT_DARKENING, T_COAT_ROTATION, T_FUZZ_WEIGHT, T_FUZZ_ROUGHNESS, T_EMISSION_LUMINANCE,
    T_GEOMETRY_OPACITY
};
constexpr uint32_t NO_TEXTURE = 0xffffffffu;

// load_textures (integrate.glsl:219-266), in its order.
inline MaterialConstants load_textures(const Material& m, const std::vector<Texture>& tex, v2 uv, float lod) {
    MaterialConstants c = m.constants;
    auto fetch = [&](int slot, v4& out) {
        uint32_t i = m.textures[slot];
        if (i == NO_TEXTURE) return false;
        out = sample_texture(tex[i], uv, lod);
        return true;
    };
    v4 rgba;
    if (fetch(T_BASE_COLOR, rgba)) c.base_color = rgba;
    if (fetch(T_SPECULAR_COLOR, rgba)) c.specular_color = rgba;
    if (fetch(T_TRANSMISSION_COLOR, rgba)) c.transmission_color = rgba;
    if (fetch(T_COAT_COLOR, rgba)) c.coat_color = rgba;
    if (fetch(T_FUZZ_COLOR, rgba)) c.fuzz_color = rgba;
    if (fetch(T_GEOMETRY_NORMAL, rgba)) {
        v3 n = octahedron_decode(v2{rgba.x, rgba.y});
        c.geometry_normal = v4{n.x, n.y, n.z, n.x};
    }
    if (fetch(T_BASE_METALNESS, rgba)) c.base_metalness = rgba.x;
    if (fetch(T_BASE_DIFFUSE_ROUGHNESS, rgba)) c.base_diffuse_roughness = rgba.x;
    if (fetch(T_SPECULAR_WEIGHT, rgba)) c.specular_weight = rgba.x;
    if (fetch(T_SPECULAR_ROUGHNESS, rgba)) c.specular_roughness = rgba.x;
    if (fetch(T_SPECULAR_ROUGHNESS_ANISOTROPY, rgba)) c.specular_roughness_anisotropy = rgba.x;
    if (fetch(T_SPECULAR_IOR, rgba)) c.specular_ior = rgba.x;
    if (fetch(T_SPECULAR_ROTATION, rgba)) c.specular_rotation = rgba.x;
    if (fetch(T_TRANSMISSION_WEIGHT, rgba)) c.transmission_weight = rgba.x;
    if (fetch(T_COAT_WEIGHT, rgba)) c.coat_weight = rgba.x;
    if (fetch(T_COAT_DARKENING, rgba)) c.coat_darkening = rgba.x;
    if (fetch(T_COAT_ROTATION, rgba)) c.coat_rotation = rgba.x;
    if (fetch(T_FUZZ_WEIGHT, rgba)) c.fuzz_weight = rgba.x;
    if (fetch(T_FUZZ_ROUGHNESS, rgba)) c.fuzz_roughness = rgba.x;
    if (fetch(T_GEOMETRY_OPACITY, rgba)) c.geometry_opacity = rgba.x;
    return c;
}

// material_emissive (integrate.glsl:148-154)
inline v3 material_emissive(const Material& m, const std::vector<Texture>& tex, v2 uv, float lod) {
    v4 color = m.constants.emission_color;
    v4 luminance = v4{m.constants.emission_luminance, 0.0f, 0.0f, 0.0f};
    if (m.textures[T_EMISSION_COLOR] != NO_TEXTURE) color = sample_texture(tex[m.textures[T_EMISSION_COLOR]], uv, lod);
    if (m.textures[T_EMISSION_LUMINANCE] != NO_TEXTURE)
        luminance = sample_texture(tex[m.textures[T_EMISSION_LUMINANCE]], uv, lod);
    return v3{color.x, color.y, color.z} * luminance.x;
}

// triangle_intersection (src/includes/math.glsl:113-125)
inline v3 triangle_intersection(const v3* p, v3 origin, v3 dir) {
    v3 eo = origin - p[0];
    v3 e2 = p[2] - p[0];
    v3 e1 = p[1] - p[0];
    v3 r = cross(dir, e2);
    v3 s = cross(eo, e1);
    float inv = 1.0f / dot(r, e1);
    float v1 = dot(r, eo);
    float v2_ = dot(s, dir);
    float b = v1 * inv;
    float c = v2_ * inv;
    return v3{1.0f - b - c, b, c};
}

// calculate_mip_level (integrate.glsl:134-139); log2 is tlog * log2(e).
inline float calculate_mip_level(v2 ddx, v2 ddy, const uint32_t* screen) {
    float sw = (float)screen[0], sh = (float)screen[1];
    v2 sx = v2{ddx.x * sw, ddx.y * sh}, sy = v2{ddy.x * sw, ddy.y * sh};
    float gx = sx.x * sx.x + sx.y * sx.y, gy = sy.x * sy.x + sy.y * sy.y;
    return 0.5f * (tlog(fmx(gx, gy)) * LOG2E);
}

}  // namespace ref
