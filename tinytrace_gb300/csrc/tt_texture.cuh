// Textured materials of src/integrate/integrate.glsl:134-154, 219-266: texture coordinates
// and their ray differentials at the primary hit, the mip level they select, and
// textureLod through the scene sampler (src/scene.rs:121-128: linear minification,
// magnification and mip filtering, repeat addressing; the LOD is explicit, so anisotropy
// does not apply) for the four formats ProcessedTexture produces (src/asset/texture.rs):
// BC1 sRGB colour, BC5 unorm normal maps, R8 unorm and R16 float scalars.
//
// Decoding and filtering are done in software with float weights, in a fixed operation
// order, so that the CPU oracle reproduces every bit; the texture units' fixed-point
// weights and BC palette rounding are not specified to that precision.  Definitions:
//   BC1    endpoints 5:6:5 expanded by bit replication; c0 > c1: palette c2 = (2 c0 + c1 + 1) / 3,
//          c3 = (c0 + 2 c1 + 1) / 3 per 8-bit channel (integer division); otherwise
//          c2 = (c0 + c1 + 1) / 2 and c3 transparent black; sRGB to linear by a 256-entry
//          table; alpha 1 (0 for the transparent entry).
//   BC4/5  per channel: index 0 -> e0 / 255, 1 -> e1 / 255; e0 > e1: k = 2..7 ->
//          ((8 - k) e0 + (k - 1) e1) / 1785; otherwise k = 2..5 -> ((6 - k) e0 + (k - 1) e1) / 1275,
//          6 -> 0, 7 -> 1.  BC5 returns (red, green, 0, 1).
//   R8     v / 255 -> (v, 0, 0, 1);  R16F  half -> (v, 0, 0, 1).
//   level  lambda = min(max(lod, 0), levels - 1) (NaN -> 0); levels floor(lambda) and the next,
//          blended (1 - f) a + f b when f = lambda - floor(lambda) > 0.
//   texel  level extent max(1, size >> level); u' = (u - floor(u)) (non-finite -> 0), then
//          x = u' w - 0.5, i = floor(x), alpha = x - i, columns i and i + 1 wrapped modulo w
//          (rows likewise); weights (1-a)(1-b), a(1-b), (1-a)b, ab summed in that order.
#pragma once

#include <cuda_fp16.h>

#include "tt_bsdf.cuh"
#include "tt_bvh.cuh"

namespace tt {

constexpr uint32_t TEX_BC1_SRGB = 1u, TEX_BC5_UNORM = 2u, TEX_R8_UNORM = 3u, TEX_R16_FLOAT = 4u;
constexpr uint32_t TEXTURE_NONE = 0xffffffffu;

// Material texture slots (MaterialTextures, src/material/material.glsl:40-68)
enum TexSlot : uint32_t {
    SLOT_BASE_COLOR = 0, SLOT_SPECULAR_COLOR, SLOT_TRANSMISSION_COLOR, SLOT_COAT_COLOR, SLOT_FUZZ_COLOR,
    SLOT_EMISSION_COLOR, SLOT_GEOMETRY_NORMAL, SLOT_BASE_WEIGHT, SLOT_BASE_METALNESS,
    SLOT_BASE_DIFFUSE_ROUGHNESS, SLOT_SPECULAR_WEIGHT, SLOT_SPECULAR_ROUGHNESS,
    SLOT_SPECULAR_ROUGHNESS_ANISOTROPY, SLOT_SPECULAR_IOR, SLOT_SPECULAR_ROTATION, SLOT_TRANSMISSION_WEIGHT,
    SLOT_TRANSMISSION_DEPTH, SLOT_COAT_WEIGHT, SLOT_COAT_ROUGHNESS, SLOT_COAT_ROUGHNESS_ANISOTROPY,
    SLOT_COAT_IOR, SLOT_COAT_DARKENING, SLOT_COAT_ROTATION, SLOT_FUZZ_WEIGHT, SLOT_FUZZ_ROUGHNESS,
    SLOT_EMISSION_LUMINANCE, SLOT_GEOMETRY_OPACITY, SLOT_COUNT
};
// The slots load_textures reads (integrate.glsl:219-266); base_weight, transmission_depth,
// coat_roughness, coat_roughness_anisotropy and coat_ior are uploaded but never sampled.
constexpr uint32_t LOAD_SLOTS = (1u << SLOT_BASE_COLOR) | (1u << SLOT_SPECULAR_COLOR) |
                                (1u << SLOT_TRANSMISSION_COLOR) | (1u << SLOT_COAT_COLOR) | (1u << SLOT_FUZZ_COLOR) |
                                (1u << SLOT_GEOMETRY_NORMAL) | (1u << SLOT_BASE_METALNESS) |
                                (1u << SLOT_BASE_DIFFUSE_ROUGHNESS) | (1u << SLOT_SPECULAR_WEIGHT) |
                                (1u << SLOT_SPECULAR_ROUGHNESS) | (1u << SLOT_SPECULAR_ROUGHNESS_ANISOTROPY) |
                                (1u << SLOT_SPECULAR_IOR) | (1u << SLOT_SPECULAR_ROTATION) |
                                (1u << SLOT_TRANSMISSION_WEIGHT) | (1u << SLOT_COAT_WEIGHT) |
                                (1u << SLOT_COAT_DARKENING) | (1u << SLOT_COAT_ROTATION) | (1u << SLOT_FUZZ_WEIGHT) |
                                (1u << SLOT_FUZZ_ROUGHNESS) | (1u << SLOT_GEOMETRY_OPACITY);
constexpr uint32_t EMISSION_SLOTS = (1u << SLOT_EMISSION_COLOR) | (1u << SLOT_EMISSION_LUMINANCE);

__device__ __forceinline__ int wrap_index(int i, int n) {
    int r = i % n;
    return r < 0 ? r + n : r;
}

__device__ __forceinline__ float bc4_value(uint32_t e0, uint32_t e1, uint32_t k) {
    if (k == 0u) return (float)e0 / 255.0f;
    if (k == 1u) return (float)e1 / 255.0f;
    if (e0 > e1) return (float)((8u - k) * e0 + (k - 1u) * e1) / 1785.0f;
    if (k == 6u) return 0.0f;
    if (k == 7u) return 1.0f;
    return (float)((6u - k) * e0 + (k - 1u) * e1) / 1275.0f;
}

__device__ __forceinline__ float bc4_texel(uint2 block, uint32_t t) {
    uint32_t e0 = block.x & 0xffu, e1 = (block.x >> 8) & 0xffu;
    // 48 index bits: bytes 2..7 of the block, little-endian
    uint64_t bits = ((uint64_t)block.y << 16) | (uint64_t)(block.x >> 16);
    uint32_t k = (uint32_t)(bits >> (3u * t)) & 7u;
    return bc4_value(e0, e1, k);
}

__device__ __forceinline__ uint32_t expand5(uint32_t v) { return (v << 3) | (v >> 2); }
__device__ __forceinline__ uint32_t expand6(uint32_t v) { return (v << 2) | (v >> 4); }

__device__ __forceinline__ float4 fetch_texel(const DevScene& sc, const DevTexture& tx, const uint8_t* level,
                                              uint32_t w, uint32_t x, uint32_t y) {
    switch (tx.format) {
        case TEX_BC1_SRGB: {
            uint32_t bw = (w + 3u) >> 2;
            uint2 b = __ldg(reinterpret_cast<const uint2*>(level) + (uint64_t)(y >> 2) * bw + (x >> 2));
            uint32_t c0 = b.x & 0xffffu, c1 = b.x >> 16;
            uint32_t sel = (b.y >> (2u * ((y & 3u) * 4u + (x & 3u)))) & 3u;
            uint32_t a[3] = {expand5(c0 >> 11), expand6((c0 >> 5) & 63u), expand5(c0 & 31u)};
            uint32_t e[3] = {expand5(c1 >> 11), expand6((c1 >> 5) & 63u), expand5(c1 & 31u)};
            uint32_t r[3];
            float alpha = 1.0f;
#pragma unroll
            for (int ch = 0; ch < 3; ++ch) {
                uint32_t v;
                if (sel == 0u) v = a[ch];
                else if (sel == 1u) v = e[ch];
                else if (c0 > c1) v = sel == 2u ? (2u * a[ch] + e[ch] + 1u) / 3u : (a[ch] + 2u * e[ch] + 1u) / 3u;
                else v = sel == 2u ? (a[ch] + e[ch] + 1u) / 2u : 0u;
                r[ch] = v;
            }
            if (c0 <= c1 && sel == 3u) alpha = 0.0f;
            return make_float4(__ldg(sc.srgb + r[0]), __ldg(sc.srgb + r[1]), __ldg(sc.srgb + r[2]), alpha);
        }
        case TEX_BC5_UNORM: {
            uint32_t bw = (w + 3u) >> 2;
            uint4 b = __ldg(reinterpret_cast<const uint4*>(level) + (uint64_t)(y >> 2) * bw + (x >> 2));
            uint32_t t = (y & 3u) * 4u + (x & 3u);
            return make_float4(bc4_texel(make_uint2(b.x, b.y), t), bc4_texel(make_uint2(b.z, b.w), t), 0.0f, 1.0f);
        }
        case TEX_R8_UNORM:
            return make_float4((float)__ldg(level + (uint64_t)y * w + x) / 255.0f, 0.0f, 0.0f, 1.0f);
        default: {  // TEX_R16_FLOAT
            uint16_t h = __ldg(reinterpret_cast<const unsigned short*>(level) + (uint64_t)y * w + x);
            return make_float4(__half2float(__ushort_as_half(h)), 0.0f, 0.0f, 1.0f);
        }
    }
}

__device__ __forceinline__ float4 add4(float4 a, float4 b) {
    return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}
__device__ __forceinline__ float4 mul4(float4 a, float s) { return make_float4(a.x * s, a.y * s, a.z * s, a.w * s); }

__device__ __forceinline__ float wrap_coordinate(float u) {
    float f = u - floorf(u);
    return isfinite(f) ? f : 0.0f;
}

static __device__ float4 sample_level(const DevScene& sc, const DevTexture& tx, uint32_t level, f2 uv) {
    uint32_t w = max(1u, tx.width >> level), h = max(1u, tx.height >> level);
    const uint8_t* base = sc.tex_data + tx.offset[level];
    float x = wrap_coordinate(uv.x) * (float)w - 0.5f;
    float y = wrap_coordinate(uv.y) * (float)h - 0.5f;
    float xf = floorf(x), yf = floorf(y);
    float a = x - xf, b = y - yf;
    int xi = (int)xf, yi = (int)yf;
    uint32_t x0 = (uint32_t)wrap_index(xi, (int)w), x1 = (uint32_t)wrap_index(xi + 1, (int)w);
    uint32_t y0 = (uint32_t)wrap_index(yi, (int)h), y1 = (uint32_t)wrap_index(yi + 1, (int)h);
    float4 t00 = fetch_texel(sc, tx, base, w, x0, y0);
    float4 t10 = fetch_texel(sc, tx, base, w, x1, y0);
    float4 t01 = fetch_texel(sc, tx, base, w, x0, y1);
    float4 t11 = fetch_texel(sc, tx, base, w, x1, y1);
    float ia = 1.0f - a, ib = 1.0f - b;
    float4 r = mul4(t00, ia * ib);
    r = add4(r, mul4(t10, a * ib));
    r = add4(r, mul4(t01, ia * b));
    r = add4(r, mul4(t11, a * b));
    return r;
}

// textureLod(textures[index], uv, lod)
static __device__ float4 sample_texture(const DevScene& sc, uint32_t index, f2 uv, float lod) {
    const DevTexture& tx = sc.textures[index];
    float q = (float)(tx.levels - 1u);
    float d = fminf(fmaxf(lod, 0.0f), q);
    float lf = floorf(d);
    uint32_t l0 = (uint32_t)lf;
    float f = d - lf;
    float4 r = sample_level(sc, tx, l0, uv);
    if (f > 0.0f) r = add4(mul4(r, 1.0f - f), mul4(sample_level(sc, tx, l0 + 1u, uv), f));
    return r;
}

// interpolate(barycentric, f16vec2 a, b, c) of math.glsl:94-96; each argument packs the two
// f16 coordinates (u in the low half).
__device__ __forceinline__ f2 half2_of(uint32_t t) {
    return f2{__half2float(__ushort_as_half((unsigned short)(t & 0xffffu))),
              __half2float(__ushort_as_half((unsigned short)(t >> 16)))};
}
__device__ __forceinline__ f2 interp_uv(f3 b, uint32_t t0, uint32_t t1, uint32_t t2) {
    f2 a0 = half2_of(t0), a1 = half2_of(t1), a2 = half2_of(t2);
    return f2{b.x * a0.x + b.y * a1.x + b.z * a2.x, b.x * a0.y + b.y * a1.y + b.z * a2.y};
}

// triangle_intersection (math.glsl:113-125): barycentrics of the ray's crossing of the plane.
__device__ __forceinline__ f3 triangle_barycentrics(const f3* p, f3 origin, f3 dir) {
    f3 eo = origin - p[0];
    f3 e2 = p[2] - p[0];
    f3 e1 = p[1] - p[0];
    f3 r = cross(dir, e2);
    f3 s = cross(eo, e1);
    float inv = 1.0f / dot(r, e1);
    float v1 = dot(r, eo);
    float v2 = dot(s, dir);
    float b = v1 * inv;
    float c = v2 * inv;
    return f3{1.0f - b - c, b, c};
}

// The texture values a material slot receives (integrate.glsl:141-146, 219-266).
__device__ __forceinline__ void apply_texture(MatC& m, uint32_t slot, float4 v) {
    switch (slot) {
        case SLOT_BASE_COLOR: m.base_color[0] = v.x, m.base_color[1] = v.y, m.base_color[2] = v.z, m.base_color[3] = v.w; break;
        case SLOT_SPECULAR_COLOR: m.specular_color[0] = v.x, m.specular_color[1] = v.y, m.specular_color[2] = v.z, m.specular_color[3] = v.w; break;
        case SLOT_TRANSMISSION_COLOR: m.transmission_color[0] = v.x, m.transmission_color[1] = v.y, m.transmission_color[2] = v.z, m.transmission_color[3] = v.w; break;
        case SLOT_COAT_COLOR: m.coat_color[0] = v.x, m.coat_color[1] = v.y, m.coat_color[2] = v.z, m.coat_color[3] = v.w; break;
        case SLOT_FUZZ_COLOR: m.fuzz_color[0] = v.x, m.fuzz_color[1] = v.y, m.fuzz_color[2] = v.z, m.fuzz_color[3] = v.w; break;
        case SLOT_GEOMETRY_NORMAL: {
            f3 n = octahedron_decode(f2{v.x, v.y});
            m.geometry_normal[0] = n.x, m.geometry_normal[1] = n.y, m.geometry_normal[2] = n.z, m.geometry_normal[3] = n.x;
            break;
        }
        case SLOT_BASE_METALNESS: m.base_metalness = v.x; break;
        case SLOT_BASE_DIFFUSE_ROUGHNESS: m.base_diffuse_roughness = v.x; break;
        case SLOT_SPECULAR_WEIGHT: m.specular_weight = v.x; break;
        case SLOT_SPECULAR_ROUGHNESS: m.specular_roughness = v.x; break;
        case SLOT_SPECULAR_ROUGHNESS_ANISOTROPY: m.specular_roughness_anisotropy = v.x; break;
        case SLOT_SPECULAR_IOR: m.specular_ior = v.x; break;
        case SLOT_SPECULAR_ROTATION: m.specular_rotation = v.x; break;
        case SLOT_TRANSMISSION_WEIGHT: m.transmission_weight = v.x; break;
        case SLOT_COAT_WEIGHT: m.coat_weight = v.x; break;
        case SLOT_COAT_DARKENING: m.coat_darkening = v.x; break;
        case SLOT_COAT_ROTATION: m.coat_rotation = v.x; break;
        case SLOT_FUZZ_WEIGHT: m.fuzz_weight = v.x; break;
        case SLOT_FUZZ_ROUGHNESS: m.fuzz_roughness = v.x; break;
        default: m.geometry_opacity = v.x; break;  // SLOT_GEOMETRY_OPACITY
    }
}

// load_textures (integrate.glsl:219-266).  `mask` holds the material's set slots (the device
// copy of the material keeps it in its padding word).
__device__ __forceinline__ void load_textures(const DevScene& sc, const tt_material* mat, uint32_t mask, f2 uv,
                                              float lod, MatC& m) {
    uint32_t todo = mask & LOAD_SLOTS;
    while (todo) {
        uint32_t slot = (uint32_t)(__ffs(todo) - 1);
        todo &= todo - 1u;
        apply_texture(m, slot, sample_texture(sc, __ldg(&mat->textures[slot]), uv, lod));
    }
}

// material_emissive (integrate.glsl:148-154)
__device__ __forceinline__ f3 material_emissive_textured(const DevScene& sc, const tt_material* mat, uint32_t mask,
                                                         f2 uv, float lod) {
    const MatC& m = mat->constants;
    float4 color = make_float4(m.emission_color[0], m.emission_color[1], m.emission_color[2], m.emission_color[3]);
    float luminance = m.emission_luminance;
    if (mask & (1u << SLOT_EMISSION_COLOR)) color = sample_texture(sc, __ldg(&mat->textures[SLOT_EMISSION_COLOR]), uv, lod);
    if (mask & (1u << SLOT_EMISSION_LUMINANCE))
        luminance = sample_texture(sc, __ldg(&mat->textures[SLOT_EMISSION_LUMINANCE]), uv, lod).x;
    return f3{color.x, color.y, color.z} * luminance;
}

}  // namespace tt
