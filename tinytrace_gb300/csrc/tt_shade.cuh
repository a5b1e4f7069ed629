// Shading pieces of src/integrate/integrate.glsl shared by the megakernel and the wavefront
// integrator: camera rays, hit reconstruction, emission, the shading basis and emissive-
// triangle sampling for next-event estimation.  Both integrators call these functions, so a
// path performs the same operations in the same order whichever integrator runs it.
#pragma once

#include "tt_bsdf.cuh"
#include "tt_bvh.cuh"
#include "tt_texture.cuh"

namespace tt {

constexpr float EXTENSION_TMIN = 1.0e-3f, EXTENSION_TMAX = 1000.0f;  // integrate.glsl:114-117
constexpr float SHADOW_TMIN = 1.0e-3f, SHADOW_TMAX = 10000.0f;       // integrate.glsl:168-172

// integrate.glsl:129-132 (the two draws come from the pixel generator)
TT_HD f2 pixel_ndc_from_draws(uint32_t px, uint32_t py, uint32_t W, uint32_t H, float ox, float oy) {
    f2 off = f2{ox - 0.5f, oy - 0.5f};
    return f2{(((float)px + off.x) / (float)W) * 2.0f - 1.0f, (((float)py + off.y) / (float)H) * 2.0f - 1.0f};
}
TT_HD f2 pixel_ndc(uint32_t px, uint32_t py, uint32_t W, uint32_t H, uint32_t& pixel_gen) {
    float ox = random_float(pixel_gen);
    float oy = random_float(pixel_gen);
    return pixel_ndc_from_draws(px, py, W, H, ox, oy);
}

// integrate.glsl:17-20
TT_HD f3 camera_ray_direction(const tt_constants& c, f2 ndc) {
    float4 vsp = mat4_mul(c.inverse_proj, make_float4(-ndc.x, -ndc.y, 1.0f, 1.0f));
    float4 wd = mat4_mul(c.inverse_view, make_float4(vsp.x, vsp.y, vsp.z, 0.0f));
    return normalize(f3{wd.x, wd.y, wd.z});
}

// Index of pixel (x, y) in the band order of the wavefront integrator's work items (bands of 8
// rows, column by column within a band): the index of rasterised primary-visibility keys.
TT_HD uint32_t band_index(uint32_t x, uint32_t y, uint32_t W, uint32_t H) {
    uint32_t band = y / 8u;
    uint32_t rows = H - 8u * band < 8u ? H - 8u * band : 8u;
    return band * 8u * W + x * rows + (y - 8u * band);
}

// The closest hit of the camera ray (o, d) from its rasterised primary-visibility key (t bits <<
// 32 | scene triangle index, ~0: no hit; primary.cu): the key's record, tested with the ray's own
// set-up, gives the t, u, v the traversal reports.  A key the test does not confirm sets
// ERR_PRIMARY_MISMATCH and counts as a miss.
__device__ __forceinline__ Hit primary_resolve(const DevScene& sc, unsigned long long key, f3 o, f3 d, uint32_t* err) {
    Hit h;
    h.hit = 0;
    h.t = h.u = h.v = 0.0f;
    h.instance = h.prim = 0u;
    if (key == ~0ull) return h;
    const uint32_t rec = __ldg(sc.tri_record + (uint32_t)key);
    const float4 a = __ldg(sc.tris + 3ull * rec), b = __ldg(sc.tris + 3ull * rec + 1), c = __ldg(sc.tris + 3ull * rec + 2);
    const uint32_t inst = __float_as_uint(b.w);
    f3 oo, od;
    uint32_t mesh;
    instance_ray(sc, inst, o, d, oo, od, mesh);
    RayPre rp = ray_precompute(oo, od);
    float t, u, v;
    bool ok = finite3(od) &&
              intersect_triangle(rp, tri_vertex(a), tri_vertex(b), tri_vertex(c), true, EXTENSION_TMIN, EXTENSION_TMAX,
                                 t, u, v) &&
              __float_as_uint(t) == (uint32_t)(key >> 32);
    if (!ok) {
        atomicOr(err, ERR_PRIMARY_MISMATCH);
        return h;
    }
    h.hit = 1;
    h.t = t;
    h.u = u;
    h.v = v;
    h.instance = inst;
    h.prim = __float_as_uint(a.w);
    return h;
}

struct ShadeHit {
    f3 world_position;
    Basis tangent_space;
    uint32_t material_index;
    // texturing inputs (dead code unless a textured instantiation reads them)
    f2 uv;                // interpolated texture coordinates
    f3 bary;              // barycentrics of the hit
    f3 world[3];          // world-space triangle vertices
    uint32_t tc[3];       // the vertices' f16 texture coordinates
};

// integrate.glsl:22-110; the ray differentials of the primary hit are primary_mip_level.
__device__ __forceinline__ ShadeHit get_ray_hit(const DevScene& sc, uint32_t instance, uint32_t prim, float u,
                                                float v) {
    ShadeHit hit;
    const tt_instance* in = sc.instances + instance;
    hit.material_index = __ldg(&in->material_index);
    uint32_t index_offset = __ldg(&in->index_offset), vertex_offset = __ldg(&in->vertex_offset);
    float m[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) m[k] = __ldg(&in->transform[k]);
    uint32_t base = 3u * prim + index_offset;
    f3 pos[3];
    TangentFrame tf[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        uint32_t vi = __ldg(sc.indices + base + k) + vertex_offset;
        const int16_t* s = sc.positions + 3ull * vi;
        f3 p = f3{dequant_snorm16(__ldg(s + 0)), dequant_snorm16(__ldg(s + 1)), dequant_snorm16(__ldg(s + 2))};
        pos[k] = mat43_point(m, p);
        tf[k] = decode_tangent_frame(__ldg(&sc.vertices[vi].tangent_frame));
        hit.tc[k] = __ldg(reinterpret_cast<const uint32_t*>(&sc.vertices[vi].texture_coordinates));
        hit.world[k] = pos[k];
    }
    f3 bary = f3{0.0f, u, v};
    bary.x = 1.0f - bary.y - bary.z;
    float nt[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) nt[k] = k < 11 ? __ldg(&in->normal_transform[k]) : 0.0f;
    hit.tangent_space.normal = normalize(mat3_vec(nt, interp3(bary, tf[0].normal, tf[1].normal, tf[2].normal)));
    hit.tangent_space.tangent = normalize(mat3_vec(nt, interp3(bary, tf[0].tangent, tf[1].tangent, tf[2].tangent)));
    float bs = signf(tf[0].bitangent_sign * bary.x + tf[1].bitangent_sign * bary.y + tf[2].bitangent_sign * bary.z);
    hit.tangent_space.bitangent = normalize(bs * cross(hit.tangent_space.normal, hit.tangent_space.tangent));
    hit.world_position = bary.x * pos[0] + bary.y * pos[1] + bary.z * pos[2];
    hit.bary = bary;
    hit.uv = interp_uv(bary, hit.tc[0], hit.tc[1], hit.tc[2]);
    return hit;
}

// calculate_mip_level (integrate.glsl:134-139) of the texture-coordinate differentials of the
// primary hit (integrate.glsl:91-106): the camera rays one texel right and one texel up,
// crossed with the hit triangle's plane.
__device__ __forceinline__ float primary_mip_level(const tt_constants& c, const ShadeHit& hit, f3 origin, f2 ndc) {
    f2 texel = f2{2.0f / (float)c.screen_size[0], 2.0f / (float)c.screen_size[1]};
    f3 hx = triangle_barycentrics(hit.world, origin, camera_ray_direction(c, f2{ndc.x + texel.x, ndc.y}));
    f3 hy = triangle_barycentrics(hit.world, origin, camera_ray_direction(c, f2{ndc.x, ndc.y + texel.y}));
    f2 ddx = interp_uv(hit.bary - hx, hit.tc[0], hit.tc[1], hit.tc[2]);
    f2 ddy = interp_uv(hit.bary - hy, hit.tc[0], hit.tc[1], hit.tc[2]);
    float sw = (float)c.screen_size[0], sh = (float)c.screen_size[1];
    f2 sx = f2{ddx.x * sw, ddx.y * sh}, sy = f2{ddy.x * sw, ddy.y * sh};
    float gx = sx.x * sx.x + sx.y * sx.y, gy = sy.x * sy.x + sy.y * sy.y;
    return 0.5f * (tlog(fmx(gx, gy)) * LOG2E);
}

// The material constants a hit shades with: the material's own, or (textured) a copy with
// the sampled slots replaced; `local` holds the copy.
template <bool TEX>
__device__ __forceinline__ const MatC& hit_material(const DevScene& sc, const tt_material* mat, f2 uv, float lod,
                                                    MatC& local) {
    if (TEX) {
        uint32_t mask = __ldg(&mat->padding);
        if (mask & LOAD_SLOTS) {
            local = mat->constants;
            load_textures(sc, mat, mask, uv, lod, local);
            return local;
        }
    }
    return mat->constants;
}

template <bool TEX>
__device__ __forceinline__ f3 hit_emissive(const DevScene& sc, const tt_material* mat, f2 uv, float lod) {
    if (TEX) {
        uint32_t mask = __ldg(&mat->padding);
        if (mask & EMISSION_SLOTS) return material_emissive_textured(sc, mat, mask, uv, lod);
    }
    const MatC& m = mat->constants;
    return col3(m.emission_color) * m.emission_luminance;
}

// integrate.glsl:148-154 (constant materials)
__device__ __forceinline__ f3 material_emissive(const tt_material* mat) {
    const MatC& m = mat->constants;
    return col3(m.emission_color) * m.emission_luminance;
}

// integrate.glsl:195-201
__device__ __forceinline__ Basis create_surface_basis(const Basis& ts, f3 n) {
    Basis b;
    b.normal = transform_to_basis(ts, n);
    b.tangent = gram_schmidt(b.normal, ts.tangent);
    b.bitangent = normalize(cross(b.normal, b.tangent));
    return b;
}

// scene.glsl:114-136 followed by the geometry part of integrate.glsl:160-167: the light
// sample, the shadow ray towards it and the solid-angle density.
struct LightSample {
    f3 wo;          // direction to the light in the shading basis
    f3 dir;         // world-space shadow ray direction
    float density;  // solid-angle density times the light selection probability
    uint32_t instance, hash;
    uint32_t prim;  // primitive of the light triangle in its instance's mesh (exact visibility)
    uint32_t light; // emissive triangle index (its light record)
    f2 uv;          // texture coordinates of the light point (read by textured shading only)
};
// The triangle's world vertices, area and normal come from its light record, which
// light_records_kernel computes once per scene with the operations of scene.glsl:114-136
// (instance transform of the dequantised positions, cross product of the edges).
__device__ __forceinline__ LightSample sample_light(const DevScene& sc, f3 position, const Basis& basis,
                                                    uint32_t& g) {
    uint32_t light = xor_shift(g) % sc.emissive_count;
    float light_probability = 1.0f / (float)sc.emissive_count;
    if (sc.light_power) {  // alias table: keep `light` with its probability, else take its alias
        float4 e = __ldg(sc.light_alias + light);
        float coin = random_float(g);
        if (!(coin < e.x)) light = __float_as_uint(e.y);
        light_probability = __ldg(&sc.light_alias[light].z);
    }
    const float4* rec = sc.light_rec + (uint64_t)LIGHT_RECORD * light;
    f2 rnd = random_vec2(g);
    f3 bary = sample_triangle(rnd);
    float4 r0 = __ldg(rec + 0), r1 = __ldg(rec + 1), r2 = __ldg(rec + 2), r3 = __ldg(rec + 3), r5 = __ldg(rec + 5);
    LightSample ls;
    ls.light = light;
    ls.instance = __float_as_uint(r1.w);
    float area = r0.w;
    f3 lnormal = f3{r3.x, r3.y, r3.z};
    f3 lpos = interp3(bary, f3{r0.x, r0.y, r0.z}, f3{r1.x, r1.y, r1.z}, f3{r2.x, r2.y, r2.z});
    ls.uv = interp_uv(bary, __float_as_uint(r5.x), __float_as_uint(r5.y), __float_as_uint(r5.z));
    ls.hash = __float_as_uint(r2.w);
    ls.prim = sc.light_exact ? __float_as_uint(r5.w) : 0xffffffffu;
    f3 to_light = lpos - position;
    ls.wo = transform_from_basis(basis, to_light);
    float d2 = dot(to_light, to_light);
    ls.dir = to_light / sqrtf(d2);
    ls.density = (1.0f / area) * d2 / saturate(dot(-ls.dir, lnormal)) * light_probability;
    return ls;
}

// Emission of a light point: the record's constant emission, or the material's emission
// textures at `uv` when it has some (textured scenes).
template <bool TEX>
__device__ __forceinline__ f3 light_emission(const DevScene& sc, uint32_t light, f2 uv, float lod) {
    const float4* rec = sc.light_rec + (uint64_t)LIGHT_RECORD * light;
    float4 r4 = __ldg(rec + 4);
    if (TEX) {
        uint32_t mask = __float_as_uint(__ldg(&rec[3].w));
        if (mask) return material_emissive_textured(sc, sc.materials + __float_as_uint(r4.w), mask, uv, lod);
    }
    return f3{r4.x, r4.y, r4.z};
}

// The contribution of integrate.glsl:186-192 when the light is visible (the light's emission
// textures are sampled at mip level 4, integrate.glsl:188-189).
template <bool TEX = false, uint32_t LS = LOBE_SET_ALL>
__device__ __forceinline__ f3 light_contribution(const DevScene& sc, const LightSample& ls, const MatC& mat,
                                                 const Lobes& lobes, f3 wi) {
    f3 emissive = light_emission<TEX>(sc, ls.light, ls.uv, 4.0f);
    float bd = 0.0f;
    f3 bsdf = bsdf_evaluate<LS>(mat, lobes, wi, ls.wo, bd);
    return bsdf * emissive * fabsf(cos_theta(ls.wo)) / fmx(ls.density, PDF_EPSILON);
}

// The triangle the visibility test of integrate.glsl:175-185 accepts, found before the shadow
// ray is traced.  In a light instance of at most 65,535 triangles exactly one primitive p can
// satisfy (p + index_offset / 3) % 0xffff == hash (none when hash == 0xffff or p would lie past
// the mesh): the ray is visible iff its closest hit is that triangle.  Returns
//   0  no primitive qualifies, or the ray misses it: not visible, nothing to trace;
//   1  `best`/`tbest` hold the ray's hit on it: trace for a closer hit (any closer hit occludes);
//   2  the instance has more than 65,535 triangles: trace plainly and test the closest hit.
// The hit is computed exactly as the traversal computes it (object ray of the instance, the
// same watertight test on the same dequantised vertices), so a traversal seeded with it finds
// the same closest hit as an unseeded one.
// The hit of ray (o, d) on primitive `prim` of instance `inst` (no culling, t in [tmin, tmax])
// exactly as the traversal computes it: the instance's object ray, the watertight test on the
// dequantised snorm16 vertices.  On a hit, `best` and `tbest` hold it and the result is true.
__device__ __forceinline__ bool seed_triangle_hit(const DevScene& sc, uint32_t inst, uint32_t prim,
                                                  uint32_t index_offset, uint32_t vertex_offset, f3 o, f3 d,
                                                  float tmin, float tmax, Hit& best, float& tbest) {
    f3 oo, od;
    uint32_t mesh;
    instance_ray(sc, inst, o, d, oo, od, mesh);
    if (!finite3(d) || !finite3(od)) return false;
    f3 p[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int16_t* s = sc.positions + 3ull * (__ldg(sc.indices + index_offset + 3u * prim + k) + vertex_offset);
        p[k] = f3{dequant_snorm16(__ldg(s + 0)), dequant_snorm16(__ldg(s + 1)), dequant_snorm16(__ldg(s + 2))};
    }
    float t, u, v;
    if (!intersect_triangle(ray_precompute(oo, od), p[0], p[1], p[2], false, tmin, tmax, t, u, v)) return false;
    best.hit = 1;
    best.t = t;
    best.u = u;
    best.v = v;
    best.instance = inst;
    best.prim = prim;
    tbest = t;
    return true;
}

__device__ __forceinline__ int shadow_target(const DevScene& sc, uint32_t light_instance, uint32_t hash,
                                             uint32_t exact_prim, f3 o, f3 d, float tmin, float tmax, Hit& best,
                                             float& tbest) {
    const tt_instance* in = sc.instances + light_instance;
    uint32_t index_offset = __ldg(&in->index_offset), vertex_offset = __ldg(&in->vertex_offset);
    uint32_t tri_count = __ldg(&sc.meshes[__ldg(&in->mesh_index)].index_count) / 3u;
    uint32_t prim;
    if (sc.light_exact) {  // the sampled triangle itself
        prim = exact_prim;
        if (prim >= tri_count) return 0;
    } else {
        if (tri_count > 0xffffu) return 2;
        if (hash >= 0xffffu) return 0;
        uint32_t r = (index_offset / 3u) % 0xffffu;
        prim = hash >= r ? hash - r : hash + 0xffffu - r;
        if (prim >= tri_count) return 0;
    }
    return seed_triangle_hit(sc, light_instance, prim, index_offset, vertex_offset, o, d, tmin, tmax, best, tbest) ? 1 : 0;
}

// integrate.glsl:175-185: the closest shadow hit must be the sampled light triangle.
__device__ __forceinline__ bool light_visible(const DevScene& sc, const Hit& h, uint32_t light_instance,
                                              uint32_t hash, uint32_t exact_prim) {
    if (!h.hit) return false;
    if (h.instance != light_instance) return false;
    if (sc.light_exact) return h.prim == exact_prim;
    uint32_t tri_index = h.prim + __ldg(&sc.instances[h.instance].index_offset) / 3u;
    return tri_index % 0xffffu == hash;
}

}  // namespace tt
