// ReSTIR DI (spatiotemporal reservoir resampling for direct lighting; Bitterli, Wyman, Pharr,
// Shirley, Lefohn & Jarosz, SIGGRAPH 2020) on the emissive triangles of the scene.  This is an
// addition: the reference samples one light per vertex (src/includes/scene.glsl:114-136).
//
// Per pixel and frame (1 sample per pixel, direct light at the primary hit):
//   G-buffer   camera ray (the path tracer's jitter), closest hit with back faces culled,
//              shading basis, outgoing direction, material, the generator state before
//              bsdf_prepare (each pass rebuilds the same stochastic lobe albedos from it);
//   initial    C candidates x_i = (light, r1, r2) from the source density p = 1 / (lights *
//              area) in area measure, streaming RIS with weight p^(x) / p(x), where the target
//              p^(x) is the luminance of the unshadowed contribution f * Le * |cos| * cosL / d^2;
//              then the chosen sample's visibility (shadow ray; occluded => W = 0);
//   temporal   reprojection of the primary hit into the previous frame's camera; when the
//              previous pixel's surface is similar (normal within 25 degrees, camera distance
//              within 10 %) its reservoir is merged, its M capped at 20 x C;
//   spatial    up to 5 neighbours in a 30-pixel disk with similar surfaces are merged;
//   shade      the final sample's contribution times W and its visibility (a second shadow
//              ray), plus the primary hit's emission; misses see the white sky.
// Reservoir merging is the biased combination of the paper (no 1/Z correction).  Visibility
// means the closest hit is the light sample's own triangle (instance and primitive), with the
// shadow rays' semantics of the path tracer (no culling, t in [1e-3, 1e4]).
//
// Random streams: the G-buffer pass uses the pixel generator of the path tracer (two jitter
// draws); every later pass starts its own stream from jenkins_hash(seed + pass), where seed is
// the stored generator state.  The CPU oracle restates every pass with the same operations,
// and the tests compare the images and reservoirs bit for bit.
#pragma once

#include "tt_kernels.h"
#include "tt_shade.cuh"

namespace tt {

struct Reservoir {
    uint32_t light;    // emissive triangle index (0xffffffff: empty)
    float r1, r2;      // the sample_triangle random numbers of the chosen point
    float w_sum;       // running sum of resampling weights
    float M;           // candidates represented
    float W;           // unbiased contribution weight of the chosen sample
    float pad0, pad1;  // 32-byte records
};

constexpr uint32_t NO_LIGHT = 0xffffffffu;
constexpr uint32_t NO_SURFACE = 0xffffffffu;

// G-buffer record of one pixel (64 bytes).
struct Surface {
    float4 pos_dist;      // world position, distance from the camera
    float4 normal_mat;    // shading normal, material index bits (NO_SURFACE: the camera ray missed)
    float4 tangent_inst;  // shading tangent, instance bits
    float4 wi_seed;       // outgoing direction in the shading basis, generator state bits
};

TT_HD float luminance(f3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }

// The primary hit's prepared lobes (bsdf_prepare from the G-buffer's generator state), stored
// by the G-buffer pass so that the later passes read them instead of preparing again.
static_assert(sizeof(Lobes) == 16 * LOBE_RECORD, "Lobes is 24 floats");
TT_HD void store_lobes(float4* dst, const Lobes& l) {
    float v[4 * LOBE_RECORD];
    memcpy(v, &l, sizeof(v));
#pragma unroll
    for (int k = 0; k < LOBE_RECORD; ++k) dst[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
}
TT_HD Lobes load_lobes(const float4* src) {
    float v[4 * LOBE_RECORD];
#pragma unroll
    for (int k = 0; k < LOBE_RECORD; ++k) {
        float4 q = src[k];
        v[4 * k] = q.x;
        v[4 * k + 1] = q.y;
        v[4 * k + 2] = q.z;
        v[4 * k + 3] = q.w;
    }
    Lobes l;
    memcpy(&l, v, sizeof(v));
    return l;
}

// World position, normal (one-sided, cross(p1-p0, p2-p0)), area and emission of a light point.
struct LightPoint {
    f3 pos, normal, emission;
    float area;
    uint32_t instance;
};
template <bool TEX>
__device__ __forceinline__ LightPoint light_point(const DevScene& sc, uint32_t light, float r1, float r2) {
    const float4* rec = sc.light_rec + (uint64_t)LIGHT_RECORD * light;
    float4 q0 = __ldg(rec + 0), q1 = __ldg(rec + 1), q2 = __ldg(rec + 2), q3 = __ldg(rec + 3);
    LightPoint lp;
    lp.instance = __float_as_uint(q1.w);
    lp.area = q0.w;
    lp.normal = f3{q3.x, q3.y, q3.z};
    f3 bary = sample_triangle(f2{r1, r2});
    lp.pos = interp3(bary, f3{q0.x, q0.y, q0.z}, f3{q1.x, q1.y, q1.z}, f3{q2.x, q2.y, q2.z});
    f2 uv = f2{0.0f, 0.0f};
    if (TEX) {
        float4 q5 = __ldg(rec + 5);
        uv = interp_uv(bary, __float_as_uint(q5.x), __float_as_uint(q5.y), __float_as_uint(q5.z));
    }
    lp.emission = light_emission<TEX>(sc, light, uv, 4.0f);
    return lp;
}

// Unshadowed contribution f * Le * |cos| * cosL / d^2 of light point lp at the surface (the
// surface's material has its lobe set within LS).
template <uint32_t LS = LOBE_SET_ALL>
__device__ __forceinline__ f3 restir_contribution(const MatC& mc, const Lobes& lobes, const Basis& basis, f3 wi,
                                                  f3 pos, const LightPoint& lp) {
    f3 d = lp.pos - pos;
    float d2 = dot(d, d);
    f3 dir = d / sqrtf(d2);
    float cos_light = dot(-dir, lp.normal);
    if (!(cos_light > 0.0f) || !(d2 > 0.0f)) return splat(0.0f);
    f3 wo = transform_from_basis(basis, d);
    float density = 0.0f;
    f3 f = bsdf_evaluate<LS>(mc, lobes, wi, wo, density);
    return f * lp.emission * (fabsf(cos_theta(wo)) * cos_light / d2);
}

// Weighted reservoir update: the candidate replaces the sample with probability w / w_sum.
TT_HD bool reservoir_update(Reservoir& r, uint32_t light, float r1, float r2, float w, float m, uint32_t& g) {
    r.w_sum += w;
    r.M += m;
    float u = random_float(g);
    bool take = w > 0.0f && u * r.w_sum < w;
    if (take) {
        r.light = light;
        r.r1 = r1;
        r.r2 = r2;
    }
    return take;
}

TT_HD Reservoir empty_reservoir() {
    Reservoir r;
    r.light = NO_LIGHT;
    r.r1 = r.r2 = 0.0f;
    r.w_sum = 0.0f;
    r.M = 0.0f;
    r.W = 0.0f;
    r.pad0 = r.pad1 = 0.0f;
    return r;
}

// Visibility of a light point: the closest hit along the shadow ray is its own triangle.  The
// traversal starts from the ray's hit on that triangle (seed_triangle_hit, computed as the
// traversal computes it), so it only searches for a closer hit and stops at the first one:
// the same answer as a full closest-hit query followed by the comparison.
template <bool COUNT, int ACCEL = ACCEL_ANY>
__device__ __forceinline__ bool restir_visible(const DevScene& sc, f3 pos, const LightPoint& lp, uint32_t light,
                                               uint32_t* stack, int stride, uint32_t* err) {
    f3 d = lp.pos - pos;
    f3 dir = d / sqrtf(dot(d, d));
    uint32_t prim = __float_as_uint(__ldg(&sc.light_rec[(uint64_t)LIGHT_RECORD * light + 5].w));
    const tt_instance* in = sc.instances + lp.instance;
    TraceState st;
    trace_init(st, sc, pos, dir, SHADOW_TMIN, SHADOW_TMAX, false);
    if (!st.have) return false;  // NaN direction or empty scene: the closest-hit query misses
    if (!seed_triangle_hit(sc, lp.instance, prim, __ldg(&in->index_offset), __ldg(&in->vertex_offset), pos, dir,
                           SHADOW_TMIN, SHADOW_TMAX, st.best, st.tbest))
        return false;
    Counters cnt{0u, 0u, 0u, 0u};
    while (!trace_step<COUNT, ACCEL, true>(st, sc, stack, stride, err, cnt))
        if (st.best.prim != prim || st.best.instance != lp.instance) return false;  // a closer hit occludes
    return st.best.hit && st.best.instance == lp.instance && st.best.prim == prim;
}

}  // namespace tt
