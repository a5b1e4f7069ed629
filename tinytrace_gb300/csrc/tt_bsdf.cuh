// OpenPBR six-lobe BSDF on the device, restated from the reference GLSL
// (src/material/{bsdf,fresnel,microfacet,diffuse_brdf,coat_brdf,fuzz_brdf,metal_brdf,
// specular_brdf,specular_btdf}.glsl).  Each function cites the GLSL it follows.
//
// GLSL leaves an `out` parameter that the callee never writes undefined; here every such
// value is zero (all locals the reference declares without an initialiser start at zero).
// Material constants are read through a pointer into global memory so that the 192-byte
// record is not held in registers.
#pragma once

#include "tt_common.cuh"

namespace tt {

using MatC = tt_material_constants;

// Lobe evaluate/sample functions are compiled out of line: inlined at every call site (albedo
// estimates, next-event estimation, lobe sampling) they made the shading kernel larger than the
// instruction cache.  Define TT_INLINE_LOBES to inline them.
#ifdef TT_INLINE_LOBES
#define TT_LOBE TT_HD
#else
#define TT_LOBE static __device__ __noinline__
#endif

constexpr float DENOM_TOLERANCE = 1.0e-10f;  // material.glsl:4-8
constexpr float RADIANCE_EPSILON = 1.0e-12f;
constexpr float PDF_EPSILON = 1.0e-6f;
constexpr float IOR_EPSILON = 1.0e-5f;

TT_HD f3 col3(const float* c) { return f3{c[0], c[1], c[2]}; }

// ---------------------------------------------------------------- math.glsl:35-92
struct LocalRotation {
    float t00, t01, t10, t11, i00, i01, i10, i11;
};
TT_HD LocalRotation local_frame_rotation(float angle) {
    LocalRotation r;
    if (angle == 0.0f || angle == 2.0f * PI) {
        r.t00 = 1.0f; r.t01 = 0.0f; r.t10 = 0.0f; r.t11 = 1.0f;
        r.i00 = 1.0f; r.i01 = 0.0f; r.i10 = 0.0f; r.i11 = 1.0f;
    } else {
        float s, c;
        tsincos(angle, &s, &c);
        r.t00 = c; r.t01 = s; r.t10 = -s; r.t11 = c;
        r.i00 = c; r.i01 = -s; r.i10 = s; r.i11 = c;
    }
    return r;
}
TT_HD f3 rotate_local(f3 l, const LocalRotation& r) {
    return f3{r.t00 * l.x + r.t10 * l.y, r.t01 * l.x + r.t11 * l.y, l.z};
}
TT_HD f3 inverse_rotate_local(f3 l, const LocalRotation& r) {
    return f3{r.i00 * l.x + r.i10 * l.y, r.i01 * l.x + r.i11 * l.y, l.z};
}
TT_HD f3 safe_normalize(f3 v) { return v * (1.0f / fmx(length(v), 1e-8f)); }
TT_HD float pow2(float v) { return v * v; }
TT_HD f3 pow2v(f3 v) { return v * v; }
TT_HD float pow5(float v) { return v * pow2(v) * pow2(v); }
TT_HD float pow6(float v) { return v * pow5(v); }
TT_HD float length_squared(f3 v) { return dot(v, v); }
TT_HD float cos_theta(f3 d) { return d.z; }
TT_HD float cos_theta_squared(f3 d) { return pow2(d.z); }
TT_HD float sin_theta_squared(f3 d) { return fmx(0.0f, 1.0f - cos_theta_squared(d)); }
TT_HD float sin_theta(f3 d) { return sqrtf(sin_theta_squared(d)); }
TT_HD float tan_theta_squared(f3 d) { return sin_theta_squared(d) / cos_theta_squared(d); }
TT_HD float sin_phi(f3 d) {
    float st = sin_theta(d);
    return fabsf(st) < 0.0001f ? 0.0f : clampf(d.y / st, -1.0f, 1.0f);
}
TT_HD float cos_phi(f3 d) {
    float st = sin_theta(d);
    return fabsf(st) < 0.0001f ? 1.0f : clampf(d.x / st, -1.0f, 1.0f);
}
TT_HD bool is_same_hemisphere(f3 a, f3 b) { return cos_theta(a) * cos_theta(b) >= 0.0f; }

// ---------------------------------------------------------------- fresnel.glsl:6-39
TT_HD f3 fresnel_schlick(f3 f0, float ct) { return f0 + pow5(1.0f - ct) * (1.0f - f0); }
TT_HD float fresnel_at_normal_incident(float ior) { return pow2((ior - 1.0f) / (ior + 1.0f)); }
TT_HD float dieletric_fresnel_factor(float ior) {
    return tlog((10893.0f * ior - 1438.2f) / (-774.4f * pow2(ior) + 10212.0f * ior + 1.0f));
}
TT_HD float fresnel_dielectric(float cti, float ior) {
    float sti2 = 1.0f - pow2(cti);
    float stt2 = sti2 / pow2(ior);
    if (stt2 >= 1.0f) return 1.0f;
    float ctt = sqrtf(1.0f - stt2);
    float par = (ior * cti - ctt) / (ior * cti + ctt);
    float per = (cti - ior * ctt) / (cti + ior * ctt);
    return 0.5f * (pow2(par) + pow2(per));
}
TT_HD float average_dielectric_fresnel(float ior) {
    if (ior > 1.0f) return dieletric_fresnel_factor(ior);
    if (ior < 1.0f) return 1.0f - pow2(ior) * (1.0f - dieletric_fresnel_factor(1.0f / ior));
    return 0.0f;
}

// ---------------------------------------------------------------- microfacet.glsl:7-54
TT_HD float microfacet_distribution(f2 alpha, f3 m) {
    float t2 = tan_theta_squared(m);
    if (isinf(t2)) return 0.0f;
    float e = t2 * (pow2(cos_phi(m) / alpha.x) + pow2(sin_phi(m) / alpha.y));
    return 1.0f / (PI * alpha.x * alpha.y * pow2(cos_theta_squared(m)) * pow2(1.0f + e));
}
TT_HD float microfacet_lambda(f2 alpha, f3 v) {
    float t2 = tan_theta_squared(v);
    if (isinf(t2)) return 0.0f;
    float a2 = pow2(cos_phi(v) * alpha.x) + pow2(sin_phi(v) * alpha.y);
    return (sqrtf(1.0f + a2 * t2) - 1.0f) / 2.0f;
}
TT_HD float microfacet_visibility(f2 alpha, f3 i, f3 o) {
    return 1.0f / (1.0f + microfacet_lambda(alpha, o) + microfacet_lambda(alpha, i));
}
TT_HD float microfacet_masking(f2 alpha, f3 v) { return 1.0f / (1.0f + microfacet_lambda(alpha, v)); }
TT_HD f3 microfacet_sample(f2 alpha, f3 view, f2 rnd) {
    view = normalize(f3{view.x * alpha.x, view.y * alpha.y, view.z});
    float phi = 2.0f * PI * rnd.x;
    float z = (1.0f - rnd.y) * (1.0f + view.z) - view.z;
    float st = sqrtf(saturate(1.0f - pow2(z)));
    float s, c;
    tsincos(phi, &s, &c);
    f3 h = f3{st * c, st * s, z} + view;
    return normalize(f3{h.x * alpha.x, h.y * alpha.y, h.z});
}
TT_HD f2 microfacet_roughness_to_alpha(float roughness, float anisotropy) {
    float r2 = pow2(roughness);
    float ax = r2 * sqrtf(2.0f / (1.0f + pow2(1.0f - anisotropy)));
    float ay = (1.0f - anisotropy) * ax;
    return f2{fmx(1e-4f, ax), fmx(1e-4f, ay)};
}

// ---------------------------------------------------------------- diffuse_brdf.glsl:9-61
TT_HD float oren_nayar(float ct, float s2) {
    float a = 1.0f - 0.5f * (s2 / (s2 + 0.33f));
    float b = 0.45f * s2 / (s2 + 0.09f);
    float s = sqrtf(1.0f - pow2(ct));
    float g = s * (tacos(ct) - s * ct) + (s / fmx(1e-7f, ct)) * (1.0f - (s * s * s)) * 2.0f / 3.0f;
    return a + (b * INVERSE_PI) * g;
}
TT_HD f3 energy_compensated_oren_nayar(f3 rho, float sigma, f3 wi, f3 wo) {
    float s2 = pow2(sigma);
    float s = dot(wi, wo) - cos_theta(wi) * cos_theta(wo);
    float s_over_t = s > 0.0f ? s / fmx(cos_theta(wi), cos_theta(wo)) : 0.0f;
    float a = 1.0f - 0.5f * (s2 / (s2 + 0.33f));
    float b = 0.45f * s2 / (s2 + 0.09f);
    float on_o = oren_nayar(cos_theta(wo), s2);
    float on_i = oren_nayar(cos_theta(wi), s2);
    float avg = a + (2.0f / 3.0f - 64.0f / (45.0f * PI)) * b;
    f3 rho_ms = pow2v(rho) * avg / (splat(1.0f) - rho * fmx(0.0f, 1.0f - avg));
    return (rho * INVERSE_PI) * (a + b * s_over_t) +
           (rho_ms * INVERSE_PI) * fmx(1e-7f, 1.0f - on_o) * fmx(1e-7f, 1.0f - on_i) /
               fmx(1e-7f, 1.0f - avg);
}
TT_HD f3 diffuse_rho(const MatC& m) { return m.base_weight * col3(m.base_color); }
TT_LOBE f3 diffuse_brdf_evaluate(const MatC& m, f3 wi, f3 wo, float& density) {
    if (cos_theta(wi) < DENOM_TOLERANCE || cos_theta(wo) < DENOM_TOLERANCE) return splat(0.0f);
    density = cosine_hemisphere_density(cos_theta(wo));
    return energy_compensated_oren_nayar(diffuse_rho(m), PI / 2.0f * m.base_diffuse_roughness, wi, wo);
}
TT_LOBE f3 diffuse_brdf_sample(const MatC& m, f3 wi, uint32_t& g, f3& wo, float& density) {
    if (cos_theta(wi) < DENOM_TOLERANCE) return splat(0.0f);
    wo = cosine_hemisphere_sample(random_vec2(g));
    density = cosine_hemisphere_density(cos_theta(wo));
    return energy_compensated_oren_nayar(diffuse_rho(m), PI / 2.0f * m.base_diffuse_roughness, wi, wo);
}
TT_HD f3 diffuse_brdf_albedo(const MatC& m, f3 wi) {
    if (cos_theta(wi) < DENOM_TOLERANCE) return splat(0.0f);
    return diffuse_rho(m);
}

// ---------------------------------------------------------------- coat_brdf.glsl:8-73
TT_HD f3 coat_brdf(f3 wi, f3 wo, f3 wir, f3 wor, float ior, f2 alpha, float& density) {
    f3 mn = normalize(wor + wir);
    float wdn = dot(wir, mn);
    float dist = microfacet_distribution(alpha, mn);
    float vn = dist * microfacet_masking(alpha, wir) * fmx(0.0f, wdn) / cos_theta(wir);
    float jac = 1.0f / fmx(fabsf(4.0f * wdn), DENOM_TOLERANCE);
    density = vn * jac;
    float fres = fresnel_dielectric(fabsf(wdn), ior);
    return splat(fres) * dist * microfacet_visibility(alpha, wir, wor) /
           fmx(4.0f * fabsf(cos_theta(wo)) * fabsf(cos_theta(wi)), DENOM_TOLERANCE);
}
TT_LOBE f3 coat_brdf_evaluate(const MatC& m, f3 wi, f3 wo, float& density) {
    if (!is_same_hemisphere(wo, wi)) return splat(0.0f);
    float ior = cos_theta(wi) > 0.0f ? m.coat_ior : 1.0f / m.coat_ior;
    if (fabsf(ior - 1.0f) < IOR_EPSILON) return splat(0.0f);
    f2 alpha = microfacet_roughness_to_alpha(m.coat_roughness, m.coat_roughness_anisotropy);
    LocalRotation rot = local_frame_rotation(2.0f * PI * m.coat_rotation);
    return coat_brdf(wi, wo, rotate_local(wi, rot), rotate_local(wo, rot), ior, alpha, density);
}
TT_LOBE f3 coat_brdf_sample(const MatC& m, f3 wi, uint32_t& g, f3& wo, float& density) {
    float ior = cos_theta(wi) > 0.0f ? m.coat_ior / 1.0f : 1.0f / m.coat_ior;
    if (fabsf(ior - 1.0f) < IOR_EPSILON) return splat(0.0f);
    f2 alpha = microfacet_roughness_to_alpha(m.coat_roughness, m.coat_roughness_anisotropy);
    LocalRotation rot = local_frame_rotation(2.0f * PI * m.coat_rotation);
    f3 wir = rotate_local(wi, rot);
    f3 mn = microfacet_sample(alpha, wir, random_vec2(g));
    if (cos_theta(wir) <= 0.0f) return splat(0.0f);
    f3 wor = -reflect(wir, mn);
    if (!is_same_hemisphere(wir, wor)) return splat(0.0f);
    wo = inverse_rotate_local(wor, rot);
    return coat_brdf(wi, wo, wir, wor, ior, alpha, density);
}
TT_HD f3 coat_brdf_albedo(const MatC& m, f3 wi, uint32_t& g) {
    float ior = m.coat_ior / 1.0f;
    if (fabsf(ior - 1.0f) < IOR_EPSILON) return splat(0.0f);
    f3 albedo = splat(0.0f), wo = splat(0.0f);
    float density = 0.0f;
    f3 brdf = coat_brdf_sample(m, wi, g, wo, density);
    if (length(brdf) > RADIANCE_EPSILON) albedo += brdf * fabsf(cos_theta(wo)) / fmx(PDF_EPSILON, density);
    return albedo / 1.0f;
}

// ---------------------------------------------------------------- fuzz_brdf.glsl:11-73
TT_HD float fuzz_albedo(float x, float y) {
    float s = y * (0.0206607f + 1.58491f * y) / (0.0379424f + y * (1.32227f + y));
    float mm = y * (-0.193854f + y * (-1.14885f + y * (1.7932f - 0.95943f * y * y))) / (0.046391f + y);
    float o = y * (0.000654023f + (-0.0207818f + 0.119681f * y) * y) / (1.26264f + y * (-1.92021f + y));
    return texp(-0.5f * pow2((x - mm) / s)) / (s * sqrtf(2.0f * PI)) + o;
}
TT_HD f2 ltc_inverse_coeffs(float x, float y) {
    float a = (2.58126f * x + 0.813703f * y) * y / (1.0f + 0.310327f * x * x + 2.60994f * x * y);
    float b = sqrtf(1.0f - x) * (y - 1.0f) * y * y * y /
              (0.0000254053f + 1.71228f * x - 1.71506f * x * y + 1.34174f * y * y);
    return f2{a, b};
}
struct LtcBasis {
    f3 c0, c1, c2;
};
TT_HD LtcBasis orthonormal_basis_ltc(f3 n) {
    float ls = n.x * n.x + n.y * n.y;
    f3 t = ls > 0.0f ? f3{n.x, n.y, 0.0f} * (1.0f / sqrtf(ls)) : f3{1.0f, 0.0f, 0.0f};
    return LtcBasis{t, f3{-t.y, t.x, 0.0f}, f3{0.0f, 0.0f, 1.0f}};
}
TT_HD f3 fuzz_density_and_brdf(const MatC& m, f3 dir, f3 wi, float a_inv, float roughness, float& density) {
    float jac = pow2(a_inv / length_squared(dir));
    density = fmx(cos_theta(dir), 0.0f) * INVERSE_PI * jac;
    float alb = fuzz_albedo(cos_theta(wi), roughness);
    return col3(m.fuzz_color) * alb * INVERSE_PI * jac;
}
TT_LOBE f3 fuzz_brdf_evaluate(const MatC& m, f3 wi, f3 wo, float& density) {
    if (cos_theta(wi) < DENOM_TOLERANCE || cos_theta(wo) < DENOM_TOLERANCE) return splat(0.0f);
    float roughness = clampf(m.fuzz_roughness, 0.01f, 1.0f);
    LtcBasis b = orthonormal_basis_ltc(wi);
    f3 w = f3{dot(b.c0, wo), dot(b.c1, wo), dot(b.c2, wo)};
    f2 ic = ltc_inverse_coeffs(cos_theta(wi), roughness);
    f3 dir = f3{ic.x * w.x + ic.y * w.z, ic.x * w.y, w.z};
    return fuzz_density_and_brdf(m, dir, wi, ic.x, roughness, density);
}
TT_LOBE f3 fuzz_brdf_sample(const MatC& m, f3 wi, uint32_t& g, f3& wo, float& density) {
    if (cos_theta(wi) < DENOM_TOLERANCE) return splat(0.0f);
    float roughness = clampf(m.fuzz_roughness, 0.01f, 1.0f);
    f3 dir = cosine_hemisphere_sample(random_vec2(g));
    f2 ic = ltc_inverse_coeffs(cos_theta(wi), roughness);
    f3 w = f3{dir.x / ic.x - dir.z * ic.y / ic.x, dir.y / ic.x, dir.z};
    LtcBasis b = orthonormal_basis_ltc(wi);
    f3 nw = normalize(w);
    wo = b.c0 * nw.x + b.c1 * nw.y + b.c2 * nw.z;
    return fuzz_density_and_brdf(m, dir, wi, ic.x, roughness, density);
}
TT_HD f3 fuzz_brdf_albedo(const MatC& m, f3 wi) { return splat(fuzz_albedo(cos_theta(wi), m.fuzz_roughness)); }

// ---------------------------------------------------------------- specular_brdf.glsl:8-116
TT_HD float specular_ior(const MatC& m) { return m.specular_ior / mixf(1.0f, m.coat_ior, m.coat_weight); }
TT_HD float specular_ior_ratio(const MatC& m) {
    float ior = specular_ior(m);
    float f0 = fresnel_at_normal_incident(ior);
    float csw = clampf(m.specular_weight, 0.0f, 1.0f / fmx(f0, DENOM_TOLERANCE));
    float eps = signf(ior - 1.0f) * sqrtf(csw * f0);
    return (1.0f + eps) / fmx(1.0f - eps, DENOM_TOLERANCE);
}
TT_HD f3 specular_fresnel_with_coat(const MatC& m, float ct, float ior) {
    float cra = sqrtf(1.0f - (1.0f - pow2(ct)) / pow2(m.coat_ior));
    float ior_mix = mixf(m.specular_ior, ior, m.coat_weight);
    return splat(fresnel_dielectric(cra, ior_mix));
}
TT_HD f3 specular_brdf(const MatC& m, f3 wi, f3 wo, f3 wir, f3 wor, f3 mn, f2 alpha, float ior, float& density) {
    float dist = microfacet_distribution(alpha, mn);
    float vn = dist * microfacet_masking(alpha, wir) * fmx(0.0f, dot(wir, mn)) / fmx(DENOM_TOLERANCE, cos_theta(wir));
    float jac = 1.0f / fmx(fabsf(4.0f * dot(wir, mn)), DENOM_TOLERANCE);
    density = vn * jac;
    f3 fres;
    if (cos_theta(wir) > 0.0f) fres = specular_fresnel_with_coat(m, fabsf(dot(wir, mn)), ior);
    else fres = splat(fresnel_dielectric(fabsf(dot(wir, mn)), ior));
    f3 brdf = fres * dist * microfacet_visibility(alpha, wir, wor) /
              fmx(4.0f * fabsf(cos_theta(wo)) * fabsf(cos_theta(wi)), DENOM_TOLERANCE);
    return brdf * col3(m.specular_color);
}
TT_LOBE f3 specular_brdf_evaluate(const MatC& m, f3 wi, f3 wo, float& density) {
    if (!is_same_hemisphere(wo, wi)) return splat(0.0f);
    float ratio = specular_ior_ratio(m);
    float ior = cos_theta(wi) > 0.0f ? ratio : 1.0f / ratio;
    if (fabsf(ior - 1.0f) < IOR_EPSILON) return splat(0.0f);
    f2 alpha = microfacet_roughness_to_alpha(m.specular_roughness, m.specular_roughness_anisotropy);
    LocalRotation rot = local_frame_rotation(2.0f * PI * m.specular_rotation);
    f3 wir = rotate_local(wi, rot), wor = rotate_local(wo, rot);
    f3 mn = normalize(wor + wir);
    if (dot(mn, wir) * cos_theta(wir) < 0.0f || dot(mn, wor) * cos_theta(wor) < 0.0f) return splat(0.0f);
    return specular_brdf(m, wi, wo, wir, wor, mn, alpha, ior, density);
}
TT_LOBE f3 specular_brdf_sample(const MatC& m, f3 wi, uint32_t& g, f3& wo, float& density) {
    float ratio = specular_ior_ratio(m);
    float ior = cos_theta(wi) > 0.0f ? ratio : 1.0f / ratio;
    if (fabsf(ior - 1.0f) < IOR_EPSILON) return splat(0.0f);
    f2 alpha = microfacet_roughness_to_alpha(m.specular_roughness, m.specular_roughness_anisotropy);
    LocalRotation rot = local_frame_rotation(2.0f * PI * m.specular_rotation);
    f3 wir = rotate_local(wi, rot);
    f3 mn;
    if (cos_theta(wir) > 0.0f) {
        mn = microfacet_sample(alpha, wir, random_vec2(g));
    } else {
        mn = microfacet_sample(alpha, f3{wir.x, wir.y, -wir.z}, random_vec2(g));
        mn.z *= -1.0f;
    }
    f3 wor = -reflect(wir, mn);
    if (!is_same_hemisphere(wir, wor)) {
        density = 1.0f;
        return splat(0.0f);
    }
    wo = inverse_rotate_local(wor, rot);
    return specular_brdf(m, wi, wo, wir, wor, mn, alpha, ior, density);
}
TT_HD f3 specular_brdf_albedo(const MatC& m, f3 wi, uint32_t& g) {
    if (fabsf(specular_ior_ratio(m) - 1.0f) < IOR_EPSILON) return splat(0.0f);
    f3 albedo = splat(0.0f), wo = splat(0.0f);
    float density = 0.0f;
    f3 brdf = specular_brdf_sample(m, wi, g, wo, density);
    if (length(brdf) > RADIANCE_EPSILON) albedo += brdf * fabsf(cos_theta(wo)) / fmx(DENOM_TOLERANCE, density);
    return albedo / 1.0f;
}

// ---------------------------------------------------------------- metal_brdf.glsl:9-82
TT_HD f3 fresnel_metal(float ct, f3 f0, f3 tint) {
    const float mu_bar = 1.0f / 7.0f;
    const float denom = mu_bar * pow6(1.0f - mu_bar);
    return fresnel_schlick(f0, ct) - ct * pow6(1.0f - ct) * (1.0f - tint) * fresnel_schlick(f0, mu_bar) / denom;
}
TT_HD f3 metal_brdf(const MatC& m, f2 alpha, f3 mn, f3 wi, f3 wo, f3 wir, f3 wor, float& density) {
    float dist = microfacet_distribution(alpha, mn);
    float vn = dist * microfacet_masking(alpha, wir) * fmx(0.0f, dot(wir, mn)) / fmx(DENOM_TOLERANCE, cos_theta(wir));
    float jac = 1.0f / fmx(fabsf(4.0f * dot(wir, mn)), DENOM_TOLERANCE);
    density = fmx(PDF_EPSILON, vn * jac);
    f3 fres = fresnel_metal(fabsf(dot(wir, mn)), m.base_weight * col3(m.base_color),
                            m.specular_weight * col3(m.specular_color));
    float vis = microfacet_visibility(alpha, wir, wor);
    return fres * dist * vis / fmx(4.0f * fabsf(cos_theta(wo)) * fabsf(cos_theta(wi)), DENOM_TOLERANCE);
}
TT_LOBE f3 metal_brdf_evaluate(const MatC& m, f3 wi, f3 wo, float& density) {
    if (cos_theta(wi) < DENOM_TOLERANCE || cos_theta(wo) < DENOM_TOLERANCE) {
        density = PDF_EPSILON;
        return splat(0.0f);
    }
    LocalRotation rot = local_frame_rotation(2.0f * PI * m.specular_rotation);
    f3 wir = rotate_local(wi, rot), wor = rotate_local(wo, rot);
    f2 alpha = microfacet_roughness_to_alpha(m.specular_roughness, m.specular_roughness_anisotropy);
    f3 mn = normalize(wor + wir);
    return metal_brdf(m, alpha, mn, wi, wo, wir, wor, density);
}
TT_LOBE f3 metal_brdf_sample(const MatC& m, f3 wi, uint32_t& g, f3& wo, float& density) {
    if (cos_theta(wi) < DENOM_TOLERANCE) {
        density = PDF_EPSILON;
        return splat(0.0f);
    }
    f2 alpha = microfacet_roughness_to_alpha(m.specular_roughness, m.specular_roughness_anisotropy);
    LocalRotation rot = local_frame_rotation(2.0f * PI * m.specular_rotation);
    f3 wir = rotate_local(wi, rot);
    f3 mn = microfacet_sample(alpha, wir, random_vec2(g));
    f3 wor = -reflect(wir, mn);
    if (!is_same_hemisphere(wir, wor)) return splat(0.0f);
    wo = inverse_rotate_local(wor, rot);
    return metal_brdf(m, alpha, mn, wi, wo, wir, wor, density);
}
TT_HD f3 metal_brdf_albedo(const MatC& m, f3 wi, uint32_t& g) {
    if (cos_theta(wi) < DENOM_TOLERANCE) return splat(0.0f);
    f3 albedo = splat(0.0f), wo = splat(0.0f);
    float density = 0.0f;
    f3 brdf = metal_brdf_sample(m, wi, g, wo, density);
    if (length(brdf) > RADIANCE_EPSILON) albedo += brdf * fabsf(cos_theta(wo)) / fmx(PDF_EPSILON, density);
    return albedo / 1.0f;
}

// ---------------------------------------------------------------- specular_btdf.glsl:8-119
TT_HD f3 btdf_tint(const MatC& m) {
    return m.transmission_depth == 0.0f ? col3(m.transmission_color) : splat(1.0f);
}
TT_HD f3 specular_btdf(const MatC& m, f3 mn, f2 alpha, f3 wi, f3 wo, f3 wir, f3 wor, float ior, float& density) {
    float jac = pow2(ior) * fabsf(cos_theta(wi)) / fmx(pow2(cos_theta(wo) + ior * cos_theta(wi)), DENOM_TOLERANCE);
    float dist = microfacet_distribution(alpha, mn);
    float vn = dist * microfacet_masking(alpha, wir) * fmx(0.0f, dot(wir, mn)) /
               fmx(DENOM_TOLERANCE, fabsf(cos_theta(wir)));
    density = vn * jac;
    float vis = microfacet_visibility(alpha, wir, wor);
    float trans = fmx(0.0f, 1.0f - fresnel_dielectric(fabsf(dot(wir, mn)), 1.0f / ior));
    float btdf = trans * fabsf(dot(wir, mn)) * jac * vis * dist /
                 fmx(fabsf(cos_theta(wo)) * fabsf(cos_theta(wi)), DENOM_TOLERANCE);
    return btdf * btdf_tint(m);
}
TT_LOBE f3 specular_btdf_evaluate(const MatC& m, f3 wi, f3 wo, float& density) {
    if (is_same_hemisphere(wo, wi)) {
        density = 1.0f;
        return splat(0.0f);
    }
    float ior = cos_theta(wi) > 0.0f ? 1.0f / m.specular_ior : m.specular_ior;
    if (fabsf(ior - 1.0f) < IOR_EPSILON) {
        f3 tint = btdf_tint(m);
        density = 1.0f / PDF_EPSILON;
        return tint * density / fmx(DENOM_TOLERANCE, fabsf(cos_theta(wo)));
    }
    LocalRotation rot = local_frame_rotation(2.0f * PI * m.specular_rotation);
    f3 wir = rotate_local(wi, rot), wor = rotate_local(wo, rot);
    f3 mn = -wor - ior * wir;
    if (length_squared(mn) == 0.0f) return splat(0.0f);
    mn = safe_normalize(mn);
    if (cos_theta(mn) <= 0.0f) mn = mn * -1.0f;
    f2 alpha = microfacet_roughness_to_alpha(m.specular_roughness, m.specular_roughness_anisotropy);
    return specular_btdf(m, mn, alpha, wi, wo, wir, wor, ior, density);
}
TT_HD bool refraction_direction(f3 n, float ior, f3 wi, f3& dir) {
    float cti = dot(wi, n);
    float sti2 = fmx(0.0f, 1.0f - pow2(cti));
    float stt2 = pow2(ior) * sti2;
    if (stt2 >= 1.0f) return false;
    float ctt = sqrtf(1.0f - stt2);
    dir = ior * -wi + (ior * cti - ctt) * n;
    return true;
}
TT_LOBE f3 specular_btdf_sample(const MatC& m, f3 wi, uint32_t& g, f3& wo, float& density) {
    float ior = cos_theta(wi) > 0.0f ? 1.0f / m.specular_ior : m.specular_ior;
    if (fabsf(ior - 1.0f) < IOR_EPSILON) {
        wo = -wi;
        density = 1.0f / PDF_EPSILON;
        f3 tint = btdf_tint(m);
        return tint * density / fmx(DENOM_TOLERANCE, fabsf(cos_theta(wo)));
    }
    LocalRotation rot = local_frame_rotation(2.0f * PI * m.specular_rotation);
    f3 wir = rotate_local(wi, rot);
    f2 alpha = microfacet_roughness_to_alpha(m.specular_roughness, m.specular_roughness_anisotropy);
    f3 mn;
    if (cos_theta(wir) > 0.0f) {
        mn = microfacet_sample(alpha, wir, random_vec2(g));
    } else {
        mn = microfacet_sample(alpha, f3{wir.x, wir.y, -cos_theta(wir)}, random_vec2(g));
        mn.z *= -1.0f;
    }
    f3 rd = splat(0.0f);
    if (!refraction_direction(mn, ior, wir, rd)) {
        density = PDF_EPSILON;
        return splat(0.0f);
    }
    f3 wor = -safe_normalize(rd);
    wo = inverse_rotate_local(wor, rot);
    return specular_btdf(m, mn, alpha, wi, wo, wir, wor, ior, density);
}
TT_HD f3 specular_btdf_albedo(const MatC& m, f3 wi, uint32_t& g) {
    if (fabsf(m.specular_ior - 1.0f) < IOR_EPSILON) return btdf_tint(m);
    f3 albedo = splat(0.0f), wo = splat(0.0f);
    float density = 0.0f;
    f3 btdf = specular_btdf_sample(m, wi, g, wo, density);
    if (length(btdf) > RADIANCE_EPSILON) albedo += btdf * fabsf(cos_theta(wo)) / fmx(DENOM_TOLERANCE, density);
    return albedo / 1.0f;
}

// ---------------------------------------------------------------- bsdf.glsl:15-203
enum { FUZZ = 0, COAT = 1, METAL = 2, SPEC_BRDF = 3, SPEC_BTDF = 4, DIFFUSE = 5, LOBE_COUNT = 6 };
struct Lobes {
    f3 weights[LOBE_COUNT];
    float probs[LOBE_COUNT];
};

// Lobe sets: bit i stands for lobe i.  A material can carry weight in lobe i only where the
// albedo condition of bsdf_prepare holds for it (lobe_set_of); elsewhere the lobe's albedo is
// zero, so its probability is zero (or NaN), it is never evaluated and never sampled.  The BSDF
// functions below take the lobe set LS their callers' materials fall into and compile the lobes
// outside it away: for every material whose lobe_set_of is a subset of LS they compute exactly
// what the six-lobe code computes (same operations, same generator draws).
constexpr uint32_t LOBE_SET_ALL = (1u << LOBE_COUNT) - 1u;
constexpr uint32_t LOBE_SET_DIELECTRIC = (1u << SPEC_BRDF) | (1u << DIFFUSE);  // opaque, no coat or fuzz
constexpr uint32_t LOBE_SET_METAL = 1u << METAL;                               // fully metallic
constexpr uint32_t LOBE_SET_BASE = LOBE_SET_DIELECTRIC | LOBE_SET_METAL;        // partly metallic

// The lobes whose albedo bsdf_prepare computes for material m (the conditions of bsdf.glsl:39-59).
__host__ __device__ inline uint32_t lobe_set_of(const MatC& m) {
    bool fully_metallic = m.base_metalness == 1.0f;
    uint32_t set = 0u;
    if (m.fuzz_weight > 0.0f) set |= 1u << FUZZ;
    if (m.coat_weight > 0.0f) set |= 1u << COAT;
    if (m.base_metalness > 0.0f) set |= 1u << METAL;
    if (!fully_metallic) set |= 1u << SPEC_BRDF;
    if (!fully_metallic && m.transmission_weight > 0.0f) set |= 1u << SPEC_BTDF;
    if (!fully_metallic && m.transmission_weight != 1.0f) set |= 1u << DIFFUSE;
    return set;
}

template <uint32_t LS, int LOBE>
TT_HD constexpr bool has_lobe() { return (LS >> LOBE) & 1u; }

// lobe_weights + lobe_probabilities (bsdf.glsl:33-120).  Albedos are needed only here.
template <uint32_t LS = LOBE_SET_ALL>
TT_HD Lobes bsdf_prepare(const MatC& m, f3 wi, uint32_t& g) {
    Lobes l;
    f3 alb[LOBE_COUNT];
    bool fully_metallic = m.base_metalness == 1.0f;
    bool fully_transmissive = m.transmission_weight == 1.0f;
    alb[FUZZ] = has_lobe<LS, FUZZ>() && m.fuzz_weight > 0.0f ? fuzz_brdf_albedo(m, wi) : splat(0.0f);
    alb[COAT] = has_lobe<LS, COAT>() && m.coat_weight > 0.0f ? coat_brdf_albedo(m, wi, g) : splat(0.0f);
    alb[METAL] = has_lobe<LS, METAL>() && m.base_metalness > 0.0f ? metal_brdf_albedo(m, wi, g) : splat(0.0f);
    alb[SPEC_BRDF] = has_lobe<LS, SPEC_BRDF>() && !fully_metallic ? specular_brdf_albedo(m, wi, g) : splat(0.0f);
    alb[SPEC_BTDF] = has_lobe<LS, SPEC_BTDF>() && !fully_metallic && m.transmission_weight > 0.0f
                         ? specular_btdf_albedo(m, wi, g)
                         : splat(0.0f);
    alb[DIFFUSE] = has_lobe<LS, DIFFUSE>() && !fully_metallic && !fully_transmissive ? diffuse_brdf_albedo(m, wi)
                                                                                      : splat(0.0f);

    l.weights[FUZZ] = splat(m.fuzz_weight);
    f3 coated_base_weight = mix3(splat(1.0f), 1.0f - alb[FUZZ], m.fuzz_weight);
    l.weights[COAT] = coated_base_weight * m.coat_weight;
    f3 base_darkening = splat(1.0f);
    if (has_lobe<LS, COAT>() && m.coat_weight > 0.0f && m.coat_darkening > 0.0f) {
        float fresnel_weight = saturate(m.specular_weight * fresnel_at_normal_incident(specular_ior(m)));
        float dielectric_roughness = mixf(1.0f, m.specular_roughness, fresnel_weight);
        float base_roughness = mixf(dielectric_roughness, m.specular_roughness, m.base_metalness);
        float average_fresnel = 1.0f - (1.0f - average_dielectric_fresnel(m.coat_ior)) / pow2(m.coat_ior);
        float fres = fresnel_dielectric(fabsf(cos_theta(wi)), m.coat_ior);
        float drc = mixf(fres, average_fresnel, base_roughness);
        f3 dielectric_base_albedo = mix3(alb[DIFFUSE], alb[SPEC_BTDF], m.transmission_weight);
        f3 base_albedo = mix3(dielectric_base_albedo, alb[METAL], m.base_metalness);
        f3 darkening_factor = (1.0f - drc) / (1.0f - base_albedo * drc);
        base_darkening = mix3(splat(1.0f), darkening_factor, m.coat_weight * m.coat_darkening);
    }
    f3 base_weight = coated_base_weight *
                     mix3(splat(1.0f), base_darkening * col3(m.coat_color) * (1.0f - alb[COAT]), m.coat_weight);
    l.weights[METAL] = base_weight * m.base_metalness;
    f3 dielectric_base_weight = base_weight * splat(1.0f - m.base_metalness);
    l.weights[SPEC_BRDF] = dielectric_base_weight;
    l.weights[SPEC_BTDF] = dielectric_base_weight * m.transmission_weight;
    f3 opaque = dielectric_base_weight * (1.0f - m.transmission_weight);
    l.weights[DIFFUSE] = opaque * (1.0f - alb[SPEC_BRDF]);

    float total = 0.0f;
#pragma unroll
    for (int i = 0; i < LOBE_COUNT; ++i) {
        l.probs[i] = length(l.weights[i] * alb[i]);
        total += l.probs[i];
    }
    total = fmx(DENOM_TOLERANCE, total);
#pragma unroll
    for (int i = 0; i < LOBE_COUNT; ++i) l.probs[i] /= total;
    return l;
}

template <uint32_t LS = LOBE_SET_ALL>
TT_HD f3 bsdf_evaluate_lobes(const MatC& m, const Lobes& l, f3 wi, f3 wo, int skip, float* dens) {
    f3 b = splat(0.0f);
    if (has_lobe<LS, FUZZ>() && skip != FUZZ && l.probs[FUZZ] > 0.0f)
        b += l.weights[FUZZ] * fuzz_brdf_evaluate(m, wi, wo, dens[FUZZ]);
    if (has_lobe<LS, COAT>() && skip != COAT && l.probs[COAT] > 0.0f)
        b += l.weights[COAT] * coat_brdf_evaluate(m, wi, wo, dens[COAT]);
    if (has_lobe<LS, METAL>() && skip != METAL && l.probs[METAL] > 0.0f)
        b += l.weights[METAL] * metal_brdf_evaluate(m, wi, wo, dens[METAL]);
    if (has_lobe<LS, SPEC_BRDF>() && skip != SPEC_BRDF && l.probs[SPEC_BRDF] > 0.0f)
        b += l.weights[SPEC_BRDF] * specular_brdf_evaluate(m, wi, wo, dens[SPEC_BRDF]);
    if (has_lobe<LS, DIFFUSE>() && skip != DIFFUSE && l.probs[DIFFUSE] > 0.0f)
        b += l.weights[DIFFUSE] * diffuse_brdf_evaluate(m, wi, wo, dens[DIFFUSE]);
    if (has_lobe<LS, SPEC_BTDF>() && skip != SPEC_BTDF && l.probs[SPEC_BTDF] > 0.0f)
        b += l.weights[SPEC_BTDF] * specular_btdf_evaluate(m, wi, wo, dens[SPEC_BTDF]);
    return b;
}
TT_HD float bsdf_total_pdf(const Lobes& l, const float* dens) {
    float d = 0.0f;
#pragma unroll
    for (int i = 0; i < LOBE_COUNT; ++i) d += l.probs[i] * dens[i];
    return d;
}
template <uint32_t LS = LOBE_SET_ALL>
TT_HD f3 bsdf_evaluate(const MatC& m, const Lobes& l, f3 wi, f3 wo, float& density) {
    float dens[LOBE_COUNT] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    f3 b = bsdf_evaluate_lobes<LS>(m, l, wi, wo, -1, dens);
    density = bsdf_total_pdf(l, dens);
    return b;
}
// A lobe outside LS has probability zero (or NaN) and is never the sampled one: its case below
// is unreachable and compiled away.
template <uint32_t LS = LOBE_SET_ALL>
TT_HD f3 bsdf_sample(const MatC& m, const Lobes& l, f3 wi, uint32_t& g, f3& wo, float& density, int& sampled) {
    static_assert(LS == LOBE_SET_ALL || (LS & ~LOBE_SET_BASE) == 0u, "lobe sets: all six, or within metal + dielectric");
    float rnd = random_float(g);
    float acc = 0.0f;
    int lobe = -1;
#pragma unroll
    for (int i = 0; i < LOBE_COUNT; ++i) {
        acc += l.probs[i];
        if (lobe < 0 && rnd < acc) lobe = i;
    }
    if (lobe < 0) {
        sampled = -1;
        density = 1.0f;
        return splat(0.0f);
    }
    float lobe_density = 0.0f;
    f3 lobe_bsdf = splat(0.0f);
    if (LS == LOBE_SET_ALL) {
        switch (lobe) {
            case FUZZ: lobe_bsdf = fuzz_brdf_sample(m, wi, g, wo, lobe_density); break;
            case COAT: lobe_bsdf = coat_brdf_sample(m, wi, g, wo, lobe_density); break;
            case METAL: lobe_bsdf = metal_brdf_sample(m, wi, g, wo, lobe_density); break;
            case SPEC_BRDF: lobe_bsdf = specular_brdf_sample(m, wi, g, wo, lobe_density); break;
            case SPEC_BTDF: lobe_bsdf = specular_btdf_sample(m, wi, g, wo, lobe_density); break;
            default: lobe_bsdf = diffuse_brdf_sample(m, wi, g, wo, lobe_density); break;
        }
    } else if (has_lobe<LS, METAL>() && (LS == LOBE_SET_METAL || lobe == METAL)) {
        lobe_bsdf = metal_brdf_sample(m, wi, g, wo, lobe_density);
    } else if (has_lobe<LS, SPEC_BRDF>() && lobe == SPEC_BRDF) {
        lobe_bsdf = specular_brdf_sample(m, wi, g, wo, lobe_density);
    } else if (has_lobe<LS, DIFFUSE>()) {
        lobe_bsdf = diffuse_brdf_sample(m, wi, g, wo, lobe_density);
    }
    float dens[LOBE_COUNT] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    f3 b = bsdf_evaluate_lobes<LS>(m, l, wi, wo, lobe, dens);
    f3 w = splat(0.0f);
#pragma unroll
    for (int i = 0; i < LOBE_COUNT; ++i) {  // unrolled selects keep both arrays in registers
        if (i == lobe) {
            dens[i] = lobe_density;
            w = l.weights[i];
        }
    }
    density = bsdf_total_pdf(l, dens);
    sampled = lobe;
    return b + w * lobe_bsdf;
}

}  // namespace tt
