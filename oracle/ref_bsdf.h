// TEST INFRASTRUCTURE — the CPU oracle for the tinytrace rendering hot path (the checker,
// never the product; only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg
// may load it).
//
// The OpenPBR six-lobe BSDF restated from src/material/*.glsl.
//
// GLSL leaves `out` parameters that a callee never writes undefined; this restatement (and
// the CUDA implementation) defines every such value as zero: all locals that the reference
// declares without an initialiser start at zero here.
#pragma once

#include "ref_scene.h"

namespace ref {

constexpr float DENOM_TOLERANCE = 1.0e-10f;  // material.glsl:4
constexpr float RADIANCE_EPSILON = 1.0e-12f;
constexpr float THROUGHPUT_EPSILON = 1.0e-6f;
constexpr float PDF_EPSILON = 1.0e-6f;
constexpr float IOR_EPSILON = 1.0e-5f;

// ---------------------------------------------------------------- math.glsl:35-92
struct LocalRotation {
    float t00, t01, t10, t11;  // column-major mat2: col0 = (t00, t01), col1 = (t10, t11)
    float i00, i01, i10, i11;
};
inline LocalRotation local_frame_rotation(float angle) {
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
// mat2 * v.xy (column-major): x = m00*v.x + m10*v.y, y = m01*v.x + m11*v.y
inline v3 rotate_local(v3 l, const LocalRotation& r) {
    return v3{r.t00 * l.x + r.t10 * l.y, r.t01 * l.x + r.t11 * l.y, l.z};
}
inline v3 inverse_rotate_local(v3 l, const LocalRotation& r) {
    return v3{r.i00 * l.x + r.i10 * l.y, r.i01 * l.x + r.i11 * l.y, l.z};
}
inline v3 safe_normalize(v3 v) { return v * (1.0f / fmx(length(v), 1e-8f)); }
inline float pow2(float v) { return v * v; }
inline v3 pow2v(v3 v) { return v * v; }
inline float pow5(float v) { return v * pow2(v) * pow2(v); }
inline float pow6(float v) { return v * pow5(v); }
inline float length_squared(v3 v) { return dot(v, v); }
inline float length_squared2(v2 v) { return dot2(v, v); }
inline float cos_theta(v3 d) { return d.z; }
inline float cos_theta_squared(v3 d) { return pow2(d.z); }
inline float sin_theta_squared(v3 d) { return fmx(0.0f, 1.0f - cos_theta_squared(d)); }
inline float sin_theta(v3 d) { return std::sqrt(sin_theta_squared(d)); }
inline float tan_theta_squared(v3 d) { return sin_theta_squared(d) / cos_theta_squared(d); }
inline float sin_phi(v3 d) {
    float st = sin_theta(d);
    return std::fabs(st) < 0.0001f ? 0.0f : clampf(d.y / st, -1.0f, 1.0f);
}
inline float cos_phi(v3 d) {
    float st = sin_theta(d);
    return std::fabs(st) < 0.0001f ? 1.0f : clampf(d.x / st, -1.0f, 1.0f);
}
inline bool is_same_hemisphere(v3 a, v3 b) { return cos_theta(a) * cos_theta(b) >= 0.0f; }
inline float lengthv(v3 v) { return length(v); }

// ---------------------------------------------------------------- fresnel.glsl
inline v3 fresnel_schlick(v3 f0, float ct) { return f0 + pow5(1.0f - ct) * (1.0f - f0); }
inline float fresnel_at_normal_incident(float ior) {
    return pow2((ior - 1.0f) / (ior + 1.0f));
}
inline float dieletric_fresnel_factor(float ior) {
    return tlog((10893.0f * ior - 1438.2f) / (-774.4f * pow2(ior) + 10212.0f * ior + 1.0f));
}
inline float fresnel_dielectric(float cti, float ior) {
    float sti2 = 1.0f - pow2(cti);
    float stt2 = sti2 / pow2(ior);
    if (stt2 >= 1.0f) return 1.0f;
    float ctt = std::sqrt(1.0f - stt2);
    float par = (ior * cti - ctt) / (ior * cti + ctt);
    float per = (cti - ior * ctt) / (cti + ior * ctt);
    return 0.5f * (pow2(par) + pow2(per));
}
inline float average_dielectric_fresnel(float ior) {
    if (ior > 1.0f) return dieletric_fresnel_factor(ior);
    if (ior < 1.0f) return 1.0f - pow2(ior) * (1.0f - dieletric_fresnel_factor(1.0f / ior));
    return 0.0f;
}

// ---------------------------------------------------------------- microfacet.glsl
inline float microfacet_distribution(v2 alpha, v3 m) {
    float t2 = tan_theta_squared(m);
    if (std::isinf(t2)) return 0.0f;
    float e = t2 * (pow2(cos_phi(m) / alpha.x) + pow2(sin_phi(m) / alpha.y));
    return 1.0f / (PI * alpha.x * alpha.y * pow2(cos_theta_squared(m)) * pow2(1.0f + e));
}
inline float microfacet_lambda(v2 alpha, v3 v) {
    float t2 = tan_theta_squared(v);
    if (std::isinf(t2)) return 0.0f;
    float a2 = pow2(cos_phi(v) * alpha.x) + pow2(sin_phi(v) * alpha.y);
    return (std::sqrt(1.0f + a2 * t2) - 1.0f) / 2.0f;
}
inline float microfacet_visibility(v2 alpha, v3 i, v3 o) {
    return 1.0f / (1.0f + microfacet_lambda(alpha, o) + microfacet_lambda(alpha, i));
}
inline float microfacet_masking(v2 alpha, v3 v) {
    return 1.0f / (1.0f + microfacet_lambda(alpha, v));
}
inline v3 microfacet_sample(v2 alpha, v3 view, v2 rnd) {
    view = normalize(v3{view.x * alpha.x, view.y * alpha.y, view.z});
    float phi = 2.0f * PI * rnd.x;
    float z = (1.0f - rnd.y) * (1.0f + view.z) - view.z;
    float st = std::sqrt(saturate(1.0f - pow2(z)));
    float s, c;
    tsincos(phi, &s, &c);
    v3 h = v3{st * c, st * s, z} + view;
    return normalize(v3{h.x * alpha.x, h.y * alpha.y, h.z});
}
inline v2 microfacet_roughness_to_alpha(float roughness, float anisotropy) {
    float r2 = pow2(roughness);
    float ax = r2 * std::sqrt(2.0f / (1.0f + pow2(1.0f - anisotropy)));
    float ay = (1.0f - anisotropy) * ax;
    return v2{fmx(1e-4f, ax), fmx(1e-4f, ay)};
}

// ---------------------------------------------------------------- diffuse_brdf.glsl
inline float oren_nayar(float ct, float s2) {
    float a = 1.0f - 0.5f * (s2 / (s2 + 0.33f));
    float b = 0.45f * s2 / (s2 + 0.09f);
    float s = std::sqrt(1.0f - pow2(ct));
    float g = s * (tacos(ct) - s * ct) + (s / fmx(1e-7f, ct)) * (1.0f - (s * s * s)) * 2.0f / 3.0f;
    return a + (b * INVERSE_PI) * g;
}
inline v3 energy_compensated_oren_nayar(v3 rho, float sigma, v3 wi, v3 wo) {
    float s2 = pow2(sigma);
    float s = dot(wi, wo) - cos_theta(wi) * cos_theta(wo);
    float s_over_t = s > 0.0f ? s / fmx(cos_theta(wi), cos_theta(wo)) : 0.0f;
    float a = 1.0f - 0.5f * (s2 / (s2 + 0.33f));
    float b = 0.45f * s2 / (s2 + 0.09f);
    float on_o = oren_nayar(cos_theta(wo), s2);
    float on_i = oren_nayar(cos_theta(wi), s2);
    float avg = a + (2.0f / 3.0f - 64.0f / (45.0f * PI)) * b;
    v3 rho_ms = pow2v(rho) * avg / (splat3(1.0f) - rho * fmx(0.0f, 1.0f - avg));
    return (rho * INVERSE_PI) * (a + b * s_over_t) +
           (rho_ms * INVERSE_PI) * fmx(1e-7f, 1.0f - on_o) * fmx(1e-7f, 1.0f - on_i) /
               fmx(1e-7f, 1.0f - avg);
}
inline v3 diffuse_brdf_evaluate(const MaterialConstants& m, v3 wi, v3 wo, float& density) {
    if (cos_theta(wi) < DENOM_TOLERANCE || cos_theta(wo) < DENOM_TOLERANCE) return splat3(0.0f);
    density = cosine_hemisphere_density(cos_theta(wo));
    return energy_compensated_oren_nayar(m.base_weight * xyz(m.base_color),
                                         PI / 2.0f * m.base_diffuse_roughness, wi, wo);
}
inline v3 diffuse_brdf_sample(const MaterialConstants& m, v3 wi, Generator& g, v3& wo,
                              float& density) {
    if (cos_theta(wi) < DENOM_TOLERANCE) return splat3(0.0f);
    wo = cosine_hemisphere_sample(random_vec2(g));
    density = cosine_hemisphere_density(cos_theta(wo));
    return energy_compensated_oren_nayar(m.base_weight * xyz(m.base_color),
                                         PI / 2.0f * m.base_diffuse_roughness, wi, wo);
}
inline v3 diffuse_brdf_albedo(const MaterialConstants& m, v3 wi) {
    if (cos_theta(wi) < DENOM_TOLERANCE) return splat3(0.0f);
    return m.base_weight * xyz(m.base_color);
}

// ---------------------------------------------------------------- coat_brdf.glsl
inline v3 coat_brdf(const MaterialConstants& m, v3 wi, v3 wo, v3 wir, v3 wor, float ior,
                    v2 alpha, float& density) {
    (void)m;
    v3 mn = normalize(wor + wir);
    float wi_dot_n = dot(wir, mn);
    float dist = microfacet_distribution(alpha, mn);
    float vis_normals = dist * microfacet_masking(alpha, wir) * fmx(0.0f, wi_dot_n) / cos_theta(wir);
    float jac = 1.0f / fmx(std::fabs(4.0f * wi_dot_n), DENOM_TOLERANCE);
    density = vis_normals * jac;
    float fres = fresnel_dielectric(std::fabs(wi_dot_n), ior);
    return splat3(fres) * dist * microfacet_visibility(alpha, wir, wor) /
           fmx(4.0f * std::fabs(cos_theta(wo)) * std::fabs(cos_theta(wi)), DENOM_TOLERANCE);
}
inline v3 coat_brdf_evaluate(const MaterialConstants& m, v3 wi, v3 wo, float& density) {
    if (!is_same_hemisphere(wo, wi)) return splat3(0.0f);
    float ior = cos_theta(wi) > 0.0f ? m.coat_ior : 1.0f / m.coat_ior;
    if (std::fabs(ior - 1.0f) < IOR_EPSILON) return splat3(0.0f);
    v2 alpha = microfacet_roughness_to_alpha(m.coat_roughness, m.coat_roughness_anisotropy);
    LocalRotation rot = local_frame_rotation(2.0f * PI * m.coat_rotation);
    return coat_brdf(m, wi, wo, rotate_local(wi, rot), rotate_local(wo, rot), ior, alpha, density);
}
inline v3 coat_brdf_sample(const MaterialConstants& m, v3 wi, Generator& g, v3& wo,
                           float& density) {
    float ior = cos_theta(wi) > 0.0f ? m.coat_ior / 1.0f : 1.0f / m.coat_ior;
    if (std::fabs(ior - 1.0f) < IOR_EPSILON) return splat3(0.0f);
    v2 alpha = microfacet_roughness_to_alpha(m.coat_roughness, m.coat_roughness_anisotropy);
    LocalRotation rot = local_frame_rotation(2.0f * PI * m.coat_rotation);
    v3 wir = rotate_local(wi, rot);
    v3 mn = microfacet_sample(alpha, wir, random_vec2(g));
    if (cos_theta(wir) <= 0.0f) return splat3(0.0f);
    v3 wor = -reflect(wir, mn);
    if (!is_same_hemisphere(wir, wor)) return splat3(0.0f);
    wo = inverse_rotate_local(wor, rot);
    return coat_brdf(m, wi, wo, wir, wor, ior, alpha, density);
}
inline v3 coat_brdf_albedo(const MaterialConstants& m, v3 wi, Generator& g) {
    float ior = m.coat_ior / 1.0f;
    if (std::fabs(ior - 1.0f) < IOR_EPSILON) return splat3(0.0f);
    v3 albedo = splat3(0.0f);
    v3 wo = splat3(0.0f);
    float density = 0.0f;
    v3 brdf = coat_brdf_sample(m, wi, g, wo, density);
    if (length(brdf) > RADIANCE_EPSILON)
        albedo += brdf * std::fabs(cos_theta(wo)) / fmx(PDF_EPSILON, density);
    return albedo / 1.0f;
}

// ---------------------------------------------------------------- fuzz_brdf.glsl
inline float fuzz_albedo(float x, float y) {
    float s = y * (0.0206607f + 1.58491f * y) / (0.0379424f + y * (1.32227f + y));
    float mm = y * (-0.193854f + y * (-1.14885f + y * (1.7932f - 0.95943f * y * y))) /
               (0.046391f + y);
    float o = y * (0.000654023f + (-0.0207818f + 0.119681f * y) * y) /
              (1.26264f + y * (-1.92021f + y));
    return texp(-0.5f * pow2((x - mm) / s)) / (s * std::sqrt(2.0f * PI)) + o;
}
inline v2 ltc_inverse_coeffs(float x, float y) {
    float a = (2.58126f * x + 0.813703f * y) * y / (1.0f + 0.310327f * x * x + 2.60994f * x * y);
    float b = std::sqrt(1.0f - x) * (y - 1.0f) * y * y * y /
              (0.0000254053f + 1.71228f * x - 1.71506f * x * y + 1.34174f * y * y);
    return v2{a, b};
}
struct Mat3 {
    v3 c0, c1, c2;
};
inline Mat3 orthonormal_basis_ltc(v3 n) {
    float ls = length_squared2(v2{n.x, n.y});
    v3 t = ls > 0.0f ? v3{n.x, n.y, 0.0f} * (1.0f / std::sqrt(ls)) : v3{1.0f, 0.0f, 0.0f};
    v3 b = v3{-t.y, t.x, 0.0f};
    return Mat3{t, b, v3{0.0f, 0.0f, 1.0f}};
}
inline v3 fuzz_density_and_brdf(const MaterialConstants& m, v3 dir, v3 wi, float a_inv,
                                float roughness, float& density) {
    float jac = pow2(a_inv / length_squared(dir));
    density = fmx(cos_theta(dir), 0.0f) * INVERSE_PI * jac;
    float alb = fuzz_albedo(cos_theta(wi), roughness);
    return xyz(m.fuzz_color) * alb * INVERSE_PI * jac;
}
inline v3 fuzz_brdf_evaluate(const MaterialConstants& m, v3 wi, v3 wo, float& density) {
    if (cos_theta(wi) < DENOM_TOLERANCE || cos_theta(wo) < DENOM_TOLERANCE) return splat3(0.0f);
    float roughness = clampf(m.fuzz_roughness, 0.01f, 1.0f);
    Mat3 b = orthonormal_basis_ltc(wi);
    v3 w = v3{dot(b.c0, wo), dot(b.c1, wo), dot(b.c2, wo)};  // transpose(B) * wo
    v2 ic = ltc_inverse_coeffs(cos_theta(wi), roughness);
    v3 dir = v3{ic.x * w.x + ic.y * w.z, ic.x * w.y, w.z};
    return fuzz_density_and_brdf(m, dir, wi, ic.x, roughness, density);
}
inline v3 fuzz_brdf_sample(const MaterialConstants& m, v3 wi, Generator& g, v3& wo,
                           float& density) {
    if (cos_theta(wi) < DENOM_TOLERANCE) return splat3(0.0f);
    float roughness = clampf(m.fuzz_roughness, 0.01f, 1.0f);
    v3 dir = cosine_hemisphere_sample(random_vec2(g));
    v2 ic = ltc_inverse_coeffs(cos_theta(wi), roughness);
    v3 w = v3{dir.x / ic.x - dir.z * ic.y / ic.x, dir.y / ic.x, dir.z};
    Mat3 b = orthonormal_basis_ltc(wi);
    v3 nw = normalize(w);
    wo = b.c0 * nw.x + b.c1 * nw.y + b.c2 * nw.z;  // B * normalize(w)
    return fuzz_density_and_brdf(m, dir, wi, ic.x, roughness, density);
}
inline v3 fuzz_brdf_albedo(const MaterialConstants& m, v3 wi) {
    return splat3(fuzz_albedo(cos_theta(wi), m.fuzz_roughness));
}

// ---------------------------------------------------------------- specular_brdf.glsl
inline float specular_ior(const MaterialConstants& m) {
    return m.specular_ior / mixf(1.0f, m.coat_ior, m.coat_weight);
}
inline float specular_ior_ratio(const MaterialConstants& m) {
    float ior = specular_ior(m);
    float f0 = fresnel_at_normal_incident(ior);
    float csw = clampf(m.specular_weight, 0.0f, 1.0f / fmx(f0, DENOM_TOLERANCE));
    float eps = signf(ior - 1.0f) * std::sqrt(csw * f0);
    return (1.0f + eps) / fmx(1.0f - eps, DENOM_TOLERANCE);
}
inline v3 specular_fresnel_with_coat(const MaterialConstants& m, float ct, float ior) {
    float cra = std::sqrt(1.0f - (1.0f - pow2(ct)) / pow2(m.coat_ior));
    float ior_mix = mixf(m.specular_ior, ior, m.coat_weight);
    return splat3(fresnel_dielectric(cra, ior_mix));
}
inline v3 specular_brdf(const MaterialConstants& m, v3 wi, v3 wo, v3 wir, v3 wor, v3 mn,
                        v2 alpha, float ior, float& density) {
    float dist = microfacet_distribution(alpha, mn);
    float vis_normals = dist * microfacet_masking(alpha, wir) * fmx(0.0f, dot(wir, mn)) /
                        fmx(DENOM_TOLERANCE, cos_theta(wir));
    float jac = 1.0f / fmx(std::fabs(4.0f * dot(wir, mn)), DENOM_TOLERANCE);
    density = vis_normals * jac;
    v3 fres;
    if (cos_theta(wir) > 0.0f) fres = specular_fresnel_with_coat(m, std::fabs(dot(wir, mn)), ior);
    else fres = splat3(fresnel_dielectric(std::fabs(dot(wir, mn)), ior));
    v3 brdf = fres * dist * microfacet_visibility(alpha, wir, wor) /
              fmx(4.0f * std::fabs(cos_theta(wo)) * std::fabs(cos_theta(wi)), DENOM_TOLERANCE);
    return brdf * xyz(m.specular_color);
}
inline v3 specular_brdf_evaluate(const MaterialConstants& m, v3 wi, v3 wo, float& density) {
    if (!is_same_hemisphere(wo, wi)) return splat3(0.0f);
    float ratio = specular_ior_ratio(m);
    float ior = cos_theta(wi) > 0.0f ? ratio : 1.0f / ratio;
    if (std::fabs(ior - 1.0f) < IOR_EPSILON) return splat3(0.0f);
    v2 alpha = microfacet_roughness_to_alpha(m.specular_roughness, m.specular_roughness_anisotropy);
    LocalRotation rot = local_frame_rotation(2.0f * PI * m.specular_rotation);
    v3 wir = rotate_local(wi, rot), wor = rotate_local(wo, rot);
    v3 mn = normalize(wor + wir);
    if (dot(mn, wir) * cos_theta(wir) < 0.0f || dot(mn, wor) * cos_theta(wor) < 0.0f)
        return splat3(0.0f);
    return specular_brdf(m, wi, wo, wir, wor, mn, alpha, ior, density);
}
inline v3 specular_brdf_sample(const MaterialConstants& m, v3 wi, Generator& g, v3& wo,
                               float& density) {
    float ratio = specular_ior_ratio(m);
    float ior = cos_theta(wi) > 0.0f ? ratio : 1.0f / ratio;
    if (std::fabs(ior - 1.0f) < IOR_EPSILON) return splat3(0.0f);
    v2 alpha = microfacet_roughness_to_alpha(m.specular_roughness, m.specular_roughness_anisotropy);
    LocalRotation rot = local_frame_rotation(2.0f * PI * m.specular_rotation);
    v3 wir = rotate_local(wi, rot);
    v3 mn;
    if (cos_theta(wir) > 0.0f) {
        mn = microfacet_sample(alpha, wir, random_vec2(g));
    } else {
        mn = microfacet_sample(alpha, v3{wir.x, wir.y, -wir.z}, random_vec2(g));
        mn.z *= -1.0f;
    }
    v3 wor = -reflect(wir, mn);
    if (!is_same_hemisphere(wir, wor)) {
        density = 1.0f;
        return splat3(0.0f);
    }
    wo = inverse_rotate_local(wor, rot);
    return specular_brdf(m, wi, wo, wir, wor, mn, alpha, ior, density);
}
inline v3 specular_brdf_albedo(const MaterialConstants& m, v3 wi, Generator& g) {
    if (std::fabs(specular_ior_ratio(m) - 1.0f) < IOR_EPSILON) return splat3(0.0f);
    v3 albedo = splat3(0.0f);
    v3 wo = splat3(0.0f);
    float density = 0.0f;
    v3 brdf = specular_brdf_sample(m, wi, g, wo, density);
    if (length(brdf) > RADIANCE_EPSILON)
        albedo += brdf * std::fabs(cos_theta(wo)) / fmx(DENOM_TOLERANCE, density);
    return albedo / 1.0f;
}

// ---------------------------------------------------------------- metal_brdf.glsl
inline v3 fresnel_metal(float ct, v3 f0, v3 tint) {
    const float mu_bar = 1.0f / 7.0f;
    const float denom = mu_bar * pow6(1.0f - mu_bar);
    return fresnel_schlick(f0, ct) -
           ct * pow6(1.0f - ct) * (1.0f - tint) * fresnel_schlick(f0, mu_bar) / denom;
}
inline v3 metal_brdf(const MaterialConstants& m, v2 alpha, v3 mn, v3 wi, v3 wo, v3 wir, v3 wor,
                     float& density) {
    float dist = microfacet_distribution(alpha, mn);
    float vis_normals = dist * microfacet_masking(alpha, wir) * fmx(0.0f, dot(wir, mn)) /
                        fmx(DENOM_TOLERANCE, cos_theta(wir));
    float jac = 1.0f / fmx(std::fabs(4.0f * dot(wir, mn)), DENOM_TOLERANCE);
    density = fmx(PDF_EPSILON, vis_normals * jac);
    v3 fres = fresnel_metal(std::fabs(dot(wir, mn)), m.base_weight * xyz(m.base_color),
                            m.specular_weight * xyz(m.specular_color));
    float vis = microfacet_visibility(alpha, wir, wor);
    return fres * dist * vis /
           fmx(4.0f * std::fabs(cos_theta(wo)) * std::fabs(cos_theta(wi)), DENOM_TOLERANCE);
}
inline v3 metal_brdf_evaluate(const MaterialConstants& m, v3 wi, v3 wo, float& density) {
    if (cos_theta(wi) < DENOM_TOLERANCE || cos_theta(wo) < DENOM_TOLERANCE) {
        density = PDF_EPSILON;
        return splat3(0.0f);
    }
    LocalRotation rot = local_frame_rotation(2.0f * PI * m.specular_rotation);
    v3 wir = rotate_local(wi, rot), wor = rotate_local(wo, rot);
    v2 alpha = microfacet_roughness_to_alpha(m.specular_roughness, m.specular_roughness_anisotropy);
    v3 mn = normalize(wor + wir);
    return metal_brdf(m, alpha, mn, wi, wo, wir, wor, density);
}
inline v3 metal_brdf_sample(const MaterialConstants& m, v3 wi, Generator& g, v3& wo,
                            float& density) {
    if (cos_theta(wi) < DENOM_TOLERANCE) {
        density = PDF_EPSILON;
        return splat3(0.0f);
    }
    v2 alpha = microfacet_roughness_to_alpha(m.specular_roughness, m.specular_roughness_anisotropy);
    LocalRotation rot = local_frame_rotation(2.0f * PI * m.specular_rotation);
    v3 wir = rotate_local(wi, rot);
    v3 mn = microfacet_sample(alpha, wir, random_vec2(g));
    v3 wor = -reflect(wir, mn);
    if (!is_same_hemisphere(wir, wor)) return splat3(0.0f);
    wo = inverse_rotate_local(wor, rot);
    return metal_brdf(m, alpha, mn, wi, wo, wir, wor, density);
}
inline v3 metal_brdf_albedo(const MaterialConstants& m, v3 wi, Generator& g) {
    if (cos_theta(wi) < DENOM_TOLERANCE) return splat3(0.0f);
    v3 albedo = splat3(0.0f);
    v3 wo = splat3(0.0f);
    float density = 0.0f;
    v3 brdf = metal_brdf_sample(m, wi, g, wo, density);
    if (length(brdf) > RADIANCE_EPSILON)
        albedo += brdf * std::fabs(cos_theta(wo)) / fmx(PDF_EPSILON, density);
    return albedo / 1.0f;
}

// ---------------------------------------------------------------- specular_btdf.glsl
inline v3 btdf_tint(const MaterialConstants& m) {
    return m.transmission_depth == 0.0f ? xyz(m.transmission_color) : splat3(1.0f);
}
inline v3 specular_btdf(const MaterialConstants& m, v3 mn, v2 alpha, v3 wi, v3 wo, v3 wir, v3 wor,
                        float ior, float& density) {
    float jac = pow2(ior) * std::fabs(cos_theta(wi)) /
                fmx(pow2(cos_theta(wo) + ior * cos_theta(wi)), DENOM_TOLERANCE);
    float dist = microfacet_distribution(alpha, mn);
    float vis_normals = dist * microfacet_masking(alpha, wir) * fmx(0.0f, dot(wir, mn)) /
                        fmx(DENOM_TOLERANCE, std::fabs(cos_theta(wir)));
    density = vis_normals * jac;
    float vis = microfacet_visibility(alpha, wir, wor);
    float trans = fmx(0.0f, 1.0f - fresnel_dielectric(std::fabs(dot(wir, mn)), 1.0f / ior));
    float btdf = trans * std::fabs(dot(wir, mn)) * jac * vis * dist /
                 fmx(std::fabs(cos_theta(wo)) * std::fabs(cos_theta(wi)), DENOM_TOLERANCE);
    return btdf * btdf_tint(m);
}
inline v3 specular_btdf_evaluate(const MaterialConstants& m, v3 wi, v3 wo, float& density) {
    if (is_same_hemisphere(wo, wi)) {
        density = 1.0f;
        return splat3(0.0f);
    }
    float ior = cos_theta(wi) > 0.0f ? 1.0f / m.specular_ior : m.specular_ior;
    if (std::fabs(ior - 1.0f) < IOR_EPSILON) {
        v3 tint = btdf_tint(m);
        density = 1.0f / PDF_EPSILON;
        return tint * density / fmx(DENOM_TOLERANCE, std::fabs(cos_theta(wo)));
    }
    LocalRotation rot = local_frame_rotation(2.0f * PI * m.specular_rotation);
    v3 wir = rotate_local(wi, rot), wor = rotate_local(wo, rot);
    v3 mn = -wor - ior * wir;
    if (length_squared(mn) == 0.0f) return splat3(0.0f);
    mn = safe_normalize(mn);
    if (cos_theta(mn) <= 0.0f) mn = mn * -1.0f;
    v2 alpha = microfacet_roughness_to_alpha(m.specular_roughness, m.specular_roughness_anisotropy);
    return specular_btdf(m, mn, alpha, wi, wo, wir, wor, ior, density);
}
inline bool refraction_direction(v3 n, float ior, v3 wi, v3& dir) {
    float cti = dot(wi, n);
    float sti2 = fmx(0.0f, 1.0f - pow2(cti));
    float stt2 = pow2(ior) * sti2;
    if (stt2 >= 1.0f) return false;
    float ctt = std::sqrt(1.0f - stt2);
    dir = ior * -wi + (ior * cti - ctt) * n;
    return true;
}
inline v3 specular_btdf_sample(const MaterialConstants& m, v3 wi, Generator& g, v3& wo,
                               float& density) {
    float ior = cos_theta(wi) > 0.0f ? 1.0f / m.specular_ior : m.specular_ior;
    if (std::fabs(ior - 1.0f) < IOR_EPSILON) {
        wo = -wi;
        density = 1.0f / PDF_EPSILON;
        v3 tint = btdf_tint(m);
        return tint * density / fmx(DENOM_TOLERANCE, std::fabs(cos_theta(wo)));
    }
    LocalRotation rot = local_frame_rotation(2.0f * PI * m.specular_rotation);
    v3 wir = rotate_local(wi, rot);
    v2 alpha = microfacet_roughness_to_alpha(m.specular_roughness, m.specular_roughness_anisotropy);
    v3 mn;
    if (cos_theta(wir) > 0.0f) {
        mn = microfacet_sample(alpha, wir, random_vec2(g));
    } else {
        mn = microfacet_sample(alpha, v3{wir.x, wir.y, -cos_theta(wir)}, random_vec2(g));
        mn.z *= -1.0f;
    }
    v3 rd = splat3(0.0f);
    if (!refraction_direction(mn, ior, wir, rd)) {
        density = PDF_EPSILON;
        return splat3(0.0f);
    }
    v3 wor = -safe_normalize(rd);
    wo = inverse_rotate_local(wor, rot);
    return specular_btdf(m, mn, alpha, wi, wo, wir, wor, ior, density);
}
inline v3 specular_btdf_albedo(const MaterialConstants& m, v3 wi, Generator& g) {
    if (std::fabs(m.specular_ior - 1.0f) < IOR_EPSILON) return btdf_tint(m);
    v3 albedo = splat3(0.0f);
    v3 wo = splat3(0.0f);
    float density = 0.0f;
    v3 btdf = specular_btdf_sample(m, wi, g, wo, density);
    if (length(btdf) > RADIANCE_EPSILON)
        albedo += btdf * std::fabs(cos_theta(wo)) / fmx(DENOM_TOLERANCE, density);
    return albedo / 1.0f;
}

// ---------------------------------------------------------------- bsdf.glsl
constexpr int FUZZ = 0, COAT = 1, METAL = 2, SPEC_BRDF = 3, SPEC_BTDF = 4, DIFFUSE = 5;
constexpr int LOBE_COUNT = 6;
struct Lobes {
    v3 weights[LOBE_COUNT];
    v3 albedos[LOBE_COUNT];
    float probs[LOBE_COUNT];
};
inline void lobe_weights(const MaterialConstants& m, v3 wi, Generator& g, Lobes& l) {
    bool fully_metallic = m.base_metalness == 1.0f;
    bool fully_transmissive = m.transmission_weight == 1.0f;
    l.albedos[FUZZ] = m.fuzz_weight > 0.0f ? fuzz_brdf_albedo(m, wi) : splat3(0.0f);
    l.albedos[COAT] = m.coat_weight > 0.0f ? coat_brdf_albedo(m, wi, g) : splat3(0.0f);
    l.albedos[METAL] = m.base_metalness > 0.0f ? metal_brdf_albedo(m, wi, g) : splat3(0.0f);
    l.albedos[SPEC_BRDF] = !fully_metallic ? specular_brdf_albedo(m, wi, g) : splat3(0.0f);
    l.albedos[SPEC_BTDF] = !fully_metallic && m.transmission_weight > 0.0f
                               ? specular_btdf_albedo(m, wi, g)
                               : splat3(0.0f);
    l.albedos[DIFFUSE] =
        !fully_metallic && !fully_transmissive ? diffuse_brdf_albedo(m, wi) : splat3(0.0f);

    l.weights[FUZZ] = splat3(m.fuzz_weight);
    v3 coated_base_weight = mix3(splat3(1.0f), 1.0f - l.albedos[FUZZ], m.fuzz_weight);
    l.weights[COAT] = coated_base_weight * m.coat_weight;

    v3 base_darkening = splat3(1.0f);
    if (m.coat_weight > 0.0f && m.coat_darkening > 0.0f) {
        float fresnel_weight =
            saturate(m.specular_weight * fresnel_at_normal_incident(specular_ior(m)));
        float dielectric_roughness = mixf(1.0f, m.specular_roughness, fresnel_weight);
        float base_roughness = mixf(dielectric_roughness, m.specular_roughness, m.base_metalness);
        float average_fresnel =
            1.0f - (1.0f - average_dielectric_fresnel(m.coat_ior)) / pow2(m.coat_ior);
        float fres = fresnel_dielectric(std::fabs(cos_theta(wi)), m.coat_ior);
        float drc = mixf(fres, average_fresnel, base_roughness);
        v3 dielectric_base_albedo =
            mix3(l.albedos[DIFFUSE], l.albedos[SPEC_BTDF], m.transmission_weight);
        v3 base_albedo = mix3(dielectric_base_albedo, l.albedos[METAL], m.base_metalness);
        v3 darkening_factor = (1.0f - drc) / (1.0f - base_albedo * drc);
        base_darkening = mix3(splat3(1.0f), darkening_factor, m.coat_weight * m.coat_darkening);
    }
    v3 base_weight = coated_base_weight *
                     mix3(splat3(1.0f),
                          base_darkening * xyz(m.coat_color) * (1.0f - l.albedos[COAT]),
                          m.coat_weight);
    l.weights[METAL] = base_weight * m.base_metalness;
    v3 dielectric_base_weight = base_weight * splat3(1.0f - m.base_metalness);
    l.weights[SPEC_BRDF] = dielectric_base_weight;
    l.weights[SPEC_BTDF] = dielectric_base_weight * m.transmission_weight;
    v3 opaque = dielectric_base_weight * (1.0f - m.transmission_weight);
    l.weights[DIFFUSE] = opaque * (1.0f - l.albedos[SPEC_BRDF]);
}
inline void lobe_probabilities(Lobes& l) {
    float total = 0.0f;
    for (int i = 0; i < LOBE_COUNT; ++i) {
        l.probs[i] = length(l.weights[i] * l.albedos[i]);
        total += l.probs[i];
    }
    total = fmx(DENOM_TOLERANCE, total);
    for (int i = 0; i < LOBE_COUNT; ++i) l.probs[i] /= total;
}
inline Lobes bsdf_prepare(const MaterialConstants& m, v3 wi, Generator& g) {
    Lobes l;
    lobe_weights(m, wi, g, l);
    lobe_probabilities(l);
    return l;
}
inline v3 bsdf_evaluate_lobes(const MaterialConstants& m, const Lobes& l, v3 wi, v3 wo, int skip,
                              float* dens) {
    v3 b = splat3(0.0f);
    if (skip != FUZZ && l.probs[FUZZ] > 0.0f)
        b += l.weights[FUZZ] * fuzz_brdf_evaluate(m, wi, wo, dens[FUZZ]);
    if (skip != COAT && l.probs[COAT] > 0.0f)
        b += l.weights[COAT] * coat_brdf_evaluate(m, wi, wo, dens[COAT]);
    if (skip != METAL && l.probs[METAL] > 0.0f)
        b += l.weights[METAL] * metal_brdf_evaluate(m, wi, wo, dens[METAL]);
    if (skip != SPEC_BRDF && l.probs[SPEC_BRDF] > 0.0f)
        b += l.weights[SPEC_BRDF] * specular_brdf_evaluate(m, wi, wo, dens[SPEC_BRDF]);
    if (skip != DIFFUSE && l.probs[DIFFUSE] > 0.0f)
        b += l.weights[DIFFUSE] * diffuse_brdf_evaluate(m, wi, wo, dens[DIFFUSE]);
    if (skip != SPEC_BTDF && l.probs[SPEC_BTDF] > 0.0f)
        b += l.weights[SPEC_BTDF] * specular_btdf_evaluate(m, wi, wo, dens[SPEC_BTDF]);
    return b;
}
inline float bsdf_total_pdf(const Lobes& l, const float* dens) {
    float d = 0.0f;
    for (int i = 0; i < LOBE_COUNT; ++i) d += l.probs[i] * dens[i];
    return d;
}
inline v3 bsdf_evaluate(const MaterialConstants& m, const Lobes& l, v3 wi, v3 wo, float& density) {
    float dens[7] = {0, 0, 0, 0, 0, 0, 0};
    v3 b = bsdf_evaluate_lobes(m, l, wi, wo, -1, dens);
    density = bsdf_total_pdf(l, dens);
    return b;
}
inline v3 bsdf_sample(const MaterialConstants& m, const Lobes& l, v3 wi, Generator& g, v3& wo,
                      float& density, int& sampled) {
    float rnd = random_float(g);
    float acc = 0.0f;
    for (int i = 0; i < LOBE_COUNT; ++i) {
        acc += l.probs[i];
        if (rnd < acc) {
            float lobe_density = 0.0f;
            v3 lobe_bsdf = splat3(0.0f);
            if (i == FUZZ) lobe_bsdf = fuzz_brdf_sample(m, wi, g, wo, lobe_density);
            else if (i == COAT) lobe_bsdf = coat_brdf_sample(m, wi, g, wo, lobe_density);
            else if (i == METAL) lobe_bsdf = metal_brdf_sample(m, wi, g, wo, lobe_density);
            else if (i == SPEC_BRDF) lobe_bsdf = specular_brdf_sample(m, wi, g, wo, lobe_density);
            else if (i == SPEC_BTDF) lobe_bsdf = specular_btdf_sample(m, wi, g, wo, lobe_density);
            else lobe_bsdf = diffuse_brdf_sample(m, wi, g, wo, lobe_density);
            float dens[7] = {0, 0, 0, 0, 0, 0, 0};
            v3 b = bsdf_evaluate_lobes(m, l, wi, wo, i, dens);
            dens[i] = lobe_density;
            density = bsdf_total_pdf(l, dens);
            sampled = i;
            return b + l.weights[i] * lobe_bsdf;
        }
    }
    sampled = -1;
    density = 1.0f;
    return splat3(0.0f);
}

}  // namespace ref
