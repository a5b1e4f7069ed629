// TEST INFRASTRUCTURE — the CPU oracle for the tinytrace rendering hot path.
// Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg may load this
// library; it is the checker, never the thing measured as the product or shipped.
//
// A CPU restatement of the reference path tracer (src/integrate/integrate.glsl), its
// OpenPBR BSDF (src/material/*.glsl), emissive-triangle light sampling
// (src/includes/scene.glsl:114-136) and the neutral tonemap
// (src/post_process/tonemap.glsl:17-26, display.glsl:6-12), plus the project's LBVH.
// Parity status: the reference's own tests hold no golden vectors for any of this
// (src/material/test.rs asserts nothing), and the reference cannot run here (no Rust
// toolchain, no Vulkan), so this oracle is "parity unpinned" against the reference; it is
// pinned by analytic checks in tests/ (reciprocity, energy, furnace, convergence).
//
// Exported with a C ABI for ctypes.
#include <cstdio>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "ref_bsdf.h"
#include "ref_bvh.h"
#include "ref_ingest.h"
#include "ref_texture.h"

using namespace ref;

namespace {

constexpr float EXTENSION_TMIN = 1.0e-3f, EXTENSION_TMAX = 1000.0f;  // integrate.glsl:116-117
constexpr float SHADOW_TMIN = 1.0e-3f, SHADOW_TMAX = 10000.0f;       // integrate.glsl:170-171

struct OracleScene {
    std::vector<int16_t> positions;
    std::vector<uint32_t> indices;
    std::vector<Vertex> vertices;
    std::vector<Material> materials;
    std::vector<Mesh> meshes;
    std::vector<Instance> instances;
    std::vector<EmissiveTriangle> emissive;
    std::vector<Texture> textures;
    SceneBvh bvh;
    std::vector<uint32_t> light_prim;  // primitive of each emissive triangle in its instance's mesh
    std::vector<LightAlias> light_alias;  // power-proportional selection (built for every scene)
    bool light_power = false;             // next-event estimation picks lights through light_alias
    bool light_exact = false;          // visibility tests the sampled triangle itself (full id)
    bool use_bvh = true;
    bool flat = false;  // the integrator traces through the flat BVH instead of the two-level one
    Geometry geom() const {
        return Geometry{positions.data(), indices.data(), instances.data(),
                        (uint32_t)instances.size(), meshes.data(), (uint32_t)meshes.size()};
    }
    SceneView view() const {
        return SceneView{positions.data(), indices.data(), vertices.data(), materials.data(),
                         instances.data(), emissive.data(), (uint32_t)emissive.size(),
                         light_power && !light_alias.empty() ? light_alias.data() : nullptr};
    }
};

Hit trace(const OracleScene& s, v3 o, v3 d, float tmin, float tmax, bool cull) {
    Geometry g = s.geom();
    if (!s.use_bvh) return trace_brute(g, o, d, tmin, tmax, cull);
    return s.flat ? trace_flat(g, s.bvh, o, d, tmin, tmax, cull) : trace_bvh(g, s.bvh, o, d, tmin, tmax, cull);
}

struct Ray {
    v3 direction, origin;
};

// integrate.glsl:17-20
v3 camera_ray_direction(const Constants& c, v2 ndc) {
    v4 vsp = mat4_mul(c.inverse_proj, v4{-ndc.x, -ndc.y, 1.0f, 1.0f});
    v4 w = mat4_mul(c.inverse_view, v4{vsp.x, vsp.y, vsp.z, 0.0f});
    return normalize(v3{w.x, w.y, w.z});
}

struct RayHit {
    v3 world_position;
    Basis tangent_space;
    v2 uv, uv_ddx, uv_ddy;
    uint32_t instance_index, material_index;
};

// integrate.glsl:22-110; `bounce`, `ndc` and `origin` feed the ray differentials of the
// primary hit (integrate.glsl:89-106).
RayHit get_ray_hit(const OracleScene& s, const Constants& c, const Hit& h, uint32_t bounce, v2 ndc, v3 origin) {
    RayHit hit;
    const Instance& in = s.instances[h.instance];
    hit.instance_index = h.instance;
    hit.material_index = in.material_index;
    uint32_t base = 3u * h.prim + in.index_offset;
    uint32_t ti[3];
    v3 pos[3];
    for (int k = 0; k < 3; ++k) {
        ti[k] = s.indices[base + k] + in.vertex_offset;
        pos[k] = mat43_point(in.transform, dequantize_snorm3(&s.positions[3u * ti[k]]));
    }
    const Vertex* tv[3] = {&s.vertices[ti[0]], &s.vertices[ti[1]], &s.vertices[ti[2]]};
    v3 bary = v3{0.0f, h.u, h.v};
    bary.x = 1.0f - bary.y - bary.z;
    TangentFrame tf[3];
    for (int k = 0; k < 3; ++k) tf[k] = decode_tangent_frame(tv[k]->tangent_frame);
    hit.tangent_space.normal =
        normalize(mat3_vec(in.normal_transform, interp3(bary, tf[0].normal, tf[1].normal, tf[2].normal)));
    hit.tangent_space.tangent = normalize(
        mat3_vec(in.normal_transform, interp3(bary, tf[0].tangent, tf[1].tangent, tf[2].tangent)));
    float bs = signf(tf[0].bitangent_sign * bary.x + tf[1].bitangent_sign * bary.y +
                     tf[2].bitangent_sign * bary.z);
    hit.tangent_space.bitangent =
        normalize(bs * cross(hit.tangent_space.normal, hit.tangent_space.tangent));
    hit.uv = interp2(bary, uv_of(tv[0]->uv), uv_of(tv[1]->uv), uv_of(tv[2]->uv));
    hit.world_position = bary.x * pos[0] + bary.y * pos[1] + bary.z * pos[2];
    hit.uv_ddx = hit.uv_ddy = v2{0.0f, 0.0f};
    if (bounce == 0) {
        v2 texel = v2{2.0f / (float)c.screen_size[0], 2.0f / (float)c.screen_size[1]};
        v3 hx = triangle_intersection(pos, origin, camera_ray_direction(c, v2{ndc.x + texel.x, ndc.y}));
        v3 hy = triangle_intersection(pos, origin, camera_ray_direction(c, v2{ndc.x, ndc.y + texel.y}));
        hit.uv_ddx = interp2(bary - hx, uv_of(tv[0]->uv), uv_of(tv[1]->uv), uv_of(tv[2]->uv));
        hit.uv_ddy = interp2(bary - hy, uv_of(tv[0]->uv), uv_of(tv[1]->uv), uv_of(tv[2]->uv));
    }
    return hit;
}

// integrate.glsl:148-154 for a material without emission textures
v3 material_emissive(const Material& m) {
    return xyz(m.constants.emission_color) * m.constants.emission_luminance;
}

// integrate.glsl:156-193
v3 direct_light_contribution(const OracleScene& s, v3 position, v3 wi, const Basis& basis,
                             const MaterialConstants& mat, const Lobes& lobes, Generator& g) {
    SceneView sv = s.view();
    DirectLightSample ls = sample_random_light(sv, g);
    v3 to_light = ls.position - position;
    v3 wo = transform_from_basis(basis, to_light);
    float d2 = length_squared(to_light);
    Ray ray{to_light / std::sqrt(d2), position};
    float density = (1.0f / ls.area) * d2 / saturate(dot(-ray.direction, ls.normal)) *
                    ls.light_probability;
    Hit h = trace(s, ray.origin, ray.direction, SHADOW_TMIN, SHADOW_TMAX, false);
    if (!h.hit) return splat3(0.0f);
    if (h.instance != ls.instance) return splat3(0.0f);
    if (s.light_exact) {
        if (h.prim != s.light_prim[ls.index]) return splat3(0.0f);
    } else {
        uint32_t tri = h.prim + s.instances[h.instance].index_offset / 3u;
        if (tri % 0xffffu != ls.hash) return splat3(0.0f);
    }
    const Material& lm = s.materials[s.instances[ls.instance].material_index];
    v3 emissive = material_emissive(lm, s.textures, ls.uv, 4.0f);  // integrate.glsl:188-189
    float bd = 0.0f;
    v3 bsdf = bsdf_evaluate(mat, lobes, wi, wo, bd);
    return bsdf * emissive * std::fabs(cos_theta(wo)) / fmx(density, PDF_EPSILON);
}

// integrate.glsl:195-201
Basis create_surface_basis(const Basis& ts, v3 n) {
    Basis b;
    b.normal = transform_to_basis(ts, n);
    b.tangent = gram_schmidt(b.normal, ts.tangent);
    b.bitangent = normalize(cross(b.normal, b.tangent));
    return b;
}

struct PathState {
    v3 accumulated, throughput;
    Generator generator;
    v2 ndc;
    float mip_level;
    Ray ray;
};

// integrate.glsl:270-321
bool next_path_segment(const OracleScene& s, const Constants& c, PathState& ps, uint32_t bounce) {
    Hit h = trace(s, ps.ray.origin, ps.ray.direction, EXTENSION_TMIN, EXTENSION_TMAX, true);
    if (!h.hit) {
        ps.accumulated += splat3(1.0f) * ps.throughput;
        return false;
    }
    RayHit hit = get_ray_hit(s, c, h, bounce, ps.ndc, ps.ray.origin);
    if (bounce == 0) ps.mip_level = calculate_mip_level(hit.uv_ddx, hit.uv_ddy, c.screen_size);
    const Material& material = s.materials[hit.material_index];
    const MaterialConstants mc = load_textures(material, s.textures, hit.uv, ps.mip_level);
    Basis basis = create_surface_basis(hit.tangent_space, xyz(mc.geometry_normal));
    v3 wi = transform_from_basis(basis, -ps.ray.direction);
    Lobes lobes = bsdf_prepare(mc, wi, ps.generator);
    bool nee = c.light_sampling == LIGHT_SAMPLING_NEXT_EVENT_ESTIMATION && !s.emissive.empty() &&
               mc.specular_roughness > 0.15f;
    if (nee) {
        v3 direct = direct_light_contribution(s, hit.world_position, wi, basis, mc, lobes,
                                              ps.generator);
        ps.accumulated += ps.throughput * direct;
    }
    if (bounce == 0 || !nee) {
        v3 emissive = material_emissive(material, s.textures, hit.uv, ps.mip_level);
        ps.accumulated += emissive * ps.throughput;
    }
    float density = 1.0f;
    v3 wo = splat3(0.0f);
    int lobe = 0;
    v3 bsdf = bsdf_sample(mc, lobes, wi, ps.generator, wo, density, lobe);
    ps.ray.direction = transform_to_basis(basis, wo);
    ps.ray.origin = hit.world_position;
    ps.throughput *= bsdf / fmx(density, PDF_EPSILON) * std::fabs(cos_theta(wo));
    return true;
}

// integrate.glsl:323-347 for one pixel.
v3 render_pixel(const OracleScene& s, const Constants& c, uint32_t px, uint32_t py) {
    uint32_t W = c.screen_size[0], H = c.screen_size[1];
    Generator g = init_generator_from_pixel(px, py, W, c.frame_index);
    v3 acc = splat3(0.0f);
    for (uint32_t si = 0; si < c.sample_count; ++si) {
        float ox = random_float(g);
        float oy = random_float(g);
        v2 off = v2{ox - 0.5f, oy - 0.5f};
        v2 ndc = v2{(((float)px + off.x) / (float)W) * 2.0f - 1.0f,
                    (((float)py + off.y) / (float)H) * 2.0f - 1.0f};
        Ray ray{camera_ray_direction(c, ndc), xyz(c.camera_position)};
        PathState ps{splat3(0.0f), splat3(1.0f), g, ndc, 1.0f, ray};
        for (uint32_t b = 0; b < c.bounce_count; ++b)
            if (!next_path_segment(s, c, ps, b)) break;
        acc += ps.accumulated;
    }
    return acc / (float)c.sample_count;
}

// ---------------------------------------------------------------- ReSTIR DI
// The project's spatiotemporal reservoir resampling for direct light (Bitterli et al. 2020),
// restated pass by pass on the CPU as the checker of tinytrace_gb300/csrc/restir.cu; the
// reference has no such pass.  Same operations and random-number order as the device code.
struct RSurface {
    bool hit = false;
    v3 pos{}, normal{}, tangent{}, wi{};
    float dist = 0.0f;
    uint32_t material = 0, instance = 0, seed = 0;
    v2 uv{};          // texture coordinates of the hit
    float mip = 0.0f; // mip level of the primary hit (integrate.glsl:134-139)
};
struct RRes {
    uint32_t light;
    float r1, r2, w_sum, M, W, pad0, pad1;
};
static_assert(sizeof(RRes) == 32, "reservoir record");
constexpr uint32_t R_NO_LIGHT = 0xffffffffu;

RRes r_empty() { return RRes{R_NO_LIGHT, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f}; }

struct RState {  // shading state rebuilt from a G-buffer record
    v3 pos, wi;
    Basis basis;
    MaterialConstants mat;  // the material with its textures sampled at the hit
    const MaterialConstants* mc;
    Lobes lobes;
    uint32_t seed;
    float dist;
    v2 uv;
    float mip;
};
bool r_load(const OracleScene& s, const RSurface& q, RState& st) {
    if (!q.hit) return false;
    st.pos = q.pos;
    st.dist = q.dist;
    st.basis.normal = q.normal;
    st.basis.tangent = q.tangent;
    st.basis.bitangent = normalize(cross(q.normal, q.tangent));
    st.wi = q.wi;
    st.seed = q.seed;
    st.uv = q.uv;
    st.mip = q.mip;
    st.mat = load_textures(s.materials[q.material], s.textures, q.uv, q.mip);
    st.mc = &st.mat;
    Generator g{q.seed};
    st.lobes = bsdf_prepare(*st.mc, st.wi, g);
    return true;
}

struct RLight {
    v3 pos, normal, emission;
    float area;
    uint32_t instance;
};
RLight r_light(const OracleScene& s, uint32_t light, float r1, float r2) {
    const EmissiveTriangle& t = s.emissive[light];
    const Instance& in = s.instances[t.instance_index];
    v3 p[3];
    for (int k = 0; k < 3; ++k) p[k] = mat43_point(in.transform, dequantize_snorm3(t.positions[k]));
    v3 e = cross(p[1] - p[0], p[2] - p[0]);
    RLight L;
    L.area = fmx(0.00001f, 0.5f * length(e));
    L.normal = normalize(e);
    v3 bary = sample_triangle(v2{r1, r2});
    L.pos = interp3(bary, p[0], p[1], p[2]);
    v2 uv = interp2(bary, uv_of(t.uv[0]), uv_of(t.uv[1]), uv_of(t.uv[2]));
    L.emission = material_emissive(s.materials[in.material_index], s.textures, uv, 4.0f);
    L.instance = t.instance_index;
    return L;
}

float r_luminance(v3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }

// f * Le * |cos| * cosL / d^2 (unshadowed, area measure)
v3 r_contribution(const RState& st, const RLight& L) {
    v3 d = L.pos - st.pos;
    float d2 = dot(d, d);
    v3 dir = d / std::sqrt(d2);
    float cos_light = dot(-dir, L.normal);
    if (!(cos_light > 0.0f) || !(d2 > 0.0f)) return splat3(0.0f);
    v3 wo = transform_from_basis(st.basis, d);
    float density = 0.0f;
    v3 f = bsdf_evaluate(*st.mc, st.lobes, st.wi, wo, density);
    return f * L.emission * (std::fabs(cos_theta(wo)) * cos_light / d2);
}

bool r_update(RRes& r, uint32_t light, float r1, float r2, float w, float m, Generator& g) {
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

struct RestirOracle {
    const OracleScene* s = nullptr;
    uint32_t W = 0, H = 0, cur = 0;
    std::vector<RSurface> gb[2];
    std::vector<RRes> fin[2], init, temp;
    std::vector<uint32_t> light_prim;
    bool hist_valid = false;
    float hist_cam[3] = {0, 0, 0}, hist_view[16] = {}, hist_ip[16] = {};
    uint32_t candidates = 32, neighbours = 5;
    float m_cap_factor = 20.0f, radius = 30.0f;
};

bool r_visible(const RestirOracle& R, v3 pos, const RLight& L, uint32_t light) {
    v3 d = L.pos - pos;
    v3 dir = d / std::sqrt(dot(d, d));
    Hit h = trace(*R.s, pos, dir, SHADOW_TMIN, SHADOW_TMAX, false);
    return h.hit && h.instance == L.instance && h.prim == R.light_prim[light];
}

// The emissive triangle's primitive in its instance's mesh: the triangle with the same snorm16
// positions, the running index first.
std::vector<uint32_t> r_light_prims(const OracleScene& s) {
    std::vector<uint32_t> out(s.emissive.size(), 0xffffffffu);
    std::vector<uint32_t> next(s.instances.size(), 0);
    for (size_t e = 0; e < s.emissive.size(); ++e) {
        const EmissiveTriangle& t = s.emissive[e];
        const Instance& in = s.instances[t.instance_index];
        const Mesh& me = s.meshes[in.mesh_index];
        uint32_t tris = me.index_count / 3u;
        auto same = [&](uint32_t p) {
            for (int k = 0; k < 3; ++k) {
                const int16_t* v = &s.positions[3u * (me.vertex_offset + s.indices[me.index_offset + 3u * p + k])];
                for (int a = 0; a < 3; ++a)
                    if (v[a] != t.positions[k][a]) return false;
            }
            return true;
        };
        uint32_t guess = next[t.instance_index];
        if (guess < tris && same(guess)) out[e] = guess;
        else
            for (uint32_t p = 0; p < tris; ++p)
                if (same(p)) {
                    out[e] = p;
                    break;
                }
        if (out[e] != 0xffffffffu) next[t.instance_index] = out[e] + 1u;
    }
    return out;
}

RSurface r_gbuffer(const RestirOracle& R, const Constants& c, uint32_t x, uint32_t y) {
    const OracleScene& s = *R.s;
    uint32_t W = c.screen_size[0], H = c.screen_size[1];
    Generator g = init_generator_from_pixel(x, y, W, c.frame_index);
    float ox = random_float(g);
    float oy = random_float(g);
    v2 ndc = v2{(((float)x + (ox - 0.5f)) / (float)W) * 2.0f - 1.0f, (((float)y + (oy - 0.5f)) / (float)H) * 2.0f - 1.0f};
    v3 dir = camera_ray_direction(c, ndc);
    v3 org = xyz(c.camera_position);
    Hit h = trace(s, org, dir, EXTENSION_TMIN, EXTENSION_TMAX, true);
    RSurface q;
    q.seed = g.state;
    if (!h.hit) return q;
    RayHit hit = get_ray_hit(s, c, h, 0u, ndc, org);
    q.mip = calculate_mip_level(hit.uv_ddx, hit.uv_ddy, c.screen_size);
    q.uv = hit.uv;
    const MaterialConstants mc = load_textures(s.materials[hit.material_index], s.textures, q.uv, q.mip);
    Basis basis = create_surface_basis(hit.tangent_space, xyz(mc.geometry_normal));
    q.hit = true;
    q.pos = hit.world_position;
    q.dist = length(hit.world_position - org);
    q.normal = basis.normal;
    q.tangent = basis.tangent;
    q.wi = transform_from_basis(basis, -dir);
    q.material = hit.material_index;
    q.instance = h.instance;
    return q;
}

RRes r_initial(const RestirOracle& R, const RSurface& q) {
    const OracleScene& s = *R.s;
    RState st;
    RRes r = r_empty();
    if (!r_load(s, q, st) || s.emissive.empty()) return r;
    Generator g{jenkins_hash(st.seed + 1u)};
    float lights = (float)s.emissive.size();
    float chosen = 0.0f;
    for (uint32_t k = 0; k < R.candidates; ++k) {
        uint32_t light = random_uint(g, (uint32_t)s.emissive.size());
        float inv_p = lights;
        if (s.light_power) {  // candidates by emitted power
            float coin = random_float(g);
            if (!(coin < s.light_alias[light].keep)) light = s.light_alias[light].alias;
            inv_p = 1.0f / s.light_alias[light].pdf;
        }
        float r1 = random_float(g);
        float r2 = random_float(g);
        RLight L = r_light(s, light, r1, r2);
        float ph = r_luminance(r_contribution(st, L));
        float w = ph * (inv_p * L.area);
        if (r_update(r, light, r1, r2, w, 1.0f, g)) chosen = ph;
    }
    r.W = chosen > 0.0f ? r.w_sum / (r.M * chosen) : 0.0f;
    if (r.W > 0.0f && !r_visible(R, st.pos, r_light(s, r.light, r.r1, r.r2), r.light)) r.W = 0.0f;
    return r;
}

float r_target(const RestirOracle& R, const RState& st, uint32_t light, float r1, float r2) {
    if (light == R_NO_LIGHT) return 0.0f;
    return r_luminance(r_contribution(st, r_light(*R.s, light, r1, r2)));
}

void r_merge(const RestirOracle& R, const RState& st, RRes& r, const RRes& q, float cap, float& chosen, Generator& g) {
    float m = fmn(q.M, cap);
    float ph = r_target(R, st, q.light, q.r1, q.r2);
    float w = ph * q.W * m;
    if (r_update(r, q.light, q.r1, q.r2, w, m, g)) chosen = ph;
}

bool r_similar(const RSurface& q, v3 normal, float dist) {
    if (!q.hit) return false;
    return dot(q.normal, normal) > 0.90630779f && std::fabs(q.dist - dist) <= 0.1f * dist;
}

bool r_reproject(const RestirOracle& R, v3 pos, uint32_t& px, uint32_t& py) {
    v3 d = pos - v3{R.hist_cam[0], R.hist_cam[1], R.hist_cam[2]};
    const float* v = R.hist_view;
    v3 u = v3{v[0] * d.x + v[4] * d.y + v[8] * d.z, v[1] * d.x + v[5] * d.y + v[9] * d.z,
              v[2] * d.x + v[6] * d.y + v[10] * d.z};
    const float* ip = R.hist_ip;
    v3 a = v3{ip[0], ip[1], ip[2]}, b = v3{ip[4], ip[5], ip[6]};
    v3 cc = v3{ip[8] + ip[12], ip[9] + ip[13], ip[10] + ip[14]};
    v3 c0 = -a, c1 = -b, c2 = -u, rhs = -cc;
    float det = dot(c0, cross(c1, c2));
    if (!(std::fabs(det) > 0.0f)) return false;
    float nx = dot(rhs, cross(c1, c2)) / det;
    float ny = dot(c0, cross(rhs, c2)) / det;
    float sc = dot(c0, cross(c1, rhs)) / det;
    if (!(sc > 0.0f)) return false;
    float fx = (nx + 1.0f) * 0.5f * (float)R.W, fy = (ny + 1.0f) * 0.5f * (float)R.H;
    if (!(fx >= 0.0f && fx < (float)R.W && fy >= 0.0f && fy < (float)R.H)) return false;
    px = (uint32_t)fx;
    py = (uint32_t)fy;
    return true;
}

// One ReSTIR frame into `target` (W*H RGBA32F, read for accumulation).
void restir_frame(RestirOracle& R, const Constants& c, float* target) {
    const OracleScene& s = *R.s;
    uint32_t W = R.W, H = R.H;
    uint64_t n = (uint64_t)W * H;
    std::vector<RSurface>& gb = R.gb[R.cur];
    const std::vector<RSurface>& pgb = R.gb[R.cur ^ 1u];
    std::vector<RRes>& out = R.fin[R.cur];
    const std::vector<RRes>& prev = R.fin[R.cur ^ 1u];
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < (int64_t)n; ++i) gb[i] = r_gbuffer(R, c, (uint32_t)(i % W), (uint32_t)(i / W));
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < (int64_t)n; ++i) R.init[i] = r_initial(R, gb[i]);
    float cap = R.m_cap_factor * (float)R.candidates;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < (int64_t)n; ++i) {  // temporal
        RRes cur = R.init[i];
        RState st;
        uint32_t px, py;
        if (!R.hist_valid || !r_load(s, gb[i], st) || !r_reproject(R, st.pos, px, py)) {
            R.temp[i] = cur;
            continue;
        }
        uint64_t j = (uint64_t)py * W + px;
        v3 from_prev = st.pos - v3{R.hist_cam[0], R.hist_cam[1], R.hist_cam[2]};
        if (!r_similar(pgb[j], st.basis.normal, length(from_prev))) {
            R.temp[i] = cur;
            continue;
        }
        Generator g{jenkins_hash(st.seed + 2u)};
        RRes r = r_empty();
        float chosen = 0.0f;
        r_merge(R, st, r, cur, cur.M, chosen, g);
        r_merge(R, st, r, prev[j], cap, chosen, g);
        r.W = chosen > 0.0f ? r.w_sum / (r.M * chosen) : 0.0f;
        R.temp[i] = r;
    }
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < (int64_t)n; ++i) {  // spatial
        uint32_t x = (uint32_t)(i % W), y = (uint32_t)(i / W);
        RState st;
        RRes cur = R.temp[i];
        if (!r_load(s, gb[i], st)) {
            out[i] = cur;
            continue;
        }
        Generator g{jenkins_hash(st.seed + 3u)};
        RRes r = r_empty();
        float chosen = 0.0f;
        r_merge(R, st, r, cur, cur.M, chosen, g);
        for (uint32_t k = 0; k < R.neighbours; ++k) {
            float rr = R.radius * std::sqrt(random_float(g));
            float angle = TAU * random_float(g);
            float sn, cs;
            tsincos(angle, &sn, &cs);
            float qx = (float)x + rr * cs, qy = (float)y + rr * sn;
            if (!(qx >= 0.0f && qx < (float)W && qy >= 0.0f && qy < (float)H)) continue;
            uint64_t j = (uint64_t)(uint32_t)qy * W + (uint32_t)qx;
            if (j == (uint64_t)i || !r_similar(gb[j], st.basis.normal, st.dist)) continue;
            r_merge(R, st, r, R.temp[j], R.temp[j].M, chosen, g);
        }
        r.W = chosen > 0.0f ? r.w_sum / (r.M * chosen) : 0.0f;
        out[i] = r;
    }
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < (int64_t)n; ++i) {  // shade
        RState st;
        v3 radiance;
        if (!r_load(s, gb[i], st)) {
            radiance = splat3(1.0f);
        } else {
            radiance = material_emissive(s.materials[gb[i].material], s.textures, st.uv, st.mip);
            const RRes& r = out[i];
            if (r.light != R_NO_LIGHT && r.W > 0.0f) {
                RLight L = r_light(s, r.light, r.r1, r.r2);
                v3 contrib = r_contribution(st, L);
                if (r_visible(R, st.pos, L, r.light)) radiance += contrib * r.W;
            }
        }
        float* t = target + 4ull * i;
        if (c.accumulated_frame_count != 0) {
            v3 prevc = v3{t[0], t[1], t[2]};
            radiance = (prevc * (float)(c.accumulated_frame_count - 1u) + radiance) / (float)c.accumulated_frame_count;
        }
        t[0] = radiance.x;
        t[1] = radiance.y;
        t[2] = radiance.z;
        t[3] = 1.0f;
    }
    std::memcpy(R.hist_cam, &c.camera_position, sizeof(R.hist_cam));
    std::memcpy(R.hist_view, c.view, sizeof(R.hist_view));
    std::memcpy(R.hist_ip, c.inverse_proj, sizeof(R.hist_ip));
    R.hist_valid = true;
    R.cur ^= 1u;
}

// tonemap.glsl:1-26
v3 neutral_tonemap(v3 col) {
    v3 y = v3{0.2126f * col.x + 0.7152f * col.y + 0.0722f * col.z,
              -0.1146f * col.x + -0.3854f * col.y + 0.5f * col.z,
              0.5f * col.x + -0.4542f * col.y + -0.0458f * col.z};
    float bt = 1.0f - texp(-(std::sqrt(y.y * y.y + y.z * y.z) * 2.4f));
    float desat = fmx((bt - 0.7f) * 0.8f, 0.0f);
    desat *= desat;
    v3 desat_color = mix3(col, splat3(y.x), desat);
    float tm_lum = 1.0f - texp(-y.x);
    float lum = 0.2126f * col.x + 0.7152f * col.y + 0.0722f * col.z;
    v3 tm0 = col * fmx(0.0f, tm_lum / fmx(1e-5f, lum));
    v3 tm1 = v3{1.0f - texp(-desat_color.x), 1.0f - texp(-desat_color.y),
                1.0f - texp(-desat_color.z)};
    return mix3(tm0, tm1, bt * bt) * 0.97f;
}

template <class T>
void copy_in(std::vector<T>& dst, const void* src, uint64_t count) {
    dst.resize(count);
    if (count) std::memcpy(dst.data(), src, count * sizeof(T));
}

}  // namespace

extern "C" {

// Alias table by emitted power: emission_luminance x luminance(emission_color) x world-space
// area in double precision (area alone for textured emission), Vose's method with index-ordered
// work stacks, as the library builds it (the table is an input the CUDA path receives).
std::vector<LightAlias> build_light_alias(const OracleScene& s) {
    uint32_t n = (uint32_t)s.emissive.size();
    std::vector<LightAlias> out(n);
    if (n == 0) return out;
    std::vector<double> power(n);
    double total = 0.0;
    for (uint32_t e = 0; e < n; ++e) {
        const EmissiveTriangle& t = s.emissive[e];
        const Instance& in = s.instances[t.instance_index];
        const Material& m = s.materials[in.material_index];
        double p[3][3];
        for (int k = 0; k < 3; ++k) {
            double v[3] = {t.positions[k][0] / 32767.0, t.positions[k][1] / 32767.0, t.positions[k][2] / 32767.0};
            for (int r = 0; r < 3; ++r)
                p[k][r] = in.transform[r] * v[0] + in.transform[4 + r] * v[1] + in.transform[8 + r] * v[2] +
                          in.transform[12 + r];
        }
        double e1[3] = {p[1][0] - p[0][0], p[1][1] - p[0][1], p[1][2] - p[0][2]};
        double e2[3] = {p[2][0] - p[0][0], p[2][1] - p[0][1], p[2][2] - p[0][2]};
        double c[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        double area = 0.5 * std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        bool textured = m.textures[T_EMISSION_COLOR] != NO_TEXTURE || m.textures[T_EMISSION_LUMINANCE] != NO_TEXTURE;
        const MaterialConstants& mc = m.constants;
        double lum = 0.2126 * mc.emission_color.x + 0.7152 * mc.emission_color.y + 0.0722 * mc.emission_color.z;
        double pw = textured ? area : (double)mc.emission_luminance * lum * area;
        power[e] = std::isfinite(pw) && pw > 0.0 ? pw : 0.0;
        total += power[e];
    }
    if (!(total > 0.0)) {
        for (uint32_t e = 0; e < n; ++e) out[e] = LightAlias{1.0f, e, (float)(1.0 / n)};
        return out;
    }
    std::vector<double> scaled(n), keep(n, 1.0);
    std::vector<uint32_t> small, large, alias(n);
    for (uint32_t e = 0; e < n; ++e) {
        scaled[e] = power[e] / total * (double)n;
        (scaled[e] < 1.0 ? small : large).push_back(e);
        alias[e] = e;
    }
    while (!small.empty() && !large.empty()) {
        uint32_t sm = small.back(), lg = large.back();
        small.pop_back();
        large.pop_back();
        keep[sm] = scaled[sm];
        alias[sm] = lg;
        scaled[lg] = (scaled[lg] + scaled[sm]) - 1.0;
        (scaled[lg] < 1.0 ? small : large).push_back(lg);
    }
    for (uint32_t e = 0; e < n; ++e) out[e] = LightAlias{(float)keep[e], alias[e], (float)(power[e] / total)};
    return out;
}

// Layout of tt_scene_desc (include/tinytrace_cuda.h): pointers + counts.
struct OracleSceneDesc {
    const int16_t* positions;
    uint64_t position_count;
    const uint32_t* indices;
    uint64_t index_count;
    const Vertex* vertices;
    uint64_t vertex_count;
    const Material* materials;
    uint32_t material_count;
    uint32_t mesh_count;
    const Mesh* meshes;
    const Instance* instances;
    uint32_t instance_count;
    uint32_t emissive_count;
    const EmissiveTriangle* emissive;
    const TextureDesc* textures;
    uint32_t texture_count;
    uint32_t reserved;
};

// accel: 0 brute force, 1 two-level BVH, 2 flat BVH (the structure render() traces through;
// both BVHs are built whenever accel != 0), 3 the flat BVH plus its compressed 8-wide format
// (render() traces through the flat BVH; the wide format is for comparison with the GPU build).
void* oracle_scene_create(const OracleSceneDesc* d, int accel, int leaf_max) {
    OracleScene* s = new OracleScene();
    copy_in(s->positions, d->positions, d->position_count * 3u);
    copy_in(s->indices, d->indices, d->index_count);
    copy_in(s->vertices, d->vertices, d->vertex_count);
    copy_in(s->materials, d->materials, d->material_count);
    copy_in(s->meshes, d->meshes, d->mesh_count);
    copy_in(s->instances, d->instances, d->instance_count);
    copy_in(s->emissive, d->emissive, d->emissive_count);
    s->textures.resize(d->texture_count);
    for (uint32_t t = 0; t < d->texture_count; ++t) {
        const TextureDesc& td = d->textures[t];
        Texture& tx = s->textures[t];
        tx.format = td.format;
        tx.width = td.width;
        tx.height = td.height;
        uint64_t at = 0;
        for (uint32_t l = 0; l < td.level_count; ++l) {
            uint64_t n = texture_level_bytes(td.format, td.width >> l, td.height >> l);
            tx.levels.emplace_back(td.data + at, td.data + at + n);
            at += n;
        }
    }
    s->light_prim = r_light_prims(*s);
    s->light_alias = build_light_alias(*s);
    s->use_bvh = accel != 0;
    s->flat = accel == 2 || accel == 3;
    if (s->use_bvh) s->bvh = build_scene_bvh(s->geom(), leaf_max);
    if (accel == 3) build_wide_bvh(s->geom(), s->bvh);
    return s;
}

void oracle_scene_destroy(void* p) { delete static_cast<OracleScene*>(p); }

// 0: the reference's uniform light pick; 1: power-proportional through the alias table.
void oracle_scene_set_light_power(void* p, int power) { static_cast<OracleScene*>(p)->light_power = power != 0; }

// 0: the reference's 16-bit hash visibility test; 1: the sampled triangle itself.
void oracle_scene_set_light_exact(void* p, int exact) { static_cast<OracleScene*>(p)->light_exact = exact != 0; }

// BVH arrays for node-for-node comparison with the GPU build.
void oracle_scene_bvh_info(void* p, uint64_t* out /* blas_nodes, tris, tlas_nodes, blas_levels, tlas_levels,
                                                    flat_nodes, flat_tris, flat_levels, wide_nodes,
                                                    wide_tris, wide_levels */) {
    OracleScene* s = static_cast<OracleScene*>(p);
    out[0] = s->bvh.blas.size();
    out[1] = s->bvh.tris.size();
    out[2] = s->bvh.tlas.size();
    out[3] = (uint64_t)s->bvh.blas_levels;
    out[4] = (uint64_t)s->bvh.tlas_levels;
    out[5] = s->bvh.flat.size();
    out[6] = s->bvh.flat_tris.size();
    out[7] = (uint64_t)s->bvh.flat_levels;
    out[8] = s->bvh.wide.size();
    out[9] = s->bvh.wide_tris.size();
    out[10] = (uint64_t)s->bvh.wide_levels;
}
void oracle_scene_wide_copy(void* p, void* nodes, void* tris) {
    OracleScene* s = static_cast<OracleScene*>(p);
    if (nodes) std::memcpy(nodes, s->bvh.wide.data(), s->bvh.wide.size() * sizeof(Node8));
    if (tris) std::memcpy(tris, s->bvh.wide_tris.data(), s->bvh.wide_tris.size() * sizeof(TriRecord));
}
void oracle_scene_flat_copy(void* p, void* nodes, void* tris) {
    OracleScene* s = static_cast<OracleScene*>(p);
    if (nodes) std::memcpy(nodes, s->bvh.flat.data(), s->bvh.flat.size() * sizeof(Node4));
    if (tris) std::memcpy(tris, s->bvh.flat_tris.data(), s->bvh.flat_tris.size() * sizeof(TriRecord));
}
void oracle_scene_bvh_copy(void* p, void* blas, void* tris, void* tlas) {
    OracleScene* s = static_cast<OracleScene*>(p);
    if (blas) std::memcpy(blas, s->bvh.blas.data(), s->bvh.blas.size() * sizeof(Node4));
    if (tris) std::memcpy(tris, s->bvh.tris.data(), s->bvh.tris.size() * sizeof(TriRecord));
    if (tlas) std::memcpy(tlas, s->bvh.tlas.data(), s->bvh.tlas.size() * sizeof(Node4));
}

// rays: n x 8 floats (origin xyz, tmin, direction xyz, tmax); hits: n x 8 words
// (hit, t, u, v, instance, prim, 0, 0).  flags bit0 = cull back faces, bit1 = brute force,
// bit2 = the flat BVH, bit3 = the wide format of the flat BVH (scene created with accel 3).
void oracle_trace_batch(void* p, const float* rays, uint32_t n, uint32_t flags, uint32_t* hits,
                        int threads) {
    OracleScene* s = static_cast<OracleScene*>(p);
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 64)
#endif
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        const float* r = rays + 8 * i;
        v3 o{r[0], r[1], r[2]}, d{r[4], r[5], r[6]};
        bool cull = flags & 1u;
        Geometry g = s->geom();
        Hit h = (flags & 2u) || !s->use_bvh ? trace_brute(g, o, d, r[3], r[7], cull)
                : (flags & 8u)                  ? trace_wide(g, s->bvh, o, d, r[3], r[7], cull)
                : (flags & 4u)                  ? trace_flat(g, s->bvh, o, d, r[3], r[7], cull)
                                                : trace_bvh(g, s->bvh, o, d, r[3], r[7], cull);
        uint32_t* out = hits + 8 * i;
        out[0] = (uint32_t)h.hit;
        out[1] = h.hit ? fbits(h.t) : 0u;
        out[2] = h.hit ? fbits(h.u) : 0u;
        out[3] = h.hit ? fbits(h.v) : 0u;
        out[4] = h.hit ? h.instance : 0u;
        out[5] = h.hit ? h.prim : 0u;
        out[6] = 0u;
        out[7] = 0u;
    }
}

// Renders rows [y0, y1) into `target` (W*H RGBA32F, read for accumulation).
void oracle_render(void* p, const Constants* c, float* target, uint32_t y0, uint32_t y1,
                   uint32_t x0, uint32_t x1, int threads) {
    OracleScene* s = static_cast<OracleScene*>(p);
    uint32_t W = c->screen_size[0];
    int64_t cols = (int64_t)x1 - x0;
    int64_t total = ((int64_t)y1 - y0) * cols;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
    for (int64_t k = 0; k < total; ++k) {
        uint32_t py = y0 + (uint32_t)(k / cols), px = x0 + (uint32_t)(k % cols);
        v3 acc = render_pixel(*s, *c, px, py);
        float* t = target + 4ull * ((uint64_t)py * W + px);
        if (c->accumulated_frame_count != 0) {
            v3 prev = v3{t[0], t[1], t[2]};
            acc = (prev * (float)(c->accumulated_frame_count - 1u) + acc) /
                  (float)c->accumulated_frame_count;
        }
        t[0] = acc.x;
        t[1] = acc.y;
        t[2] = acc.z;
        t[3] = 1.0f;
    }
}

// display.glsl:6-12 on n RGBA32F pixels -> RGBA32F.
void oracle_tonemap(const float* in, uint64_t n, int tonemap, float* out) {
    for (uint64_t i = 0; i < n; ++i) {
        v3 col{in[4 * i], in[4 * i + 1], in[4 * i + 2]};
        if (tonemap) col = neutral_tonemap(col);
        out[4 * i] = col.x;
        out[4 * i + 1] = col.y;
        out[4 * i + 2] = col.z;
        out[4 * i + 3] = 1.0f;
    }
}

// material/test.rs harness: per sample, bsdf_prepare with Generator(seed) then
// bsdf_evaluate(wi, wo).  samples: n x 8 floats (wi xyz, seed bits, wo xyz, 0);
// results: n x 8 floats (bsdf rgb, pdf, lobe probabilities 0..3) — see tt_bsdf_eval_batch.
void oracle_bsdf_eval_batch(const MaterialConstants* m, const float* samples, uint32_t n,
                            float* results) {
    for (uint32_t i = 0; i < n; ++i) {
        const float* sm = samples + 8 * i;
        Generator g{fbits(sm[3])};
        v3 wi{sm[0], sm[1], sm[2]}, wo{sm[4], sm[5], sm[6]};
        Lobes l = bsdf_prepare(*m, wi, g);
        float pdf = 0.0f;
        v3 b = bsdf_evaluate(*m, l, wi, wo, pdf);
        float* r = results + 8 * i;
        r[0] = b.x; r[1] = b.y; r[2] = b.z; r[3] = pdf;
        r[4] = bitsf(g.state); r[5] = l.probs[5]; r[6] = l.probs[2]; r[7] = l.probs[3];
    }
}

// bsdf_prepare + bsdf_sample.  samples: n x 4 (wi xyz, seed bits); results: n x 12
// (bsdf rgb, pdf, wo xyz, lobe, final state bits, 0, 0, 0).
void oracle_bsdf_sample_batch(const MaterialConstants* m, const float* samples, uint32_t n,
                              float* results) {
    for (uint32_t i = 0; i < n; ++i) {
        const float* sm = samples + 4 * i;
        Generator g{fbits(sm[3])};
        v3 wi{sm[0], sm[1], sm[2]};
        Lobes l = bsdf_prepare(*m, wi, g);
        v3 wo = splat3(0.0f);
        float pdf = 0.0f;
        int lobe = 0;
        v3 b = bsdf_sample(*m, l, wi, g, wo, pdf, lobe);
        float* r = results + 12 * i;
        r[0] = b.x; r[1] = b.y; r[2] = b.z; r[3] = pdf;
        r[4] = wo.x; r[5] = wo.y; r[6] = wo.z; r[7] = (float)lobe;
        r[8] = bitsf(g.state); r[9] = 0.0f; r[10] = 0.0f; r[11] = 0.0f;
    }
}

// New instance transforms (same count, meshes, materials): refits both world structures.
void oracle_scene_update_instances(void* p, const Instance* instances, uint32_t count) {
    OracleScene* s = static_cast<OracleScene*>(p);
    if (count != s->instances.size()) return;
    std::memcpy(s->instances.data(), instances, sizeof(Instance) * count);
    if (s->use_bvh) refit_world_structures(s->geom(), s->bvh);
    if (!s->bvh.wide.empty()) build_wide_bvh(s->geom(), s->bvh);  // quantised boxes: rebuilt, not refitted
    s->light_alias = build_light_alias(*s);
}

// ReSTIR DI state of the oracle: config = {candidates, m_cap_factor, neighbours, radius}.
void* oracle_restir_create(void* scene, uint32_t width, uint32_t height, uint32_t candidates, float m_cap_factor,
                           uint32_t neighbours, float radius) {
    RestirOracle* R = new RestirOracle();
    R->s = static_cast<OracleScene*>(scene);
    R->W = width;
    R->H = height;
    uint64_t n = (uint64_t)width * height;
    for (int k = 0; k < 2; ++k) {
        R->gb[k].assign(n, RSurface{});
        R->fin[k].assign(n, r_empty());
    }
    R->init.assign(n, r_empty());
    R->temp.assign(n, r_empty());
    R->light_prim = r_light_prims(*R->s);
    R->candidates = candidates;
    R->m_cap_factor = m_cap_factor;
    R->neighbours = neighbours;
    R->radius = radius;
    return R;
}
void oracle_restir_destroy(void* p) { delete static_cast<RestirOracle*>(p); }
void oracle_restir_frame(void* p, const Constants* c, float* target, int threads) {
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
    restir_frame(*static_cast<RestirOracle*>(p), *c, target);
}
// Final reservoirs of the last frame (W*H records of 32 bytes).
void oracle_restir_reservoirs(void* p, void* out) {
    RestirOracle* R = static_cast<RestirOracle*>(p);
    const std::vector<RRes>& f = R->fin[R->cur ^ 1u];
    std::memcpy(out, f.data(), f.size() * sizeof(RRes));
}

// Elementary functions, for accuracy tests against libm.
void oracle_math(int which, const float* x, uint64_t n, float* y) {
    for (uint64_t i = 0; i < n; ++i) {
        switch (which) {
            case 0: y[i] = tsin(x[i]); break;
            case 1: y[i] = tcos(x[i]); break;
            case 2: y[i] = texp(x[i]); break;
            case 3: y[i] = tlog(x[i]); break;
            case 4: y[i] = tacos(x[i]); break;
            default: y[i] = 0.0f;
        }
    }
}

// textureLod of texture `index` of a scene at n (u, v, lod) triples -> n RGBA.
void oracle_texture_sample(void* p, uint32_t index, const float* uvl, uint32_t n, float* rgba) {
    const OracleScene* s = static_cast<const OracleScene*>(p);
    for (uint32_t i = 0; i < n; ++i) {
        v4 r = sample_texture(s->textures[index], v2{uvl[3 * i], uvl[3 * i + 1]}, uvl[3 * i + 2]);
        rgba[4 * i] = r.x;
        rgba[4 * i + 1] = r.y;
        rgba[4 * i + 2] = r.z;
        rgba[4 * i + 3] = r.w;
    }
}

// atan2 of the tangent-frame encoding, for accuracy tests against libm.
void oracle_atan2(const float* y, const float* x, uint64_t n, float* out) {
    for (uint64_t i = 0; i < n; ++i) out[i] = tatan2(y[i], x[i]);
}

// Scene::insert_mesh restated (ref_ingest.h); vertices are 8-byte ProcessedVertex records.
int oracle_mesh_ingest(const float* positions, const float* uv, const uint32_t* indices, const float* normals,
                       const float* tangents, uint32_t n, uint32_t m, int16_t* out_positions, void* out_vertices,
                       float* sphere) {
    return ref::mesh_ingest(positions, uv, indices, normals, tangents, n, m, out_positions,
                            static_cast<ref::IngestVertex*>(out_vertices), sphere);
}

int oracle_abi_version(void) { return 1; }

}  // extern "C"
