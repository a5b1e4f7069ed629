// ReSTIR DI kernels (the passes described in tt_restir.cuh), one thread per pixel in 16 x 8
// tiles; each pass reads and writes whole-frame arrays in HBM:
//   G-buffer 64 B / pixel (current and previous frame), prepared lobes 96 B / pixel (current
//   frame), reservoirs 32 B / pixel
//   (initial, temporal, final; the final array of frame n is the history of frame n + 1).
//
// The BSDF lobes are inlined in this translation unit (the path tracer's shading kernel calls
// them out of line to stay within the instruction cache): the passes evaluate lobes in loops over
// candidates and neighbours, where the calls cost more (5.72 -> 5.56 ms per 1080p frame).
#define TT_INLINE_LOBES 1
#include <cuda_runtime.h>

#include "tt_internal.h"
#include "tt_kernels.h"
#include "tt_restir.cuh"

namespace tt {

constexpr int RT_TILE_X = 16, RT_TILE_Y = 8, RT_BLOCK = RT_TILE_X * RT_TILE_Y;
// resident blocks per SM the candidate, reuse and shading passes are compiled for (a register cap
// of 80): the 1080p frame took 5.55 ms uncapped (105 registers, 4 blocks), 5.26 ms at 5 blocks,
// 5.15 ms at 6 despite some spilling, and 5.33 ms at 7
#ifndef TT_RESTIR_MIN_BLOCKS
#define TT_RESTIR_MIN_BLOCKS 6
#endif
constexpr uint32_t PASS_INITIAL = 1u, PASS_TEMPORAL = 2u, PASS_SPATIAL = 3u;

__device__ __forceinline__ bool pixel_of_thread(const tt_constants& c, uint32_t& x, uint32_t& y) {
    x = blockIdx.x * RT_TILE_X + threadIdx.x % RT_TILE_X;
    y = blockIdx.y * RT_TILE_Y + threadIdx.x / RT_TILE_X;
    return x < c.screen_size[0] && y < c.screen_size[1];
}

// Appends each thread's pixel to its bucket's queue (bucket == HIT_BUCKETS: to none).  Warp
// ballots count the block's pixels per bucket in shared memory, and one thread per bucket takes
// the block's range of the queue with a single global atomic, so the four counters see one
// atomic per block instead of one per warp.  Every thread of the block must call it.
__device__ __forceinline__ void block_queue_append(const RestirParams& rp, uint32_t bucket, uint32_t pixel,
                                                   uint64_t WH) {
    __shared__ uint32_t s_count[HIT_BUCKETS], s_base[HIT_BUCKETS];
    if (threadIdx.x < HIT_BUCKETS) s_count[threadIdx.x] = 0u;
    __syncthreads();
    uint32_t lane = threadIdx.x & 31u, pos = 0u;
#pragma unroll
    for (uint32_t b = 0; b < HIT_BUCKETS; ++b) {
        uint32_t mask = __ballot_sync(0xffffffffu, bucket == b);
        uint32_t wbase = 0u;
        if (lane == 0u && mask != 0u) wbase = atomicAdd(&s_count[b], (uint32_t)__popc(mask));
        wbase = __shfl_sync(0xffffffffu, wbase, 0);
        if (bucket == b) pos = wbase + (uint32_t)__popc(mask & ((1u << lane) - 1u));
    }
    __syncthreads();
    if (threadIdx.x < HIT_BUCKETS)
        s_base[threadIdx.x] = s_count[threadIdx.x] ? atomicAdd(rp.queue_count + threadIdx.x, s_count[threadIdx.x]) : 0u;
    __syncthreads();
    if (bucket < HIT_BUCKETS) rp.queue[(uint64_t)bucket * WH + s_base[bucket] + pos] = pixel;
}

// Pixel of queue entry q: the bucket queues are concatenated in bucket order; with PAD each
// queue starts on a block boundary, so that a block holds one bucket's pixels.  `bucket`
// receives the bucket of a queued pixel.
template <bool PAD = false>
__device__ __forceinline__ bool queued_pixel(const RestirParams& rp, uint32_t WH, uint32_t q, uint64_t& i,
                                             uint32_t& bucket) {
    uint32_t start = 0u;
#pragma unroll
    for (uint32_t b = 0; b < HIT_BUCKETS; ++b) {
        uint32_t n = rp.queue_count[b];
        if (q < start + n) {
            i = rp.queue[(uint64_t)b * WH + (q - start)];
            bucket = b;
            return true;
        }
        start += PAD ? (n + RT_BLOCK - 1u) / RT_BLOCK * RT_BLOCK : n;
        if (q < start) return false;  // the padding after bucket b's queue
    }
    return false;
}

// The accumulation rule of tt_render for one pixel of the target.
__device__ __forceinline__ void write_target(const RenderParams& p, uint64_t i, f3 radiance) {
    const tt_constants& c = p.c;
    float4* tp = p.target + i;
    if (c.accumulated_frame_count != 0) {
        float4 prev = *tp;
        radiance = (f3{prev.x, prev.y, prev.z} * (float)(c.accumulated_frame_count - 1u) + radiance) /
                   (float)c.accumulated_frame_count;
    }
    *tp = make_float4(radiance.x, radiance.y, radiance.z, 1.0f);
}

// Rebuilds the pixel's shading state from its G-buffer record.
struct ShadingState {
    f3 pos, wi;
    Basis basis;
    const tt_material* material;
    const MatC* mc;  // the material's constants, or `local` with its textures sampled
    MatC local;
    Lobes lobes;
    uint32_t seed;
    float dist;
    f2 uv;
    float mip;
};
template <bool TEX>
__device__ __forceinline__ bool load_surface(const DevScene& sc, const Surface& s, const float4* gtex,
                                             const float4* glob, uint64_t i, ShadingState& st) {
    uint32_t mat = __float_as_uint(s.normal_mat.w);
    if (mat == NO_SURFACE) return false;
    st.pos = f3{s.pos_dist.x, s.pos_dist.y, s.pos_dist.z};
    st.dist = s.pos_dist.w;
    st.basis.normal = f3{s.normal_mat.x, s.normal_mat.y, s.normal_mat.z};
    st.basis.tangent = f3{s.tangent_inst.x, s.tangent_inst.y, s.tangent_inst.z};
    st.basis.bitangent = normalize(cross(st.basis.normal, st.basis.tangent));
    st.wi = f3{s.wi_seed.x, s.wi_seed.y, s.wi_seed.z};
    st.seed = __float_as_uint(s.wi_seed.w);
    st.material = sc.materials + mat;
    st.uv = f2{0.0f, 0.0f};
    st.mip = 0.0f;
    if (TEX) {
        float4 t = gtex[i];
        st.uv = f2{t.x, t.y};
        st.mip = t.z;
    }
    st.mc = &hit_material<TEX>(sc, st.material, st.uv, st.mip, st.local);
    st.lobes = load_lobes(glob + LOBE_RECORD * i);  // bsdf_prepare(*st.mc, st.wi, seed), stored by the G-buffer pass
    return true;
}

template <bool TEX>
__device__ __forceinline__ float target_of(const DevScene& sc, const ShadingState& st, uint32_t light, float r1,
                                           float r2) {
    if (light == NO_LIGHT) return 0.0f;
    LightPoint lp = light_point<TEX>(sc, light, r1, r2);
    return luminance(restir_contribution(*st.mc, st.lobes, st.basis, st.wi, st.pos, lp));
}

// The G-buffer pass for pixel (x, y); returns the material bucket of its primary hit, or
// HIT_BUCKETS for a sky pixel (finished here).
template <bool TEX, int ACCEL>
__device__ __forceinline__ uint32_t gbuffer_pixel(const RenderParams& p, const RestirParams& rp, Surface* gbuf,
                                                  float4* gtex, float4* glob, uint32_t x, uint32_t y, uint32_t g,
                                                  f2 ndc, f3 dir, const Hit& h) {
    const tt_constants& c = p.c;
    const DevScene& sc = p.sc;
    uint32_t W = c.screen_size[0];
    f3 org = f3{c.camera_position[0], c.camera_position[1], c.camera_position[2]};
    Surface s;
    uint64_t i = (uint64_t)y * W + x;
    // surface pixels go to their material bucket's queue for the candidate and shade passes; sky
    // pixels are finished here: empty initial reservoir, the white sky (integrate.glsl:272-276)
    uint32_t bucket = h.hit ? (uint32_t)__ldg(sc.inst_bucket + h.instance) : HIT_BUCKETS;
    if (!h.hit) {
        rp.initial[i] = empty_reservoir();
        write_target(p, i, splat(1.0f));
        s.pos_dist = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        s.normal_mat = make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(NO_SURFACE));
        s.tangent_inst = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        s.wi_seed = make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(g));
    } else {
        ShadeHit hit = get_ray_hit(sc, h.instance, h.prim, h.u, h.v);
        float mip = 0.0f;
        if (TEX) {
            mip = primary_mip_level(c, hit, org, ndc);
            gtex[(uint64_t)y * W + x] = make_float4(hit.uv.x, hit.uv.y, mip, 0.0f);
        }
        MatC local;
        const MatC& mc = hit_material<TEX>(sc, sc.materials + hit.material_index, hit.uv, mip, local);
        Basis basis = create_surface_basis(hit.tangent_space, col3(mc.geometry_normal));
        f3 wi = transform_from_basis(basis, -dir);
        f3 to = hit.world_position - org;
        s.pos_dist = make_float4(hit.world_position.x, hit.world_position.y, hit.world_position.z, length(to));
        s.normal_mat = make_float4(basis.normal.x, basis.normal.y, basis.normal.z, __uint_as_float(hit.material_index));
        s.tangent_inst = make_float4(basis.tangent.x, basis.tangent.y, basis.tangent.z, __uint_as_float(h.instance));
        s.wi_seed = make_float4(wi.x, wi.y, wi.z, __uint_as_float(g));
        uint32_t gp = g;
        store_lobes(glob + LOBE_RECORD * ((uint64_t)y * W + x), bsdf_prepare(mc, wi, gp));
    }
    gbuf[(uint64_t)y * W + x] = s;
    return bucket;
}

template <bool TEX, int ACCEL>
__global__ void __launch_bounds__(RT_BLOCK) restir_gbuffer_kernel(const __grid_constant__ RenderParams p,
                                                                  const __grid_constant__ RestirParams rp,
                                                                  Surface* gbuf, float4* gtex, float4* glob) {
    // the flat BVH: the camera rays' hits from their rasterised keys, or the warp's camera rays (a
    // 16 x 2 pixel strip) traced as one packet
    constexpr bool PACKET = ACCEL == ACCEL_FLAT_ONLY;
    __shared__ uint32_t s_stack[PACKET ? 1 : TRAVERSAL_STACK * RT_BLOCK];
    __shared__ uint2 s_packet[PACKET ? RT_BLOCK / 32 : 1][PACKET ? PACKET_STACK : 1];
    uint32_t x, y;
    const tt_constants& c = p.c;
    uint32_t W = c.screen_size[0], H = c.screen_size[1];
    const bool inside = pixel_of_thread(c, x, y);
    uint32_t g = inside ? jenkins_hash((x + y * W) ^ jenkins_hash(c.frame_index)) : 0u;
    f2 ndc = inside ? pixel_ndc(x, y, W, H, g) : f2{0.0f, 0.0f};
    f3 dir = inside ? camera_ray_direction(c, ndc) : f3{0.0f, 0.0f, 1.0f};
    f3 org = f3{c.camera_position[0], c.camera_position[1], c.camera_position[2]};
    Hit h{};
    if (PACKET && rp.vis != nullptr && *rp.vis_ok != 0u) {
        if (inside) h = primary_resolve(p.sc, rp.vis[band_index(x, y, W, H)], org, dir, p.err);
    } else if (PACKET) {
        h = packet_trace_flat(p.sc, org, dir, inside, EXTENSION_TMIN, EXTENSION_TMAX, true, s_packet[threadIdx.x >> 5],
                              p.err);
    } else if (inside) {
        Counters cnt{0u, 0u, 0u, 0u};
        h = trace_closest<false, ACCEL>(p.sc, org, dir, EXTENSION_TMIN, EXTENSION_TMAX, true, s_stack + threadIdx.x,
                                        RT_BLOCK, p.err, cnt);
    }
    // threads outside the image take part in the block's queue append only
    uint32_t bucket = HIT_BUCKETS;
    if (inside) bucket = gbuffer_pixel<TEX, ACCEL>(p, rp, gbuf, gtex, glob, x, y, g, ndc, dir, h);
    block_queue_append(rp, bucket, y * W + x, (uint64_t)W * H);
}

// Candidate generation for queued pixel i, with the BSDF compiled for lobe set LS (the lobe sets
// of all materials of the pixel's bucket lie within LS, so the result is the six-lobe code's).
template <bool TEX, int ACCEL, uint32_t LS>
__device__ __forceinline__ Reservoir initial_pixel(const RenderParams& p, const Surface* gbuf, const float4* gtex,
                                                   const float4* glob, uint64_t i, uint32_t candidates,
                                                   uint32_t* stack) {
    const DevScene& sc = p.sc;
    ShadingState st;
    Reservoir r = empty_reservoir();
    if (load_surface<TEX>(sc, gbuf[i], gtex, glob, i, st) && sc.emissive_count > 0) {
        uint32_t g = jenkins_hash(st.seed + PASS_INITIAL);
        float inv_p_pick = (float)sc.emissive_count;
        float chosen = 0.0f;
        for (uint32_t k = 0; k < candidates; ++k) {
            uint32_t light = xor_shift(g) % sc.emissive_count;
            float inv_p = inv_p_pick;
            if (sc.light_power) {  // candidates by emitted power (TT_LIGHT_SELECTION_POWER)
                float4 e = __ldg(sc.light_alias + light);
                float coin = random_float(g);
                if (!(coin < e.x)) light = __float_as_uint(e.y);
                inv_p = 1.0f / __ldg(&sc.light_alias[light].z);
            }
            float r1 = random_float(g);
            float r2 = random_float(g);
            LightPoint lp = light_point<TEX>(sc, light, r1, r2);
            float ph = luminance(restir_contribution<LS>(*st.mc, st.lobes, st.basis, st.wi, st.pos, lp));
            float w = ph * (inv_p * lp.area);  // p^ / p, p = pick probability / area
            if (reservoir_update(r, light, r1, r2, w, 1.0f, g)) chosen = ph;
        }
        r.W = chosen > 0.0f ? r.w_sum / (r.M * chosen) : 0.0f;
        if (r.W > 0.0f) {
            LightPoint lp = light_point<TEX>(sc, r.light, r.r1, r.r2);
            if (!restir_visible<false, ACCEL>(sc, st.pos, lp, r.light, stack, RT_BLOCK, p.err)) r.W = 0.0f;
        }
    }
    return r;
}

// Untextured scenes: the bucket queues are padded to block boundaries and each block evaluates
// its candidates with the BSDF of its bucket's lobe set (metal, opaque dielectric, the two, or
// all six lobes), which leaves the absent lobes' code and registers out of the candidate loop.
// Textured materials can take metalness or transmission from a texel: they use all six lobes.
template <bool TEX, int ACCEL>
__global__ void __launch_bounds__(RT_BLOCK, TT_RESTIR_MIN_BLOCKS) restir_initial_kernel(const __grid_constant__ RenderParams p,
                                                                  const __grid_constant__ RestirParams rp,
                                                                  const Surface* gbuf, const float4* gtex, const float4* glob,
                                                                  Reservoir* out, uint32_t candidates) {
    __shared__ uint32_t s_stack[TRAVERSAL_STACK * RT_BLOCK];
    const tt_constants& c = p.c;
    uint64_t i = 0;
    uint32_t bucket = 0;
    if (!queued_pixel<!TEX>(rp, c.screen_size[0] * c.screen_size[1], blockIdx.x * RT_BLOCK + threadIdx.x, i, bucket))
        return;
    uint32_t* stack = s_stack + threadIdx.x;
    Reservoir r;
    uint32_t ls = TEX ? LOBE_SET_ALL : (p.sc.bucket_lobes >> (8u * bucket)) & LOBE_SET_ALL;
    if ((ls & ~LOBE_SET_METAL) == 0u) r = initial_pixel<TEX, ACCEL, LOBE_SET_METAL>(p, gbuf, gtex, glob, i, candidates, stack);
    else if ((ls & ~LOBE_SET_DIELECTRIC) == 0u)
        r = initial_pixel<TEX, ACCEL, LOBE_SET_DIELECTRIC>(p, gbuf, gtex, glob, i, candidates, stack);
    else if ((ls & ~LOBE_SET_BASE) == 0u)
        r = initial_pixel<TEX, ACCEL, LOBE_SET_BASE>(p, gbuf, gtex, glob, i, candidates, stack);
    else r = initial_pixel<TEX, ACCEL, LOBE_SET_ALL>(p, gbuf, gtex, glob, i, candidates, stack);
    out[i] = r;
}

// Merges reservoir q (from another pixel or frame) into r, re-targeted at this pixel.
template <bool TEX>
__device__ __forceinline__ void merge(const DevScene& sc, const ShadingState& st, Reservoir& r, const Reservoir& q,
                                      float m_cap, float& chosen, uint32_t& g) {
    float m = fmn(q.M, m_cap);
    float ph = target_of<TEX>(sc, st, q.light, q.r1, q.r2);
    float w = ph * q.W * m;
    if (reservoir_update(r, q.light, q.r1, q.r2, w, m, g)) chosen = ph;
}

// Pixel of the previous frame that saw world position pos, or false (behind the camera or
// outside the image).  Solves  s * u = -nx * a - ny * b + c  for (nx, ny, s), where u is the
// position in the previous camera's view space and a, b, c are the inverse projection's
// columns that map NDC to view-space ray directions (the camera ray of integrate.glsl:17-20).
__device__ __forceinline__ bool reproject(const RestirHistory& hist, f3 pos, uint32_t W, uint32_t H, uint32_t& px,
                                          uint32_t& py) {
    f3 d = pos - f3{hist.camera_position[0], hist.camera_position[1], hist.camera_position[2]};
    const float* v = hist.view;  // column-major
    f3 u = f3{v[0] * d.x + v[4] * d.y + v[8] * d.z, v[1] * d.x + v[5] * d.y + v[9] * d.z,
              v[2] * d.x + v[6] * d.y + v[10] * d.z};
    const float* ip = hist.inverse_proj;
    f3 a = f3{ip[0], ip[1], ip[2]}, b = f3{ip[4], ip[5], ip[6]};
    f3 cc = f3{ip[8] + ip[12], ip[9] + ip[13], ip[10] + ip[14]};
    // columns of the system matrix: -a, -b, -u; right-hand side: -c
    f3 c0 = -a, c1 = -b, c2 = -u, rhs = -cc;
    float det = dot(c0, cross(c1, c2));
    if (!(fabsf(det) > 0.0f)) return false;
    float nx = dot(rhs, cross(c1, c2)) / det;
    float ny = dot(c0, cross(rhs, c2)) / det;
    float s = dot(c0, cross(c1, rhs)) / det;
    if (!(s > 0.0f)) return false;
    float fx = (nx + 1.0f) * 0.5f * (float)W, fy = (ny + 1.0f) * 0.5f * (float)H;
    if (!(fx >= 0.0f && fx < (float)W && fy >= 0.0f && fy < (float)H)) return false;
    px = (uint32_t)fx;
    py = (uint32_t)fy;
    return true;
}

// Surfaces similar enough to share samples: normals within 25 degrees, camera distances
// within 10 %.
__device__ __forceinline__ bool similar(const Surface& q, f3 normal, float dist) {
    if (__float_as_uint(q.normal_mat.w) == NO_SURFACE) return false;
    f3 n = f3{q.normal_mat.x, q.normal_mat.y, q.normal_mat.z};
    return dot(n, normal) > 0.90630779f && fabsf(q.pos_dist.w - dist) <= 0.1f * dist;
}

template <bool TEX, int ACCEL>
__global__ void __launch_bounds__(RT_BLOCK, TT_RESTIR_MIN_BLOCKS) restir_temporal_kernel(const __grid_constant__ RenderParams p,
                                                                   const __grid_constant__ RestirHistory hist,
                                                                   const Surface* gbuf, const float4* gtex, const float4* glob,
                                                                   const Surface* prev_gbuf,
                                                                   const Reservoir* initial, const Reservoir* prev,
                                                                   Reservoir* out, float m_cap) {
    uint32_t x, y;
    const tt_constants& c = p.c;
    if (!pixel_of_thread(c, x, y)) return;
    const DevScene& sc = p.sc;
    uint32_t W = c.screen_size[0], H = c.screen_size[1];
    uint64_t i = (uint64_t)y * W + x;
    Reservoir cur = initial[i];
    ShadingState st;
    uint32_t px, py;
    if (!hist.valid || !load_surface<TEX>(sc, gbuf[i], gtex, glob, i, st) || !reproject(hist, st.pos, W, H, px, py)) {
        out[i] = cur;
        return;
    }
    uint64_t j = (uint64_t)py * W + px;
    f3 from_prev = st.pos - f3{hist.camera_position[0], hist.camera_position[1], hist.camera_position[2]};
    if (!similar(prev_gbuf[j], st.basis.normal, length(from_prev))) {
        out[i] = cur;
        return;
    }
    uint32_t g = jenkins_hash(st.seed + PASS_TEMPORAL);
    Reservoir r = empty_reservoir();
    float chosen = 0.0f;
    merge<TEX>(sc, st, r, cur, cur.M, chosen, g);
    merge<TEX>(sc, st, r, prev[j], m_cap, chosen, g);
    r.W = chosen > 0.0f ? r.w_sum / (r.M * chosen) : 0.0f;
    out[i] = r;
}

template <bool TEX, int ACCEL>
__global__ void __launch_bounds__(RT_BLOCK, TT_RESTIR_MIN_BLOCKS) restir_spatial_kernel(const __grid_constant__ RenderParams p,
                                                                  const Surface* gbuf, const float4* gtex, const float4* glob,
                                                                  const Reservoir* in,
                                                                  Reservoir* out, uint32_t neighbours, float radius) {
    uint32_t x, y;
    const tt_constants& c = p.c;
    if (!pixel_of_thread(c, x, y)) return;
    const DevScene& sc = p.sc;
    uint32_t W = c.screen_size[0], H = c.screen_size[1];
    uint64_t i = (uint64_t)y * W + x;
    ShadingState st;
    Reservoir cur = in[i];
    if (!load_surface<TEX>(sc, gbuf[i], gtex, glob, i, st)) {
        out[i] = cur;
        return;
    }
    uint32_t g = jenkins_hash(st.seed + PASS_SPATIAL);
    Reservoir r = empty_reservoir();
    float chosen = 0.0f;
    merge<TEX>(sc, st, r, cur, cur.M, chosen, g);
    for (uint32_t k = 0; k < neighbours; ++k) {
        float rr = radius * sqrtf(random_float(g));
        float angle = TAU * random_float(g);
        float sn, cs;
        tsincos(angle, &sn, &cs);
        float qx = (float)x + rr * cs, qy = (float)y + rr * sn;
        if (!(qx >= 0.0f && qx < (float)W && qy >= 0.0f && qy < (float)H)) continue;
        uint64_t j = (uint64_t)(uint32_t)qy * W + (uint32_t)qx;
        if (j == i || !similar(gbuf[j], st.basis.normal, st.dist)) continue;
        const Reservoir q = in[j];
        merge<TEX>(sc, st, r, q, q.M, chosen, g);
    }
    r.W = chosen > 0.0f ? r.w_sum / (r.M * chosen) : 0.0f;
    out[i] = r;
}

template <bool TEX, int ACCEL>
__global__ void __launch_bounds__(RT_BLOCK, TT_RESTIR_MIN_BLOCKS) restir_shade_kernel(const __grid_constant__ RenderParams p,
                                                                const __grid_constant__ RestirParams rp,
                                                                const Surface* gbuf, const float4* gtex, const float4* glob,
                                                                const Reservoir* res) {
    __shared__ uint32_t s_stack[TRAVERSAL_STACK * RT_BLOCK];
    const tt_constants& c = p.c;
    uint64_t i = 0;
    uint32_t bucket = 0;
    if (!queued_pixel(rp, c.screen_size[0] * c.screen_size[1], blockIdx.x * RT_BLOCK + threadIdx.x, i, bucket)) return;
    const DevScene& sc = p.sc;
    ShadingState st;
    f3 radiance;
    if (!load_surface<TEX>(sc, gbuf[i], gtex, glob, i, st)) {
        radiance = splat(1.0f);  // the white sky of integrate.glsl:272-276
    } else {
        radiance = hit_emissive<TEX>(sc, st.material, st.uv, st.mip);
        Reservoir r = res[i];
        if (r.light != NO_LIGHT && r.W > 0.0f) {
            LightPoint lp = light_point<TEX>(sc, r.light, r.r1, r.r2);
            f3 contrib = restir_contribution(*st.mc, st.lobes, st.basis, st.wi, st.pos, lp);
            if (restir_visible<false, ACCEL>(sc, st.pos, lp, r.light, s_stack + threadIdx.x, RT_BLOCK, p.err))
                radiance += contrib * r.W;
        }
    }
    write_target(p, i, radiance);
}

template <bool TEX, int ACCEL>
static void restir_passes(const RenderParams& p, const RestirParams& rp, cudaStream_t st, StageTimer* timer) {
    const tt_constants& c = p.c;
    dim3 grid((c.screen_size[0] + RT_TILE_X - 1) / RT_TILE_X, (c.screen_size[1] + RT_TILE_Y - 1) / RT_TILE_Y);
    uint64_t WH = (uint64_t)c.screen_size[0] * c.screen_size[1];
    unsigned qgrid = (unsigned)((WH + RT_BLOCK - 1) / RT_BLOCK);  // enough blocks for every pixel queued
    unsigned padded_qgrid = qgrid + HIT_BUCKETS;                       // and for each queue padded to a block
    check_cuda(cudaMemsetAsync(rp.queue_count, 0, 4ull * HIT_BUCKETS, st), "memset");
    stage_begin(timer, TT_STAGE_RESTIR_GBUFFER, st);
    restir_gbuffer_kernel<TEX, ACCEL><<<grid, RT_BLOCK, 0, st>>>(p, rp, rp.gbuf, rp.gtex, rp.glob);
    stage_end(timer, st);
    stage_begin(timer, TT_STAGE_RESTIR_INITIAL, st);
    restir_initial_kernel<TEX, ACCEL><<<padded_qgrid, RT_BLOCK, 0, st>>>(p, rp, rp.gbuf, rp.gtex, rp.glob, rp.initial,
                                                                 rp.candidates);
    stage_end(timer, st);
    stage_begin(timer, TT_STAGE_RESTIR_TEMPORAL, st);
    restir_temporal_kernel<TEX, ACCEL><<<grid, RT_BLOCK, 0, st>>>(p, rp.history, rp.gbuf, rp.gtex, rp.glob, rp.prev_gbuf,
                                                           rp.initial, rp.prev, rp.temporal, rp.m_cap);
    stage_end(timer, st);
    stage_begin(timer, TT_STAGE_RESTIR_SPATIAL, st);
    restir_spatial_kernel<TEX, ACCEL><<<grid, RT_BLOCK, 0, st>>>(p, rp.gbuf, rp.gtex, rp.glob, rp.temporal, rp.final_out,
                                                          rp.neighbours, rp.radius);
    stage_end(timer, st);
    stage_begin(timer, TT_STAGE_RESTIR_SHADE, st);
    restir_shade_kernel<TEX, ACCEL><<<qgrid, RT_BLOCK, 0, st>>>(p, rp, rp.gbuf, rp.gtex, rp.glob, rp.final_out);
    stage_end(timer, st);
}

void render_restir(const RenderParams& p, const RestirParams& rp, cudaStream_t st, StageTimer* timer) {
    dispatch_accel(p.sc, [&](auto accel) {
        if (p.sc.textured && rp.gtex) restir_passes<true, decltype(accel)::value>(p, rp, st, timer);
        else restir_passes<false, decltype(accel)::value>(p, rp, st, timer);
    });
}

}  // namespace tt
