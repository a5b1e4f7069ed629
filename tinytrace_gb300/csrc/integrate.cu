// Path tracer megakernel, tonemap and parity kernels for sm_103a.
//
// integrate_kernel restates src/integrate/integrate.glsl:10-347 (the reference's only hot
// kernel) over the project's BVH4 ray queries.  One thread owns one pixel and runs its
// sample and bounce loops exactly as the reference does, so every pixel's RNG stream and
// float operation sequence match the CPU oracle bit for bit.  Threads of a block cover a
// 16 x 8 pixel tile (coherent primary rays); the traversal stack of each thread is a column
// of a shared-memory array.
#include <cuda_runtime.h>

#include <mutex>

#include "tt_shade.cuh"
#include "tt_internal.h"
#include "tt_kernels.h"

namespace tt {

constexpr int TILE_W = 16, TILE_H = 8, BLOCK = TILE_W * TILE_H;

template <bool COUNT, bool TEX, int ACCEL>
__global__ void __launch_bounds__(BLOCK) integrate_kernel(const __grid_constant__ RenderParams p) {
    __shared__ uint32_t s_stack[TRAVERSAL_STACK * BLOCK];
    const tt_constants& c = p.c;
    const DevScene& sc = p.sc;
    uint32_t W = c.screen_size[0], H = c.screen_size[1];
    uint32_t px = blockIdx.x * TILE_W + (threadIdx.x % TILE_W);
    uint32_t py = blockIdx.y * TILE_H + (threadIdx.x / TILE_W);
    Counters cnt{0u, 0u, 0u, 0u};
    uint32_t rays = 0, hits = 0;
    if (px < W && py < H) {
        uint32_t* stack = s_stack + threadIdx.x;
        uint32_t pixel_gen = jenkins_hash((px + py * W) ^ jenkins_hash(c.frame_index));
        f3 acc = splat(0.0f);
        f3 cam = f3{c.camera_position[0], c.camera_position[1], c.camera_position[2]};
        for (uint32_t si = 0; si < c.sample_count; ++si) {
            f2 ndc = pixel_ndc(px, py, W, H, pixel_gen);
            f3 ray_dir = camera_ray_direction(c, ndc);
            f3 ray_org = cam;
            uint32_t g = pixel_gen;
            f3 path_acc = splat(0.0f), thr = splat(1.0f);
            float mip_level = 1.0f;  // integrate.glsl:215-216
            for (uint32_t bounce = 0; bounce < c.bounce_count; ++bounce) {
                if (COUNT) rays++;
                Hit h = trace_closest<COUNT, ACCEL>(sc, ray_org, ray_dir, EXTENSION_TMIN, EXTENSION_TMAX, true,
                                             stack, BLOCK, p.err, cnt);
                if (!h.hit) {
                    path_acc += splat(1.0f) * thr;
                    break;
                }
                if (COUNT) hits++;
                ShadeHit hit = get_ray_hit(sc, h.instance, h.prim, h.u, h.v);
                if (TEX && bounce == 0) mip_level = primary_mip_level(c, hit, ray_org, ndc);
                const tt_material* material = sc.materials + hit.material_index;
                MatC local;
                const MatC& mc = hit_material<TEX>(sc, material, hit.uv, mip_level, local);
                Basis basis = create_surface_basis(hit.tangent_space, col3(mc.geometry_normal));
                f3 wi = transform_from_basis(basis, -ray_dir);
                Lobes lobes = bsdf_prepare(mc, wi, g);
                bool nee = c.light_sampling == LIGHT_SAMPLING_NEE && sc.emissive_count > 0 &&
                           mc.specular_roughness > 0.15f;
                if (nee) {
                    if (COUNT) rays++;
                    LightSample ls = sample_light(sc, hit.world_position, basis, g);
                    Hit hs = trace_closest<COUNT, ACCEL>(sc, hit.world_position, ls.dir, SHADOW_TMIN, SHADOW_TMAX, false,
                                                  stack, BLOCK, p.err, cnt);
                    f3 direct = light_visible(sc, hs, ls.instance, ls.hash, ls.prim) ? light_contribution<TEX>(sc, ls, mc, lobes, wi)
                                                                           : splat(0.0f);
                    path_acc += thr * direct;
                }
                if (bounce == 0 || !nee) path_acc += hit_emissive<TEX>(sc, material, hit.uv, mip_level) * thr;
                float density = 1.0f;
                f3 wo = splat(0.0f);
                int lobe = 0;
                f3 bsdf = bsdf_sample(mc, lobes, wi, g, wo, density, lobe);
                ray_dir = transform_to_basis(basis, wo);
                ray_org = hit.world_position;
                thr *= bsdf / fmx(density, PDF_EPSILON) * fabsf(cos_theta(wo));
            }
            acc += path_acc;
        }
        acc = acc / (float)c.sample_count;
        float4* t = p.target + (uint64_t)py * W + px;
        if (c.accumulated_frame_count != 0) {
            float4 prev = *t;
            f3 pv = f3{prev.x, prev.y, prev.z};
            acc = (pv * (float)(c.accumulated_frame_count - 1u) + acc) / (float)c.accumulated_frame_count;
        }
        *t = make_float4(acc.x, acc.y, acc.z, 1.0f);
    }
    if (COUNT) {
        unsigned long long v[6] = {rays, cnt.blas_nodes, cnt.tlas_nodes, cnt.triangles, cnt.instances, hits};
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            unsigned long long x = v[k];
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            if ((threadIdx.x & 31) == 0) atomicAdd(p.counters + k, x);
        }
    }
}

// ---------------------------------------------------------------- tonemap (tonemap.glsl:1-26)
__device__ __forceinline__ f3 neutral_tonemap(f3 col) {
    f3 y = f3{0.2126f * col.x + 0.7152f * col.y + 0.0722f * col.z,
              -0.1146f * col.x + -0.3854f * col.y + 0.5f * col.z,
              0.5f * col.x + -0.4542f * col.y + -0.0458f * col.z};
    float bt = 1.0f - texp(-(sqrtf(y.y * y.y + y.z * y.z) * 2.4f));
    float desat = fmx((bt - 0.7f) * 0.8f, 0.0f);
    desat *= desat;
    f3 desat_color = mix3(col, splat(y.x), desat);
    float tm_lum = 1.0f - texp(-y.x);
    float lum = 0.2126f * col.x + 0.7152f * col.y + 0.0722f * col.z;
    f3 tm0 = col * fmx(0.0f, tm_lum / fmx(1e-5f, lum));
    f3 tm1 = f3{1.0f - texp(-desat_color.x), 1.0f - texp(-desat_color.y), 1.0f - texp(-desat_color.z)};
    return mix3(tm0, tm1, bt * bt) * 0.97f;
}

// display.glsl:6-12, headless: writes RGBA32F or RGBA8 (unorm, round to nearest).
__global__ void tonemap_kernel(const float4* in, uint64_t n, uint32_t tonemap, uint32_t format,
                               void* out) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 v = in[i];
    f3 col = f3{v.x, v.y, v.z};
    if (tonemap != 0u) col = neutral_tonemap(col);
    if (format == TT_FORMAT_RGBA32F) {
        static_cast<float4*>(out)[i] = make_float4(col.x, col.y, col.z, 1.0f);
    } else {
        uint32_t r = (uint32_t)(saturate(col.x) * 255.0f + 0.5f);
        uint32_t g = (uint32_t)(saturate(col.y) * 255.0f + 0.5f);
        uint32_t b = (uint32_t)(saturate(col.z) * 255.0f + 0.5f);
        static_cast<uint32_t*>(out)[i] = r | (g << 8) | (b << 16) | (255u << 24);
    }
}

// ---------------------------------------------------------------- parity kernels
// src/material/test.rs:67-80: bsdf_prepare with Generator(seed) then bsdf_evaluate(wi, wo).
__global__ void bsdf_eval_kernel(const MatC* m, const float4* samples, uint32_t n, float4* results) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 a = samples[2 * i], b = samples[2 * i + 1];
    uint32_t g = __float_as_uint(a.w);
    f3 wi = f3{a.x, a.y, a.z}, wo = f3{b.x, b.y, b.z};
    Lobes l = bsdf_prepare(*m, wi, g);
    float pdf = 0.0f;
    f3 r = bsdf_evaluate(*m, l, wi, wo, pdf);
    results[2 * i] = make_float4(r.x, r.y, r.z, pdf);
    results[2 * i + 1] = make_float4(__uint_as_float(g), l.probs[DIFFUSE], l.probs[METAL], l.probs[SPEC_BRDF]);
}
__global__ void bsdf_sample_kernel(const MatC* m, const float4* samples, uint32_t n, float4* results) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 a = samples[i];
    uint32_t g = __float_as_uint(a.w);
    f3 wi = f3{a.x, a.y, a.z};
    Lobes l = bsdf_prepare(*m, wi, g);
    f3 wo = splat(0.0f);
    float pdf = 0.0f;
    int lobe = 0;
    f3 r = bsdf_sample(*m, l, wi, g, wo, pdf, lobe);
    results[3 * i] = make_float4(r.x, r.y, r.z, pdf);
    results[3 * i + 1] = make_float4(wo.x, wo.y, wo.z, (float)lobe);
    results[3 * i + 2] = make_float4(__uint_as_float(g), 0.0f, 0.0f, 0.0f);
}
template <int ACCEL>
__global__ void __launch_bounds__(BLOCK) trace_kernel(DevScene sc, const float4* rays, uint32_t n,
                                                      uint32_t flags, uint4* hits, uint32_t* err) {
    __shared__ uint32_t s_stack[TRAVERSAL_STACK * BLOCK];
    uint32_t i = blockIdx.x * BLOCK + threadIdx.x;
    if (i >= n) return;
    float4 a = rays[2 * i], b = rays[2 * i + 1];
    Counters cnt{0u, 0u, 0u, 0u};
    Hit h = trace_closest<false, ACCEL>(sc, f3{a.x, a.y, a.z}, f3{b.x, b.y, b.z}, a.w, b.w,
                                 (flags & TT_TRACE_CULL_BACK_FACES) != 0u, s_stack + threadIdx.x,
                                 BLOCK, err, cnt);
    if (h.hit) {
        hits[2 * i] = make_uint4(1u, __float_as_uint(h.t), __float_as_uint(h.u), __float_as_uint(h.v));
        hits[2 * i + 1] = make_uint4(h.instance, h.prim, 0u, 0u);
    } else {
        hits[2 * i] = make_uint4(0u, 0u, 0u, 0u);
        hits[2 * i + 1] = make_uint4(0u, 0u, 0u, 0u);
    }
}
__global__ void math_kernel(int which, const float* x, uint64_t n, float* y) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float v = x[i], r = 0.0f, s, c;
    switch (which) {
        case 0: tsincos(v, &s, &c); r = s; break;
        case 1: tsincos(v, &s, &c); r = c; break;
        case 2: r = texp(v); break;
        case 3: r = tlog(v); break;
        case 4: r = tacos(v); break;
        default: r = 0.0f;
    }
    y[i] = r;
}

// ---------------------------------------------------------------- launchers
// Light records (see LIGHT_RECORD): the world vertices, area and normal of each emissive
// triangle with the operations sample_light applied per sample (instance transform of the
// dequantised positions, cross product of the edges), the material's constant emission and its
// emission-texture slots, so that a light sample reads one record instead of the triangle, its
// instance and its material in turn.  `sc` must hold the emissive triangles, instances,
// materials (texture masks in their padding) and light primitives.
__global__ void light_records_kernel(const __grid_constant__ DevScene sc, float4* rec, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const tt_emissive_triangle* tri = sc.emissive + i;
    uint32_t inst = tri->instance_index;
    const tt_instance* in = sc.instances + inst;
    float m[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) m[k] = in->transform[k];
    f3 p[3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
        p[k] = mat43_point(m, f3{dequant_snorm16(tri->positions[k][0]), dequant_snorm16(tri->positions[k][1]),
                                 dequant_snorm16(tri->positions[k][2])});
    f3 e = cross(p[1] - p[0], p[2] - p[0]);
    float area = fmx(0.00001f, 0.5f * length(e));
    f3 nrm = normalize(e);
    uint32_t mat = in->material_index;
    f3 em = material_emissive(sc.materials + mat);
    uint32_t mask = sc.materials[mat].padding & EMISSION_SLOTS;
    const uint32_t* tc = reinterpret_cast<const uint32_t*>(tri->texture_coordinates);
    float4* r = rec + (uint64_t)LIGHT_RECORD * i;
    r[0] = make_float4(p[0].x, p[0].y, p[0].z, area);
    r[1] = make_float4(p[1].x, p[1].y, p[1].z, __uint_as_float(inst));
    r[2] = make_float4(p[2].x, p[2].y, p[2].z, __uint_as_float((uint32_t)tri->hash));
    r[3] = make_float4(nrm.x, nrm.y, nrm.z, __uint_as_float(mask));
    r[4] = make_float4(em.x, em.y, em.z, __uint_as_float(mat));
    r[5] = make_float4(__uint_as_float(tc[0]), __uint_as_float(tc[1]), __uint_as_float(tc[2]),
                       __uint_as_float(sc.light_prim[i]));
}

void launch_light_records(const DevScene& sc, float4* rec, uint32_t n, cudaStream_t st) {
    if (n) light_records_kernel<<<(n + 255) / 256, 256, 0, st>>>(sc, rec, n);
}

void launch_integrate(const RenderParams& p, bool counted, cudaStream_t st) {
    dim3 grid((p.c.screen_size[0] + TILE_W - 1) / TILE_W, (p.c.screen_size[1] + TILE_H - 1) / TILE_H);
    dispatch_accel(p.sc, [&](auto accel) {
        constexpr int A = decltype(accel)::value;
        if (p.sc.textured) {
            if (counted) integrate_kernel<true, true, A><<<grid, BLOCK, 0, st>>>(p);
            else integrate_kernel<false, true, A><<<grid, BLOCK, 0, st>>>(p);
        } else {
            if (counted) integrate_kernel<true, false, A><<<grid, BLOCK, 0, st>>>(p);
            else integrate_kernel<false, false, A><<<grid, BLOCK, 0, st>>>(p);
        }
    });
}
void launch_tonemap(const float4* in, uint64_t n, uint32_t tonemap, uint32_t format, void* out, cudaStream_t st) {
    if (n == 0) return;
    tonemap_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(in, n, tonemap, format, out);
}
void launch_bsdf_eval(const MatC* m, const float4* s, uint32_t n, float4* r, cudaStream_t st) {
    if (n) bsdf_eval_kernel<<<(n + 127) / 128, 128, 0, st>>>(m, s, n, r);
}
void launch_bsdf_sample(const MatC* m, const float4* s, uint32_t n, float4* r, cudaStream_t st) {
    if (n) bsdf_sample_kernel<<<(n + 127) / 128, 128, 0, st>>>(m, s, n, r);
}
void launch_trace(const DevScene& sc, const float4* rays, uint32_t n, uint32_t flags, uint4* hits,
                  uint32_t* err, cudaStream_t st) {
    if (n)
        dispatch_accel(sc, [&](auto accel) {
            trace_kernel<decltype(accel)::value><<<(n + BLOCK - 1) / BLOCK, BLOCK, 0, st>>>(sc, rays, n, flags, hits, err);
        });
}
// textureLod of one texture at (u, v, lod) triples, for parity tests of the decoders and filter.
__global__ void texture_sample_kernel(DevScene sc, uint32_t index, const float* uvl, uint32_t n, float4* out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = sample_texture(sc, index, f2{uvl[3ull * i], uvl[3ull * i + 1]}, uvl[3ull * i + 2]);
}
void launch_texture_sample(const DevScene& sc, uint32_t index, const float* uvl, uint32_t n, float4* out,
                           cudaStream_t st) {
    if (n) texture_sample_kernel<<<(n + 127) / 128, 128, 0, st>>>(sc, index, uvl, n, out);
}

void launch_math(int which, const float* x, uint64_t n, float* y, cudaStream_t st) {
    if (n) math_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(which, x, n, y);
}


// ---------------------------------------------------------------- allocation-free ray queries
// tt_trace_batch_noalloc serves callers that cannot allocate device memory while they query
// rays (an application owning the device-memory budget, a frame loop that must not stall on
// an allocation's synchronisation).  Its staging lives in this file-scope array: the error
// word in the first 256 bytes, then TT_TRACE_NOALLOC_MAX_RAYS rays (32 bytes each), then as
// many hits (32 bytes each).  Every GPU that loads the library holds the array until exit;
// all calls share it, so calls whose GPU work overlaps race on it.
constexpr uint64_t NOALLOC_RAYS_OFFSET = 256;
constexpr uint64_t NOALLOC_HITS_OFFSET = NOALLOC_RAYS_OFFSET + 32ull * TT_TRACE_NOALLOC_MAX_RAYS;
constexpr uint64_t NOALLOC_BYTES = NOALLOC_HITS_OFFSET + 32ull * TT_TRACE_NOALLOC_MAX_RAYS;
static __device__ __align__(256) unsigned char g_trace_scratch[NOALLOC_BYTES];

// Device address of g_trace_scratch on `device`, looked up once per device with that device
// current (in host code the symbol itself is only a host-side stand-in).  The address is kept
// for the life of the process: a device reset (cudaDeviceReset by the application or another
// library) makes it stale, and tt_trace_batch_noalloc must not be called on that device again.
static unsigned char* trace_scratch_address(int device) {
    constexpr int MAX_DEVICES = 64;
    static std::mutex mutex;
    static void* address[MAX_DEVICES] = {};
    if (device < 0 || device >= MAX_DEVICES) fail(TT_ERR_INVALID_ARGUMENT, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(mutex);
    if (!address[device]) {
        void* p = nullptr;
        check_cuda(cudaGetSymbolAddress(&p, g_trace_scratch), "cudaGetSymbolAddress(g_trace_scratch)");
        address[device] = p;
    }
    return static_cast<unsigned char*>(address[device]);
}

void trace_batch_noalloc(int device, const DevScene& sc, const float* rays_host, uint32_t n,
                         uint32_t flags, uint32_t* hits_host, cudaStream_t st) {
    if (n > TT_TRACE_NOALLOC_MAX_RAYS)
        fail(TT_ERR_INVALID_ARGUMENT, "tt_trace_batch_noalloc: n exceeds TT_TRACE_NOALLOC_MAX_RAYS (" +
                                          std::to_string(TT_TRACE_NOALLOC_MAX_RAYS) + ")");
    unsigned char* base = trace_scratch_address(device);
    uint32_t* err = reinterpret_cast<uint32_t*>(base);
    float4* rays = reinterpret_cast<float4*>(base + NOALLOC_RAYS_OFFSET);
    uint4* hits = reinterpret_cast<uint4*>(base + NOALLOC_HITS_OFFSET);
    check_cuda(cudaMemsetAsync(err, 0, 4, st), "clear error word");
    if (n) check_cuda(cudaMemcpyAsync(rays, rays_host, 32ull * n, cudaMemcpyHostToDevice, st), "stage rays");
    launch_trace(sc, rays, n, flags, hits, err, st);
    check_cuda(cudaGetLastError(), "trace launch");
    uint32_t err_value = 0;
    if (n) check_cuda(cudaMemcpyAsync(hits_host, hits, 32ull * n, cudaMemcpyDeviceToHost, st), "read hits");
    check_cuda(cudaMemcpyAsync(&err_value, err, 4, cudaMemcpyDeviceToHost, st), "read error word");
    check_cuda(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    raise_device_error(err_value);
}

}  // namespace tt
