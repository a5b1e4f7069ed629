// Wavefront path tracer for sm_103a: the same per-path computation as integrate_kernel
// (src/integrate/integrate.glsl), reorganised into stages over compacted queues so that the
// SIMT lanes of a warp always work on live paths.
//
// Work items are (pixel, sample) pairs.  A pool of P path slots holds paths in flight; each
// iteration runs
//   regen  (all slots): write finished paths' radiance to the per-sample buffer, give free
//                       slots the next work items (camera ray: the pixel generator advanced by
//                       2 draws per earlier sample, then the two jitter draws), and append the
//                       live slots to the active queue;
//   extend (active):    closest hit, back faces culled; a miss adds the sky and ends the path,
//                       a hit is appended to the shading queue;
//   shade  (hits):      hit reconstruction, bsdf_prepare, next-event estimation (light sample
//                       and its unoccluded contribution; the shadow ray goes to a queue),
//                       emission, bsdf_sample and the throughput update;
//   shadow (queue):     closest hit, light visibility, then the pending additions in the
//                       reference's order (direct light, then bounce-0 emission).
// A reduction sums each pixel's samples in sample order and applies the frame accumulation,
// so the image is bit-identical to the megakernel's and to the CPU oracle's.
//
// Slot state in HBM (structure of arrays, 16-byte records): origin + bounce, direction +
// generator, throughput + work item, path radiance + flags; pending NEE additions (3 x 16 B);
// shading queue (slot + 16-byte hit record); shadow queue entries (32 B).
#include <cuda_runtime.h>

#include <algorithm>

#include "tt_cache.cuh"
#include "tt_internal.h"
#include "tt_kernels.h"
#include "tt_shade.cuh"

namespace tt {

// Path flags (acc.w): live, terminated (radiance ready), training path of the radiance cache,
// waiting for its radiance-cache query.
constexpr uint32_t F_LIVE = 1u, F_TERM = 2u, F_TRAIN = 4u, F_CACHE = 8u;
constexpr uint32_t NO_HIT = 0xffffffffu;
constexpr int WF_BLOCK = 128;

__device__ __forceinline__ uint32_t lane_mask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}
// Warp-aggregated append: every lane of the warp must call it; lanes with `pred` get
// consecutive positions from one atomicAdd on `counter`.
__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, bool pred) {
    uint32_t mask = __ballot_sync(0xffffffffu, pred);
    if (mask == 0u) return 0u;
    int leader = __ffs(mask) - 1;
    uint32_t base = 0u;
    if ((int)(threadIdx.x & 31u) == leader) base = atomicAdd(counter, (uint32_t)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    return base + (uint32_t)__popc(mask & lane_mask_lt());
}

// Block-aggregated append: every thread of the block must call it; threads with `pred` get
// consecutive positions from one atomicAdd per block on `counter` (the position order
// inside the block is irrelevant to the results).  `s_warp` holds BLOCK / 32 + 1 words.
template <int BLOCK>
__device__ __forceinline__ uint32_t block_append(uint32_t* counter, bool pred, uint32_t* s_warp) {
    constexpr int WARPS = BLOCK / 32;
    uint32_t mask = __ballot_sync(0xffffffffu, pred);
    int warp = (int)(threadIdx.x >> 5), lane = (int)(threadIdx.x & 31u);
    if (lane == 0) s_warp[warp] = (uint32_t)__popc(mask);
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t sum = 0u;
        for (int k = 0; k < WARPS; ++k) {
            uint32_t c = s_warp[k];
            s_warp[k] = sum;
            sum += c;
        }
        s_warp[WARPS] = sum ? atomicAdd(counter, sum) : 0u;
    }
    __syncthreads();
    uint32_t pos = s_warp[WARPS] + s_warp[warp] + (uint32_t)__popc(mask & lane_mask_lt());
    __syncthreads();
    return pos;
}

// Block-aggregated append to the two parts of the active queue: threads with `camera` get
// positions from counters[WF_CAMERA] (the block's camera rays consecutive, in thread order),
// threads with `continuing` from counters[WF_CONTINUING]; counters[1] counts both.  One atomic
// per block and counter.  Every thread of the block must call it; `s_warp` holds
// 2 BLOCK / 32 + 3 words.
template <int BLOCK>
__device__ __forceinline__ uint32_t block_append_split(uint32_t* counters, bool camera, bool continuing,
                                                       uint32_t* s_warp) {
    constexpr int WARPS = BLOCK / 32;
    uint32_t ma = __ballot_sync(0xffffffffu, camera), mb = __ballot_sync(0xffffffffu, continuing);
    int warp = (int)(threadIdx.x >> 5), lane = (int)(threadIdx.x & 31u);
    if (lane == 0) {
        s_warp[warp] = (uint32_t)__popc(ma);
        s_warp[WARPS + warp] = (uint32_t)__popc(mb);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t sa = 0u, sb = 0u;
        for (int k = 0; k < WARPS; ++k) {
            uint32_t ca = s_warp[k], cb = s_warp[WARPS + k];
            s_warp[k] = sa;
            s_warp[WARPS + k] = sb;
            sa += ca;
            sb += cb;
        }
        s_warp[2 * WARPS] = sa ? atomicAdd(&counters[WF_CAMERA], sa) : 0u;
        s_warp[2 * WARPS + 1] = sb ? atomicAdd(&counters[WF_CONTINUING], sb) : 0u;
        if (sa + sb) atomicAdd(&counters[1], sa + sb);
    }
    __syncthreads();
    uint32_t below = lane_mask_lt();
    uint32_t pos = camera ? s_warp[2 * WARPS] + s_warp[warp] + (uint32_t)__popc(ma & below)
                          : s_warp[2 * WARPS + 1] + s_warp[WARPS + warp] + (uint32_t)__popc(mb & below);
    __syncthreads();
    return pos;
}

// Slot of active-queue entry i when the camera rays (n_camera of them, from the front) and the
// continuing paths (from the back) are taken as one sequence.
__device__ __forceinline__ uint32_t active_slot(const WfParams& w, uint32_t n_camera, uint32_t i) {
    return i < n_camera ? w.active[i] : w.active[w.P - 1u - (i - n_camera)];
}

// Pixel of band-ordered index t: bands of 8 rows, column-major inside a band, so a warp's 32
// consecutive items cover a 4 x 8 pixel block (coherent camera rays).
__device__ __forceinline__ void band_pixel(uint32_t t, uint32_t W, uint32_t H, uint32_t& x, uint32_t& y) {
    uint32_t band = t / (8u * W);
    uint32_t j = t - band * 8u * W;
    uint32_t rows = min(8u, H - 8u * band);
    x = j / rows;
    y = 8u * band + j % rows;
}

__device__ __forceinline__ f3 xyz(float4 v) { return f3{v.x, v.y, v.z}; }
__device__ __forceinline__ float4 pack(f3 v, uint32_t w) { return make_float4(v.x, v.y, v.z, __uint_as_float(w)); }

constexpr int REGEN_BLOCK = 512;

// M^(2 s) for s = 0..64: the generator of sample chunk_sample0 + s of a pixel is its seed
// advanced by chunk_jump and then by the entry of s (2 draws per earlier sample), 64 selects
// per path instead of 2 (chunk_sample0 + s) xor_shift steps.
struct XsJumpTable {
    XsJump m[65];
};
constexpr XsJumpTable xs_jump_table() {
    XsJumpTable t{};
    XsJump two = xs_power(2u);
    t.m[0] = xs_power(0u);
    for (int s = 1; s < 65; ++s) t.m[s] = xs_compose(two, t.m[s - 1]);
    return t;
}
__constant__ XsJumpTable c_xs_jump = xs_jump_table();

// The camera ray of sample chunk_sample0 + s_local of pixel t (band order) into slot s.
__device__ __forceinline__ void regen_path(const WfParams& w, const tt_constants& c, const XsJump& chunk_jump,
                                           uint32_t chunk_sample0, uint32_t WH, uint32_t item, uint32_t s,
                                           uint32_t org_w) {
    uint32_t W = c.screen_size[0], H = c.screen_size[1];
    uint32_t s_local = item / WH, t = item - s_local * WH;
    uint32_t x, y;
    band_pixel(t, W, H, x, y);
    uint32_t pg = jenkins_hash((x + y * W) ^ jenkins_hash(c.frame_index));
    if (chunk_sample0) pg = xs_apply(chunk_jump, pg);
    for (uint32_t r = s_local; r >= 64u; r -= 64u) pg = xs_apply(c_xs_jump.m[64], pg);  // chunks hold <= 64
    pg = xs_apply(c_xs_jump.m[s_local & 63u], pg);
    f2 ndc = pixel_ndc(x, y, W, H, pg);
    f3 d = camera_ray_direction(c, ndc);
    if (w.ndc_mip) w.ndc_mip[s] = make_float2(ndc.x, ndc.y);
    w.org[s] = make_float4(c.camera_position[0], c.camera_position[1], c.camera_position[2], __uint_as_float(org_w));
    w.dir[s] = pack(d, pg);
    w.thr[s] = pack(splat(1.0f), item);
}

// Index of the last of the n ascending `base` entries that is <= v (base[0] == 0 <= v).
__device__ __forceinline__ uint32_t last_at_most(const uint32_t* base, uint32_t n, uint32_t v) {
    uint32_t lo = 0u, hi = n;  // base[lo] <= v < base[hi] (base[n] = infinity)
    while (hi - lo > 1u) {
        uint32_t mid = (lo + hi) >> 1;
        if (base[mid] <= v) lo = mid;
        else hi = mid;
    }
    return lo;
}

// MULTI: a shared-pool round (BatchParams); the work items of every request of the round are
// drawn from one counter, and a finished path's radiance goes to its own request's buffer.
template <bool MULTI>
__global__ void __launch_bounds__(REGEN_BLOCK) wf_regen_kernel(const __grid_constant__ RenderParams p,
                                                               const __grid_constant__ WfParams w,
                                                               const __grid_constant__ BatchParams b) {
    __shared__ uint32_t s_warp[REGEN_BLOCK / 32 + 1];
    __shared__ uint32_t s_warp2[2 * (REGEN_BLOCK / 32) + 3];
    __shared__ uint32_t s_base[MULTI ? BATCH_MAX_REQUESTS : 1];
    __shared__ uint32_t s_next, s_nreq, s_total;
    uint32_t s = blockIdx.x * REGEN_BLOCK + threadIdx.x;
    bool valid = s < w.P;
    float4 a = valid ? w.acc[s] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    uint32_t flags = __float_as_uint(a.w);
    if (valid && (flags & F_TERM)) {
        uint32_t item = __float_as_uint(w.thr[s].w);
        if (MULTI) {
            uint32_t r = (__float_as_uint(w.org[s].w) >> BATCH_BOUNCE_BITS) & 0xffu;
            b.reqs[r].samples[item] = make_float4(a.x, a.y, a.z, 0.0f);
        } else {
            w.samples[item] = make_float4(a.x, a.y, a.z, 0.0f);
            if (flags & F_TRAIN)
                w.train_final[((uint64_t)w.chunk_sample0 * w.WH + item) / w.train_stride] =
                    make_float4(a.x, a.y, a.z, 0.0f);
        }
        flags = 0u;
        w.acc[s] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    bool live = valid && (flags & F_LIVE);
    // whether work items remain: one read of the shared counter per block (a stale value only
    // makes some free slots draw item numbers past the chunk, which they skip)
    if (threadIdx.x == 0) {
        s_next = *(volatile uint32_t*)&w.counters[0];
        if (MULTI) {
            s_nreq = b.round->nreq;
            s_total = b.round->items;
        }
    }
    if (MULTI && threadIdx.x < BATCH_MAX_REQUESTS) s_base[threadIdx.x] = b.reqs[threadIdx.x].item_base;
    __syncthreads();
    uint32_t total = MULTI ? s_total : w.chunk_items;
    bool need = valid && !live && s_next < total;
    uint32_t item = block_append<REGEN_BLOCK>(&w.counters[0], need, s_warp);
    bool fresh = need && item < total;
    if (fresh) {
        if (MULTI) {
            uint32_t r = last_at_most(s_base, s_nreq, item);
            const BatchRequest& R = b.reqs[r];
            regen_path(w, R.c, R.chunk_jump, R.chunk_sample0, R.WH, item - s_base[r], s, r << BATCH_BOUNCE_BITS);
            w.acc[s] = pack(splat(0.0f), F_LIVE);
        } else {
            regen_path(w, p.c, w.chunk_jump, w.chunk_sample0, w.WH, item, s, 0u);
            bool train = w.cache_on && ((uint64_t)w.chunk_sample0 * w.WH + item) % w.train_stride == 0u;
            if (w.cache_on) w.spread[s] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            w.acc[s] = pack(splat(0.0f), F_LIVE | (train ? F_TRAIN : 0u));
        }
        live = true;
    }
    // new camera rays to the front of the active queue, continuing paths to its back: trace warps
    // take runs of coherent camera rays (consecutive work items of neighbouring pixels) apart
    // from the scattered secondary rays
    uint32_t q = block_append_split<REGEN_BLOCK>(w.counters, fresh, live && !fresh, s_warp2);
    if (fresh) w.active[q] = s;
    else if (live) w.active[w.P - 1u - q] = s;
}

// Extension and shadow rays: persistent warps with per-lane refill.  Each lane traces one ray
// at a time; when fewer than w.refill lanes of a warp still have a ray, the idle lanes
// fetch new rays from the queue (one atomicAdd per warp), so warps keep their lanes busy
// instead of waiting for their longest ray (the dynamic fetch of Aila & Laine 2009).  Reserving
// queue items 32 at a time per warp (fewer atomics) measured slower: extension 81.4 -> 86.9 ms,
// shadow 16.6 -> 19.2 ms per frame of the 1080p benchmark.
#ifndef TT_TRACE_MIN_BLOCKS
#define TT_TRACE_MIN_BLOCKS 6
#endif
constexpr int TR_BLOCK = 128;

// The end of an extension ray (fin): a hit goes to the shading queue of its material bucket,
// so that the shade stage's warps share lobe sets; a miss adds the sky (integrate.glsl:272-276)
// and ends the path.  Every lane of the warp must call it.
__device__ __forceinline__ bool extension_result(const WfParams& w, const DevScene& sc, uint32_t slot, bool fin,
                                                 const Hit& h) {
    bool is_hit = fin && h.hit;
    uint32_t bucket = is_hit ? (uint32_t)__ldg(sc.inst_bucket + h.instance) : 0u;
    uint32_t pos = 0u;
#pragma unroll
    for (uint32_t b = 0; b < HIT_BUCKETS; ++b) {
        uint32_t pb = warp_append(&w.counters[5 + b], is_hit && bucket == b);
        pos = bucket == b ? pb : pos;
    }
    if (is_hit) {
        uint64_t at = (uint64_t)bucket * w.P + pos;
        w.hslot[at] = slot;
        w.hit[at] = make_uint4(__float_as_uint(h.u), __float_as_uint(h.v), h.instance, h.prim);
    } else if (fin) {
        f3 thr = xyz(w.thr[slot]);
        float4 a4 = w.acc[slot];
        f3 acc = xyz(a4);
        acc += splat(1.0f) * thr;
        w.acc[slot] = pack(acc, F_TERM | (__float_as_uint(a4.w) & F_TRAIN));
    }
    return is_hit;
}

// The closest hit of the camera ray in `slot` from the chunk's rasterised key of its work item.
__device__ __forceinline__ Hit primary_hit(const WfParams& w, const DevScene& sc, uint32_t slot, bool valid,
                                           uint32_t* err) {
    if (!valid) return primary_resolve(sc, ~0ull, splat(0.0f), splat(0.0f), err);
    return primary_resolve(sc, w.vis[__float_as_uint(w.thr[slot].w)], xyz(w.org[slot]), xyz(w.dir[slot]), err);
}

// MULTI: a shared-pool round; each lane traces in the scene of its ray's request and reports
// traversal errors to that request's error word.
// KEYS: the flat-BVH extension kernel of renders with rasterised camera-ray keys (no packet code).
template <bool COUNT, bool SHADOW, int ACCEL, int STACK = TRAVERSAL_STACK, bool MULTI = false, bool KEYS = false>
__global__ void __launch_bounds__(TR_BLOCK, TT_TRACE_MIN_BLOCKS) wf_trace_kernel(const __grid_constant__ RenderParams p,
                                                                const __grid_constant__ WfParams w,
                                                                const __grid_constant__ BatchParams b) {
    // CAMERA: the camera rays go first, 32 at a time per warp: from their rasterised closest hits
    // when the chunk has them (w.vis), else, in the uninstrumented kernel (PACKET), through the
    // warp-wide traversal of the flat BVH; the per-lane loop below then takes the continuing
    // paths only
    constexpr bool CAMERA = !SHADOW && ACCEL == ACCEL_FLAT_ONLY && (!MULTI || KEYS);
    constexpr bool PACKET = CAMERA && !COUNT && !KEYS;
    __shared__ uint32_t s_stack[STACK * TR_BLOCK];
    __shared__ uint2 s_packet[PACKET ? TR_BLOCK / 32 : 1][PACKET ? PACKET_STACK : 1];
    uint32_t* stack = s_stack + threadIdx.x;
    uint32_t lane_req = 0u, lane_scene = 0u;  // MULTI: request and scene of the lane's ray
#define TT_SC (MULTI ? b.scenes[lane_scene] : p.sc)
#define TT_ERR (MULTI ? b.reqs[lane_req].err : p.err)
    const uint32_t n_camera = SHADOW ? 0u : w.counters[WF_CAMERA];
    Counters cnt{0u, 0u, 0u, 0u};
    uint32_t rays = 0, hits = 0;
    const bool raster = CAMERA && (MULTI ? b.round->keys != 0u : w.vis != nullptr && *w.vis_ok != 0u);
    const bool camera_phase = raster || PACKET;
    if (CAMERA && camera_phase) {
        uint32_t* phead = &w.counters[WF_PACKET_HEAD];
        const uint32_t lane = threadIdx.x & 31u;
        while (true) {
            uint32_t base = 0u;
            if (lane == 0u) base = atomicAdd(phead, 32u);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base >= n_camera) break;
            uint32_t i = base + lane;
            bool valid = i < n_camera;
            uint32_t pslot = valid ? w.active[i] : 0u;
            Hit h{};
            if (MULTI && raster) {  // the key of the ray's request, indexed by its item in that request
                const uint32_t req = valid ? (__float_as_uint(w.org[pslot].w) >> BATCH_BOUNCE_BITS) & 0xffu : 0u;
                const BatchRequest& R = b.reqs[req];
                h = valid ? primary_resolve(b.scenes[R.scene], R.vis[__float_as_uint(w.thr[pslot].w)],
                                            xyz(w.org[pslot]), xyz(w.dir[pslot]), R.err)
                          : Hit{};
            } else if (raster) {
                h = primary_hit(w, p.sc, pslot, valid, p.err);
                if (COUNT && valid) {  // one record test and one object-ray set-up per hit
                    rays++;
                    cnt.triangles += h.hit ? 1u : 0u;
                    cnt.instances += h.hit ? 1u : 0u;
                }
            } else if constexpr (PACKET) {
                float4 o = valid ? w.org[pslot] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                float4 d = valid ? w.dir[pslot] : make_float4(0.0f, 0.0f, 1.0f, 0.0f);
                h = packet_trace_flat(p.sc, xyz(o), xyz(d), valid, EXTENSION_TMIN, EXTENSION_TMAX, true,
                                      s_packet[threadIdx.x >> 5], p.err);
            }
            if (MULTI) {
                const uint32_t req = valid ? (__float_as_uint(w.org[pslot].w) >> BATCH_BOUNCE_BITS) & 0xffu : 0u;
                extension_result(w, b.scenes[b.reqs[req].scene], pslot, valid, h);
            } else if (extension_result(w, p.sc, pslot, valid, h) && COUNT) {
                hits++;
            }
        }
    }
    // the per-lane loop's queue: shadow rays, or the active paths (camera rays, unless the camera
    // phase took them, then the continuing paths)
    const uint32_t skip = camera_phase ? n_camera : 0u;
    const uint32_t n = SHADOW ? w.counters[2] : w.counters[WF_CAMERA] + w.counters[WF_CONTINUING] - skip;
    uint32_t* head = &w.counters[SHADOW ? 4 : 3];
    TraceState st;
    uint32_t item = 0, slot = 0, light = 0, target_prim = 0;
    bool active = false;
    bool seeded = false;  // shadow ray seeded with its light triangle: any change of the closest hit occludes
    bool drained = false;  // warp-uniform: the queue has no more rays
    unsigned long long warp_steps = 0, lane_steps = 0;  // step-level lane occupancy (instrumented kernel)
    while (true) {
        if (!drained) {
            bool idle = !active;
            uint32_t mask = __ballot_sync(0xffffffffu, idle);
            if (mask) {
                int leader = __ffs(mask) - 1;
                uint32_t base = 0;
                if ((int)(threadIdx.x & 31u) == leader) base = atomicAdd(head, (uint32_t)__popc(mask));
                base = __shfl_sync(0xffffffffu, base, leader);
                uint32_t my = base + (uint32_t)__popc(mask & lane_mask_lt());
                if (idle && my < n) {
                    item = my;
                    float4 o, d;
                    uint32_t org_w;
                    if (SHADOW) {
                        o = w.shadow[2ull * item];
                        d = w.shadow[2ull * item + 1];
                        slot = __float_as_uint(o.w);
                        light = __float_as_uint(d.w);
                        org_w = MULTI ? __float_as_uint(w.org[slot].w) : 0u;
                    } else {
                        slot = active_slot(w, n_camera, skip + item);
                        o = w.org[slot];
                        d = w.dir[slot];
                        org_w = __float_as_uint(o.w);
                    }
                    if (MULTI) {
                        lane_req = (org_w >> BATCH_BOUNCE_BITS) & 0xffu;
                        lane_scene = b.reqs[lane_req].scene;
                    }
                    trace_init(st, TT_SC, xyz(o), xyz(d), SHADOW ? SHADOW_TMIN : EXTENSION_TMIN,
                               SHADOW ? SHADOW_TMAX : EXTENSION_TMAX, !SHADOW);
                    if (SHADOW) {
                        uint32_t hash = __float_as_uint(w.pa1[slot].w) >> 16;
                        uint32_t exact = __float_as_uint(w.pa0[slot].w);
                        int mode = shadow_target(TT_SC, light, hash, exact, xyz(o), xyz(d), SHADOW_TMIN, SHADOW_TMAX,
                                                 st.best, st.tbest);
                        if (mode == 0) trace_stop(st);  // not visible: the first step finishes
                        seeded = mode == 1;
                        target_prim = st.best.prim;
                    }
                    active = true;
                    if (COUNT) rays++;
                }
                drained = __any_sync(0xffffffffu, idle && my >= n);
            }
        }
        if (!__any_sync(0xffffffffu, active)) break;
        while (true) {
            bool fin = false;
            if (active && (trace_step<COUNT, ACCEL, SHADOW, STACK>(st, TT_SC, stack, TR_BLOCK, TT_ERR, cnt) ||
                           (SHADOW && seeded && (st.best.prim != target_prim || st.best.instance != light)))) {
                fin = true;
                active = false;
            }
            const Hit& h = st.best;
            if (SHADOW) {
                if (fin) {
                    float4 a1 = w.pa1[slot];
                    uint32_t pflags = __float_as_uint(a1.w);
                    float4 a0 = w.pa0[slot];
                    bool vis = light_visible(TT_SC, h, light, pflags >> 16, __float_as_uint(a0.w));
                    float4 a4 = w.acc[slot];
                    f3 acc = xyz(a4);
                    acc += vis ? xyz(a1) : xyz(a0);
                    if (pflags & 1u) acc += xyz(w.pe[slot]);
                    w.acc[slot] = make_float4(acc.x, acc.y, acc.z, a4.w);
                }
            } else {
                if (extension_result(w, TT_SC, slot, fin, h) && COUNT) hits++;
            }
            uint32_t am = __ballot_sync(0xffffffffu, active);
            if (COUNT && (threadIdx.x & 31u) == 0u) {
                warp_steps++;
                lane_steps += (uint32_t)__popc(am);
            }
            if (am == 0u || (!drained && (uint32_t)__popc(am) < w.refill)) break;
        }
    }
    if (COUNT) {
        unsigned long long v[8] = {rays, cnt.blas_nodes, cnt.tlas_nodes, cnt.triangles, cnt.instances, hits,
                                   warp_steps, lane_steps};
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            unsigned long long x = v[k];
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            if ((threadIdx.x & 31) == 0 && x) atomicAdd(p.counters + k, x);
        }
    }
}
#undef TT_SC
#undef TT_ERR

// 8 resident blocks (64 registers, 32 warps per SM): shade 20.6 -> 19.5 ms per 1080p frame against
// 6 blocks (80 registers), despite more spilling; 10 and 12 blocks gave 19.6 and 19.8 ms
#ifndef TT_SHADE_MIN_BLOCKS
#define TT_SHADE_MIN_BLOCKS 8
#endif
// What the shading of one hit leaves for the block's appends (shadow ray, cache query, training record).
struct ShadeOut {
    bool want_shadow = false, want_cache = false, want_record = false;
    uint32_t s = 0, light = 0;
    f3 sh_org = splat(0.0f), sh_dir = splat(0.0f);
    float qv[12];  // radiance-cache query of this vertex (cache or training record)
    f3 rec_thr = splat(0.0f), rec_before = splat(0.0f);
    uint32_t rec_path = 0;
};

// The shading of the hit at queue entry `at`, with the BSDF compiled for lobe set LS: every
// material of the hit's bucket has its lobe set within LS, so the result is the six-lobe code's.
template <bool CACHE, bool TEX, bool MULTI, uint32_t LS>
__device__ __forceinline__ void shade_hit(const RenderParams& p, const WfParams& w, const BatchParams& b, uint64_t at,
                                          ShadeOut& o) {
    uint32_t s = w.hslot[at];
    o.s = s;
    uint4 hv = w.hit[at];
    float4 o4 = w.org[s], d4 = w.dir[s], t4 = w.thr[s], a4 = w.acc[s];
    uint32_t ow = __float_as_uint(o4.w);
    uint32_t req = MULTI ? (ow >> BATCH_BOUNCE_BITS) & 0xffu : 0u;
    const tt_constants& c = MULTI ? b.reqs[req].c : p.c;
    const DevScene& sc = MULTI ? b.scenes[b.reqs[req].scene] : p.sc;
    f3 thr = xyz(t4), acc = xyz(a4), ray_dir = xyz(d4);
    uint32_t g = __float_as_uint(d4.w), bounce = MULTI ? ow & ((1u << BATCH_BOUNCE_BITS) - 1u) : ow;
    uint32_t train = __float_as_uint(a4.w) & F_TRAIN;
    ShadeHit hit = get_ray_hit(sc, hv.z, hv.w, __uint_as_float(hv.x), __uint_as_float(hv.y));
    float mip_level = 1.0f;
    if (TEX) {
        float2 nm = w.ndc_mip[s];
        if (bounce == 0u) {
            mip_level = primary_mip_level(c, hit, xyz(o4), f2{nm.x, nm.y});
            w.ndc_mip[s] = make_float2(mip_level, nm.y);
        } else {
            mip_level = nm.x;
        }
    }
    const tt_material* material = sc.materials + hit.material_index;
    MatC local;
    const MatC& mc = hit_material<TEX>(sc, material, hit.uv, mip_level, local);
    Basis basis = create_surface_basis(hit.tangent_space, col3(mc.geometry_normal));
    {
        if (CACHE) {
            float ib = 0.5f / w.cache_bound;
            o.qv[0] = hit.world_position.x * ib + 0.5f;
            o.qv[1] = hit.world_position.y * ib + 0.5f;
            o.qv[2] = hit.world_position.z * ib + 0.5f;
            o.qv[3] = -ray_dir.x;
            o.qv[4] = -ray_dir.y;
            o.qv[5] = -ray_dir.z;
            o.qv[6] = basis.normal.x;
            o.qv[7] = basis.normal.y;
            o.qv[8] = basis.normal.z;
            o.qv[9] = mc.specular_roughness;
            o.qv[10] = o.qv[11] = 0.0f;
            if (w.spread_c > 0.0f) {
                // path spread (neural radiance caching, Mueller et al. 2021, section 4):
                // a += sqrt(d^2 / (p |cos|)) per vertex after the first, a0 from a uniform
                // sphere pdf at the first; the path ends in the cache once a > c a0
                float4 sp = w.spread[s];
                f3 seg = hit.world_position - xyz(o4);
                float d2 = dot(seg, seg);
                float cs = fmaxf(fabsf(dot(basis.normal, ray_dir)), 1e-4f);
                if (bounce == 0u) sp.y = sqrtf(d2 / (4.0f * PI * cs));
                else sp.x += sqrtf(d2 / (fmaxf(sp.z, 1e-20f) * cs));
                w.spread[s] = sp;
                o.want_cache = !train && bounce >= w.cache_depth && sp.x > w.spread_c * sp.y;
            } else {
                o.want_cache = !train && bounce == w.cache_depth;
            }
            o.want_record = train != 0u;
            o.rec_thr = thr;
            o.rec_before = acc;
            o.rec_path = (uint32_t)(((uint64_t)w.chunk_sample0 * w.WH + __float_as_uint(t4.w)) / w.train_stride);
        }
    }
    if (o.want_cache) {  // the path ends in the cache: its radiance comes from the query
        w.acc[s] = pack(acc, F_CACHE);
    } else {
        f3 wi = transform_from_basis(basis, -ray_dir);
        Lobes lobes = bsdf_prepare<LS>(mc, wi, g);
        bool nee = c.light_sampling == LIGHT_SAMPLING_NEE && sc.emissive_count > 0 && mc.specular_roughness > 0.15f;
        f3 em = hit_emissive<TEX>(sc, material, hit.uv, mip_level);
        if (nee) {
            LightSample ls = sample_light(sc, hit.world_position, basis, g);
            f3 contrib = light_contribution<TEX, LS>(sc, ls, mc, lobes, wi);
            f3 a1 = thr * contrib, a0 = thr * splat(0.0f);
            // When the visible and the occluded update have the same bits (the light faces
            // away, or the BSDF is zero towards it) the shadow ray cannot change the result:
            // apply the update here, in the order the shadow stage would, and trace nothing.
            bool same = __float_as_uint(a1.x) == __float_as_uint(a0.x) &&
                        __float_as_uint(a1.y) == __float_as_uint(a0.y) &&
                        __float_as_uint(a1.z) == __float_as_uint(a0.z);
            if (same) {
                acc += a1;
                if (bounce == 0u) acc += em * thr;
            } else {
                uint32_t pflags = (bounce == 0u ? 1u : 0u) | (ls.hash << 16);
                w.pa1[s] = pack(a1, pflags);
                w.pa0[s] = pack(a0, ls.prim);
                w.pe[s] = pack(em * thr, 0u);
                o.want_shadow = true;
                o.light = ls.instance;
                o.sh_org = hit.world_position;
                o.sh_dir = ls.dir;
            }
        } else {
            acc += em * thr;
        }
        uint32_t next = bounce + 1u;
        if (next == c.bounce_count) {
            // last vertex: the continuation ray would never be traced, so its BSDF sample
            // (which changes only the generator and the throughput) is skipped
            w.acc[s] = pack(acc, F_TERM | train);
        } else {
            float density = 1.0f;
            f3 wo = splat(0.0f);
            int lobe = 0;
            f3 bsdf = bsdf_sample<LS>(mc, lobes, wi, g, wo, density, lobe);
            if (CACHE && w.spread_c > 0.0f) w.spread[s].z = density;
            f3 new_dir = transform_to_basis(basis, wo);
            thr *= bsdf / fmx(density, PDF_EPSILON) * fabsf(cos_theta(wo));
            w.org[s] = pack(hit.world_position, MULTI ? next | (req << BATCH_BOUNCE_BITS) : next);
            w.dir[s] = pack(new_dir, g);
            w.thr[s] = pack(thr, __float_as_uint(t4.w));
            w.acc[s] = pack(acc, F_LIVE | train);
        }
    }
}

// MULTI: a shared-pool round; each path shades with its request's Constants and scene.
// Single-request, untextured scenes: each bucket's queue starts on a block boundary, so a block
// shades one bucket, and the block runs the shading compiled for the smallest lobe set covering
// the bucket's materials (opaque dielectric, fully metallic, the two, or all six lobes).  The
// variants leave out the code of lobes that carry no weight, and the registers it needs.
// Textured materials can take metalness or transmission from a texel; they and shared-pool
// rounds (whose buckets mix the requests' scenes) shade with all six lobes.
template <bool CACHE, bool TEX, bool MULTI = false>
__global__ void __launch_bounds__(WF_BLOCK, TT_SHADE_MIN_BLOCKS) wf_shade_kernel(const __grid_constant__ RenderParams p,
                                                            const __grid_constant__ WfParams w,
                                                            const __grid_constant__ BatchParams b) {
    constexpr bool VARIANTS = !TEX && !MULTI;
    // thread q shades entry q of the bucket queues laid end to end (VARIANTS: each queue padded
    // to a multiple of the block)
    uint32_t q = blockIdx.x * WF_BLOCK + threadIdx.x;
    uint64_t at = 0;
    uint32_t start = 0, bucket = HIT_BUCKETS;
    bool have = false;
#pragma unroll
    for (uint32_t k = 0; k < HIT_BUCKETS; ++k) {
        uint32_t cnt = w.counters[5 + k];
        uint32_t span = VARIANTS ? (cnt + WF_BLOCK - 1u) / WF_BLOCK * WF_BLOCK : cnt;
        bool in = !have && q >= start && q < start + cnt;
        bucket = bucket == HIT_BUCKETS && q >= start && q < start + span ? k : bucket;
        at = in ? (uint64_t)k * w.P + (q - start) : at;
        have = have || in;
        start += span;
    }
    ShadeOut o;
    if (VARIANTS) {
        uint32_t ls = bucket < HIT_BUCKETS ? (p.sc.bucket_lobes >> (8u * bucket)) & LOBE_SET_ALL : LOBE_SET_ALL;
        if (!have) {
        } else if ((ls & ~LOBE_SET_METAL) == 0u) {
            shade_hit<CACHE, TEX, MULTI, LOBE_SET_METAL>(p, w, b, at, o);
        } else if ((ls & ~LOBE_SET_DIELECTRIC) == 0u) {
            shade_hit<CACHE, TEX, MULTI, LOBE_SET_DIELECTRIC>(p, w, b, at, o);
        } else if ((ls & ~LOBE_SET_BASE) == 0u) {
            shade_hit<CACHE, TEX, MULTI, LOBE_SET_BASE>(p, w, b, at, o);
        } else {
            shade_hit<CACHE, TEX, MULTI, LOBE_SET_ALL>(p, w, b, at, o);
        }
    } else if (have) {
        shade_hit<CACHE, TEX, MULTI, LOBE_SET_ALL>(p, w, b, at, o);
    }
    const bool want_shadow = o.want_shadow, want_cache = o.want_cache, want_record = o.want_record;
    const uint32_t s = o.s, light = o.light, rec_path = o.rec_path;
    const f3 sh_org = o.sh_org, sh_dir = o.sh_dir, rec_thr = o.rec_thr, rec_before = o.rec_before;
    const float* qv = o.qv;
    __shared__ uint32_t s_warp[WF_BLOCK / 32 + 1];
    uint32_t e = block_append<WF_BLOCK>(&w.counters[2], want_shadow, s_warp);
    if (want_shadow) {
        w.shadow[2ull * e] = pack(sh_org, s);
        w.shadow[2ull * e + 1] = pack(sh_dir, light);
    }
    if (CACHE) {
        uint32_t cq = block_append<WF_BLOCK>(&w.counters[CACHE_QUEUE], want_cache, s_warp);
        if (want_cache) {
            float4* dst = reinterpret_cast<float4*>(w.cq) + 3ull * cq;
            dst[0] = make_float4(qv[0], qv[1], qv[2], qv[3]);
            dst[1] = make_float4(qv[4], qv[5], qv[6], qv[7]);
            dst[2] = make_float4(qv[8], qv[9], qv[10], qv[11]);
            w.cq_slot[cq] = s;
        }
        uint32_t r = block_append<WF_BLOCK>(&w.counters[CTRL_RECORDS], want_record, s_warp);
        if (want_record && r < w.rec_cap) {
            float4* dst = reinterpret_cast<float4*>(w.rec + r);
            dst[0] = make_float4(qv[0], qv[1], qv[2], qv[3]);
            dst[1] = make_float4(qv[4], qv[5], qv[6], qv[7]);
            dst[2] = make_float4(qv[8], qv[9], qv[10], qv[11]);
            dst[3] = make_float4(rec_thr.x, rec_thr.y, rec_thr.z, rec_before.x);
            dst[4] = make_float4(rec_before.y, rec_before.z, __uint_as_float(rec_path), 0.0f);
        }
    }
}

// Radiance-cache results of this iteration's queued paths: acc += throughput * max(L, 0).
__global__ void wf_cache_apply_kernel(const __grid_constant__ WfParams w) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.counters[CACHE_QUEUE]) return;
    uint32_t s = w.cq_slot[i];
    f3 L = f3{fmaxf(w.cq_out[3ull * i], 0.0f), fmaxf(w.cq_out[3ull * i + 1], 0.0f), fmaxf(w.cq_out[3ull * i + 2], 0.0f)};
    f3 acc = xyz(w.acc[s]) + xyz(w.thr[s]) * L;
    w.acc[s] = pack(acc, F_TERM);
}

// Per pixel: samples of this chunk added in sample order to the running sum; after the last
// chunk, divide by the sample count and apply the frame accumulation (integrate.glsl:338-346).
__device__ __forceinline__ void reduce_pixel(const tt_constants& c, uint32_t WH, uint32_t chunk_sample0,
                                             uint32_t chunk_spp, const float4* samples, float4* running,
                                             float4* target, bool last, uint32_t t) {
    f3 acc = chunk_sample0 == 0u ? splat(0.0f) : xyz(running[t]);
    for (uint32_t sl = 0; sl < chunk_spp; ++sl) acc += xyz(samples[(uint64_t)sl * WH + t]);
    if (!last) {
        running[t] = make_float4(acc.x, acc.y, acc.z, 0.0f);
        return;
    }
    uint32_t x, y;
    band_pixel(t, c.screen_size[0], c.screen_size[1], x, y);
    acc = acc / (float)c.sample_count;
    float4* tp = target + (uint64_t)y * c.screen_size[0] + x;
    if (c.accumulated_frame_count != 0) {
        float4 prev = *tp;
        acc = (xyz(prev) * (float)(c.accumulated_frame_count - 1u) + acc) / (float)c.accumulated_frame_count;
    }
    *tp = make_float4(acc.x, acc.y, acc.z, 1.0f);
}

__global__ void wf_reduce_kernel(const __grid_constant__ RenderParams p, const __grid_constant__ WfParams w,
                                 int last) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= w.WH) return;
    reduce_pixel(p.c, w.WH, w.chunk_sample0, w.chunk_spp, w.samples, w.running, p.target, last != 0, t);
}

// The reductions of a shared-pool round: the requests' pixels laid end to end (request r owns
// [pixel_base, pixel_base + WH)), grid-stride over all of them.
__global__ void __launch_bounds__(256) wf_reduce_batch_kernel(const __grid_constant__ BatchParams b) {
    __shared__ uint32_t s_base[BATCH_MAX_REQUESTS];
    if (threadIdx.x < BATCH_MAX_REQUESTS) s_base[threadIdx.x] = b.reqs[threadIdx.x].pixel_base;
    __syncthreads();
    uint32_t nreq = b.round->nreq, total = b.round->pixels;
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
        uint32_t r = last_at_most(s_base, nreq, g);
        const BatchRequest& R = b.reqs[r];
        reduce_pixel(R.c, R.WH, R.chunk_sample0, R.chunk_spp, R.samples, R.running, R.target, R.last != 0u,
                     g - s_base[r]);
    }
}

template <bool SHADOW>
// The short-stack kernels serve scenes whose structure needs at most SHORT_TRAVERSAL_STACK
// entries (measured on the 1080p benchmark: 1169 -> 1184 Msamples/s); the instrumented
// kernels always use the full stack.
static void launch_trace(const RenderParams& p, const WfParams& w, unsigned grid, bool counted, cudaStream_t st) {
    bool short_stack = !counted && p.sc.stack_need <= (uint32_t)SHORT_TRAVERSAL_STACK;
    if (p.sc.wide) {
        if (counted) wf_trace_kernel<true, SHADOW, ACCEL_WIDE_ONLY><<<grid, TR_BLOCK, 0, st>>>(p, w, BatchParams{});
        else if (short_stack)
            wf_trace_kernel<false, SHADOW, ACCEL_WIDE_ONLY, SHORT_TRAVERSAL_STACK><<<grid, TR_BLOCK, 0, st>>>(p, w, BatchParams{});
        else wf_trace_kernel<false, SHADOW, ACCEL_WIDE_ONLY><<<grid, TR_BLOCK, 0, st>>>(p, w, BatchParams{});
    } else if (p.sc.flat) {
        if (counted) wf_trace_kernel<true, SHADOW, ACCEL_FLAT_ONLY><<<grid, TR_BLOCK, 0, st>>>(p, w, BatchParams{});
        else if (!SHADOW && w.vis && short_stack)
            wf_trace_kernel<false, SHADOW, ACCEL_FLAT_ONLY, SHORT_TRAVERSAL_STACK, false, true>
                <<<grid, TR_BLOCK, 0, st>>>(p, w, BatchParams{});
        else if (!SHADOW && w.vis)
            wf_trace_kernel<false, SHADOW, ACCEL_FLAT_ONLY, TRAVERSAL_STACK, false, true><<<grid, TR_BLOCK, 0, st>>>(p, w, BatchParams{});
        else if (short_stack)
            wf_trace_kernel<false, SHADOW, ACCEL_FLAT_ONLY, SHORT_TRAVERSAL_STACK><<<grid, TR_BLOCK, 0, st>>>(p, w, BatchParams{});
        else wf_trace_kernel<false, SHADOW, ACCEL_FLAT_ONLY><<<grid, TR_BLOCK, 0, st>>>(p, w, BatchParams{});
    } else {
        if (counted) wf_trace_kernel<true, SHADOW, ACCEL_TWO_LEVEL_ONLY><<<grid, TR_BLOCK, 0, st>>>(p, w, BatchParams{});
        else if (short_stack)
            wf_trace_kernel<false, SHADOW, ACCEL_TWO_LEVEL_ONLY, SHORT_TRAVERSAL_STACK><<<grid, TR_BLOCK, 0, st>>>(p, w, BatchParams{});
        else wf_trace_kernel<false, SHADOW, ACCEL_TWO_LEVEL_ONLY><<<grid, TR_BLOCK, 0, st>>>(p, w, BatchParams{});
    }
}

// `grid` covers the hits; each bucket's queue can be padded to a block boundary (one more block each).
static void launch_shade(const RenderParams& p, const WfParams& w, unsigned grid, cudaStream_t st) {
    bool tex = p.sc.textured != 0u;
    grid += HIT_BUCKETS;
    if (w.cache_on) {
        if (tex) wf_shade_kernel<true, true><<<grid, WF_BLOCK, 0, st>>>(p, w, BatchParams{});
        else wf_shade_kernel<true, false><<<grid, WF_BLOCK, 0, st>>>(p, w, BatchParams{});
    } else {
        if (tex) wf_shade_kernel<false, true><<<grid, WF_BLOCK, 0, st>>>(p, w, BatchParams{});
        else wf_shade_kernel<false, false><<<grid, WF_BLOCK, 0, st>>>(p, w, BatchParams{});
    }
}

// Device-side loop control: counts the chunk's iterations and keeps the graph's while loop
// running while paths are live, for at most `limit` iterations (then ERR_ITERATION_LIMIT).
__global__ void wf_control_kernel(uint32_t* counters, cudaGraphConditionalHandle handle, uint32_t limit,
                                  uint32_t* err) {
    uint32_t n = counters[1];
    uint32_t it = ++counters[CTRL_ITERATION];
    bool more = n > 0u && it < limit;
    if (n > 0u && it >= limit) atomicOr(err, ERR_ITERATION_LIMIT);
    cudaGraphSetConditional(handle, more ? 1u : 0u);
}

// The same control for a shared-pool round, whose iteration limit is in the round header.
__global__ void wf_control_batch_kernel(uint32_t* counters, cudaGraphConditionalHandle handle,
                                        const BatchRound* round, uint32_t* err) {
    uint32_t n = counters[1];
    uint32_t it = ++counters[CTRL_ITERATION];
    uint32_t limit = round->limit;
    bool more = n > 0u && it < limit;
    if (n > 0u && it >= limit) atomicOr(err, ERR_ITERATION_LIMIT);
    cudaGraphSetConditional(handle, more ? 1u : 0u);
}

void trace_occupancy(int* sms, int* blocks_per_sm) {
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    check_cuda(cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, dev), "sm count");
    check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, wf_trace_kernel<false, false, ACCEL_FLAT_ONLY>,
                                                             TR_BLOCK, 0),
               "occupancy");
}

void render_wavefront_graph(const RenderParams& p, WfParams w, bool counted, cudaStream_t st, cudaStream_t cs,
                            cudaStream_t body_stream, const PrimaryParams* prim) {
    const tt_constants& c = p.c;
    uint32_t WH = c.screen_size[0] * c.screen_size[1];
    uint32_t spp = c.sample_count;
    uint32_t max_chunk = w.chunk_spp;
    w.WH = WH;
    unsigned regen_grid = (w.P + REGEN_BLOCK - 1) / REGEN_BLOCK;
    unsigned shade_grid = (w.P + WF_BLOCK - 1) / WF_BLOCK;
    unsigned tgrid = w.trace_blocks;
    cudaGraph_t g = nullptr;
    check_cuda(cudaGraphCreate(&g, 0), "cudaGraphCreate");
    check_cuda(cudaStreamBeginCaptureToGraph(cs, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed), "capture");
    check_cuda(cudaMemsetAsync(w.acc, 0, 16ull * w.P, cs), "memset");  // every slot starts free
    check_cuda(cudaMemsetAsync(w.counters + CTRL_RECORDS, 0, 4, cs), "memset");
    for (uint32_t s0 = 0; s0 < spp; s0 += max_chunk) {
        w.chunk_sample0 = s0;
        w.chunk_jump = xs_power(2ull * s0);
        w.chunk_spp = std::min(max_chunk, spp - s0);
        w.chunk_items = WH * w.chunk_spp;
        check_cuda(cudaMemsetAsync(w.counters, 0, 4ull * CHUNK_WORDS, cs), "memset");
        check_cuda(cudaMemsetAsync(w.counters + CTRL_ITERATION, 0, 4, cs), "memset");
        if (prim) primary_chunk(p, *prim, w, cs);
        // while (paths are live) { regen; extend; shade; shadow }
        cudaStreamCaptureStatus status;
        cudaGraph_t cg = nullptr;
        const cudaGraphNode_t* deps = nullptr;
        size_t ndeps = 0;
        check_cuda(cudaStreamGetCaptureInfo(cs, &status, nullptr, &cg, &deps, nullptr, &ndeps), "capture info");
        cudaGraphConditionalHandle handle;
        check_cuda(cudaGraphConditionalHandleCreate(&handle, cg, 1u, cudaGraphCondAssignDefault), "conditional handle");
        cudaGraphNodeParams cp{};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = handle;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t loop;
        check_cuda(cudaGraphAddNode(&loop, cg, deps, nullptr, ndeps, &cp), "conditional node");
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        check_cuda(cudaStreamBeginCaptureToGraph(body_stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed),
                   "body capture");
        uint64_t rounds = (uint64_t)w.chunk_items / w.P + 1u;
        uint32_t limit = (uint32_t)std::min<uint64_t>(2ull * rounds * (c.bounce_count + 2u) + 16u, 0x7fffffffu);
        check_cuda(cudaMemsetAsync(w.counters + 1, 0, 4ull * (WF_COUNTERS - 1), body_stream), "memset");
        wf_regen_kernel<false><<<regen_grid, REGEN_BLOCK, 0, body_stream>>>(p, w, BatchParams{});
        wf_control_kernel<<<1, 1, 0, body_stream>>>(w.counters, handle, limit, p.err);
        launch_trace<false>(p, w, tgrid, counted, body_stream);
        launch_shade(p, w, shade_grid, body_stream);
        launch_trace<true>(p, w, tgrid, counted, body_stream);
        if (w.cache_on) {
            cache_infer_queue(w.cache_grid, w.cache_w16, w.cq, w.counters + CACHE_QUEUE, w.P, w.cq_out, p.err,
                              body_stream);
            wf_cache_apply_kernel<<<(w.P + 255) / 256, 256, 0, body_stream>>>(w);
        }
        check_cuda(cudaStreamEndCapture(body_stream, &body), "body capture end");
        check_cuda(cudaStreamUpdateCaptureDependencies(cs, &loop, nullptr, 1, cudaStreamSetCaptureDependencies),
                   "capture dependencies");
        wf_reduce_kernel<<<(WH + 255) / 256, 256, 0, cs>>>(p, w, s0 + w.chunk_spp >= spp ? 1 : 0);
    }
    check_cuda(cudaStreamEndCapture(cs, &g), "capture end");
    cudaGraphExec_t exec = nullptr;
    cudaError_t e = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    check_cuda(e, "cudaGraphInstantiate");
    e = cudaGraphLaunch(exec, st);
    cudaGraphExecDestroy(exec);  // freed when the launch completes
    check_cuda(e, "cudaGraphLaunch");
}

template <int ACCEL, int STACK>
static cudaGraphExec_t batch_graph(const WfParams& w, const BatchParams& b, bool tex, uint32_t* batch_err,
                                   cudaStream_t cs, cudaStream_t body_stream) {
    RenderParams p{};  // the shared-pool kernels read only its batch error word
    p.err = batch_err;
    unsigned regen_grid = (w.P + REGEN_BLOCK - 1) / REGEN_BLOCK;
    unsigned shade_grid = (w.P + WF_BLOCK - 1) / WF_BLOCK;
    int sms = 0, dev = 0, ext_per_sm = 0, shadow_per_sm = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "sm count");
    auto ext = wf_trace_kernel<false, false, ACCEL, STACK, true, ACCEL == ACCEL_FLAT_ONLY>;
    auto shadow = wf_trace_kernel<false, true, ACCEL, STACK, true>;
    check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ext_per_sm, ext, TR_BLOCK, 0), "occupancy");
    check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&shadow_per_sm, shadow, TR_BLOCK, 0), "occupancy");
    unsigned ext_grid = (unsigned)std::max(1, sms * ext_per_sm), shadow_grid = (unsigned)std::max(1, sms * shadow_per_sm);
    cudaGraph_t g = nullptr;
    check_cuda(cudaGraphCreate(&g, 0), "cudaGraphCreate");
    check_cuda(cudaStreamBeginCaptureToGraph(cs, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed), "capture");
    check_cuda(cudaMemsetAsync(w.acc, 0, 16ull * w.P, cs), "memset");  // every slot starts free
    check_cuda(cudaMemsetAsync(w.counters, 0, 4ull * CTRL_WORDS, cs), "memset");
    cudaStreamCaptureStatus status;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    check_cuda(cudaStreamGetCaptureInfo(cs, &status, nullptr, &cg, &deps, nullptr, &ndeps), "capture info");
    cudaGraphConditionalHandle handle;
    check_cuda(cudaGraphConditionalHandleCreate(&handle, cg, 1u, cudaGraphCondAssignDefault), "conditional handle");
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = handle;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t loop;
    check_cuda(cudaGraphAddNode(&loop, cg, deps, nullptr, ndeps, &cp), "conditional node");
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    check_cuda(cudaStreamBeginCaptureToGraph(body_stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed),
               "body capture");
    check_cuda(cudaMemsetAsync(w.counters + 1, 0, 4ull * (WF_COUNTERS - 1), body_stream), "memset");
    wf_regen_kernel<true><<<regen_grid, REGEN_BLOCK, 0, body_stream>>>(p, w, b);
    wf_control_batch_kernel<<<1, 1, 0, body_stream>>>(w.counters, handle, b.round, batch_err);
    ext<<<ext_grid, TR_BLOCK, 0, body_stream>>>(p, w, b);
    if (tex) wf_shade_kernel<false, true, true><<<shade_grid, WF_BLOCK, 0, body_stream>>>(p, w, b);
    else wf_shade_kernel<false, false, true><<<shade_grid, WF_BLOCK, 0, body_stream>>>(p, w, b);
    shadow<<<shadow_grid, TR_BLOCK, 0, body_stream>>>(p, w, b);
    check_cuda(cudaStreamEndCapture(body_stream, &body), "body capture end");
    check_cuda(cudaStreamUpdateCaptureDependencies(cs, &loop, nullptr, 1, cudaStreamSetCaptureDependencies),
               "capture dependencies");
    wf_reduce_batch_kernel<<<(unsigned)(4 * sms), 256, 0, cs>>>(b);
    check_cuda(cudaStreamEndCapture(cs, &g), "capture end");
    cudaGraphExec_t exec = nullptr;
    cudaError_t e = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    check_cuda(e, "cudaGraphInstantiate");
    return exec;
}

cudaGraphExec_t build_batch_graph(const WfParams& w, const BatchParams& b, bool tex, int structures,
                                  bool short_stack, uint32_t* batch_err, cudaStream_t cs, cudaStream_t body_stream) {
    if (structures == BATCH_FLAT)
        return short_stack ? batch_graph<ACCEL_FLAT_ONLY, SHORT_TRAVERSAL_STACK>(w, b, tex, batch_err, cs, body_stream)
                           : batch_graph<ACCEL_FLAT_ONLY, TRAVERSAL_STACK>(w, b, tex, batch_err, cs, body_stream);
    if (structures == BATCH_NO_WIDE)
        return short_stack ? batch_graph<ACCEL_NO_WIDE, SHORT_TRAVERSAL_STACK>(w, b, tex, batch_err, cs, body_stream)
                           : batch_graph<ACCEL_NO_WIDE, TRAVERSAL_STACK>(w, b, tex, batch_err, cs, body_stream);
    return batch_graph<ACCEL_ANY, TRAVERSAL_STACK>(w, b, tex, batch_err, cs, body_stream);
}

void render_wavefront(const RenderParams& p, WfParams w, uint32_t* host_count, bool counted, cudaStream_t st,
                      StageTimer* timer, const PrimaryParams* prim) {
    const tt_constants& c = p.c;
    uint32_t WH = c.screen_size[0] * c.screen_size[1];
    uint32_t spp = c.sample_count;
    uint32_t max_chunk = w.chunk_spp;
    w.WH = WH;
    unsigned regen_grid = (w.P + REGEN_BLOCK - 1) / REGEN_BLOCK;
    unsigned trace_blocks = w.trace_blocks;
    check_cuda(cudaMemsetAsync(w.acc, 0, 16ull * w.P, st), "memset");  // every slot starts free
    check_cuda(cudaMemsetAsync(w.counters + CTRL_RECORDS, 0, 4, st), "memset");
    for (uint32_t s0 = 0; s0 < spp; s0 += max_chunk) {
        w.chunk_sample0 = s0;
        w.chunk_jump = xs_power(2ull * s0);
        w.chunk_spp = std::min(max_chunk, spp - s0);
        w.chunk_items = WH * w.chunk_spp;
        check_cuda(cudaMemsetAsync(w.counters, 0, 4ull * CHUNK_WORDS, st), "memset");
        if (prim) {
            stage_begin(timer, TT_STAGE_PRIMARY, st);
            primary_chunk(p, *prim, w, st);
            stage_end(timer, st);
        }
        while (true) {
            check_cuda(cudaMemsetAsync(w.counters + 1, 0, 4ull * (WF_COUNTERS - 1), st), "memset");
            stage_begin(timer, TT_STAGE_REGEN, st);
            wf_regen_kernel<false><<<regen_grid, REGEN_BLOCK, 0, st>>>(p, w, BatchParams{});
            stage_end(timer, st);
            check_cuda(cudaMemcpyAsync(host_count, w.counters + 1, 4, cudaMemcpyDeviceToHost, st), "count");
            check_cuda(cudaStreamSynchronize(st), "sync");
            uint32_t n = *host_count;
            if (n == 0) break;
            unsigned grid = (n + WF_BLOCK - 1) / WF_BLOCK;
            unsigned tgrid = std::min<unsigned>(trace_blocks, (n + TR_BLOCK - 1) / TR_BLOCK);
            stage_begin(timer, TT_STAGE_EXTEND, st);
            launch_trace<false>(p, w, tgrid, counted, st);
            stage_end(timer, st);
            stage_begin(timer, TT_STAGE_SHADE, st);
            launch_shade(p, w, grid, st);
            stage_end(timer, st);
            stage_begin(timer, TT_STAGE_SHADOW, st);
            launch_trace<true>(p, w, tgrid, counted, st);
            stage_end(timer, st);
            if (w.cache_on) {
                stage_begin(timer, TT_STAGE_CACHE, st);
                cache_infer_queue(w.cache_grid, w.cache_w16, w.cq, w.counters + CACHE_QUEUE, n, w.cq_out, p.err, st);
                wf_cache_apply_kernel<<<grid, WF_BLOCK, 0, st>>>(w);
                stage_end(timer, st);
            }
        }
        stage_begin(timer, TT_STAGE_REDUCE, st);
        wf_reduce_kernel<<<(WH + 255) / 256, 256, 0, st>>>(p, w, s0 + w.chunk_spp >= spp ? 1 : 0);
        stage_end(timer, st);
    }
}

}  // namespace tt
