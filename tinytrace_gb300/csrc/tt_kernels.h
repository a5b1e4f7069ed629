// Kernel launch interface between the C ABI (api.cu) and the device code (integrate.cu).
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <type_traits>

#include "../../include/tinytrace_cuda.h"
#include "tt_bvh.cuh"

namespace tt {

// Calls f with the traversal variant of scene sc (ACCEL_*) as a compile-time constant.
template <class F>
inline void dispatch_accel(const DevScene& sc, F&& f) {
    if (sc.wide) f(std::integral_constant<int, ACCEL_WIDE_ONLY>{});
    else if (sc.flat) f(std::integral_constant<int, ACCEL_FLAT_ONLY>{});
    else f(std::integral_constant<int, ACCEL_TWO_LEVEL_ONLY>{});
}

struct RenderParams {
    DevScene sc;
    tt_constants c;
    float4* target;
    uint32_t* err;
    unsigned long long* counters;  // 6 counters, instrumented kernel only
};

// Wavefront integrator (wavefront.cu): device pointers of the slot pool and queues.
constexpr uint32_t HIT_BUCKETS = 4;                // shading queues, one per material bucket
static_assert(HIT_BUCKETS <= 4, "DevScene::bucket_lobes holds one byte per bucket");
constexpr uint32_t CACHE_QUEUE = 5 + HIT_BUCKETS;  // counters word: queued radiance-cache queries
constexpr uint32_t WF_CAMERA = 6 + HIT_BUCKETS;    // counters word: camera rays in the active queue
constexpr uint32_t WF_CONTINUING = 7 + HIT_BUCKETS;  // counters word: continuing paths in the active queue
constexpr uint32_t WF_PACKET_HEAD = 8 + HIT_BUCKETS;  // counters word: next camera ray of the packet phase
constexpr uint32_t WF_COUNTERS = 9 + HIT_BUCKETS;  // words cleared every iteration: [1, WF_COUNTERS)
constexpr uint32_t CTRL_RECORDS = 14;              // training records of the frame (cleared per frame)
constexpr uint32_t CTRL_ITERATION = 15;            // iteration count of the device-side loop
constexpr uint32_t CTRL_WORDS = 16;                // words of WfParams::counters
constexpr uint32_t CHUNK_WORDS = 14;               // words cleared per sample chunk: [0, CHUNK_WORDS)
static_assert(WF_COUNTERS <= CHUNK_WORDS && CHUNK_WORDS <= CTRL_RECORDS, "counter words overlap");

struct CacheQuery;
// A vertex of a training path: its query, the throughput arriving at it and the path radiance
// before its contributions (the training target is (final - before) / throughput).
struct TrainRecord {
    float q[12];
    float thr[3];
    float before[3];
    uint32_t path;  // training path id (global work item / stride)
    uint32_t pad;
};
struct WfParams {
    float4 *org, *dir, *thr, *acc, *pa1, *pa0, *pe;
    uint4* hit;          // shading queues: hit records, HIT_BUCKETS x P
    uint32_t* hslot;     // shading queues: slots, HIT_BUCKETS x P
    uint32_t* active;    // P entries: camera rays from the front, continuing paths from the back
    float4* shadow;
    uint32_t* counters;  // [0] next work item, [1] active paths, [2] shadow rays, [3]/[4] trace queue heads,
                         // [5 + b] length of shading queue b, [WF_CAMERA] / [WF_CONTINUING] the two parts
                         // of the active paths
    float4* samples;     // chunk_spp x WH per-sample radiance (band order)
    float4* running;     // WH running per-pixel sums across chunks
    uint32_t P, WH;
    uint32_t chunk_sample0, chunk_spp, chunk_items;
    XsJump chunk_jump;      // xor_shift advanced by 2 * chunk_sample0 draws
    uint32_t refill;        // a trace warp refills its idle lanes when fewer than this many hold a ray
    uint32_t trace_blocks;  // grid of the persistent trace kernel (host side)
    // learned radiance cache (cache_on = 0: off)
    uint32_t cache_on, cache_depth, train_stride, rec_cap;
    float cache_bound;      // positions map to the unit cube as p / bound * 0.5 + 0.5
    float spread_c;         // > 0: end paths by their spread (tt_cache_config.spread_threshold)
    float4* spread;         // per slot: spread sum, primary footprint a0, pdf of the last direction
    CacheQuery* cq;         // queued queries (P)
    uint32_t* cq_slot;      // their slots
    float* cq_out;          // their radiance (3 P)
    TrainRecord* rec;       // training records of the frame (rec_cap)
    float4* train_final;    // final radiance of each training path
    const __half* cache_grid;   // FP16 grid features (two per entry)
    const __half* cache_w16;
    // textured scenes: per slot, the primary ray's ndc (written by regen) and then the mip
    // level of the path (x, written at bounce 0); null without textures
    float2* ndc_mip;
    // rasterised primary visibility (primary.cu): the closest-hit key of every camera ray of the
    // chunk, indexed by work item; null, or *vis_ok == 0, when the camera rays are traversed
    const unsigned long long* vis;
    const uint32_t* vis_ok;
};
// SM count and resident blocks per SM of the persistent trace kernel.
void trace_occupancy(int* sms, int* blocks_per_sm);

// Shared-pool rendering of several requests (the render server): one round renders the next
// sample chunk of every request in the batch through one path pool.  The round's work items
// are the requests' chunk items laid end to end (request r owns [item_base, item_base +
// chunk_items)); a path slot carries its request in bits 16..23 of org.w (the bounce count
// keeps bits 0..15).  Each request keeps its own Constants, scene, per-sample radiance,
// running sums, image and error word, so its image is the one it gets rendered alone.
constexpr uint32_t BATCH_MAX_REQUESTS = 64;
constexpr uint32_t BATCH_BOUNCE_BITS = 16;
struct BatchRequest {
    tt_constants c;
    XsJump chunk_jump;   // xor_shift advanced by 2 * chunk_sample0 draws
    float4* samples;     // chunk_spp x WH per-sample radiance of the round's chunk (band order)
    float4* running;     // WH running per-pixel sums across chunks
    float4* target;      // WH image
    uint32_t* err;       // the request's ERR_* word
    uint32_t scene;      // index into the round's scene table
    uint32_t WH, item_base, pixel_base;
    uint32_t chunk_sample0, chunk_spp, chunk_items, last;  // last: the chunk ends the request
    // rasterised camera-ray keys of the request's chunk (indexed by its work item) and their ok
    // word; null when the request's camera rays are traversed
    const unsigned long long* vis;
    const uint32_t* vis_ok;
};
// Round header in device memory (read by the graph's kernels, so that one instantiated graph
// serves every round): request count, total work items, total pixels, iteration limit.
struct BatchRound {
    uint32_t nreq, items, pixels, limit;
    uint32_t keys;  // 1: every request of the round has complete camera-ray keys
};
struct BatchParams {
    const BatchRequest* reqs;  // BATCH_MAX_REQUESTS entries
    const DevScene* scenes;    // BATCH_MAX_REQUESTS entries
    const BatchRound* round;
};
// Instantiates the graph of one shared-pool round: while (paths are live) { regen, extend,
// shade, shadow }, then the per-request reductions.  `w` holds the pool (no radiance cache);
// `tex`: some scene of the batch samples textures (w.ndc_mip allocated); `structures`: the
// acceleration structures of the batch's scenes (BATCH_*: only their traversal steps are
// compiled into the trace kernel); `short_stack`: every scene needs at most
// SHORT_TRAVERSAL_STACK entries (not used with wide structures).  Launch it after the request
// table, the scene table and the round header are in place.
constexpr int BATCH_FLAT = 0, BATCH_NO_WIDE = 1, BATCH_ANY = 2;
cudaGraphExec_t build_batch_graph(const WfParams& w, const BatchParams& b, bool tex, int structures,
                                  bool short_stack, uint32_t* batch_err, cudaStream_t cs, cudaStream_t body_stream);
// Optional per-launch timing: a pair of CUDA events recorded on the launching stream around
// each integrator launch, tagged with its TT_STAGE_*.  `events` holds 2 * MAX_LAUNCHES events
// owned by the context; launches past MAX_LAUNCHES are not recorded (overflow).
struct StageTimer {
    static constexpr int MAX_LAUNCHES = 4096;
    cudaEvent_t* events = nullptr;
    uint8_t stage[MAX_LAUNCHES];
    int count = 0;
    bool overflow = false, open = false;
};
inline void stage_begin(StageTimer* t, int stage, cudaStream_t st) {
    if (!t) return;
    t->open = t->count < StageTimer::MAX_LAUNCHES;
    if (!t->open) {
        t->overflow = true;
        return;
    }
    t->stage[t->count] = (uint8_t)stage;
    cudaEventRecord(t->events[2 * t->count], st);
}
inline void stage_end(StageTimer* t, cudaStream_t st) {
    if (!t || !t->open) return;
    cudaEventRecord(t->events[2 * t->count + 1], st);
    t->count++;
    t->open = false;
}

// Primary visibility by rasterisation (primary.cu).  Every camera ray of a frame starts at the
// camera position, so the triangles it can hit are found the way a rasteriser finds them: each
// triangle record of a flat BVH4 scene is bounded on the screen (its projection, widened by a
// margin that covers the rounding of the camera rays and of the ray/triangle test, clipped
// where no camera ray can reach it, back faces dropped), and every sample of every pixel in that
// rectangle is tested against it with the traversal's own ray/triangle test.  The smallest
// (t, scene triangle index) key of each sample is its closest hit: the traversal's result, since
// that key orders hits exactly as the closest-hit rule does (smallest t, then the smaller
// (instance, primitive)).  The extension kernel then rebuilds each camera ray's hit from its key
// with one ray/triangle test instead of a traversal.
struct PrimaryInstance {
    float oo[3];     // the camera position in object space, as instance_ray computes it
    float ci[9];     // (object-from-world 3x3 * B)^-1, row-major: object-space offset -> lambda (ndc, 1)
    float margin;    // screen margin in pixels (rounding of the rays, the ray/triangle test and the bound)
    uint32_t ok;     // 0: no bound (the instance's records cover the whole screen)
    float pad[2];
};
struct PrimaryParams {
    unsigned long long* key;     // chunk_spp x WH keys (t bits << 32 | scene triangle index), ~0: no hit
    float4* rect;                // per record: pixel-position rectangle x0, y0, x1, y1 (x0 > x1: none)
    float4* edge;                // per record: 3 edge functions (a, b, c, 0); a sample at pixel position
                                 // (x, y) can hit the record only where a x + b y + c >= 0 for all three
    uint32_t* count;             // records + 1: pixels of each rectangle, then their exclusive prefix
    uint32_t* live_pos;          // records + 1: 1 per record with pixels, then their exclusive prefix
    uint32_t* live_rec;          // per record with pixels (in record order): its record
    uint32_t* live_first;        // per record with pixels: its first pair; then the total pairs
    unsigned long long* total;   // pixel-record pairs of the frame
    uint32_t* ok;                // 1 when the keys are complete (the extension kernel reads them)
    uint32_t* live_n;            // records with pixels
    uint32_t* next;              // first pair of the next range the key pass hands out
    PrimaryInstance* inst;       // per instance
    double B[9];                 // row-major: (ndc.x, ndc.y, 1) -> world direction of the camera ray
    double lambda_clip;          // no camera ray hits where lambda < lambda_clip
    double pixel_scale;          // pixels per radian of direction error, an upper bound
    uint32_t records;
    int sms;                     // multiprocessors (the key pass runs one wave of resident blocks)
};
// Camera terms of `c` for primary visibility; false when the camera's ray map is singular.
bool primary_camera(const tt_constants& c, PrimaryParams& v);
// Per frame, on `st`: instance bounds, record rectangles, their prefix and the ok flag.
void primary_setup(const RenderParams& p, const PrimaryParams& v, cudaStream_t st);
// Per sample chunk (w.chunk_sample0, w.chunk_spp, w.chunk_jump): clears and fills the keys.
void primary_chunk(const RenderParams& p, const PrimaryParams& v, const WfParams& w, cudaStream_t st);
// Shared-pool rounds: round->keys stays 1 only if every request's ok word is 1 (one thread).
void primary_round_keys(const BatchRequest* reqs, BatchRound* round, cudaStream_t st);

// Renders with the wavefront integrator; w.chunk_spp is the largest chunk of samples the
// buffers hold.  Synchronises `st` once per iteration to read the active-path count.  `prim`:
// rasterised primary visibility (w.vis points to its keys), or null.
void render_wavefront(const RenderParams& p, WfParams w, uint32_t* host_count, bool counted, cudaStream_t st,
                      StageTimer* timer, const PrimaryParams* prim);
// The same loop with no host synchronisation: each sample chunk's iterations run as a
// device-side while loop (a conditional node) of one CUDA graph, captured on `cs` and
// `body_stream` and launched on `st`.
void render_wavefront_graph(const RenderParams& p, WfParams w, bool counted, cudaStream_t st, cudaStream_t cs,
                            cudaStream_t body_stream, const PrimaryParams* prim);
void launch_integrate(const RenderParams& p, bool counted, cudaStream_t st);

// ReSTIR DI (restir.cu): the previous frame's camera and the frame's buffers.
struct RestirHistory {
    float camera_position[3];
    float view[16];          // column-major, as in tt_constants
    float inverse_proj[16];  // column-major
    uint32_t valid;          // 0: no previous frame (no temporal reuse)
};
struct Surface;
struct Reservoir;
constexpr int LOBE_RECORD = 6;  // float4 per pixel of RestirParams::glob
struct RestirParams {
    Surface *gbuf, *prev_gbuf;
    float4* gtex;  // textured scenes: per pixel (u, v, mip level, 0) of the primary hit; else null
    float4* glob;  // per pixel: the primary hit's prepared lobes (LOBE_RECORD float4)
    Reservoir *initial, *temporal, *final_out, *prev;
    // pixels whose camera ray hit a surface, one queue of pixel indices per material bucket
    // (HIT_BUCKETS x width * height) with its length in queue_count[bucket]; the candidate and
    // shade passes run over the queues laid end to end, so that a warp's pixels share a lobe set
    // (sky pixels are finished by the G-buffer pass)
    uint32_t* queue;
    uint32_t* queue_count;
    RestirHistory history;
    uint32_t candidates, neighbours;
    float m_cap, radius;
    // rasterised primary visibility of the frame's camera rays (one sample per pixel, keys in band
    // order); null, or *vis_ok == 0, when the G-buffer pass traces them
    const unsigned long long* vis;
    const uint32_t* vis_ok;
};
void render_restir(const RenderParams& p, const RestirParams& rp, cudaStream_t st, StageTimer* timer);
void launch_tonemap(const float4* in, uint64_t n, uint32_t tonemap, uint32_t format, void* out,
                    cudaStream_t st);
void launch_bsdf_eval(const tt_material_constants* m, const float4* samples, uint32_t n,
                      float4* results, cudaStream_t st);
void launch_bsdf_sample(const tt_material_constants* m, const float4* samples, uint32_t n,
                        float4* results, cudaStream_t st);
void launch_trace(const DevScene& sc, const float4* rays, uint32_t n, uint32_t flags, uint4* hits,
                  uint32_t* err, cudaStream_t st);
void launch_math(int which, const float* x, uint64_t n, float* y, cudaStream_t st);
void launch_light_records(const DevScene& sc, float4* rec, uint32_t n, cudaStream_t st);
void launch_texture_sample(const DevScene& sc, uint32_t index, const float* uvl, uint32_t n, float4* out,
                           cudaStream_t st);
// Ray queries staged in the library's static device array (no device allocation).
void trace_batch_noalloc(int device, const DevScene& sc, const float* rays_host, uint32_t n,
                         uint32_t flags, uint32_t* hits_host, cudaStream_t st);

}  // namespace tt
