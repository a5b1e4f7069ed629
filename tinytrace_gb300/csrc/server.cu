// Continuous-batching render server (tt_server_*): requests of any scene, resolution and
// sample count share one wavefront path pool and one set of persistent kernels.
//
// The scheduler thread works in rounds.  A round takes the next sample chunk of the admitted
// requests (up to round_items work items in total, capped at 64 samples per pixel per request:
// split evenly across the requests under the fair policy, given to the requests with the least
// remaining work first under the smallest-first policy), lays the chunks end to end as the work items of one shared-pool
// wavefront loop (regen, extend, shade, shadow in a device-side while loop) and finishes with
// the per-request reductions; the whole round is one launch of a CUDA graph instantiated once
// per server.  Between rounds the scheduler retires finished requests (their images are copied
// out while the next round runs) and admits queued ones (in arrival order, or the smallest
// first) while the batch has room and their device memory fits in the HBM budget, so requests
// that arrive while others render join the batch at the next round boundary.
//
// Per request the device holds one stream-ordered arena (allocated from a server-owned memory
// pool): the per-sample radiance of its largest chunk, the running pixel sums, the image and
// its error word; the admission test uses the arena's exact size.  A path carries its request
// in its slot state, and every kernel reads that request's Constants, scene and buffers, so a
// request's image is the same, bit for bit, alone or among others (the reduction adds each
// pixel's samples in sample order whatever the chunking).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "tt_internal.h"
#include "tt_kernels.h"

namespace tt {
DevScene scene_view(tt_context* ctx, tt_handle scene);
int context_device(tt_context* ctx);
bool context_primary_raster(tt_context* ctx);
}  // namespace tt

using namespace tt;
using Clock = std::chrono::steady_clock;

namespace {

constexpr uint64_t DEFAULT_BUDGET = 150ull << 30;
constexpr uint32_t DEFAULT_INFLIGHT = 16;
constexpr uint32_t DEFAULT_PATHS = 1u << 21;
constexpr uint64_t DEFAULT_ROUND_ITEMS = 1ull << 26;
constexpr uint32_t MAX_CHUNK_SPP = 64;
constexpr uint64_t MAX_PIXELS = 1ull << 24;  // per request: 4096 x 4096

uint64_t align256(uint64_t b) { return (b + 255u) / 256u * 256u; }

struct Request {
    uint64_t id = 0;
    DevScene sc{};
    tt_constants c{};
    float* host = nullptr;
    uint64_t bytes = 0, arena_bytes = 0, WH = 0;
    uint32_t chunk_cap = 0;  // samples per pixel the arena's per-sample buffer holds
    uint32_t done_spp = 0;
    Clock::time_point submitted, finished;
    int32_t status = TT_REQUEST_QUEUED;
    std::string error;
    // device arena: samples (chunk_cap x WH), running sums, image, error word
    char* arena = nullptr;
    float4 *samples = nullptr, *running = nullptr, *target = nullptr;
    uint32_t* err = nullptr;
    // this round
    uint32_t chunk_spp = 0;
    bool last = false;
};

// A pinned host buffer the image of a finished request is copied into during its last round.
struct Staging {
    float* ptr = nullptr;
    uint64_t bytes = 0;
};

}  // namespace

struct tt_server {
    int device = 0;
    tt_context* ctx = nullptr;
    uint64_t budget = DEFAULT_BUDGET, round_items = DEFAULT_ROUND_ITEMS;
    uint32_t max_live = DEFAULT_INFLIGHT, paths = DEFAULT_PATHS, policy = TT_SERVER_POLICY_FAIR;
    cudaStream_t stream = nullptr, capture = nullptr, body = nullptr;
    cudaEvent_t round_start = nullptr, round_done = nullptr;
    cudaMemPool_t pool = nullptr;
    // the shared path pool and the round tables (device), their pinned host mirrors
    DeviceBuffer org, dir, thr, acc, pa1, pa0, pe, hit, hslot, active, shadow, counters, ndc_mip;
    DeviceBuffer d_reqs, d_scenes, d_round, d_batch_err;
    // rasterised camera-ray keys of flat-BVH4 rounds: one key per work item of the round, and the
    // per-request bound buffers (reused request after request) with per-request total/ok words
    DeviceBuffer keys, prim_rect, prim_edge, prim_count, prim_live_pos, prim_live_rec, prim_live_first, prim_inst,
        prim_flags;
    uint64_t key_items = 0, prim_records = 0, prim_instances = 0;
    int occupancy_sms = 0;
    bool primary = true;  // the context's TT_OPTION_PRIMARY_VISIBILITY at creation is TT_PRIMARY_RASTER
    BatchRequest* h_reqs = nullptr;
    DevScene* h_scenes = nullptr;
    BatchRound* h_round = nullptr;
    uint32_t* h_err = nullptr;  // BATCH_MAX_REQUESTS request error words + the batch word
    WfParams w{};
    cudaGraphExec_t graph[2][3][2] = {};  // [texture sampling][BATCH_* structures][short stacks]
    std::vector<Staging> staging_free;
    uint64_t round_items_now = 0;
    uint32_t round_n = 0;  // requests in the last round: live[0 .. round_n)

    std::mutex mu;
    std::condition_variable cv;       // submissions and stop (scheduler side)
    std::condition_variable done_cv;  // completions (waiter side)
    std::deque<Request*> queue;
    std::map<uint64_t, std::unique_ptr<Request>> requests;
    uint64_t next_id = 1;
    bool stop = false;
    tt_server_stats stats{};
    std::thread worker;

    void create_pool();
    void admit(std::vector<Request*>& live);
    void launch_round(std::vector<Request*>& live);
    Staging take_staging(uint64_t bytes);
    void retire(Request* r, int32_t status, const std::string& error);
    void run();
};

void tt_server::create_pool() {
    uint64_t P = (paths + 127u) / 128u * 128u;
    org.alloc(16 * P);
    dir.alloc(16 * P);
    thr.alloc(16 * P);
    acc.alloc(16 * P);
    pa1.alloc(16 * P);
    pa0.alloc(16 * P);
    pe.alloc(16 * P);
    hit.alloc(16ull * HIT_BUCKETS * P);
    hslot.alloc(4ull * HIT_BUCKETS * P);
    active.alloc(4 * P);
    shadow.alloc(32 * P);
    counters.alloc(4ull * CTRL_WORDS);
    ndc_mip.alloc(8 * P);
    d_reqs.alloc(sizeof(BatchRequest) * BATCH_MAX_REQUESTS);
    d_scenes.alloc(sizeof(DevScene) * BATCH_MAX_REQUESTS);
    d_round.alloc(sizeof(BatchRound));
    d_batch_err.alloc(256);
    check_cuda(cudaMemset(d_reqs.ptr, 0, d_reqs.bytes), "memset");
    check_cuda(cudaMemset(d_scenes.ptr, 0, d_scenes.bytes), "memset");
    check_cuda(cudaMallocHost((void**)&h_reqs, sizeof(BatchRequest) * BATCH_MAX_REQUESTS), "cudaMallocHost");
    check_cuda(cudaMallocHost((void**)&h_scenes, sizeof(DevScene) * BATCH_MAX_REQUESTS), "cudaMallocHost");
    check_cuda(cudaMallocHost((void**)&h_round, sizeof(BatchRound)), "cudaMallocHost");
    check_cuda(cudaMallocHost((void**)&h_err, 4ull * (BATCH_MAX_REQUESTS + 1)), "cudaMallocHost");
    std::memset(h_reqs, 0, sizeof(BatchRequest) * BATCH_MAX_REQUESTS);
    w = WfParams{};
    w.org = org.as<float4>();
    w.dir = dir.as<float4>();
    w.thr = thr.as<float4>();
    w.acc = acc.as<float4>();
    w.pa1 = pa1.as<float4>();
    w.pa0 = pa0.as<float4>();
    w.pe = pe.as<float4>();
    w.hit = hit.as<uint4>();
    w.hslot = hslot.as<uint32_t>();
    w.active = active.as<uint32_t>();
    w.shadow = shadow.as<float4>();
    w.counters = counters.as<uint32_t>();
    w.ndc_mip = ndc_mip.as<float2>();
    w.P = (uint32_t)P;
    w.refill = 20;
}

Staging tt_server::take_staging(uint64_t bytes) {
    for (size_t k = 0; k < staging_free.size(); ++k)
        if (staging_free[k].bytes >= bytes) {
            Staging s = staging_free[k];
            staging_free.erase(staging_free.begin() + (long)k);
            return s;
        }
    Staging s;
    check_cuda(cudaMallocHost((void**)&s.ptr, bytes), "cudaMallocHost");
    s.bytes = bytes;
    return s;
}

// Final status of r; frees its arena (stream-ordered after the work already enqueued).
void tt_server::retire(Request* r, int32_t status, const std::string& error) {
    if (r->arena) cudaFreeAsync(r->arena, stream);
    r->arena = nullptr;
    std::lock_guard<std::mutex> lk(mu);
    r->finished = Clock::now();
    r->status = status;
    r->error = error;
    stats.inflight--;
    stats.bytes_in_flight -= r->arena_bytes;
    if (status == TT_REQUEST_DONE) stats.completed++;
    else stats.failed++;
    done_cv.notify_all();
}

// Moves queued requests into the batch in arrival order while it has room and the budget allows.
void tt_server::admit(std::vector<Request*>& live) {
    std::vector<Request*> in;
    {
        std::lock_guard<std::mutex> lk(mu);
        while (!queue.empty()) {
            auto pick = queue.begin();
            if (policy == TT_SERVER_POLICY_SMALLEST_FIRST)  // fewest samples, then arrival order
                pick = std::min_element(queue.begin(), queue.end(), [](const Request* a, const Request* b) {
                    uint64_t sa = a->WH * a->c.sample_count, sb = b->WH * b->c.sample_count;
                    return sa != sb ? sa < sb : a->id < b->id;
                });
            Request* head = *pick;
            if (head->arena_bytes > budget) {  // can never fit
                queue.erase(pick);
                head->status = TT_REQUEST_FAILED;
                head->error = "request needs more device memory than the HBM budget";
                head->finished = Clock::now();
                stats.queued--;
                stats.failed++;
                done_cv.notify_all();
                continue;
            }
            if (live.size() + in.size() >= max_live || stats.bytes_in_flight + head->arena_bytes > budget) break;
            queue.erase(pick);
            head->status = TT_REQUEST_RUNNING;
            stats.queued--;
            stats.inflight++;
            stats.bytes_in_flight += head->arena_bytes;
            stats.peak_inflight = std::max(stats.peak_inflight, stats.inflight);
            stats.peak_bytes_in_flight = std::max(stats.peak_bytes_in_flight, stats.bytes_in_flight);
            in.push_back(head);
        }
    }
    for (Request* r : in) {
        try {
            check_cuda(cudaMallocFromPoolAsync((void**)&r->arena, r->arena_bytes, pool, stream), "arena");
            uint64_t at = 0;
            r->samples = reinterpret_cast<float4*>(r->arena + at);
            at += align256(16ull * r->chunk_cap * r->WH);
            r->running = reinterpret_cast<float4*>(r->arena + at);
            at += align256(16ull * r->WH);
            r->target = reinterpret_cast<float4*>(r->arena + at);
            at += align256(16ull * r->WH);
            r->err = reinterpret_cast<uint32_t*>(r->arena + at);
            check_cuda(cudaMemsetAsync(r->err, 0, 4, stream), "memset");
            live.push_back(r);
        } catch (const Error& e) {
            retire(r, TT_REQUEST_FAILED, e.message);
        }
    }
}

// Enqueues one round: picks each request's chunk by the policy (the round serves live[0 ..
// round_n)), uploads the request table, the scene table and the round header, launches the
// graph and reads the error words back; run() adds the image copies of the requests whose last
// chunk this is.
void tt_server::launch_round(std::vector<Request*>& live) {
    uint32_t n = (uint32_t)live.size();
    if (policy == TT_SERVER_POLICY_SMALLEST_FIRST) {
        // the oldest request first, with up to a quarter of the round's items (so the largest
        // requests keep progressing), then least remaining work first: full chunks until the
        // round's items are spent; the requests left out wait, after the served ones in `live`
        auto oldest = std::min_element(live.begin(), live.end(), [](const Request* a, const Request* b) {
            return a->id < b->id;
        });
        std::iter_swap(live.begin(), oldest);
        std::stable_sort(live.begin() + 1, live.end(), [](const Request* a, const Request* b) {
            return a->WH * (a->c.sample_count - a->done_spp) < b->WH * (b->c.sample_count - b->done_spp);
        });
        uint64_t room = round_items;
        uint32_t served = 0;
        for (Request* r : live) {
            uint32_t left = r->c.sample_count - r->done_spp;
            uint64_t fit = (served == 0 ? round_items / 4u : room) / r->WH;
            uint32_t spp = (uint32_t)std::min<uint64_t>(std::min(r->chunk_cap, left), served == 0 ? std::max<uint64_t>(fit, 1) : fit);
            r->chunk_spp = spp;
            if (spp == 0) break;
            room -= std::min<uint64_t>(room, (uint64_t)spp * r->WH);
            ++served;
        }
        n = served;
    } else {
        uint64_t share = std::max<uint64_t>(1, round_items / n);
        for (Request* r : live) {
            uint32_t left = r->c.sample_count - r->done_spp;
            uint32_t fair = (uint32_t)std::max<uint64_t>(1, share / r->WH);
            r->chunk_spp = std::min({r->chunk_cap, left, fair});
        }
    }
    round_n = n;
    uint64_t items = 0, pixels = 0;
    uint32_t max_bounce = 1;
    bool tex = false, wide = false, two_level = false, short_stack = true;
    for (uint32_t k = 0; k < n; ++k) {
        Request& r = *live[k];
        uint32_t left = r.c.sample_count - r.done_spp;
        r.last = r.chunk_spp == left;
        BatchRequest& b = h_reqs[k];
        b.c = r.c;
        b.chunk_jump = xs_power(2ull * r.done_spp);
        b.samples = r.samples;
        b.running = r.running;
        b.target = r.target;
        b.err = r.err;
        b.scene = k;
        b.WH = (uint32_t)r.WH;
        b.item_base = (uint32_t)items;
        b.pixel_base = (uint32_t)pixels;
        b.chunk_sample0 = r.done_spp;
        b.chunk_spp = r.chunk_spp;
        b.chunk_items = (uint32_t)(r.WH * r.chunk_spp);
        b.last = r.last ? 1u : 0u;
        h_scenes[k] = r.sc;
        items += b.chunk_items;
        pixels += r.WH;
        max_bounce = std::max(max_bounce, r.c.bounce_count);
        tex = tex || r.sc.textured != 0u;
        wide = wide || r.sc.wide != 0u;
        two_level = two_level || r.sc.flat == 0u;
        short_stack = short_stack && r.sc.stack_need <= (uint32_t)SHORT_TRAVERSAL_STACK;
    }
    h_round->nreq = n;
    h_round->items = (uint32_t)items;
    h_round->pixels = (uint32_t)pixels;
    h_round->limit = (uint32_t)std::min<uint64_t>(2ull * (items / w.P + 1u) * (max_bounce + 2u) + 16u, 0x7fffffffu);
    round_items_now = items;
    BatchParams bp{d_reqs.as<BatchRequest>(), d_scenes.as<DevScene>(), d_round.as<BatchRound>()};
    int structures = wide ? BATCH_ANY : (two_level ? BATCH_NO_WIDE : BATCH_FLAT);
    short_stack = short_stack && !wide;
    cudaGraphExec_t& g = graph[tex ? 1 : 0][structures][short_stack ? 1 : 0];
    if (!g) g = build_batch_graph(w, bp, tex, structures, short_stack, d_batch_err.as<uint32_t>(), capture, body);
    check_cuda(cudaEventRecord(round_start, stream), "event");
    // flat-BVH4 rounds: each request's camera-ray keys for its chunk, at its items in the round
    h_round->keys = 0u;
    if (structures == BATCH_FLAT && primary) {
        uint64_t recs = 0, insts = 0;
        for (uint32_t k = 0; k < n; ++k) {
            recs = std::max<uint64_t>(recs, live[k]->sc.tri_count);
            insts = std::max<uint64_t>(insts, live[k]->sc.instance_count);
        }
        if (items > key_items) {
            keys.alloc(8ull * items);
            key_items = items;
        }
        if (recs + 1 > prim_records) {
            prim_rect.alloc(16ull * recs);
            prim_edge.alloc(48ull * recs);
            prim_count.alloc(4ull * (recs + 1));
            prim_live_pos.alloc(4ull * (recs + 1));
            prim_live_rec.alloc(4ull * recs);
            prim_live_first.alloc(4ull * (recs + 1));
            prim_records = recs + 1;
        }
        if (insts > prim_instances) {
            prim_inst.alloc(sizeof(PrimaryInstance) * insts);
            prim_instances = insts;
        }
        if (!prim_flags.ptr) prim_flags.alloc(32ull * BATCH_MAX_REQUESTS);
        if (occupancy_sms == 0)
            check_cuda(cudaDeviceGetAttribute(&occupancy_sms, cudaDevAttrMultiProcessorCount, device), "sm count");
        bool all = n > 0;
        for (uint32_t k = 0; k < n; ++k) {
            Request& r = *live[k];
            BatchRequest& b = h_reqs[k];
            PrimaryParams v{};
            if (!(r.sc.tri_record && r.sc.tri_count > 0 && primary_camera(r.c, v))) {
                b.vis = nullptr;
                b.vis_ok = nullptr;
                all = false;
                continue;
            }
            v.key = keys.as<unsigned long long>() + b.item_base;
            v.rect = prim_rect.as<float4>();
            v.edge = prim_edge.as<float4>();
            v.count = prim_count.as<uint32_t>();
            v.live_pos = prim_live_pos.as<uint32_t>();
            v.live_rec = prim_live_rec.as<uint32_t>();
            v.live_first = prim_live_first.as<uint32_t>();
            v.total = reinterpret_cast<unsigned long long*>(prim_flags.as<unsigned char>() + 32ull * k);
            v.ok = reinterpret_cast<uint32_t*>(prim_flags.as<unsigned char>() + 32ull * k + 8);
            v.live_n = reinterpret_cast<uint32_t*>(prim_flags.as<unsigned char>() + 32ull * k + 12);
            v.next = reinterpret_cast<uint32_t*>(prim_flags.as<unsigned char>() + 32ull * k + 16);
            v.inst = prim_inst.as<PrimaryInstance>();
            v.records = r.sc.tri_count;
            v.sms = std::max(1, occupancy_sms);
            RenderParams rp{};
            rp.sc = r.sc;
            rp.c = r.c;
            WfParams chunk{};
            chunk.chunk_sample0 = b.chunk_sample0;
            chunk.chunk_spp = b.chunk_spp;
            chunk.chunk_jump = b.chunk_jump;
            primary_setup(rp, v, stream);
            primary_chunk(rp, v, chunk, stream);
            b.vis = v.key;
            b.vis_ok = v.ok;
        }
        h_round->keys = all ? 1u : 0u;
    } else {
        for (uint32_t k = 0; k < n; ++k) {
            h_reqs[k].vis = nullptr;
            h_reqs[k].vis_ok = nullptr;
        }
    }
    check_cuda(cudaMemcpyAsync(d_reqs.ptr, h_reqs, sizeof(BatchRequest) * n, cudaMemcpyHostToDevice, stream), "table");
    check_cuda(cudaMemcpyAsync(d_scenes.ptr, h_scenes, sizeof(DevScene) * n, cudaMemcpyHostToDevice, stream), "scenes");
    check_cuda(cudaMemcpyAsync(d_round.ptr, h_round, sizeof(BatchRound), cudaMemcpyHostToDevice, stream), "round");
    if (h_round->keys) primary_round_keys(d_reqs.as<BatchRequest>(), d_round.as<BatchRound>(), stream);
    check_cuda(cudaMemsetAsync(d_batch_err.ptr, 0, 4, stream), "memset");
    check_cuda(cudaGraphLaunch(g, stream), "cudaGraphLaunch");
    for (uint32_t k = 0; k < n; ++k)
        check_cuda(cudaMemcpyAsync(h_err + k, live[k]->err, 4, cudaMemcpyDeviceToHost, stream), "error word");
    check_cuda(cudaMemcpyAsync(h_err + BATCH_MAX_REQUESTS, d_batch_err.ptr, 4, cudaMemcpyDeviceToHost, stream),
               "error word");
}

void tt_server::run() {
    cudaSetDevice(device);
    std::vector<Request*> live;
    // finished requests of the previous round: image in pinned staging, copied out while the
    // next round renders
    std::vector<std::pair<Request*, Staging>> copy_out;
    auto ns_since = [](Clock::time_point t0) {
        return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(Clock::now() - t0).count();
    };
    uint64_t t_admit = 0, t_launch = 0, t_copy = 0, t_wait = 0, busy = 0;
    while (true) {
        Clock::time_point t0 = Clock::now();
        try {
            admit(live);
        } catch (const Error&) {
        }
        t_admit += ns_since(t0);
        t0 = Clock::now();
        bool launched = false;
        std::vector<std::pair<Request*, Staging>> finishing;
        if (!live.empty()) {
            try {
                launch_round(live);
                for (uint32_t k = 0; k < round_n; ++k)
                    if (Request* r = live[k]; r->last) {
                        Staging s = take_staging(r->bytes);
                        check_cuda(cudaMemcpyAsync(s.ptr, r->target, r->bytes, cudaMemcpyDeviceToHost, stream),
                                   "image");
                        finishing.emplace_back(r, s);
                    }
                check_cuda(cudaEventRecord(round_done, stream), "event");
                launched = true;
            } catch (const Error& e) {
                for (auto& f : finishing) staging_free.push_back(f.second);
                finishing.clear();
                cudaStreamSynchronize(stream);
                for (Request* r : live) retire(r, TT_REQUEST_FAILED, e.message);
                live.clear();
            }
        }
        t_launch += ns_since(t0);
        t0 = Clock::now();
        for (auto& [r, s] : copy_out) {
            std::memcpy(r->host, s.ptr, r->bytes);
            staging_free.push_back(s);
            retire(r, TT_REQUEST_DONE, "");
        }
        copy_out.clear();
        t_copy += ns_since(t0);
        if (launched) {
            t0 = Clock::now();
            cudaError_t q = cudaEventSynchronize(round_done);
            t_wait += ns_since(t0);
            float ms = 0.0f;
            if (q == cudaSuccess && cudaEventElapsedTime(&ms, round_start, round_done) == cudaSuccess)
                busy += (uint64_t)((double)ms * 1e6);
            {
                std::lock_guard<std::mutex> lk(mu);
                stats.rounds++;
                stats.round_items += round_items_now;
                stats.gpu_busy_ns = busy;
                stats.admit_ns = t_admit;
                stats.launch_ns = t_launch;
                stats.copy_out_ns = t_copy;
                stats.wait_ns = t_wait;
            }
            uint32_t batch_err = q == cudaSuccess ? h_err[BATCH_MAX_REQUESTS] : 0u;
            std::vector<Request*> still;
            for (size_t k = 0; k < live.size(); ++k) {
                Request* r = live[k];
                if (k >= round_n) {  // not served this round
                    still.push_back(r);
                    continue;
                }
                std::string error;
                if (q != cudaSuccess) error = std::string("device error: ") + cudaGetErrorString(q);
                else if (batch_err & ERR_ITERATION_LIMIT) error = "iteration limit reached";
                else if (h_err[k] & ERR_STACK_OVERFLOW) error = "traversal stack overflow";
                else if (h_err[k] & ERR_ITERATION_LIMIT) error = "iteration limit reached";
                auto f = std::find_if(finishing.begin(), finishing.end(), [&](auto& e) { return e.first == r; });
                if (!error.empty()) {
                    if (f != finishing.end()) {
                        staging_free.push_back(f->second);
                        finishing.erase(f);
                    }
                    retire(r, TT_REQUEST_FAILED, error);
                    continue;
                }
                r->done_spp += r->chunk_spp;
                if (f == finishing.end()) still.push_back(r);
                else if (r->arena) {
                    cudaFreeAsync(r->arena, stream);  // the image is in staging
                    r->arena = nullptr;
                }
            }
            live.swap(still);
            copy_out.swap(finishing);
            continue;
        }
        std::unique_lock<std::mutex> lk(mu);
        if (copy_out.empty() && live.empty()) {
            if (stop && queue.empty()) break;
            if (queue.empty()) cv.wait_for(lk, std::chrono::milliseconds(2));
        }
    }
}

namespace {
template <class F>
int32_t server_guarded(F&& f) {
    try {
        f();
        return TT_OK;
    } catch (const Error& e) {
        set_last_error(e.message);
        return e.code;
    } catch (const std::bad_alloc&) {
        set_last_error("host allocation failed");
        return TT_ERR_OOM;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return TT_ERR_DEVICE;
    }
}
void need(bool cond, const char* msg) {
    if (!cond) fail(TT_ERR_INVALID_ARGUMENT, msg);
}
uint64_t arena_bytes(uint64_t WH, uint32_t chunk_cap) {
    return align256(16ull * chunk_cap * WH) + 2 * align256(16ull * WH) + 256u;
}
}  // namespace

extern "C" {

int32_t tt_server_create(tt_context* ctx, const tt_server_config* config, tt_server** out) {
    return server_guarded([&] {
        need(ctx && out, "null argument");
        auto srv = std::make_unique<tt_server>();
        srv->ctx = ctx;
        srv->device = context_device(ctx);
        srv->primary = context_primary_raster(ctx);
        check_cuda(cudaSetDevice(srv->device), "cudaSetDevice");
        if (config) {
            if (config->hbm_budget_bytes) srv->budget = config->hbm_budget_bytes;
            if (config->max_inflight) srv->max_live = config->max_inflight;
            if (config->pool_paths) srv->paths = config->pool_paths;
            if (config->round_items) srv->round_items = config->round_items;
            srv->policy = config->policy;
        }
        need(srv->policy == TT_SERVER_POLICY_FAIR || srv->policy == TT_SERVER_POLICY_SMALLEST_FIRST,
             "unknown server policy");
        need(srv->max_live <= BATCH_MAX_REQUESTS, "max_inflight above 64");
        need(srv->paths <= (1u << 24), "pool_paths above 2^24");
        need(srv->round_items >= 1 && srv->round_items <= (1ull << 30), "round_items must be in [1, 2^30]");
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = srv->device;
        check_cuda(cudaMemPoolCreate(&srv->pool, &props), "cudaMemPoolCreate");
        uint64_t keep = srv->budget;  // keep freed arenas cached up to the budget
        check_cuda(cudaMemPoolSetAttribute(srv->pool, cudaMemPoolAttrReleaseThreshold, &keep), "pool attribute");
        check_cuda(cudaStreamCreateWithFlags(&srv->stream, cudaStreamNonBlocking), "stream");
        check_cuda(cudaStreamCreateWithFlags(&srv->capture, cudaStreamNonBlocking), "stream");
        check_cuda(cudaStreamCreateWithFlags(&srv->body, cudaStreamNonBlocking), "stream");
        check_cuda(cudaEventCreate(&srv->round_start), "event");
        check_cuda(cudaEventCreate(&srv->round_done), "event");
        srv->create_pool();
        tt_server* raw = srv.get();
        srv->worker = std::thread([raw] { raw->run(); });
        *out = srv.release();
    });
}

int32_t tt_server_destroy(tt_server* server) {
    return server_guarded([&] {
        if (!server) return;
        {
            std::lock_guard<std::mutex> lk(server->mu);
            server->stop = true;
        }
        server->cv.notify_all();
        if (server->worker.joinable()) server->worker.join();
        cudaSetDevice(server->device);
        cudaStreamSynchronize(server->stream);
        for (auto& by_tex : server->graph)
            for (auto& by_structures : by_tex)
                for (cudaGraphExec_t g : by_structures)
                    if (g) cudaGraphExecDestroy(g);
        cudaStreamDestroy(server->stream);
        cudaStreamDestroy(server->capture);
        cudaStreamDestroy(server->body);
        cudaEventDestroy(server->round_start);
        cudaEventDestroy(server->round_done);
        cudaFreeHost(server->h_reqs);
        cudaFreeHost(server->h_scenes);
        cudaFreeHost(server->h_round);
        cudaFreeHost(server->h_err);
        for (Staging& s : server->staging_free) cudaFreeHost(s.ptr);
        if (server->pool) cudaMemPoolDestroy(server->pool);
        delete server;
    });
}

int32_t tt_server_submit(tt_server* server, tt_handle scene, const tt_constants* constants, float* host_rgba32f,
                         uint64_t bytes, uint64_t* request_id) {
    return server_guarded([&] {
        need(server && constants && host_rgba32f && request_id, "null argument");
        need(constants->sample_count >= 1 && constants->bounce_count >= 1, "sample_count and bounce_count must be >= 1");
        need(constants->bounce_count < (1u << BATCH_BOUNCE_BITS), "bounce_count must be below 65536");
        uint64_t WH = (uint64_t)constants->screen_size[0] * constants->screen_size[1];
        need(WH > 0 && bytes == 16ull * WH, "byte count must equal width * height * 16");
        need(WH <= MAX_PIXELS, "more than 4096 x 4096 pixels");
        auto r = std::make_unique<Request>();
        r->sc = scene_view(server->ctx, scene);  // validates the handle on the caller's thread
        r->c = *constants;
        r->host = host_rgba32f;
        r->bytes = bytes;
        r->WH = WH;
        r->chunk_cap = (uint32_t)std::clamp<uint64_t>(server->round_items / WH, 1,
                                                      std::min<uint32_t>(MAX_CHUNK_SPP, constants->sample_count));
        r->arena_bytes = arena_bytes(WH, r->chunk_cap);
        r->submitted = Clock::now();
        {
            std::lock_guard<std::mutex> lk(server->mu);
            need(!server->stop, "server is stopping");
            r->id = server->next_id++;
            *request_id = r->id;
            server->queue.push_back(r.get());
            server->requests[r->id] = std::move(r);
            server->stats.submitted++;
            server->stats.queued++;
        }
        server->cv.notify_all();
    });
}

int32_t tt_server_status(tt_server* server, uint64_t request_id, int32_t* status, double* latency_ms) {
    return server_guarded([&] {
        need(server && status, "null argument");
        std::lock_guard<std::mutex> lk(server->mu);
        auto it = server->requests.find(request_id);
        if (it == server->requests.end()) fail(TT_ERR_BAD_HANDLE, "unknown request id");
        const Request& r = *it->second;
        *status = r.status;
        if (latency_ms)
            *latency_ms = r.status >= TT_REQUEST_DONE
                              ? std::chrono::duration<double, std::milli>(r.finished - r.submitted).count()
                              : 0.0;
        if (r.status == TT_REQUEST_FAILED) set_last_error(r.error);
    });
}

int32_t tt_server_wait(tt_server* server, uint64_t request_id, uint32_t timeout_ms, int32_t* status) {
    return server_guarded([&] {
        need(server, "null argument");
        std::unique_lock<std::mutex> lk(server->mu);
        auto it = server->requests.find(request_id);
        if (it == server->requests.end()) fail(TT_ERR_BAD_HANDLE, "unknown request id");
        Request* r = it->second.get();
        bool ok = server->done_cv.wait_for(lk, std::chrono::milliseconds(timeout_ms),
                                           [&] { return r->status >= TT_REQUEST_DONE; });
        if (status) *status = r->status;
        if (!ok) fail(TT_ERR_TIMEOUT, "request not finished within the timeout");
        if (r->status == TT_REQUEST_FAILED) set_last_error(r->error);
    });
}

int32_t tt_server_stats_get(tt_server* server, tt_server_stats* out) {
    return server_guarded([&] {
        need(server && out, "null argument");
        std::lock_guard<std::mutex> lk(server->mu);
        *out = server->stats;
    });
}

}  // extern "C"
