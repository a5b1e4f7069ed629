// Continuous-batching render server (tt_server_*): requests of any scene, resolution and
// sample count are admitted from an arrival-order queue whenever an execution slot and enough
// of the HBM budget are free, and run concurrently, each as one CUDA graph on its own stream.
//
// Per request the device holds one stream-ordered arena (allocated from a server-owned memory
// pool on the slot's stream and freed on it after the image is copied out): the wavefront path
// pool, its queues, the per-sample radiance of one sample chunk, the running pixel sums and the
// render target.  The admission test uses the arena's exact size, so the budget bounds what is
// in flight.  Requests share nothing mutable on the device, which makes every image identical
// to the same request rendered alone.
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
}  // namespace tt

using namespace tt;
using Clock = std::chrono::steady_clock;

namespace {

constexpr uint64_t DEFAULT_BUDGET = 150ull << 30;
constexpr uint32_t DEFAULT_INFLIGHT = 8;
constexpr uint32_t DEFAULT_PATHS = 1u << 20;
constexpr uint32_t MAX_CHUNK_SPP = 64;

struct Request {
    uint64_t id = 0;
    DevScene sc{};
    tt_constants c{};
    float* host = nullptr;
    uint64_t bytes = 0, arena_bytes = 0;
    Clock::time_point submitted, finished;
    int32_t status = TT_REQUEST_QUEUED;
    std::string error;
};

// Byte offsets of one request's arrays inside its arena (256-byte aligned).
struct Layout {
    uint32_t P = 0, chunk_spp = 0;
    uint64_t WH = 0, items = 0;
    uint64_t org, dir, thr, acc, pa1, pa0, pe, hit, hslot, active, shadow, ndc_mip, counters, samples, running, target,
        total;
};

Layout layout_for(const tt_constants& c, uint32_t paths) {
    Layout L;
    L.WH = (uint64_t)c.screen_size[0] * c.screen_size[1];
    L.chunk_spp = std::min<uint32_t>(c.sample_count, MAX_CHUNK_SPP);
    L.items = L.WH * L.chunk_spp;
    uint64_t P = std::min<uint64_t>(paths, std::max<uint64_t>(L.items, 1));
    L.P = (uint32_t)((P + 127u) / 128u * 128u);
    uint64_t at = 0;
    auto take = [&](uint64_t bytes) {
        uint64_t o = at;
        at += (bytes + 255u) / 256u * 256u;
        return o;
    };
    L.org = take(16ull * L.P);
    L.dir = take(16ull * L.P);
    L.thr = take(16ull * L.P);
    L.acc = take(16ull * L.P);
    L.pa1 = take(16ull * L.P);
    L.pa0 = take(16ull * L.P);
    L.pe = take(16ull * L.P);
    L.hit = take(16ull * HIT_BUCKETS * L.P);
    L.hslot = take(4ull * HIT_BUCKETS * L.P);
    L.active = take(4ull * L.P);
    L.shadow = take(32ull * L.P);
    L.ndc_mip = take(8ull * L.P);
    L.counters = take(4ull * CTRL_WORDS);
    L.samples = take(16ull * L.items);
    L.running = take(16ull * L.WH);
    L.target = take(16ull * L.WH);
    L.total = at + 256u;  // + the error word
    return L;
}

struct Slot {
    cudaStream_t stream = nullptr, capture = nullptr, body = nullptr;
    cudaEvent_t done = nullptr;
    uint32_t* err_dev = nullptr;   // in the arena's last 256 bytes
    uint32_t* err_host = nullptr;  // pinned
    float* staging = nullptr;      // pinned copy of the target
    uint64_t staging_bytes = 0;
    Request* req = nullptr;
};

}  // namespace

struct tt_server {
    int device = 0;
    tt_context* ctx = nullptr;
    uint64_t budget = DEFAULT_BUDGET;
    uint32_t paths = DEFAULT_PATHS;
    int trace_blocks = 0;
    cudaMemPool_t pool = nullptr;
    std::vector<Slot> slots;
    std::mutex mu;
    std::condition_variable cv;      // submissions and stop (scheduler side)
    std::condition_variable done_cv; // completions (waiter side)
    std::deque<Request*> queue;
    std::map<uint64_t, std::unique_ptr<Request>> requests;
    uint64_t next_id = 1;
    bool stop = false;
    tt_server_stats stats{};
    std::thread worker;

    void launch(Slot& s, Request& r);
    void finish(Slot& s, cudaError_t q);
    void run();
};

// Enqueues request r on slot s: arena, error word, the graph, the image and error read-back.
void tt_server::launch(Slot& s, Request& r) {
    Layout L = layout_for(r.c, paths);
    char* arena = nullptr;
    check_cuda(cudaMallocFromPoolAsync((void**)&arena, L.total, pool, s.stream), "arena");
    s.err_dev = reinterpret_cast<uint32_t*>(arena + L.total - 256u);
    uint64_t image = 16ull * L.WH;
    if (s.staging_bytes < image) {
        if (s.staging) cudaFreeHost(s.staging);
        s.staging = nullptr;
        check_cuda(cudaMallocHost((void**)&s.staging, image), "staging");
        s.staging_bytes = image;
    }
    WfParams w{};
    w.org = reinterpret_cast<float4*>(arena + L.org);
    w.dir = reinterpret_cast<float4*>(arena + L.dir);
    w.thr = reinterpret_cast<float4*>(arena + L.thr);
    w.acc = reinterpret_cast<float4*>(arena + L.acc);
    w.pa1 = reinterpret_cast<float4*>(arena + L.pa1);
    w.pa0 = reinterpret_cast<float4*>(arena + L.pa0);
    w.pe = reinterpret_cast<float4*>(arena + L.pe);
    w.hit = reinterpret_cast<uint4*>(arena + L.hit);
    w.hslot = reinterpret_cast<uint32_t*>(arena + L.hslot);
    w.active = reinterpret_cast<uint32_t*>(arena + L.active);
    w.shadow = reinterpret_cast<float4*>(arena + L.shadow);
    w.counters = reinterpret_cast<uint32_t*>(arena + L.counters);
    w.samples = reinterpret_cast<float4*>(arena + L.samples);
    w.running = reinterpret_cast<float4*>(arena + L.running);
    w.ndc_mip = r.sc.textured ? reinterpret_cast<float2*>(arena + L.ndc_mip) : nullptr;
    w.P = L.P;
    w.chunk_spp = L.chunk_spp;
    w.refill = 20;
    w.trace_blocks = (uint32_t)trace_blocks;
    RenderParams p{};
    p.sc = r.sc;
    p.c = r.c;
    p.target = reinterpret_cast<float4*>(arena + L.target);
    p.err = s.err_dev;
    p.counters = nullptr;
    try {
        check_cuda(cudaMemsetAsync(s.err_dev, 0, 4, s.stream), "memset");
        render_wavefront_graph(p, w, false, s.stream, s.capture, s.body);
        check_cuda(cudaMemcpyAsync(s.staging, p.target, image, cudaMemcpyDeviceToHost, s.stream), "image");
        check_cuda(cudaMemcpyAsync(s.err_host, s.err_dev, 4, cudaMemcpyDeviceToHost, s.stream), "error word");
    } catch (...) {
        cudaFreeAsync(arena, s.stream);
        throw;
    }
    check_cuda(cudaFreeAsync(arena, s.stream), "arena free");
    check_cuda(cudaEventRecord(s.done, s.stream), "event");
}

// Completion of slot s (its event fired, or failed with q): error word, image copy-out, stats.
void tt_server::finish(Slot& s, cudaError_t q) {
    Request& r = *s.req;
    int32_t status = TT_REQUEST_DONE;
    std::string error;
    if (q != cudaSuccess) {
        status = TT_REQUEST_FAILED;
        error = std::string("device error: ") + cudaGetErrorString(q);
    } else if (*s.err_host & ERR_STACK_OVERFLOW) {
        status = TT_REQUEST_FAILED;
        error = "traversal stack overflow";
    } else if (*s.err_host & ERR_ITERATION_LIMIT) {
        status = TT_REQUEST_FAILED;
        error = "iteration limit reached";
    } else {
        std::memcpy(r.host, s.staging, r.bytes);
    }
    std::lock_guard<std::mutex> lk(mu);
    r.finished = Clock::now();
    r.status = status;
    r.error = error;
    stats.inflight--;
    stats.bytes_in_flight -= r.arena_bytes;
    if (status == TT_REQUEST_DONE) stats.completed++;
    else stats.failed++;
    s.req = nullptr;
    done_cv.notify_all();
}

void tt_server::run() {
    cudaSetDevice(device);
    while (true) {
        bool progressed = false;
        for (Slot& s : slots) {
            if (!s.req) continue;
            cudaError_t q = cudaEventQuery(s.done);
            if (q == cudaErrorNotReady) continue;
            finish(s, q);
            progressed = true;
        }
        // admit the head of the queue while a slot and the budget allow (arrival order)
        while (true) {
            Request* r = nullptr;
            Slot* slot = nullptr;
            {
                std::lock_guard<std::mutex> lk(mu);
                if (queue.empty()) break;
                Request* head = queue.front();
                if (head->arena_bytes > budget) {  // can never fit
                    queue.pop_front();
                    head->status = TT_REQUEST_FAILED;
                    head->error = "request needs more device memory than the HBM budget";
                    head->finished = Clock::now();
                    stats.queued--;
                    stats.failed++;
                    done_cv.notify_all();
                    progressed = true;
                    continue;
                }
                for (Slot& s : slots)
                    if (!s.req) {
                        slot = &s;
                        break;
                    }
                if (!slot || stats.bytes_in_flight + head->arena_bytes > budget) break;
                queue.pop_front();
                r = head;
                r->status = TT_REQUEST_RUNNING;
                slot->req = r;
                stats.queued--;
                stats.inflight++;
                stats.bytes_in_flight += r->arena_bytes;
                stats.peak_inflight = std::max(stats.peak_inflight, stats.inflight);
                stats.peak_bytes_in_flight = std::max(stats.peak_bytes_in_flight, stats.bytes_in_flight);
            }
            progressed = true;
            try {
                launch(*slot, *r);
            } catch (const Error& e) {
                std::lock_guard<std::mutex> lk(mu);
                r->status = TT_REQUEST_FAILED;
                r->error = e.message;
                r->finished = Clock::now();
                stats.inflight--;
                stats.bytes_in_flight -= r->arena_bytes;
                stats.failed++;
                slot->req = nullptr;
                done_cv.notify_all();
            }
        }
        std::unique_lock<std::mutex> lk(mu);
        bool busy = stats.inflight > 0 || !queue.empty();
        if (stop && !busy) break;
        if (!progressed) cv.wait_for(lk, std::chrono::microseconds(busy ? 50 : 2000));
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
}  // namespace

extern "C" {

int32_t tt_server_create(tt_context* ctx, const tt_server_config* config, tt_server** out) {
    return server_guarded([&] {
        need(ctx && out, "null argument");
        auto srv = std::make_unique<tt_server>();
        srv->ctx = ctx;
        srv->device = context_device(ctx);
        check_cuda(cudaSetDevice(srv->device), "cudaSetDevice");
        uint32_t inflight = DEFAULT_INFLIGHT;
        if (config) {
            if (config->hbm_budget_bytes) srv->budget = config->hbm_budget_bytes;
            if (config->max_inflight) inflight = config->max_inflight;
            if (config->paths_per_request) srv->paths = config->paths_per_request;
        }
        need(inflight <= 64, "max_inflight above 64");
        need(srv->paths <= (1u << 24), "paths_per_request above 2^24");
        int sms = 0, per_sm = 0;
        trace_occupancy(&sms, &per_sm);
        srv->trace_blocks = std::max(1, sms * per_sm);
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = srv->device;
        check_cuda(cudaMemPoolCreate(&srv->pool, &props), "cudaMemPoolCreate");
        uint64_t keep = srv->budget;  // keep freed arenas cached up to the budget
        check_cuda(cudaMemPoolSetAttribute(srv->pool, cudaMemPoolAttrReleaseThreshold, &keep), "pool attribute");
        srv->slots.resize(inflight);
        for (Slot& s : srv->slots) {
            check_cuda(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking), "stream");
            check_cuda(cudaStreamCreateWithFlags(&s.capture, cudaStreamNonBlocking), "stream");
            check_cuda(cudaStreamCreateWithFlags(&s.body, cudaStreamNonBlocking), "stream");
            check_cuda(cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming), "event");
            check_cuda(cudaMallocHost((void**)&s.err_host, 16), "cudaMallocHost");
        }
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
        for (Slot& s : server->slots) {
            cudaStreamSynchronize(s.stream);
            cudaStreamDestroy(s.stream);
            cudaStreamDestroy(s.capture);
            cudaStreamDestroy(s.body);
            cudaEventDestroy(s.done);
            cudaFreeHost(s.err_host);
            if (s.staging) cudaFreeHost(s.staging);
        }
        if (server->pool) cudaMemPoolDestroy(server->pool);
        delete server;
    });
}

int32_t tt_server_submit(tt_server* server, tt_handle scene, const tt_constants* constants, float* host_rgba32f,
                         uint64_t bytes, uint64_t* request_id) {
    return server_guarded([&] {
        need(server && constants && host_rgba32f && request_id, "null argument");
        need(constants->sample_count >= 1 && constants->bounce_count >= 1, "sample_count and bounce_count must be >= 1");
        uint64_t WH = (uint64_t)constants->screen_size[0] * constants->screen_size[1];
        need(WH > 0 && bytes == 16ull * WH, "byte count must equal width * height * 16");
        auto r = std::make_unique<Request>();
        r->sc = scene_view(server->ctx, scene);  // validates the handle on the caller's thread
        r->c = *constants;
        r->host = host_rgba32f;
        r->bytes = bytes;
        r->arena_bytes = layout_for(*constants, server->paths).total;
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

