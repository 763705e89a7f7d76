// server.cu - the serving form: continuous batching of cull requests over
// resident scenes.
//
// Requests (scene + 1..4 views) are queued by cadr_server_submit.  A
// scheduler thread admits queued requests in arrival order while output
// memory is available (first-fit in an output arena sized from free device
// memory or the configured budget) and a batch slot is free, waits up to the
// batching window for more requests to join, and launches the batch in
// the batched form of the context's tuning on the slot's own stream and
// scratch.  Several slots are in flight at once, so requests that arrive
// while others run are admitted into the next slot and their work overlaps
// on the device.  Completion is stamped by a host callback on the slot's
// stream; results stay valid until cadr_server_release frees their output.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "capi_internal.h"

namespace cadr {

static uint64_t now_ns()
{
    return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

// First-fit allocator over one device arena (256-byte granules).
class OutputArena {
public:
    cadr_status init(size_t bytes)
    {
        bytes_ = bytes & ~size_t(255);
        cudaError_t e = cudaMalloc(&base_, bytes_ ? bytes_ : 256);
        if (e != cudaSuccess) return cuda_fail(e, "server: output arena");
        free_[0] = bytes_;
        return CADR_OK;
    }
    void release_all()
    {
        if (base_) cudaFree(base_);
        base_ = nullptr;
    }
    bool alloc(size_t bytes, size_t* off)
    {
        bytes = (bytes + 255) & ~size_t(255);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= bytes) {
                *off = it->first;
                const size_t rest = it->second - bytes, start = it->first + bytes;
                free_.erase(it);
                if (rest) free_[start] = rest;
                used_ += bytes;
                return true;
            }
        }
        return false;
    }
    void free(size_t off, size_t bytes)
    {
        bytes = (bytes + 255) & ~size_t(255);
        used_ -= bytes;
        auto it = free_.emplace(off, bytes).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    uint8_t* base() const { return static_cast<uint8_t*>(base_); }
    size_t bytes() const { return bytes_; }

private:
    void* base_ = nullptr;
    size_t bytes_ = 0, used_ = 0;
    std::map<size_t, size_t> free_;
};

struct Request {
    uint64_t id = 0;
    cadr_scene* scene = nullptr;
    cadr_view views[4];
    uint32_t num_views = 0;
    uint64_t submit_ns = 0, complete_ns = 0;
    size_t out_off = 0, out_bytes = 0;
    cadr_status status = CADR_OK;
    bool done = false;
};

struct Slot {
    cudaStream_t stream = nullptr;
    Scratch scratch;
    ViewJob* d_jobs = nullptr;
    ViewJob* h_jobs = nullptr;
    uint32_t cap = 0;
    std::vector<Request*> reqs;
    std::atomic<bool> busy{false};
    struct cadr_server* srv = nullptr;
};

}  // namespace cadr

using namespace cadr;

struct cadr_server {
    cadr_context* ctx = nullptr;
    cadr_server_config cfg = {};
    OutputArena arena;
    std::vector<Slot*> slots;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Request*> pending;
    std::deque<Request*> finished;
    std::map<uint64_t, Request*> live;
    uint64_t next_id = 1;
    std::thread worker;
    bool stop = false;
    std::atomic<uint32_t> inflight{0};
    cadr_status worker_status = CADR_OK;
};

namespace cadr {

static size_t output_bytes(const cadr_scene* sc, uint32_t views)
{
    const size_t cmds = ((size_t)sc->desc.num_drawables * 20 + 255) & ~size_t(255);
    const size_t counts = ((size_t)sc->desc.num_state_sets * 4 + 255) & ~size_t(255);
    return views * (cmds + counts);
}

static void CUDART_CB on_slot_done(void* p)
{
    Slot* slot = static_cast<Slot*>(p);
    cadr_server* srv = slot->srv;
    const uint64_t t = now_ns();
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        for (Request* r : slot->reqs) {
            r->complete_ns = t;
            r->done = true;
            srv->finished.push_back(r);
        }
        slot->reqs.clear();
        slot->busy = false;
        srv->inflight--;
    }
    srv->cv.notify_all();
}

static cadr_status launch_slot(cadr_server* srv, Slot* slot, std::vector<Request*>& batch)
{
    cadr_context* ctx = srv->ctx;
    if (__atomic_load_n(&ctx->fault, __ATOMIC_RELAXED) == CADR_FAULT_SERVER_LAUNCH)
        return fail(CADR_ERR_CUDA, "server: launch failed (injected by CADR_FAULT_SERVER_LAUNCH)");
    const cadr_tuning tu = ctx->tuning;
    uint32_t nv = 0;
    for (Request* r : batch) nv += r->num_views;
    cudaError_t e;
    if (nv > slot->cap) {
        if (slot->d_jobs) cudaFree(slot->d_jobs);
        if (slot->h_jobs) cudaFreeHost(slot->h_jobs);
        slot->cap = std::max<uint32_t>(nv, 64u);
        e = cudaMalloc(&slot->d_jobs, slot->cap * sizeof(ViewJob));
        if (e == cudaSuccess) e = cudaHostAlloc(reinterpret_cast<void**>(&slot->h_jobs), slot->cap * sizeof(ViewJob), 0);
        if (e != cudaSuccess) return cuda_fail(e, "server: job buffers");
    }
    std::vector<cadr_batch_view> bv;
    bv.reserve(nv);
    for (Request* r : batch) {
        const size_t cmds = ((size_t)r->scene->desc.num_drawables * 20 + 255) & ~size_t(255);
        const size_t counts = ((size_t)r->scene->desc.num_state_sets * 4 + 255) & ~size_t(255);
        uint8_t* p = srv->arena.base() + r->out_off;
        for (uint32_t v = 0; v < r->num_views; v++) {
            cadr_batch_view x{};
            x.scene = r->scene;
            x.view = r->views[v];
            x.cmds = reinterpret_cast<cadr_draw_indexed_cmd*>(p);
            x.counts = reinterpret_cast<uint32_t*>(p + cmds);
            x.marginal = nullptr;
            bv.push_back(x);
            p += cmds + counts;
        }
    }
    uint64_t total = 0;
    cadr_status st = build_jobs(bv.data(), nv, batched_tile(tu), slot->h_jobs, &total);
    if (st != CADR_OK) return st;
    st = scratch_reserve(ctx, slot->scratch, total);
    if (st == CADR_OK) st = scratch_reserve_planes(ctx, slot->scratch, batched_plane_words(tu, total));
    if (st != CADR_OK) return st;
    // Every batch may take the whole device (its resident grid, at most one
    // CTA per item); concurrent batches on the other slots get SMs as CTAs
    // finish.  A batch never waits on another, and a large one no longer
    // runs on a quarter of the SMs: C5's p99 went 1.25 -> 0.71 ms.
    const uint32_t grid = (uint32_t)std::min<uint64_t>(total, (uint64_t)tu.ctas_per_sm * ctx->num_sms);
    e = cudaMemcpyAsync(slot->d_jobs, slot->h_jobs, nv * sizeof(ViewJob), cudaMemcpyHostToDevice, slot->stream);
    if (e == cudaSuccess)
        e = launch_batched_cull(slot->d_jobs, nv, (uint32_t)total, slot->scratch, ctx->d_error, ctx->spin_limit_ns,
                                CADR_FAULT_NONE, tu, grid, slot->stream);
    if (e != cudaSuccess) return cuda_fail(e, "server: launch");
    ctx->launches += tu.form == kBatchedThreeLaunch ? 3 : 1;
    slot->scratch.launches++;
    slot->reqs = batch;
    e = cudaLaunchHostFunc(slot->stream, on_slot_done, slot);
    if (e != cudaSuccess) return cuda_fail(e, "server: completion callback");
    return CADR_OK;
}

static void worker_main(cadr_server* srv)
{
    // The scheduler thread belongs to the server: its current device is
    // the context's for its whole life (no caller's device to keep).
    cudaSetDevice(srv->ctx->device);
    std::unique_lock<std::mutex> lk(srv->mu);
    for (;;) {
        srv->cv.wait(lk, [&] { return srv->stop || !srv->pending.empty(); });
        if (srv->stop && srv->pending.empty()) break;
        // Batching window: from the oldest request's arrival, wait for more
        // requests, unless the batch is already full (views), the device is
        // idle (no batch in flight: waiting only adds latency), or the
        // pending work already fills the device (its resident tiles), as
        // it then gains nothing from more requests.
        const uint64_t oldest = srv->pending.front()->submit_ns;
        uint32_t views = 0;
        uint64_t items = 0;
        for (Request* r : srv->pending) {
            views += r->num_views;
            items += (uint64_t)r->num_views * r->scene->desc.num_drawables;
        }
        const uint64_t fill = (uint64_t)srv->ctx->num_sms * srv->ctx->tuning.ctas_per_sm * batched_tile(srv->ctx->tuning);
        const uint64_t t = now_ns();
        if (!srv->stop && views < srv->cfg.max_batch_views && t < oldest + srv->cfg.window_ns && srv->inflight > 0 &&
            items < fill) {
            srv->cv.wait_for(lk, std::chrono::nanoseconds(oldest + srv->cfg.window_ns - t));
            continue;
        }
        // A free slot.
        Slot* slot = nullptr;
        for (Slot* s : srv->slots)
            if (!s->busy) {
                slot = s;
                break;
            }
        if (!slot) {
            srv->cv.wait(lk, [&] { return srv->stop || srv->inflight < srv->slots.size(); });
            continue;
        }
        // Admission in arrival order while output memory lasts.
        std::vector<Request*> batch;
        uint32_t nv = 0;
        while (!srv->pending.empty()) {
            Request* r = srv->pending.front();
            if (nv + r->num_views > srv->cfg.max_batch_views && !batch.empty()) break;
            size_t off = 0;
            if (!srv->arena.alloc(r->out_bytes, &off)) break;
            r->out_off = off;
            batch.push_back(r);
            nv += r->num_views;
            srv->pending.pop_front();
        }
        if (batch.empty()) {
            // Memory is held by finished, unreleased requests or batches in
            // flight: wait for a release or a completion.
            srv->cv.wait_for(lk, std::chrono::microseconds(50));
            continue;
        }
        slot->busy = true;
        srv->inflight++;
        lk.unlock();
        cadr_status st = launch_slot(srv, slot, batch);
        // Whatever of a failed batch reached the stream has finished before
        // its output memory goes back to the arena.
        if (st != CADR_OK) cudaStreamSynchronize(slot->stream);
        lk.lock();
        if (st != CADR_OK) {
            for (Request* r : batch) {
                srv->arena.free(r->out_off, r->out_bytes);  // a failed request keeps no output
                r->status = st;
                r->done = true;
                r->complete_ns = now_ns();
                srv->finished.push_back(r);
            }
            slot->reqs.clear();
            slot->busy = false;
            srv->inflight--;
            srv->worker_status = st;
        }
    }
}

}  // namespace cadr

extern "C" {

CADR_API cadr_status cadr_server_create(cadr_context* ctx, const cadr_server_config* cfg, cadr_server** out)
{
    if (!ctx || !cfg || !out) return fail(CADR_ERR_INVALID_ARG, "server_create: null argument");
    DeviceGuard dg(ctx->device);
    *out = nullptr;
    if (cfg->max_inflight_batches == 0 || cfg->max_inflight_batches > 16 || cfg->max_batch_views == 0)
        return fail(CADR_ERR_INVALID_ARG, "server_create: 1..16 batches in flight and >= 1 view per batch");
    auto* srv = new cadr_server();
    srv->ctx = ctx;
    srv->cfg = *cfg;
    size_t budget = cfg->memory_budget_bytes;
    if (budget == 0) {
        size_t fr = 0, tot = 0;
        cudaError_t e = cudaMemGetInfo(&fr, &tot);
        if (e != cudaSuccess) {
            delete srv;
            return cuda_fail(e, "server_create: memory info");
        }
        const size_t reserve = cfg->reserve_bytes ? cfg->reserve_bytes : (size_t(4) << 30);
        budget = fr > reserve ? (fr - reserve) / 2 : 0;
    }
    cadr_status st = srv->arena.init(budget);
    if (st != CADR_OK) {
        delete srv;
        return st;
    }
    for (uint32_t i = 0; i < cfg->max_inflight_batches; i++) {
        Slot* s = new Slot();
        s->srv = srv;
        cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
        srv->slots.push_back(s);
        if (e != cudaSuccess) {
            cadr_server_destroy(srv);
            return cuda_fail(e, "server_create: stream");
        }
        st = scratch_reserve(ctx, s->scratch, 1u << 16);
        if (st != CADR_OK) {
            cadr_server_destroy(srv);
            return st;
        }
    }
    srv->worker = std::thread(worker_main, srv);
    *out = srv;
    return CADR_OK;
}

CADR_API cadr_status cadr_server_destroy(cadr_server* srv)
{
    if (!srv) return CADR_OK;
    DeviceGuard dg(srv->ctx->device);
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->stop = true;
        for (Request* r : srv->pending) {
            r->status = CADR_ERR_REJECTED;
            r->done = true;
            srv->finished.push_back(r);
        }
        srv->pending.clear();
    }
    srv->cv.notify_all();
    if (srv->worker.joinable()) srv->worker.join();
    for (Slot* s : srv->slots) {
        if (s->stream) cudaStreamSynchronize(s->stream);
    }
    for (Slot* s : srv->slots) {
        if (s->stream) cudaStreamDestroy(s->stream);
        scratch_release(s->scratch);
        if (s->d_jobs) cudaFree(s->d_jobs);
        if (s->h_jobs) cudaFreeHost(s->h_jobs);
        delete s;
    }
    srv->arena.release_all();
    for (auto& kv : srv->live) delete kv.second;
    delete srv;
    return CADR_OK;
}

CADR_API cadr_status cadr_server_submit(cadr_server* srv, cadr_scene* scene, const cadr_view* views,
                                        uint32_t num_views, uint64_t* request_id)
{
    if (!srv || !scene || !views || num_views == 0 || num_views > 4)
        return fail(CADR_ERR_INVALID_ARG, "server_submit: need a scene and 1..4 views");
    if (!scene->committed) {
        cadr_status st = cadr_scene_commit(scene);
        if (st != CADR_OK) return st;
    }
    auto* r = new Request();
    r->scene = scene;
    r->num_views = num_views;
    std::memcpy(r->views, views, num_views * sizeof(cadr_view));
    r->out_bytes = output_bytes(scene, num_views);
    if (r->out_bytes > srv->arena.bytes()) {
        delete r;
        return fail(CADR_ERR_REJECTED, "server_submit: request needs %zu output bytes, the server holds %zu",
                    output_bytes(scene, num_views), srv->arena.bytes());
    }
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        if (srv->stop) {
            delete r;
            return fail(CADR_ERR_REJECTED, "server_submit: server is stopping");
        }
        r->id = srv->next_id++;
        r->submit_ns = now_ns();
        srv->live[r->id] = r;
        srv->pending.push_back(r);
    }
    srv->cv.notify_all();
    if (request_id) *request_id = r->id;
    return CADR_OK;
}

CADR_API cadr_status cadr_server_poll(cadr_server* srv, cadr_request_result* results, uint32_t max_results,
                                      uint32_t* num_results)
{
    if (!srv || !num_results || (!results && max_results)) return fail(CADR_ERR_INVALID_ARG, "server_poll: bad argument");
    std::lock_guard<std::mutex> lk(srv->mu);
    uint32_t k = 0;
    while (k < max_results && !srv->finished.empty()) {
        Request* r = srv->finished.front();
        srv->finished.pop_front();
        cadr_request_result& o = results[k++];
        std::memset(&o, 0, sizeof(o));
        o.request_id = r->id;
        o.status = r->status;
        o.num_views = r->num_views;
        o.submit_ns = r->submit_ns;
        o.complete_ns = r->complete_ns;
        if (r->status == CADR_OK) {
            const size_t cmds = ((size_t)r->scene->desc.num_drawables * 20 + 255) & ~size_t(255);
            const size_t counts = ((size_t)r->scene->desc.num_state_sets * 4 + 255) & ~size_t(255);
            uint8_t* p = srv->arena.base() + r->out_off;
            for (uint32_t v = 0; v < r->num_views; v++) {
                o.cmds[v] = reinterpret_cast<const cadr_draw_indexed_cmd*>(p);
                o.counts[v] = reinterpret_cast<const uint32_t*>(p + cmds);
                p += cmds + counts;
            }
        }
    }
    *num_results = k;
    return CADR_OK;
}

CADR_API cadr_status cadr_server_release(cadr_server* srv, uint64_t request_id)
{
    if (!srv) return fail(CADR_ERR_INVALID_ARG, "server_release: null server");
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        auto it = srv->live.find(request_id);
        if (it == srv->live.end()) return fail(CADR_ERR_INVALID_ARG, "server_release: unknown request %llu",
                                              (unsigned long long)request_id);
        Request* r = it->second;
        if (!r->done) return fail(CADR_ERR_NOT_READY, "server_release: request still running");
        if (r->status == CADR_OK) srv->arena.free(r->out_off, r->out_bytes);
        srv->live.erase(it);
        delete r;
    }
    srv->cv.notify_all();
    return CADR_OK;
}

CADR_API cadr_status cadr_server_drain(cadr_server* srv)
{
    if (!srv) return fail(CADR_ERR_INVALID_ARG, "server_drain: null server");
    std::unique_lock<std::mutex> lk(srv->mu);
    srv->cv.wait(lk, [&] { return srv->pending.empty() && srv->inflight == 0; });
    return srv->worker_status;
}

}  // extern "C"
