// trw_server.cu -- request loop over a resident graph (continuous batching).
//
// The reference runs one compute() per process (creeper_main.h:14-72); this
// loop keeps the graph and its sampling tables resident in HBM and serves a
// stream of walk requests of different apps and sizes.  A dispatcher thread
// admits queued requests in arrival order whenever a stream slot is free and
// the request's device memory fits the budget, and launches each admitted
// request on its own stream, so requests that arrive while others run start
// at once and overlap them on the device.  A host function enqueued after each
// request's kernels timestamps its completion; latency = completion - submit.
// Every walk is a pure function of (seed, walker, step), so a request's result
// does not depend on what it ran beside.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "trw.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    trw_server *srv = nullptr;
    uint64_t ticket = 0;
    trw_request req{};
    std::vector<int32_t> schema, sources;
    size_t bytes = 0;          // device bytes held until release
    void *dmem = nullptr;
    int32_t *d_src = nullptr, *d_paths = nullptr, *d_len = nullptr, *d_vert = nullptr, *d_cnt = nullptr;
    int64_t *d_off = nullptr;
    uint64_t *d_steps = nullptr;
    int64_t capacity = 0;      // sparse PPR entries
    int stream = -1;
    Clock::time_point t_submit, t_start;
    std::atomic<int64_t> done_ns{0};  // completion time (ns since submit), 0 = running
    int status = 0;            // 0 queued, 1 running, 2 done, 3 failed
    std::string error;
};

}  // namespace

struct trw_server {
    trw_graph *g = nullptr;
    size_t budget = 0, in_use = 0;
    std::vector<cudaStream_t> streams;
    std::vector<char> stream_busy;
    std::deque<std::shared_ptr<Request>> queue;
    std::unordered_map<uint64_t, std::shared_ptr<Request>> reqs;
    std::vector<std::shared_ptr<Request>> running;
    std::mutex mu;
    std::condition_variable cv;
    std::thread dispatcher;
    bool stopping = false;
    uint64_t next_ticket = 1;
    int32_t max_queue = 1 << 16;
    // statistics
    uint64_t submitted = 0, completed = 0, failed = 0, steps = 0;
    std::vector<double> latencies_ms;
    Clock::time_point t0;
};

namespace {

// Runs on a CUDA callback thread once the request's work is done: records the
// completion time and wakes the dispatcher (no CUDA calls, no locks).
void CUDART_CB on_complete(void *arg) {
    auto *r = static_cast<Request *>(arg);
    const int64_t ns = std::chrono::duration_cast<std::chrono::nanoseconds>(Clock::now() - r->t_submit).count();
    r->done_ns.store(ns > 0 ? ns : 1);
    r->srv->cv.notify_all();
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Device bytes a request holds: sources, outputs and the step counter.
void size_request(trw_server *s, Request &r, int32_t n) {
    const trw_request &q = r.req;
    size_t b = align256(sizeof(int32_t) * (size_t)std::max<int64_t>(1, r.sources.size()));
    b += align256(sizeof(uint64_t));
    if (q.walkers_per_query > 0) {
        const double visits = (double)q.walkers_per_query / std::max(1e-6, q.desc.tp);
        r.capacity = std::min<int64_t>((int64_t)n, (int64_t)(1.25 * visits) + 1024) * (int64_t)r.sources.size();
        b += align256(sizeof(int64_t) * (r.sources.size() + 1)) + 2 * align256(sizeof(int32_t) * (size_t)r.capacity);
    } else {
        b += align256(sizeof(int32_t) * (size_t)q.num_walkers);
        if (q.path_cap > 0) b += align256(sizeof(int32_t) * (size_t)q.num_walkers * (size_t)q.path_cap);
    }
    r.bytes = b;
    (void)s;
}

// Enqueues one request on its stream (called with the server lock held).
void launch(trw_server *s, Request &r) {
    cudaStream_t st = s->streams[r.stream];
    r.t_start = Clock::now();
    r.status = 1;
    auto bad = [&](const std::string &why) { r.status = 3; r.error = why; };
    if (cudaMallocAsync(&r.dmem, r.bytes, st) != cudaSuccess) { cudaGetLastError(); return bad("device allocation failed"); }
    char *p = static_cast<char *>(r.dmem);
    auto carve = [&](size_t bytes) { char *q = p; p += align256(bytes); return q; };
    r.d_src = reinterpret_cast<int32_t *>(carve(sizeof(int32_t) * std::max<size_t>(1, r.sources.size())));
    r.d_steps = reinterpret_cast<uint64_t *>(carve(sizeof(uint64_t)));
    cudaMemcpyAsync(r.d_src, r.sources.data(), sizeof(int32_t) * r.sources.size(), cudaMemcpyHostToDevice, st);
    r.req.desc.schema = r.schema.empty() ? nullptr : r.schema.data();
    int rc;
    if (r.req.walkers_per_query > 0) {
        r.d_off = reinterpret_cast<int64_t *>(carve(sizeof(int64_t) * (r.sources.size() + 1)));
        r.d_vert = reinterpret_cast<int32_t *>(carve(sizeof(int32_t) * (size_t)r.capacity));
        r.d_cnt = reinterpret_cast<int32_t *>(carve(sizeof(int32_t) * (size_t)r.capacity));
        rc = trw_ppr_batch_sparse(s->g, &r.req.desc, r.d_src, (int64_t)r.sources.size(), r.req.walkers_per_query,
                                  r.d_off, r.d_vert, r.d_cnt, r.capacity, r.d_steps, TRW_ENGINE_PERSISTENT,
                                  reinterpret_cast<trw_stream_t>(st));
    } else {
        r.d_len = reinterpret_cast<int32_t *>(carve(sizeof(int32_t) * (size_t)r.req.num_walkers));
        if (r.req.path_cap > 0)
            r.d_paths = reinterpret_cast<int32_t *>(carve(sizeof(int32_t) * (size_t)r.req.num_walkers * r.req.path_cap));
        rc = trw_walk(s->g, &r.req.desc, r.d_src, r.req.num_walkers, r.req.id_base, r.d_paths, r.req.path_cap, r.d_len,
                      nullptr, r.d_steps, TRW_ENGINE_PERSISTENT, reinterpret_cast<trw_stream_t>(st));
    }
    if (rc != TRW_OK) return bad(trw_last_error());
    if (cudaLaunchHostFunc(st, on_complete, &r) != cudaSuccess) { cudaGetLastError(); return bad("cudaLaunchHostFunc failed"); }
}

double percentile(std::vector<double> v, double p) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const double idx = p * (double)(v.size() - 1);
    const size_t lo = (size_t)idx;
    const size_t hi = std::min(lo + 1, v.size() - 1);
    return v[lo] + (v[hi] - v[lo]) * (idx - (double)lo);
}

void dispatch_loop(trw_server *s) {
    std::unique_lock<std::mutex> lock(s->mu);
    for (;;) {
        // completions
        for (size_t i = 0; i < s->running.size();) {
            Request &r = *s->running[i];
            const int64_t ns = r.done_ns.load();
            if (r.status == 3 || ns > 0) {
                if (r.status != 3) {
                    uint64_t st = 0;
                    cudaMemcpy(&st, r.d_steps, sizeof st, cudaMemcpyDeviceToHost);
                    s->steps += st;
                    s->latencies_ms.push_back((double)ns / 1e6);
                    r.status = 2;
                    ++s->completed;
                } else {
                    ++s->failed;
                }
                s->stream_busy[r.stream] = 0;
                s->running.erase(s->running.begin() + (long)i);
                s->cv.notify_all();
            } else {
                ++i;
            }
        }
        // admissions, in arrival order
        while (!s->queue.empty()) {
            Request &r = *s->queue.front();
            int free_stream = -1;
            for (size_t k = 0; k < s->streams.size(); ++k)
                if (!s->stream_busy[k]) { free_stream = (int)k; break; }
            if (free_stream < 0 || s->in_use + r.bytes > s->budget) break;
            r.stream = free_stream;
            s->stream_busy[free_stream] = 1;
            s->in_use += r.bytes;
            launch(s, r);
            s->running.push_back(s->queue.front());
            s->queue.pop_front();
        }
        if (s->stopping && s->queue.empty() && s->running.empty()) break;
        s->cv.wait_for(lock, std::chrono::microseconds(s->running.empty() ? 2000 : 50));
    }
}

}  // namespace

extern "C" {

int trw_server_start(trw_graph *g, size_t hbm_budget_bytes, int32_t max_inflight, trw_server **out) {
    if (!g || !out || max_inflight <= 0 || max_inflight > 64) return TRW_ERR_INVALID;
    auto *s = new trw_server();
    s->g = g;
    if (hbm_budget_bytes == 0) {
        size_t free_b = 0, total_b = 0;
        cudaMemGetInfo(&free_b, &total_b);
        hbm_budget_bytes = free_b / 10 * 8;  // 80 % of what is free now
    }
    s->budget = hbm_budget_bytes;
    for (int i = 0; i < max_inflight; ++i) {
        cudaStream_t st;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
            for (cudaStream_t x : s->streams) cudaStreamDestroy(x);
            delete s;
            return TRW_ERR_CUDA;
        }
        s->streams.push_back(st);
    }
    s->stream_busy.assign(max_inflight, 0);
    s->t0 = Clock::now();
    s->dispatcher = std::thread(dispatch_loop, s);
    *out = s;
    return TRW_OK;
}

int trw_server_submit(trw_server *s, const trw_request *req, uint64_t *ticket) {
    if (!s || !req || !ticket || !req->sources) return TRW_ERR_INVALID;
    const bool ppr = req->walkers_per_query > 0;
    const int64_t nsrc = ppr ? req->num_queries : req->num_walkers;
    if (nsrc <= 0 || (ppr && req->desc.app != TRW_APP_PPR)) return TRW_ERR_INVALID;
    auto r = std::make_shared<Request>();
    r->srv = s;
    r->req = *req;
    r->sources.assign(req->sources, req->sources + nsrc);
    if (req->desc.schema && req->desc.schema_len > 0)
        r->schema.assign(req->desc.schema, req->desc.schema + req->desc.schema_len);
    int32_t n = 0;
    trw_graph_info(s->g, &n, nullptr, nullptr);
    size_request(s, *r, n);
    std::lock_guard<std::mutex> lock(s->mu);
    if (s->stopping) return TRW_ERR_INVALID;
    if ((int64_t)s->queue.size() >= s->max_queue) return TRW_ERR_BUSY;
    if (r->bytes > s->budget) return TRW_ERR_CAPACITY;
    r->ticket = s->next_ticket++;
    r->t_submit = Clock::now();
    s->reqs[r->ticket] = r;
    s->queue.push_back(r);
    ++s->submitted;
    *ticket = r->ticket;
    s->cv.notify_all();
    return TRW_OK;
}

int trw_server_wait(trw_server *s, uint64_t ticket, int32_t timeout_ms, trw_request_status *st) {
    if (!s || !st) return TRW_ERR_INVALID;
    std::unique_lock<std::mutex> lock(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return TRW_ERR_INVALID;
    std::shared_ptr<Request> r = it->second;
    const auto until = Clock::now() + std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms);
    while (r->status < 2) {
        if (timeout_ms >= 0 && Clock::now() >= until) break;
        s->cv.wait_for(lock, std::chrono::milliseconds(1));
    }
    std::memset(st, 0, sizeof *st);
    st->state = r->status;
    if (r->status == 2) {
        st->latency_ms = (double)r->done_ns.load() / 1e6;
        st->queue_ms = std::chrono::duration<double, std::milli>(r->t_start - r->t_submit).count();
        uint64_t steps = 0;
        cudaMemcpy(&steps, r->d_steps, sizeof steps, cudaMemcpyDeviceToHost);
        st->steps = steps;
        if (r->d_off) cudaMemcpy(&st->entries, r->d_off + r->sources.size(), sizeof(int64_t), cudaMemcpyDeviceToHost);
    }
    return r->status == 3 ? TRW_ERR_DEVICE : TRW_OK;
}

int trw_server_result(trw_server *s, uint64_t ticket, int32_t *paths, int32_t *lengths, int64_t *offsets,
                      int32_t *vertices, int32_t *counts, int64_t capacity) {
    if (!s) return TRW_ERR_INVALID;
    std::shared_ptr<Request> r;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        auto it = s->reqs.find(ticket);
        if (it == s->reqs.end()) return TRW_ERR_INVALID;
        r = it->second;
    }
    if (r->status != 2) return TRW_ERR_INVALID;
    if (r->d_off) {
        const size_t nq = r->sources.size();
        int64_t total = 0;
        cudaMemcpy(&total, r->d_off + nq, sizeof total, cudaMemcpyDeviceToHost);
        if (offsets) cudaMemcpy(offsets, r->d_off, sizeof(int64_t) * (nq + 1), cudaMemcpyDeviceToHost);
        if (total > capacity) return TRW_ERR_CAPACITY;
        if (vertices) cudaMemcpy(vertices, r->d_vert, sizeof(int32_t) * (size_t)total, cudaMemcpyDeviceToHost);
        if (counts) cudaMemcpy(counts, r->d_cnt, sizeof(int32_t) * (size_t)total, cudaMemcpyDeviceToHost);
    } else {
        if (lengths) cudaMemcpy(lengths, r->d_len, sizeof(int32_t) * (size_t)r->req.num_walkers, cudaMemcpyDeviceToHost);
        if (paths && r->d_paths)
            cudaMemcpy(paths, r->d_paths, sizeof(int32_t) * (size_t)r->req.num_walkers * r->req.path_cap,
                       cudaMemcpyDeviceToHost);
    }
    return TRW_OK;
}

int trw_server_release(trw_server *s, uint64_t ticket) {
    if (!s) return TRW_ERR_INVALID;
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return TRW_ERR_INVALID;
    Request &r = *it->second;
    if (r.status < 2) return TRW_ERR_BUSY;
    if (r.dmem) cudaFreeAsync(r.dmem, s->streams[r.stream]);
    s->in_use -= r.bytes;
    s->reqs.erase(it);
    s->cv.notify_all();
    return TRW_OK;
}

int trw_server_stats(trw_server *s, trw_serving_stats *out) {
    if (!s || !out) return TRW_ERR_INVALID;
    std::lock_guard<std::mutex> lock(s->mu);
    std::memset(out, 0, sizeof *out);
    out->submitted = s->submitted;
    out->completed = s->completed;
    out->failed = s->failed;
    out->steps = s->steps;
    out->queued = (int64_t)s->queue.size();
    out->running = (int64_t)s->running.size();
    out->hbm_in_use = s->in_use;
    out->p50_ms = percentile(s->latencies_ms, 0.50);
    out->p99_ms = percentile(s->latencies_ms, 0.99);
    out->max_ms = percentile(s->latencies_ms, 1.0);
    out->elapsed_s = std::chrono::duration<double>(Clock::now() - s->t0).count();
    return TRW_OK;
}

int trw_server_stop(trw_server *s) {
    if (!s) return TRW_ERR_INVALID;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stopping = true;
        s->cv.notify_all();
    }
    s->dispatcher.join();
    for (size_t k = 0; k < s->streams.size(); ++k) cudaStreamSynchronize(s->streams[k]);
    for (auto &kv : s->reqs)
        if (kv.second->dmem) cudaFreeAsync(kv.second->dmem, s->streams[kv.second->stream]);
    for (cudaStream_t st : s->streams) { cudaStreamSynchronize(st); cudaStreamDestroy(st); }
    delete s;
    return TRW_OK;
}

}  // extern "C"
