// trw_server.cu -- request loop over a resident graph (continuous batching).
//
// The reference runs one compute() per process (creeper_main.h:14-72); this
// loop keeps the graph and its sampling tables resident in HBM and serves a
// stream of walk requests of different apps and sizes.
//
// A dispatcher thread forms batches: whenever one of `max_inflight` streams
// is free it takes every queued request, in arrival order, whose device
// memory still fits the HBM budget, and runs them as one batch
// (trw::batch_walk): the walkers of all its requests that use the same
// kernel share one persistent launch and one work queue of walker chunks (the
// admission of creeper.h:321-332 over many requests), so a small request
// runs beside the others instead of occupying a launch of its own.  Batches
// on different streams overlap on the device, so requests that arrive while
// a batch runs start in the next one at once.
//
// Completion: a request whose walkers ran in a shared launch is finished when
// its last walker is (the device raises the request's flag in host-mapped
// memory and the dispatcher, polling every 20 us, timestamps it); the others
// (PPR post-processing, requests that need a launch of their own) when their
// stream reaches a host function enqueued after their work.  Latency =
// completion - submit.  Every walk is a pure function of (seed, walker, step),
// so a request's result does not depend on what it ran beside.
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
#include "trw_batch.h"

namespace {

using Clock = std::chrono::steady_clock;
constexpr int kMaxFlags = 1 << 16;     // completion flags (requests in flight at once)
constexpr int kMaxBatch = 1024;        // requests per batch

struct Request {
    trw_server *srv = nullptr;
    uint64_t ticket = 0;
    trw_request req{};
    std::vector<int32_t> schema, sources;
    size_t bytes = 0;          // device bytes held until release
    void *dmem = nullptr;
    int32_t *d_src = nullptr, *d_paths = nullptr, *d_len = nullptr, *d_vert = nullptr, *d_cnt = nullptr;
    int32_t *d_table = nullptr, *d_dist = nullptr;
    int32_t bits = 0;          // single-query PPR: table size
    int64_t *d_off = nullptr;
    uint64_t *d_steps = nullptr;
    int64_t capacity = 0;      // sparse PPR entries
    int stream = -1;
    int flag = -1;             // host-mapped completion flag (shared launches)
    Clock::time_point t_submit, t_start;
    std::atomic<int64_t> done_ns{0};  // completion time (ns since submit), 0 = running
    int status = 0;            // 0 queued, 1 running, 2 done, 3 failed
    std::string error;
};

// A batch's stream is free again once its last host function has run.
struct Batch {
    trw_server *srv = nullptr;
    int stream = -1;
    std::atomic<int> finished{0};
};

}  // namespace

struct trw_server {
    trw_graph *g = nullptr;
    int32_t n = 0;
    size_t budget = 0, in_use = 0;
    std::vector<cudaStream_t> streams;
    std::vector<char> stream_busy;
    std::vector<std::unique_ptr<Batch>> batches;  // one per stream
    std::deque<std::shared_ptr<Request>> queue;
    std::unordered_map<uint64_t, std::shared_ptr<Request>> reqs;
    std::vector<std::shared_ptr<Request>> running;
    int32_t *flags = nullptr;       // pinned, mapped: kMaxFlags completion flags
    int32_t *flags_dev = nullptr;   // their device address
    std::vector<int> free_flags;
    std::mutex mu;
    std::condition_variable cv;
    std::thread dispatcher;
    bool stopping = false;
    uint64_t next_ticket = 1;
    int32_t max_queue = 1 << 16;
    // statistics
    uint64_t submitted = 0, completed = 0, failed = 0, steps = 0, launched_batches = 0;
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

void CUDART_CB on_batch_end(void *arg) {
    auto *b = static_cast<Batch *>(arg);
    b->finished.store(1);
    b->srv->cv.notify_all();
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

bool single_ppr(const trw_request &q) { return q.walkers_per_query > 0 && q.num_queries == 1; }

// Device bytes a request holds: sources, outputs, the step counter and, for
// a single-query PPR request, its visit table and post-processing scratch.
void size_request(trw_server *s, Request &r) {
    const trw_request &q = r.req;
    size_t b = align256(sizeof(int32_t) * (size_t)std::max<int64_t>(1, r.sources.size()));
    b += align256(sizeof(uint64_t));
    if (q.walkers_per_query > 0) {
        const double visits = (double)q.walkers_per_query / std::max(1e-6, q.desc.tp);
        r.capacity = std::min<int64_t>((int64_t)s->n, (int64_t)(1.25 * visits) + 1024) * (int64_t)r.sources.size();
        b += align256(sizeof(int64_t) * (r.sources.size() + 1)) + 2 * align256(sizeof(int32_t) * (size_t)r.capacity);
        if (single_ppr(q)) {
            r.bits = trw::batch_ppr_bits(s->g, q.walkers_per_query, q.desc.tp);
            b += align256(sizeof(int32_t) * 2 * ((size_t)1 << r.bits));
            b += align256(sizeof(int32_t) * (size_t)trw::batch_ppr_distinct_ints(r.bits));
        }
    } else {
        b += align256(sizeof(int32_t) * (size_t)q.num_walkers);
        if (q.path_cap > 0) b += align256(sizeof(int32_t) * (size_t)q.num_walkers * (size_t)q.path_cap);
    }
    r.bytes = b;
}

// Carves a request's device memory and enqueues its input copy and the
// zeroing of its counters (called with the server lock held).
bool stage_request(trw_server *s, Request &r, cudaStream_t st) {
    r.t_start = Clock::now();
    r.status = 1;
    if (cudaMallocAsync(&r.dmem, r.bytes, st) != cudaSuccess) {
        cudaGetLastError();
        r.status = 3;
        r.error = "device allocation failed";
        return false;
    }
    char *p = static_cast<char *>(r.dmem);
    auto carve = [&](size_t bytes) { char *q = p; p += align256(bytes); return q; };
    r.d_src = reinterpret_cast<int32_t *>(carve(sizeof(int32_t) * std::max<size_t>(1, r.sources.size())));
    r.d_steps = reinterpret_cast<uint64_t *>(carve(sizeof(uint64_t)));
    cudaMemcpyAsync(r.d_src, r.sources.data(), sizeof(int32_t) * r.sources.size(), cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(r.d_steps, 0, sizeof(uint64_t), st);
    r.req.desc.schema = r.schema.empty() ? nullptr : r.schema.data();
    if (r.req.walkers_per_query > 0) {
        r.d_off = reinterpret_cast<int64_t *>(carve(sizeof(int64_t) * (r.sources.size() + 1)));
        r.d_vert = reinterpret_cast<int32_t *>(carve(sizeof(int32_t) * (size_t)r.capacity));
        r.d_cnt = reinterpret_cast<int32_t *>(carve(sizeof(int32_t) * (size_t)r.capacity));
        if (single_ppr(r.req)) {
            const size_t tb = sizeof(int32_t) * 2 * ((size_t)1 << r.bits);
            r.d_table = reinterpret_cast<int32_t *>(carve(tb));
            r.d_dist = reinterpret_cast<int32_t *>(carve(sizeof(int32_t) * (size_t)trw::batch_ppr_distinct_ints(r.bits)));
            cudaMemsetAsync(r.d_table, 0, tb, st);
        }
    } else {
        r.d_len = reinterpret_cast<int32_t *>(carve(sizeof(int32_t) * (size_t)r.req.num_walkers));
        if (r.req.path_cap > 0)
            r.d_paths = reinterpret_cast<int32_t *>(carve(sizeof(int32_t) * (size_t)r.req.num_walkers * r.req.path_cap));
    }
    (void)s;
    return true;
}

// Launches one batch on stream k (called with the server lock held).
void launch_batch(trw_server *s, int k, std::vector<std::shared_ptr<Request>> &batch) {
    cudaStream_t st = s->streams[(size_t)k];
    std::vector<trw::BatchItem> items;
    std::vector<Request *> item_req;   // request of each batch item
    std::vector<Request *> separate;   // multi-query PPR requests: trw_ppr_batch_sparse
    for (auto &rp : batch) {
        Request &r = *rp;
        r.stream = k;
        if (!stage_request(s, r, st)) continue;
        if (r.req.walkers_per_query > 0 && !single_ppr(r.req)) { separate.push_back(&r); continue; }
        trw::BatchItem it{};
        it.desc = r.req.desc;
        it.sources = r.d_src;
        it.steps = r.d_steps;
        if (single_ppr(r.req)) {  // every walker starts at the request's one source
            it.num_walkers = r.req.walkers_per_query;
            it.per_query = r.req.walkers_per_query;
            it.id_base = 0;
            it.table = r.d_table;
            it.table_bits = r.bits;
            it.offsets = r.d_off;
            it.vertices = r.d_vert;
            it.counts = r.d_cnt;
            it.capacity = r.capacity;
            it.distinct = r.d_dist;
        } else {
            it.num_walkers = r.req.num_walkers;
            it.id_base = r.req.id_base;
            it.paths = r.d_paths;
            it.path_cap = r.req.path_cap;
            it.lengths = r.d_len;
        }
        if (!s->free_flags.empty()) {
            r.flag = s->free_flags.back();
            s->free_flags.pop_back();
            s->flags[r.flag] = 0;
            it.done = s->flags_dev + r.flag;
        }
        items.push_back(it);
        item_req.push_back(&r);
    }
    std::vector<int> host_done;
    const int rc = items.empty() ? TRW_OK : trw::batch_walk(s->g, items, st, host_done);
    if (rc != TRW_OK) {
        for (Request *r : item_req) { r->status = 3; r->error = trw_last_error(); }
    } else {
        for (int i : host_done) cudaLaunchHostFunc(st, on_complete, item_req[(size_t)i]);
    }
    for (Request *r : separate) {
        const int prc = trw_ppr_batch_sparse(s->g, &r->req.desc, r->d_src, (int64_t)r->sources.size(),
                                             r->req.walkers_per_query, r->d_off, r->d_vert, r->d_cnt, r->capacity,
                                             r->d_steps, TRW_ENGINE_PERSISTENT, reinterpret_cast<trw_stream_t>(st));
        if (prc != TRW_OK) { r->status = 3; r->error = trw_last_error(); continue; }
        cudaLaunchHostFunc(st, on_complete, r);
    }
    Batch &b = *s->batches[(size_t)k];
    b.finished.store(0);
    cudaLaunchHostFunc(st, on_batch_end, &b);
    s->stream_busy[(size_t)k] = 1;
    ++s->launched_batches;
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
        // completions: device flags of shared launches, host functions of the rest
        for (size_t i = 0; i < s->running.size();) {
            Request &r = *s->running[i];
            if (r.flag >= 0 && r.done_ns.load() == 0 && reinterpret_cast<volatile int32_t *>(s->flags)[r.flag]) {
                const int64_t ns =
                    std::chrono::duration_cast<std::chrono::nanoseconds>(Clock::now() - r.t_submit).count();
                r.done_ns.store(ns > 0 ? ns : 1);
            }
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
                if (r.flag >= 0) { s->free_flags.push_back(r.flag); r.flag = -1; }
                s->running.erase(s->running.begin() + (long)i);
                s->cv.notify_all();
            } else {
                ++i;
            }
        }
        for (size_t k = 0; k < s->streams.size(); ++k)
            if (s->stream_busy[k] && s->batches[k]->finished.load()) s->stream_busy[k] = 0;
        // admissions, in arrival order: every queued request that fits goes
        // into one batch on a free stream
        if (!s->queue.empty()) {
            int free_stream = -1;
            for (size_t k = 0; k < s->streams.size(); ++k)
                if (!s->stream_busy[k]) { free_stream = (int)k; break; }
            if (free_stream >= 0) {
                std::vector<std::shared_ptr<Request>> batch;
                while (!s->queue.empty() && (int)batch.size() < kMaxBatch && (int)s->free_flags.size() > (int)batch.size()) {
                    Request &r = *s->queue.front();
                    if (s->in_use + r.bytes > s->budget) break;
                    s->in_use += r.bytes;
                    batch.push_back(s->queue.front());
                    s->queue.pop_front();
                }
                if (!batch.empty()) {
                    launch_batch(s, free_stream, batch);
                    for (auto &r : batch) s->running.push_back(r);
                }
            }
        }
        if (s->stopping && s->queue.empty() && s->running.empty()) break;
        s->cv.wait_for(lock, std::chrono::microseconds(s->running.empty() ? 2000 : 20));
    }
}

}  // namespace

extern "C" {

int trw_server_start(trw_graph *g, size_t hbm_budget_bytes, int32_t max_inflight, trw_server **out) {
    if (!g || !out || max_inflight <= 0 || max_inflight > 64) return TRW_ERR_INVALID;
    auto *s = new trw_server();
    s->g = g;
    trw_graph_info(g, &s->n, nullptr, nullptr);
    if (hbm_budget_bytes == 0) {
        size_t free_b = 0, total_b = 0;
        cudaMemGetInfo(&free_b, &total_b);
        hbm_budget_bytes = free_b / 10 * 8;  // 80 % of what is free now
    }
    s->budget = hbm_budget_bytes;
    auto bail = [&]() {
        for (cudaStream_t x : s->streams) cudaStreamDestroy(x);
        if (s->flags) cudaFreeHost(s->flags);
        delete s;
        return TRW_ERR_CUDA;
    };
    for (int i = 0; i < max_inflight; ++i) {
        cudaStream_t st;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return bail();
        s->streams.push_back(st);
        s->batches.push_back(std::make_unique<Batch>());
        s->batches.back()->srv = s;
        s->batches.back()->stream = i;
    }
    if (cudaHostAlloc(reinterpret_cast<void **>(&s->flags), sizeof(int32_t) * kMaxFlags, cudaHostAllocMapped) !=
            cudaSuccess ||
        cudaHostGetDevicePointer(reinterpret_cast<void **>(&s->flags_dev), s->flags, 0) != cudaSuccess)
        return bail();
    std::memset(s->flags, 0, sizeof(int32_t) * kMaxFlags);
    for (int i = kMaxFlags - 1; i >= 0; --i) s->free_flags.push_back(i);
    s->stream_busy.assign((size_t)max_inflight, 0);
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
    size_request(s, *r);
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
        // a single-query request finished when its post-processing did (its stream's host function)
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
    // stream-ordered: freed once the request's batch has left the stream
    if (r.dmem) cudaFreeAsync(r.dmem, s->streams[(size_t)r.stream]);
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
    out->batches = s->launched_batches;
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
        if (kv.second->dmem) cudaFreeAsync(kv.second->dmem, s->streams[(size_t)kv.second->stream]);
    for (cudaStream_t st : s->streams) { cudaStreamSynchronize(st); cudaStreamDestroy(st); }
    cudaFreeHost(s->flags);
    delete s;
    return TRW_OK;
}

}  // extern "C"
