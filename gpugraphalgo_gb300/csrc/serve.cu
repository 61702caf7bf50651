/*
 * Serving: a request loop over resident graphs with continuous batching.
 *
 * The reference serves nothing: one process answers one source
 * (bfs_sssp.cu:103-539).  A server keeps its graphs resident and runs the
 * batch engine (batch.cu) in supersteps on its own stream.  A superstep
 * ends at the first round in which max(1, in-flight / 8) of its queries
 * have finished -- one under light load, for the shortest turnaround; more
 * under heavy load, so the host round trip between supersteps is paid for
 * several retirements -- or after SUPERSTEP_MAX_ROUNDS rounds, so queries
 * that arrive meanwhile wait a bounded time; the launch itself leaves every slot's
 * remaining queue entries and far items in a pinned array.  Between
 * supersteps the loop
 *   - retires the queries that have none left: their distances are final
 *     (improved-vertex frontier / BFS levels), so they are copied to the
 *     callers' buffers (all copies queued, one wait) and the tickets
 *     complete;
 *   - admits waiting queries while a slot is free and their device state fits:
 *     distances + visited bits or round stamps from a pool, queue room for one
 *     entry per vertex, and unit-table room for their edges.  The pool, the
 *     queue and the unit table are sized once from mem_cap_bytes, so the
 *     server never allocates after creation;
 *   - injects the admitted sources into the next round's queue.
 * A query therefore starts at the next superstep boundary instead of waiting
 * for the batch in flight to drain.
 */
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <string.h>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "batch.cuh"

namespace {

constexpr uint32_t SUPERSTEP_MAX_ROUNDS = 128;
constexpr uint32_t QUEUE_BYTES_PER_VERTEX = 32; /* 4 arrays x 2 buffers x 4 bytes */

struct Request {
    uint64_t ticket;
    uint32_t graph, algo, src;
    uint32_t *out;
    double t_submit;
};

struct Done {
    gga_status status;
    double latency_us;
    std::string msg; /* the server thread's error message when status != GGA_OK */
};

struct Slot {
    bool busy = false;
    Request rq;
    size_t pool_off = 0, pool_words = 0;
    uint32_t n = 0, m = 0;
};

/* First-fit allocator over the state pool (offsets in words). */
struct PoolAlloc {
    std::map<size_t, size_t> free_; /* offset -> words */
    size_t total = 0;
    void init(size_t words) {
        free_.clear();
        total = words;
        if (words) free_[0] = words;
    }
    bool take(size_t words, size_t *off) {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < words) continue;
            *off = it->first;
            const size_t rest = it->second - words, at = it->first + words;
            free_.erase(it);
            if (rest) free_[at] = rest;
            return true;
        }
        return false;
    }
    void give(size_t off, size_t words) {
        auto it = free_.emplace(off, words).first;
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
};

double now_us() {
    return std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

} // namespace

struct gga_server {
    int device = 0;
    std::vector<gga_graph *> graphs;
    std::vector<const DevGraph *> dgraphs;
    std::vector<uint32_t> delta; /* SSSP bucket width per graph */
    uint32_t max_slots = 0;
    cudaStream_t st = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    MqEngine eng;
    uint32_t *pool = nullptr;
    PoolAlloc pa;
    uint64_t edges_cap = 0;
    uint64_t inflight_n = 0, inflight_m = 0, inflight_bytes = 0;
    std::vector<Slot> slots;

    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request> pending;
    std::unordered_map<uint64_t, Done> done;
    uint64_t next_ticket = 1;
    bool stop = false;
    gga_server_stats stats = {};
    std::thread th;
};

namespace {

size_t query_state_bytes(const gga_server *s, uint32_t n, uint32_t m, uint32_t algo) {
    return mq_state_words(n, algo) * 4 + (size_t)n * QUEUE_BYTES_PER_VERTEX + ((size_t)m / 2048 + 1) * 8;
}

void finish(gga_server *s, const Request &rq, gga_status st) {
    Done d;
    d.status = st;
    d.latency_us = now_us() - rq.t_submit;
    if (st != GGA_OK) d.msg = gga_last_error(); /* this thread's message, for the waiting thread */
    std::lock_guard<std::mutex> lk(s->mu);
    s->done[rq.ticket] = d;
    if (st == GGA_OK) s->stats.completed++;
    s->cv_done.notify_all();
}

void release_slot(gga_server *s, uint32_t i) {
    Slot &sl = s->slots[i];
    s->pa.give(sl.pool_off, sl.pool_words);
    s->inflight_n -= sl.n;
    s->inflight_m -= sl.m;
    s->inflight_bytes -= query_state_bytes(s, sl.n, sl.m, sl.rq.algo);
    sl.busy = false;
}

/* Fails every in-flight query with `st` and clears the engine. */
void fail_all(gga_server *s, gga_status st) {
    for (uint32_t i = 0; i < s->max_slots; ++i)
        if (s->slots[i].busy) {
            const Request rq = s->slots[i].rq;
            release_slot(s, i);
            finish(s, rq, st);
        }
    mq_engine_reset(&s->eng, s->st);
    cudaStreamSynchronize(s->st);
}

void server_loop(gga_server *s) {
    cudaSetDevice(s->device);
    std::vector<MqQuery> hq;
    std::vector<uint32_t> hslots;
    for (;;) {
        /* ---- admission */
        hq.clear();
        hslots.clear();
        uint32_t busy = 0;
        for (const Slot &sl : s->slots) busy += sl.busy;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            if (busy == 0)
                s->cv_work.wait(lk, [&] { return s->stop || !s->pending.empty(); });
            if (s->stop) break;
            while (!s->pending.empty()) {
                const Request &rq = s->pending.front();
                const DevGraph *d = s->dgraphs[rq.graph];
                uint32_t slot = UINT32_MAX;
                for (uint32_t i = 0; i < s->max_slots; ++i)
                    if (!s->slots[i].busy) {
                        slot = i;
                        break;
                    }
                if (slot == UINT32_MAX) break;
                if (s->inflight_n + d->n > s->eng.cap || s->inflight_m + d->m > s->edges_cap) break;
                const size_t words = mq_state_words(d->n, rq.algo);
                size_t off = 0;
                if (!s->pa.take(words, &off)) break;
                Slot &sl = s->slots[slot];
                sl.busy = true;
                sl.rq = rq;
                sl.pool_off = off;
                sl.pool_words = words;
                sl.n = d->n;
                sl.m = d->m;
                s->inflight_n += d->n;
                s->inflight_m += d->m;
                s->inflight_bytes += query_state_bytes(s, d->n, d->m, rq.algo);
                s->stats.state_bytes_peak = std::max<uint64_t>(s->stats.state_bytes_peak, s->inflight_bytes);
                MqQuery q;
                memset(&q, 0, sizeof q);
                q.off = d->off;
                q.col = d->col;
                q.wt = d->wt;
                q.n = d->n;
                q.m = d->m;
                q.algo = rq.algo;
                q.src = rq.src;
                q.delta = rq.algo == GGA_SSSP ? s->delta[rq.graph] : 0;
                q.tail_at = q.delta && (uint64_t)d->m >= 8ull * d->n ? d->n / 4 : 0;
                mq_state_layout(&q, s->pool + off);
                hq.push_back(q);
                hslots.push_back(slot);
                s->pending.pop_front();
                ++busy;
            }
            s->stats.max_inflight = std::max(s->stats.max_inflight, busy);
        }
        gga_status st = mq_engine_admit(&s->eng, hq.data(), hslots.data(), (uint32_t)hq.size(), s->st);
        /* ---- one superstep */
        uint32_t rounds = 0;
        const uint32_t stop_after = std::max<uint32_t>(1u, busy / 8);
        if (st == GGA_OK)
            st = mq_engine_run(&s->eng, SUPERSTEP_MAX_ROUNDS, s->st, nullptr, nullptr, &rounds, nullptr, stop_after);
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->stats.supersteps++;
        }
        if (st != GGA_OK) {
            fail_all(s, st);
            continue;
        }
        /* ---- retire finished queries: every copy queued, then one wait */
        std::vector<uint32_t> fin;
        cudaError_t e = cudaSuccess;
        for (uint32_t i = 0; i < s->max_slots; ++i) {
            Slot &sl = s->slots[i];
            if (!sl.busy || s->eng.hactive[i] != 0) continue;
            fin.push_back(i);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(sl.rq.out, s->pool + sl.pool_off, (size_t)sl.n * sizeof(uint32_t),
                                    cudaMemcpyDefault, s->st);
        }
        if (!fin.empty() && e == cudaSuccess) e = cudaStreamSynchronize(s->st);
        for (uint32_t i : fin) {
            const Request rq = s->slots[i].rq;
            const gga_status cs = e == cudaSuccess
                                      ? GGA_OK
                                      : gga_fail(GGA_ERR_CUDA, "server result copy: %s", cudaGetErrorString(e));
            release_slot(s, i);
            finish(s, rq, cs);
        }
    }
    /* stopping: cancel what is left */
    for (uint32_t i = 0; i < s->max_slots; ++i)
        if (s->slots[i].busy) {
            const Request rq = s->slots[i].rq;
            release_slot(s, i);
            finish(s, rq, GGA_ERR_NOT_READY);
        }
    cudaStreamSynchronize(s->st);
}

void server_free(gga_server *s) {
    mq_engine_free(&s->eng);
    cudaFree(s->pool);
    for (int i = 0; i < 2; ++i)
        if (s->ev[i]) cudaEventDestroy(s->ev[i]);
    if (s->st) cudaStreamDestroy(s->st);
    delete s;
}

} // namespace

gga_status gga_server_create(gga_ctx *c, uint32_t ngraphs, gga_graph *const *graphs, uint64_t mem_cap_bytes,
                             uint32_t max_slots, gga_server **out) {
    if (!out) return gga_fail(GGA_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (!c || !graphs || ngraphs == 0) return gga_fail(GGA_ERR_INVALID_ARG, "NULL context or no graphs");
    if (max_slots == 0 || max_slots > 65536) return gga_fail(GGA_ERR_INVALID_ARG, "max_slots %u (1..65536)", max_slots);
    gga_status s;
    {
        std::lock_guard<std::mutex> lk(c->mu);
        if ((s = ctx_activate(c))) return s;
        for (uint32_t i = 0; i < ngraphs; ++i) {
            if (!graphs[i]) return gga_fail(GGA_ERR_INVALID_ARG, "graph %u is NULL", i);
            if ((s = dev_graph_ensure(graphs[i], c->device, c->st))) return s;
        }
    }
    gga_server *sv = new (std::nothrow) gga_server();
    if (!sv) return gga_fail(GGA_ERR_NO_MEMORY, "server");
    sv->device = c->device;
    sv->max_slots = max_slots;
    sv->slots.resize(max_slots);
    uint64_t max_n = 1, max_m = 0;
    for (uint32_t i = 0; i < ngraphs; ++i) {
        sv->graphs.push_back(graphs[i]);
        sv->dgraphs.push_back(dev_graph_of(graphs[i]));
        sv->delta.push_back(ctx_batch_delta(graphs[i]));
        max_n = std::max<uint64_t>(max_n, graphs[i]->n);
        max_m = std::max<uint64_t>(max_m, graphs[i]->m);
    }
    /* split the cap: queue entries (32 B per vertex) and state words (<= 16 B
     * per vertex) in proportion, bounded by what max_slots queries could use */
    const uint64_t budget = mem_cap_bytes;
    uint64_t cap = std::min<uint64_t>(budget * 2 / 3 / QUEUE_BYTES_PER_VERTEX, (uint64_t)max_slots * max_n);
    cap = std::min<uint64_t>(cap, 0xFFFFFFF0ull);
    /* SSSP state is the largest: distances, stamps, far bitmap, two piles */
    uint64_t pool_words = std::min<uint64_t>(budget / 3 / 4, (uint64_t)max_slots * (4 * max_n + 320));
    sv->edges_cap = std::min<uint64_t>((uint64_t)max_slots * max_m, 0xFFFFFFFFull - 2 * 2048 - 1);
    if (cap < 1 || pool_words < 128) {
        server_free(sv);
        return gga_fail(GGA_ERR_ADMISSION, "mem_cap_bytes %llu too small", (unsigned long long)mem_cap_bytes);
    }
    cudaError_t e = cudaSetDevice(sv->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&sv->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&sv->ev[0]);
    if (e == cudaSuccess) e = cudaEventCreate(&sv->ev[1]);
    if (e == cudaSuccess) e = cudaMalloc((void **)&sv->pool, pool_words * 4);
    if (e != cudaSuccess) {
        cudaGetLastError();
        server_free(sv);
        return gga_fail(GGA_ERR_CUDA, "server setup: %s", cudaGetErrorString(e));
    }
    sv->pa.init(pool_words);
    if ((s = mq_engine_reserve(&sv->eng, sv->device, (uint32_t)cap, sv->edges_cap, max_slots)) ||
        (s = mq_engine_reset(&sv->eng, sv->st))) {
        server_free(sv);
        return s;
    }
    /* after reserve, which starts a fresh engine on its first call */
    sv->eng.nslots = max_slots;
    e = cudaStreamSynchronize(sv->st);
    if (e != cudaSuccess) {
        server_free(sv);
        return gga_fail(GGA_ERR_CUDA, "server setup: %s", cudaGetErrorString(e));
    }
    try {
        sv->th = std::thread(server_loop, sv);
    } catch (...) {
        server_free(sv);
        return gga_fail(GGA_ERR_NO_MEMORY, "server thread");
    }
    *out = sv;
    return GGA_OK;
}

gga_status gga_server_submit(gga_server *s, uint32_t graph_index, gga_algo algo, uint32_t src, uint32_t *dist_out,
                             uint64_t *ticket) {
    if (!s || !dist_out || !ticket) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    if (graph_index >= s->graphs.size())
        return gga_fail(GGA_ERR_INVALID_ARG, "graph index %u of %zu", graph_index, s->graphs.size());
    gga_graph *g = s->graphs[graph_index];
    gga_status st = ctx_validate_solve(g, algo, src);
    if (st) return st;
    const DevGraph *d = s->dgraphs[graph_index];
    std::lock_guard<std::mutex> lk(s->mu);
    if (d->n > s->eng.cap || d->m > s->edges_cap || mq_state_words(d->n, algo) > s->pa.total) {
        s->stats.rejected++;
        return gga_fail(GGA_ERR_ADMISSION, "query state for %u vertices exceeds the server's memory cap", d->n);
    }
    Request rq;
    rq.ticket = s->next_ticket++;
    rq.graph = graph_index;
    rq.algo = algo;
    rq.src = src;
    rq.out = dist_out;
    rq.t_submit = now_us();
    s->pending.push_back(rq);
    s->stats.submitted++;
    *ticket = rq.ticket;
    s->cv_work.notify_one();
    return GGA_OK;
}

gga_status gga_server_wait(gga_server *s, uint64_t ticket, uint32_t timeout_ms, double *latency_us) {
    if (!s) return gga_fail(GGA_ERR_INVALID_ARG, "NULL server");
    std::unique_lock<std::mutex> lk(s->mu);
    if (ticket == 0 || ticket >= s->next_ticket) return gga_fail(GGA_ERR_INVALID_ARG, "unknown ticket %llu",
                                                                 (unsigned long long)ticket);
    auto ready = [&] { return s->done.count(ticket) != 0; };
    if (!ready()) {
        if (timeout_ms == 0 || !s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready))
            return gga_fail(GGA_ERR_NOT_READY, "ticket %llu still running", (unsigned long long)ticket);
    }
    const Done d = s->done[ticket];
    s->done.erase(ticket);
    if (latency_us) *latency_us = d.latency_us;
    if (d.status != GGA_OK)
        return gga_fail(d.status, "ticket %llu failed: %s", (unsigned long long)ticket, d.msg.c_str());
    return GGA_OK;
}

gga_status gga_server_get_stats(gga_server *s, gga_server_stats *out) {
    if (!s || !out) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
    return GGA_OK;
}

void gga_server_destroy(gga_server *s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv_work.notify_all();
    }
    if (s->th.joinable()) s->th.join();
    cudaSetDevice(s->device);
    server_free(s);
}
