/*
 * Frontier engine: single-source BFS and SSSP as ONE persistent cooperative
 * kernel per query.
 *
 * Same answers as the reference's fixed-point loop (bfs_sssp.cu:372-468
 * around M_my_drelax, cudaKernels.h:285-344), which rescans every vertex and
 * edge each iteration with one host round trip per iteration.  Here:
 *   - the frontier is data driven: only vertices whose distance changed are
 *     expanded (BFS: level synchronous; SSSP: near-far buckets of width
 *     `delta`, or a plain improved-vertex frontier when delta = 0);
 *   - expansion is EDGE balanced: every queued vertex carries the exclusive
 *     offset of its edge range in the round's concatenated edge list, and
 *     the list is cut into fixed units of U = block_threads * unit_iters
 *     edges.  Units are dealt round-robin to the CTAs; a CTA loads its
 *     unit's queue entries into shared memory and walks the unit with
 *     consecutive threads on consecutive edges (coalesced), so a
 *     10^5-degree R-MAT hub is spread over many CTAs like any other edges;
 *   - pushes are staged per CTA in shared memory (shared atomics only) and
 *     published once per unit with ONE 64-bit atomicAdd that allocates queue
 *     slots and edge offsets together; the same flush marks the next round's
 *     unit boundaries, so no separate scan pass is needed;
 *   - deduplication: BFS by a visited bitmap, SSSP by a per-vertex round
 *     stamp (near queue) and a "far pile" bitmap;
 *   - relaxation is atomicMin on uint32 distances, as the reference does;
 *   - rounds are separated by a bounded grid barrier (no host round trip);
 *     a barrier that waits past its limit sets an error word and the kernel
 *     returns, so the host gets GGA_ERR_TIMEOUT instead of a hung GPU.
 * Synchronisation is block-uniform by construction: no warp collective is
 * reached under data-dependent control flow, and every __syncthreads is
 * reached by all threads of the CTA after decisions read from shared memory.
 * On a node-split graph (graph.h:415-522) the engine walks the split view:
 * edges target parents, reaching a parent reaches its children too (their
 * distances mirror the parent's, cudaKernels.h:326-330), and a parent's
 * queue entry covers its own and its children's contiguous edge slices.
 */
#include <stdio.h>
#include <string.h>
#include <mutex>


#include "frontier.cuh"

namespace {

constexpr uint32_t NONE = 0xffffffffu;
constexpr uint32_t MIN_UNIT = 512;  /* smallest edges-per-unit the buffers are sized for */
constexpr uint32_t MAX_UNIT = 4096; /* largest edges-per-unit (shared-memory bound) */
constexpr uint32_t STAGE_BATCH = 4; /* edges per thread in flight between staging checkpoints */
constexpr uint32_t BU_WORDS = 4;    /* bottom-up BFS: visited-bitmap words per warp step */
constexpr uint32_t BU_NBRS = 4;     /* bottom-up BFS: neighbours a lane checks per vertex per step */

struct Args {
    const uint32_t *off, *col, *wt, *cc;
    const uint32_t *first; /* split view: original -> parent split id */
    uint32_t n, m;
    uint32_t *dist, *bits, *farbits, *stamp;
    uint32_t *qv0, *qv1, *qo0, *qo1, *qb0, *qb1, *uf0, *uf1;
    uint32_t *far0, *far1, *far2;
    FrontierCtl *ctl;
    uint32_t cap;  /* queue entries */
    uint32_t ucap; /* unit-boundary entries */
    uint32_t src;
    uint32_t unit;  /* edges per unit = BS * iters */
    uint32_t iters; /* CTA-wide iterations per unit */
    uint32_t scap;  /* staging slots per CTA (>= BS * (STAGE_BATCH + 1)) */
    uint32_t delta;
    uint32_t nblocks;
    uint32_t max_rounds;
    unsigned long long timeout_ns;
    uint32_t bu;          /* BFS: bottom-up rounds allowed (symmetric, unsplit) */
    uint32_t alpha, beta; /* direction rule */
    uint32_t *trace;      /* NULL, or TRACE_ROUNDS x 4 round records then per-CTA busy kilocycles */
    /* SSSP light/heavy mode (delta-stepping edge classes), when light != NULL:
     * rows are ordered light (w < delta) first; near entries cover a vertex's
     * light edges; its heavy edges go once per bucket to a heavy list that is
     * expanded when the bucket closes.  Three heavy lists rotate by bucket. */
    const uint32_t *light; /* n: light edges per row */
    uint32_t *hstamp;      /* n: last bucket (+1) a vertex joined a heavy list */
    uint32_t *hv0, *hv1, *hv2, *ho0, *ho1, *ho2, *hb0, *hb1, *hb2, *huf0, *huf1, *huf2;
    /* bucket closes by pull (every edge's reverse has its weight): 0 never,
     * 1 when the cost rule picks it, 2 always */
    uint32_t pull;
    uint32_t *pbest; /* cap: per pull-list entry, the smallest offer its edges found (NONE: none) */
    uint32_t cw;     /* light/heavy rows: width of the heavy-edge weight classes (0: rows not class-ordered) */
    uint32_t heavy_edges; /* edges with w >= delta */
    /* SSSP: when a bucket opens with at most this many far-pile entries, the
     * threshold goes to infinity and the rest runs as one label-correcting
     * frontier over whole rows (0: never) */
    uint32_t tail_at;
};

/* Round record (block 0, thread 0) when tracing. */
__device__ __forceinline__ void trace_round(const Args &a, uint32_t round, uint32_t kind, uint32_t items,
                                            uint32_t edges, uint32_t far_items) {
    if (a.trace && blockIdx.x == 0 && threadIdx.x == 0 && round < TRACE_ROUNDS) {
        uint32_t *r = a.trace + (size_t)round * TRACE_REC;
        r[0] = kind;
        r[1] = items;
        r[2] = edges;
        r[3] = far_items;
    }
}

/* Round start time (block 0, thread 0) when tracing; round TRACE_ROUNDS'
 * slot and the one after the last round hold the end time. */
__device__ __forceinline__ void trace_time(const Args &a, uint32_t round) {
    if (a.trace && blockIdx.x == 0 && threadIdx.x == 0 && round <= TRACE_ROUNDS) {
        const unsigned long long t = global_timer_ns();
        uint32_t *r = a.trace + (size_t)round * TRACE_REC;
        r[4] = (uint32_t)t;
        r[5] = (uint32_t)(t >> 32);
    }
}

__device__ __forceinline__ uint32_t *sel(uint32_t p, uint32_t *a, uint32_t *b) { return p ? b : a; }
__device__ __forceinline__ uint32_t *sel3(uint32_t p, uint32_t *a, uint32_t *b, uint32_t *c) {
    return p == 0 ? a : (p == 1 ? b : c);
}

__device__ __forceinline__ void set_err(FrontierCtl *c, uint32_t code) { atomicCAS(&c->err, GGA_DEV_OK, code); }

/* Edge range of queue entry v: its own slice plus its split children's. */
__device__ __forceinline__ void item_range(const Args &a, uint32_t v, uint32_t &beg, uint32_t &deg) {
    beg = __ldg(a.off + v);
    const uint32_t last = a.cc ? v + a.cc[v] : v;
    deg = __ldg(a.off + last + 1) - beg;
}

/* Shared-memory layout of one CTA (dynamic shared memory):
 *   table : t_o[U+1], t_b[U+1] (+ t_du[U+1] for SSSP)   the unit's queue entries
 *   stage : sv[scap], sb[scap], sd[scap] (+ sf[scap])     staged pushes
 * Staging uses shared-memory atomics only; every collective step (flushes,
 * scans, the unit table) is entered by the whole CTA under block-uniform
 * control flow decided from shared memory after a __syncthreads. */
struct Ctrl {
    uint32_t nn, fn, fmin;   /* staged near / far counts, smallest far distance */
    uint32_t base_i, base_e; /* flush allocation */
    uint32_t nitems, total, fc, fm;
    uint32_t full; /* SSSP tail: near entries cover whole rows, no heavy lists */
    uint32_t hbase_i, hbase_e, hn, htot; /* heavy list: flush allocation, size at round start */
    uint32_t ws[32];         /* block-scan scratch */
    unsigned long long ws64[32];
};

/* Stage a near-queue vertex (any thread, any time between flushes); its
 * edge range is looked up when the stage is published. */
__device__ __forceinline__ void stage_near(const Args &a, Ctrl &C, uint32_t *sv, uint32_t v) {
    const uint32_t k = atomicAdd(&C.nn, 1u);
    if (k < a.scap) sv[k] = v;
    else set_err(a.ctl, GGA_DEV_OVERFLOW);
}

__device__ __forceinline__ void stage_far(const Args &a, Ctrl &C, uint32_t *sf, uint32_t v) {
    const uint32_t k = atomicAdd(&C.fn, 1u);
    if (k < a.scap) sf[k] = v;
    else set_err(a.ctl, GGA_DEV_OVERFLOW_FAR);
}

/* Publish the CTA's staged near-queue vertices.  Each thread takes a chunk
 * of the stage, reads the row offsets of its vertices (kept out of the edge
 * loop, whose dependent chain they would lengthen) and drops those without
 * edges; a block scan of (count << 32 | edges) pairs and ONE 64-bit atomicAdd
 * allocate queue slots (high word) and edge offsets (low word) together;
 * each thread then writes its entries and the unit boundaries k*U that fall
 * inside them, reading the (L1-resident) offsets again instead of keeping
 * them in shared memory.  In light/heavy mode a near entry covers the
 * vertex's light edges, and the vertex's heavy edges join the bucket's heavy
 * list once per bucket (second scan and allocation, same layout); the stage
 * keeps that "first time in this bucket" mark in bit 31 of the vertex id
 * (ids are below 2^31).  Called by every thread of the CTA with the same nn
 * (read from shared memory between two __syncthreads); no thread stages
 * while it runs. */
constexpr uint32_t HEAVY_MARK = 0x80000000u;

__device__ __forceinline__ void put_entry(const Args &a, uint32_t i, uint32_t o, uint32_t v, uint32_t b, uint32_t d,
                                          uint32_t *qv, uint32_t *qo, uint32_t *qb, uint32_t *uf) {
    if (i >= a.cap) {
        set_err(a.ctl, GGA_DEV_OVERFLOW);
        return;
    }
    qv[i] = v;
    qo[i] = o;
    qb[i] = b;
    /* unit boundaries inside [o, o + d): this entry holds edge k*U */
    for (uint64_t k = ((uint64_t)o + a.unit - 1) / a.unit; k * a.unit < (uint64_t)o + d; ++k) {
        if (k < a.ucap) uf[k] = i;
        else set_err(a.ctl, GGA_DEV_OVERFLOW_UNITS);
    }
}

template <int BS>
__device__ __forceinline__ void flush_near(const Args &a, Ctrl &C, uint32_t *sv, uint32_t nn, uint32_t nxt,
                                           uint32_t r3n, uint32_t bucket) {
    if (nn == 0) return;
    const uint32_t tid = threadIdx.x;
    const bool lh = a.light != nullptr && !C.full; /* the same in every thread */
    const uint32_t hl = bucket % 3;
    const uint32_t chunk = (nn + BS - 1) / BS;
    const uint32_t j0 = min(tid * chunk, nn), j1 = min(j0 + chunk, nn);
    unsigned long long local = 0, hlocal = 0;
    for (uint32_t j = j0; j < j1; ++j) {
        const uint32_t v = sv[j];
        uint32_t b, d;
        item_range(a, v, b, d);
        const uint32_t dl = lh ? __ldg(a.light + v) : d;
        if (dl) local += (1ull << 32) | dl;
        if (lh) {
            const uint32_t hd = d - dl;
            if (hd && atomicExch(a.hstamp + v, bucket + 1) != bucket + 1) {
                hlocal += (1ull << 32) | hd;
                sv[j] = v | HEAVY_MARK;
            }
        }
    }
    unsigned long long tot, htot = 0;
    unsigned long long run = block_exclusive_scan64(local, C.ws64, &tot);
    unsigned long long hrun = 0;
    if (lh) hrun = block_exclusive_scan64(hlocal, C.ws64, &htot);
    if (tid == 0) {
        const unsigned long long old = tot ? atomicAdd(&a.ctl->qctr[r3n], tot) : 0ull;
        C.base_i = (uint32_t)(old >> 32);
        C.base_e = (uint32_t)old;
        const unsigned long long hold = htot ? atomicAdd(&a.ctl->hctr[hl], htot) : 0ull;
        C.hbase_i = (uint32_t)(hold >> 32);
        C.hbase_e = (uint32_t)hold;
    }
    __syncthreads();
    const uint32_t bi = C.base_i, be = C.base_e, hbi = C.hbase_i, hbe = C.hbase_e;
    uint32_t *qv = sel(nxt, a.qv0, a.qv1), *qo = sel(nxt, a.qo0, a.qo1), *qb = sel(nxt, a.qb0, a.qb1);
    uint32_t *uf = sel(nxt, a.uf0, a.uf1);
    for (uint32_t j = j0; j < j1; ++j) {
        const uint32_t raw = sv[j], v = raw & ~HEAVY_MARK;
        uint32_t b, d;
        item_range(a, v, b, d);
        const uint32_t dl = lh ? __ldg(a.light + v) : d;
        if (dl) {
            put_entry(a, bi + (uint32_t)(run >> 32), be + (uint32_t)run, v, b, dl, qv, qo, qb, uf);
            run += (1ull << 32) | dl;
        }
        if (raw & HEAVY_MARK) { /* heavy edges start after the light ones */
            const uint32_t hd = d - dl;
            put_entry(a, hbi + (uint32_t)(hrun >> 32), hbe + (uint32_t)hrun, v, b + dl, hd,
                      sel3(hl, a.hv0, a.hv1, a.hv2), sel3(hl, a.ho0, a.ho1, a.ho2), sel3(hl, a.hb0, a.hb1, a.hb2),
                      sel3(hl, a.huf0, a.huf1, a.huf2));
            hrun += (1ull << 32) | hd;
        }
    }
    __syncthreads();
    if (tid == 0) C.nn = 0;
    __syncthreads();
}

/* Publish the CTA's staged far-pile entries (same calling rules). */
template <int BS>
__device__ __forceinline__ void flush_far(const Args &a, Ctrl &C, uint32_t *sf, uint32_t fn, uint32_t fp) {
    if (fn == 0) return;
    const uint32_t tid = threadIdx.x;
    if (tid == 0) C.base_i = atomicAdd(&a.ctl->far_count[fp], fn);
    __syncthreads();
    const uint32_t base = C.base_i;
    uint32_t *pile = sel3(fp, a.far0, a.far1, a.far2);
    for (uint32_t j = tid; j < fn; j += BS) {
        if (base + j < a.cap) pile[base + j] = sf[j];
        else set_err(a.ctl, GGA_DEV_OVERFLOW_FAR);
    }
    __syncthreads();
    if (tid == 0) C.fn = 0;
    __syncthreads();
}

/* Block-uniform checkpoint: wait for all staging, read the counts, and
 * publish a buffer when it is at least `limit` full (limit 1 = always). */
struct Stage {
    uint32_t *sv, *sf; /* staged near-queue vertices, far-pile vertices */
};

template <int BS, bool SSSP>
__device__ __forceinline__ void checkpoint(const Args &a, Ctrl &C, const Stage &S, uint32_t nxt, uint32_t r3n,
                                           uint32_t fp, uint32_t bucket, uint32_t limit) {
    __syncthreads();
    const uint32_t nn = C.nn, fn = SSSP ? C.fn : 0u;
    __syncthreads();
    if (nn >= limit) flush_near<BS>(a, C, S.sv, nn, nxt, r3n, bucket);
    if (SSSP && fn >= limit) flush_far<BS>(a, C, S.sf, fn, fp);
}

/* One bottom-up BFS round (Beamer, Asanovic, Patterson, SC 2012): every
 * unvisited vertex looks through its neighbours for one at level `round`
 * (dist == round marks the frontier exactly: later levels are round + 1 or
 * unset) and stops at the first.  A warp owns BU_WORDS 32-vertex words of
 * the visited bitmap per step, lane i vertices 32w + i of each; the warp's
 * finds are written back as whole words and appended to the next round's
 * queue with one packed 64-bit atomicAdd, so the queue has the same format
 * as after a top-down round.  Needs every edge's reverse (a symmetric graph).  The loop
 * trip count is warp-uniform; the per-lane neighbour scan reconverges before
 * the ballot. */
template <int BS>
__device__ __forceinline__ void bottom_up_round(const Args &a, uint32_t round, uint32_t nxt, uint32_t r3n,
                                                unsigned long long &relaxed) {
    constexpr unsigned FULL = 0xffffffffu;
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t gw = ((uint64_t)blockIdx.x * BS + threadIdx.x) >> 5, nw = ((uint64_t)gridDim.x * BS) >> 5;
    const uint32_t nwords = (a.n + 31) / 32;
    uint32_t *qv = sel(nxt, a.qv0, a.qv1), *qo = sel(nxt, a.qo0, a.qo1), *qb = sel(nxt, a.qb0, a.qb1);
    uint32_t *uf = sel(nxt, a.uf0, a.uf1);
    /* NW words per warp step: their loads and neighbour scans are in flight
     * together, and their finds share one queue allocation */
    constexpr uint32_t NW = BU_WORDS;
    for (uint64_t w0 = gw * NW; w0 < nwords; w0 += nw * NW) {
        uint32_t vw[NW], v[NW], b[NW], e1[NW], cur[NW];
        bool open[NW], found[NW];
#pragma unroll
        for (uint32_t k = 0; k < NW; ++k) {
            const uint64_t wk = w0 + k;
            vw[k] = wk < nwords ? __ldcg(a.bits + wk) : FULL;
            v[k] = (uint32_t)wk * 32u + lane;
            open[k] = wk < nwords && v[k] < a.n && !(vw[k] & (1u << lane));
            found[k] = false;
            b[k] = e1[k] = 0;
        }
#pragma unroll
        for (uint32_t k = 0; k < NW; ++k)
            if (open[k]) {
                b[k] = __ldg(a.off + v[k]);
                e1[k] = __ldg(a.off + v[k] + 1);
            }
#pragma unroll
        for (uint32_t k = 0; k < NW; ++k) cur[k] = b[k];
        for (;;) { /* per lane; the lanes reconverge before the ballots */
            bool act[NW], any = false;
#pragma unroll
            for (uint32_t k = 0; k < NW; ++k) {
                act[k] = open[k] && !found[k] && cur[k] < e1[k];
                any |= act[k];
            }
            if (!any) break;
            constexpr uint32_t NB = BU_NBRS;
            uint32_t u[NW][NB];
#pragma unroll
            for (uint32_t k = 0; k < NW; ++k)
#pragma unroll
                for (uint32_t q = 0; q < NB; ++q)
                    u[k][q] = act[k] && cur[k] + q < e1[k] ? __ldg(a.col + cur[k] + q) : NONE;
#pragma unroll
            for (uint32_t k = 0; k < NW; ++k) {
#pragma unroll
                for (uint32_t q = 0; q < NB; ++q)
                    if (u[k][q] != NONE && __ldcg(a.dist + u[k][q]) == round) found[k] = true;
                if (act[k]) {
                    relaxed += min(NB, e1[k] - cur[k]);
                    cur[k] += NB;
                }
            }
        }
        uint32_t fm[NW], dd[NW], incl[NW], fany = 0;
#pragma unroll
        for (uint32_t k = 0; k < NW; ++k) {
            fm[k] = __ballot_sync(FULL, found[k]);
            fany |= fm[k];
        }
        if (fany == 0) continue; /* warp-uniform */
#pragma unroll
        for (uint32_t k = 0; k < NW; ++k) {
            if (found[k]) a.dist[v[k]] = round + 1;
            /* this warp is the word's only writer this round */
            if (lane == 0 && fm[k]) a.bits[w0 + k] = vw[k] | fm[k];
            dd[k] = found[k] ? e1[k] - b[k] : 0u;
            incl[k] = dd[k];
        }
#pragma unroll
        for (int s = 1; s < 32; s <<= 1) {
#pragma unroll
            for (uint32_t k = 0; k < NW; ++k) {
                const uint32_t y = __shfl_up_sync(FULL, incl[k], s);
                if (lane >= (uint32_t)s) incl[k] += y;
            }
        }
        /* the words' finds in word order: entries before word k, edges before it */
        uint32_t pc[NW], pe[NW], allc = 0, alle = 0;
#pragma unroll
        for (uint32_t k = 0; k < NW; ++k) {
            pc[k] = allc;
            pe[k] = alle;
            allc += (uint32_t)__popc(fm[k]);
            alle += __shfl_sync(FULL, incl[k], 31);
        }
        unsigned long long old = 0;
        if (lane == 0) old = atomicAdd(&a.ctl->qctr[r3n], ((unsigned long long)allc << 32) | (unsigned long long)alle);
        old = __shfl_sync(FULL, old, 0);
#pragma unroll
        for (uint32_t k = 0; k < NW; ++k)
            if (found[k]) {
                const uint32_t idx = (uint32_t)(old >> 32) + pc[k] + (uint32_t)__popc(fm[k] & lanemask_lt());
                const uint32_t o = (uint32_t)old + pe[k] + incl[k] - dd[k];
                put_entry(a, idx, o, v[k], b[k], dd[k], qv, qo, qb, uf);
            }
    }
}

/* First half of a pulling bucket close (SSSP, light/heavy mode): list every
 * unsettled vertex (d >= thr) that has heavy edges as a queue entry over
 * those edges, in the next round's queue, where expand_units<PULL> relaxes
 * them from the settled side.  With class-ordered rows a reached vertex's
 * range is cut to the classes that can still lower its distance.  A warp
 * takes 32 x PV consecutive vertices per step, lane i vertices 32q + i, so
 * the distance, offset and light-count
 * loads are coalesced and PV of each are in flight per lane; the warp's
 * entries are allocated with one packed 64-bit atomicAdd (entries << 32 |
 * edges), as bottom_up_round does.  Trip counts are warp-uniform; no CTA
 * barrier is used. */
template <int BS>
__device__ __forceinline__ void pull_scan(const Args &a, uint32_t thr, uint32_t nxt, uint32_t r3n) {
    constexpr unsigned FULL = 0xffffffffu;
    constexpr uint32_t PV = 4;
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t gw = ((uint64_t)blockIdx.x * BS + threadIdx.x) >> 5, nw = ((uint64_t)gridDim.x * BS) >> 5;
    const uint64_t steps = ((uint64_t)a.n + 32 * PV - 1) / (32 * PV);
    uint32_t *qv = sel(nxt, a.qv0, a.qv1), *qo = sel(nxt, a.qo0, a.qo1), *qb = sel(nxt, a.qb0, a.qb1);
    uint32_t *uf = sel(nxt, a.uf0, a.uf1);
    for (uint64_t w = gw; w < steps; w += nw) {
        uint32_t b[PV], hd[PV], dv[PV];
        const uint64_t v0 = w * 32 * PV + lane;
#pragma unroll
        for (uint32_t q = 0; q < PV; ++q) dv[q] = v0 + 32 * q < a.n ? __ldcg(a.dist + v0 + 32 * q) : 0u;
        uint32_t cnt = 0, edges = 0;
#pragma unroll
        for (uint32_t q = 0; q < PV; ++q) {
            b[q] = 0;
            hd[q] = 0;
            if (dv[q] >= thr) { /* unsettled (0 past the end) */
                const uint32_t v = (uint32_t)(v0 + 32 * q);
                const uint32_t o0 = __ldg(a.off + v);
                b[q] = o0 + __ldg(a.light + v);
                hd[q] = __ldg(a.off + v + 1) - b[q];
                /* a vertex already reached (d(v) finite) can only be lowered
                 * through an edge with w < d(v): with class-ordered rows the
                 * heavy range ends where the classes start at or above d(v)
                 * (class c holds w >= delta + (c-1) cw), found by a binary
                 * search on the class, which never falls along the range */
                if (a.cw && hd[q] && dv[q] < GGA_INFINITY) {
                    const uint32_t cut_cls = 1u + (uint32_t)(((uint64_t)dv[q] - a.delta + a.cw - 1) / a.cw);
                    if (cut_cls <= LH_CLASSES) {
                        uint32_t lo = b[q], hi = b[q] + hd[q];
                        while (lo < hi) {
                            const uint32_t mid = lo + ((hi - lo) >> 1);
                            if (1u + min((__ldg(a.wt + mid) - a.delta) / a.cw, LH_CLASSES - 1) >= cut_cls) hi = mid;
                            else lo = mid + 1;
                        }
                        hd[q] = lo - b[q];
                    }
                }
                cnt += hd[q] ? 1u : 0u;
                edges += hd[q];
            }
        }
        uint32_t ic = cnt, ie = edges;
#pragma unroll
        for (int k = 1; k < 32; k <<= 1) {
            const uint32_t yc = __shfl_up_sync(FULL, ic, k), ye = __shfl_up_sync(FULL, ie, k);
            if (lane >= (uint32_t)k) {
                ic += yc;
                ie += ye;
            }
        }
        const uint32_t tc = __shfl_sync(FULL, ic, 31), te = __shfl_sync(FULL, ie, 31);
        if (tc == 0) continue; /* warp-uniform */
        unsigned long long old = 0;
        if (lane == 0) old = atomicAdd(&a.ctl->qctr[r3n], ((unsigned long long)tc << 32) | (unsigned long long)te);
        old = __shfl_sync(FULL, old, 0);
        uint32_t i = (uint32_t)(old >> 32) + ic - cnt, o = (uint32_t)old + ie - edges;
#pragma unroll
        for (uint32_t q = 0; q < PV; ++q)
            if (hd[q]) {
                put_entry(a, i, o, (uint32_t)(v0 + 32 * q), b[q], hd[q], qv, qo, qb, uf);
                if (i < a.cap) a.pbest[i] = NONE; /* the pull round's offers meet here */
                ++i;
                o += hd[q];
            }
    }
}

/* Expand one list of queue entries (the round's near queue, or a bucket's
 * heavy list): units of U edges are dealt round-robin (CTA b takes units b,
 * b + G, b + 2G, ...); each CTA loads its unit's entries into shared memory
 * and gives consecutive edges to consecutive threads.  Units hold equal edge
 * counts, so the static deal balances like a ticket counter would, without
 * an atomic on the path, and the next unit's bounds load while the current
 * one is expanded; a round with fewer units than CTAs splits each unit into
 * parts.  Each thread handles PB edges at a time in three passes (edge
 * loads, then distance/bitmap probes, then updates), so PB independent
 * memory chains are in flight per thread instead of one.  SSSP improvements
 * below thr join the next round's near queue, the rest the far pile fp.
 * Block-uniform: every thread runs the same units and checkpoints, and the
 * last barrier follows the final stage-count read.
 *
 * PULL (SSSP): the entries are unsettled vertices and their heavy edges;
 * an edge whose other end u is settled (d(u) < settled) offers d(u) + w to
 * the entry's vertex.  The offers meet in shared memory first (one shared
 * atomicMin per edge into the entry's slot of t_best, which follows t_du),
 * and each entry's best then goes to its pbest word with one fire-and-forget
 * atomicMin (an entry cut by a unit boundary gets one per unit).  Nothing is
 * returned or staged here, so a unit's chain ends at its probes; pull_apply
 * turns the pbest words into distance updates after a grid barrier. */
template <int BS, bool SSSP, bool PULL = false>
__device__ __forceinline__ void expand_units(const Args &a, Ctrl &C, const Stage &S, uint32_t *t_o, uint32_t *t_b,
                                             uint32_t *t_du, const uint32_t *qv, const uint32_t *qo,
                                             const uint32_t *qb, const uint32_t *uf, uint32_t nitems, uint32_t total,
                                             uint32_t units, uint32_t round, uint32_t thr, uint32_t settled,
                                             uint32_t nxt, uint32_t r3n, uint32_t fp, uint32_t bucket,
                                             unsigned long long &relaxed) {
    const uint32_t tid = threadIdx.x, U = a.unit, G = gridDim.x;
    FrontierCtl *ctl = a.ctl;
    uint32_t *t_best = t_du + (U + 1); /* PULL: smallest offer per entry */
    /* entries [i0, i0 + cnt) hold unit k's edges (every thread reads the
     * same two boundary words) */
    auto bounds = [&](uint32_t k, uint32_t &i0, uint32_t &cnt) {
        i0 = min(__ldcg(uf + k), nitems - 1);
        const uint32_t i1 = k + 1 < units ? min(__ldcg(uf + k + 1), nitems - 1) : nitems - 1;
        cnt = i1 >= i0 ? min(i1 - i0 + 1, U + 1) : 1u;
    };
    /* A round with fewer units than CTAs cuts each unit into SU parts of
     * U / SU edges (SU a power of two dividing iters, SU x units <= G), so
     * more CTAs share its edges and its pushes; a CTA then takes one part
     * (the unit's whole table, the part's edges). */
    uint32_t SU = 1;
    while (units * (SU * 2) <= G && a.iters % (SU * 2) == 0) SU *= 2;
    const uint32_t vunits = units * SU, its = a.iters / SU, esub = U / SU;
    uint32_t k = blockIdx.x, i0 = 0, cnt = 0; /* k: part index */
    if (k < vunits) bounds(k / SU, i0, cnt);
    for (;;) {
        __syncthreads(); /* previous unit's table reads and staging done */
        const uint32_t nn = C.nn, fn = SSSP ? C.fn : 0u;
        if (nn >= BS) flush_near<BS>(a, C, S.sv, nn, nxt, r3n, bucket);
        if (SSSP && fn >= BS) flush_far<BS>(a, C, S.sf, fn, fp);
        if (k >= vunits) break;
        const uint32_t kn = k + G;
        uint32_t ni0 = 0, ncnt = 0;
        if (kn < vunits) bounds(kn / SU, ni0, ncnt); /* used after this unit */
        /* a last unit's later parts may start past the round's last edge */
        const uint32_t ebase = (k / SU) * U + (k % SU) * esub, eend = max(ebase, min(ebase + esub, total));
        /* the unit's entries, TB per thread in flight: all entry loads, then
         * (SSSP) all distance loads, then the stores, so a table of up to
         * TB x BS entries costs two dependent L2 round trips, not 2 x TB */
        constexpr uint32_t TB = 5;
        for (uint32_t j0 = 0; j0 < cnt; j0 += TB * BS) {
            uint32_t o[TB], b[TB], x[TB];
#pragma unroll
            for (uint32_t q = 0; q < TB; ++q) {
                const uint32_t j = j0 + q * BS + tid;
                o[q] = b[q] = x[q] = 0;
                if (j < cnt) {
                    o[q] = __ldcg(qo + i0 + j);
                    b[q] = __ldcg(qb + i0 + j);
                    if (SSSP) x[q] = __ldcg(qv + i0 + j);
                }
            }
            if (SSSP && !PULL) { /* the entry's distance (a pull keeps the vertex) */
#pragma unroll
                for (uint32_t q = 0; q < TB; ++q)
                    if (j0 + q * BS + tid < cnt) x[q] = __ldcg(a.dist + x[q]);
            }
#pragma unroll
            for (uint32_t q = 0; q < TB; ++q) {
                const uint32_t j = j0 + q * BS + tid;
                if (j < cnt) {
                    t_o[j] = o[q];
                    t_b[j] = b[q];
                    if (SSSP) t_du[j] = x[q];
                    if (PULL) t_best[j] = NONE;
                }
            }
        }
        __syncthreads();
        constexpr uint32_t PB = STAGE_BATCH;
        for (uint32_t it0 = 0; it0 < its; it0 += PB) {
            if (it0) checkpoint<BS, SSSP>(a, C, S, nxt, r3n, fp, bucket, BS);
            uint32_t v[PB], alt[PB], probe[PB], tgt[PB];
            bool act[PB];
#pragma unroll
            for (uint32_t q = 0; q < PB; ++q) {
                const uint32_t e = ebase + (it0 + q) * BS + tid;
                act[q] = it0 + q < its && e < eend;
                v[q] = 0;
                alt[q] = 0;
                tgt[q] = 0;
                if (act[q]) {
                    uint32_t lo = 0, hi = cnt; /* last j with t_o[j] <= e */
                    while (hi - lo > 1) {
                        const uint32_t mid = (lo + hi) >> 1;
                        if (t_o[mid] <= e) lo = mid; else hi = mid;
                    }
                    const uint32_t ei = t_b[lo] + (e - t_o[lo]);
                    if (ei >= a.m) { /* unreachable by construction; keeps reads in bounds */
                        set_err(ctl, GGA_DEV_BAD_EDGE);
                        act[q] = false;
                    } else {
                        v[q] = __ldg(a.col + ei);
                        if (v[q] >= a.n) { /* a target outside the graph (malformed CSR): no access */
                            set_err(ctl, GGA_DEV_BAD_TARGET);
                            act[q] = false;
                            v[q] = 0;
                        } else if (PULL) {
                            alt[q] = __ldg(a.wt + ei);
                            tgt[q] = lo;
                        } else {
                            alt[q] = SSSP ? t_du[lo] + __ldg(a.wt + ei) : round + 1;
                        }
                    }
                }
            }
#pragma unroll
            for (uint32_t q = 0; q < PB; ++q)
                probe[q] = act[q] ? (SSSP ? __ldcg(a.dist + v[q]) : __ldcg(a.bits + (v[q] >> 5))) : 0u;
            if (PULL) { /* the offer d(u) + w to the entry's slot, from settled u only */
#pragma unroll
                for (uint32_t q = 0; q < PB; ++q)
                    if (act[q] && probe[q] < settled) atomicMin(t_best + tgt[q], probe[q] + alt[q]);
                continue;
            }
            /* updates in phases, so a thread's atomics for its PB edges are in
             * flight together instead of one dependent pair after another:
             * first the distance reduction / visited atomicOr of every edge,
             * then the stamp / far-bit atomic of every improved one, then the
             * shared-memory staging.  Relaxation is a min on uint32
             * distances as M_my_drelax's atomicMin is (cudaKernels.h:323-330);
             * the probe (a recent read of dist[v] or of the visited word) may
             * be stale but never lower than the truth.  SSSP takes an edge
             * whose offer beats the probe as improving v without waiting for
             * the old value: the min goes out as a fire-and-forget red.min,
             * and v is queued (once per round, by its stamp) even if a
             * concurrent offer landed lower.  Its expansion reads dist[v]
             * then, so the extra entry relaxes with the true value, and an
             * entry queued by a lower offer exists whenever one landed; the
             * distances reached are the same, one dependent L2 round trip
             * sooner per edge. */
            uint32_t won = 0; /* bit q: edge q improved v (SSSP) or visited it first (BFS) */
#pragma unroll
            for (uint32_t q = 0; q < PB; ++q) {
                if (!act[q]) continue;
                if (SSSP) {
                    if (alt[q] < probe[q]) {
                        red_min_u32(a.dist + v[q], alt[q]);
                        won |= 1u << q;
                    }
                } else {
                    const uint32_t bit = 1u << (v[q] & 31);
                    if (!(probe[q] & bit) && !(atomicOr(a.bits + (v[q] >> 5), bit) & bit)) won |= 1u << q;
                }
            }
            uint32_t nearm = 0, farm = 0, fmin = NONE;
#pragma unroll
            for (uint32_t q = 0; q < PB; ++q) {
                if (!((won >> q) & 1u)) continue;
                const uint32_t vq = v[q], aq = alt[q];
                if (a.cc) { /* split view: the children mirror the parent */
                    const uint32_t c = a.cc[vq];
                    for (uint32_t k = 1; k <= c; ++k) {
                        if (SSSP) atomicMin(a.dist + vq + k, aq);
                        else a.dist[vq + k] = aq;
                    }
                }
                if (!SSSP) {
                    a.dist[vq] = aq;
                    nearm |= 1u << q;
                } else if (aq < thr) {
                    if (atomicExch(a.stamp + vq, round + 1) != round + 1) nearm |= 1u << q;
                } else {
                    fmin = min(fmin, aq);
                    const uint32_t bit = 1u << (vq & 31);
                    if (!(atomicOr(a.farbits + (vq >> 5), bit) & bit)) farm |= 1u << q;
                }
            }
            if (nearm) {
                const uint32_t k0 = atomicAdd(&C.nn, (uint32_t)__popc(nearm));
                uint32_t k = k0;
#pragma unroll
                for (uint32_t q = 0; q < PB; ++q)
                    if ((nearm >> q) & 1u) {
                        if (k < a.scap) S.sv[k] = v[q];
                        else set_err(ctl, GGA_DEV_OVERFLOW);
                        ++k;
                    }
            }
            if (SSSP && fmin != NONE) atomicMin(&C.fmin, fmin);
            if (SSSP && farm) {
                uint32_t k = atomicAdd(&C.fn, (uint32_t)__popc(farm));
#pragma unroll
                for (uint32_t q = 0; q < PB; ++q)
                    if ((farm >> q) & 1u) {
                        if (k < a.scap) S.sf[k] = v[q];
                        else set_err(ctl, GGA_DEV_OVERFLOW_FAR);
                        ++k;
                    }
            }
        }
        if (PULL) { /* each entry's best offer, to its pbest word (result unused: a reduction) */
            __syncthreads();
            for (uint32_t j = tid; j < cnt; j += BS) {
                const uint32_t best = t_best[j];
                if (best != NONE) atomicMin(a.pbest + i0 + j, best);
            }
        }
        if (tid == 0) relaxed += eend - ebase;
        k = kn;
        i0 = ni0;
        cnt = ncnt;
    }
    /* every thread has read the final stage counts before any thread stages
     * again (a caller may stage right after, as a far pass does) */
    __syncthreads();
}

/* Far pass (SSSP): split pile fp with the new threshold thr — entries still
 * at or above it move to pile fq, entries that fell into the new bucket
 * [thr_old, thr) join the next round's near queue (once, by round stamp),
 * and entries below thr_old (settled since they were piled) are dropped.
 * Block-uniform; the caller publishes the last stage. */
template <int BS>
__device__ __forceinline__ void split_pile(const Args &a, Ctrl &C, const Stage &S, uint32_t fp, uint32_t fq,
                                           uint32_t fc, uint32_t thr, uint32_t thr_old, uint32_t round,
                                           uint32_t nxt, uint32_t r3n, uint32_t bucket) {
    const uint32_t tid = threadIdx.x;
    /* PE entries per thread per step, their loads in flight together; a
     * step stages at most PE x BS, within the stage's room after a
     * checkpoint (scap >= BS x (STAGE_BATCH + 1)) */
    constexpr uint32_t PE = STAGE_BATCH;
    const uint64_t gstep = (uint64_t)gridDim.x * BS * PE;
    const uint32_t *fin = sel3(fp, a.far0, a.far1, a.far2);
    for (uint64_t base = (uint64_t)blockIdx.x * BS * PE; base < fc; base += gstep) {
        uint32_t v[PE], d[PE];
#pragma unroll
        for (uint32_t q = 0; q < PE; ++q) {
            const uint64_t i = base + q * BS + tid;
            v[q] = i < fc ? __ldcg(fin + i) : NONE;
        }
#pragma unroll
        for (uint32_t q = 0; q < PE; ++q) d[q] = v[q] != NONE ? __ldcg(a.dist + v[q]) : 0u;
#pragma unroll
        for (uint32_t q = 0; q < PE; ++q) {
            if (v[q] == NONE) continue;
            if (d[q] >= thr) {
                atomicMin(&C.fmin, d[q]);
                stage_far(a, C, S.sf, v[q]);
            } else {
                atomicAnd(a.farbits + (v[q] >> 5), ~(1u << (v[q] & 31)));
                if (d[q] >= thr_old && atomicExch(a.stamp + v[q], round + 1) != round + 1)
                    stage_near(a, C, S.sv, v[q]);
            }
        }
        checkpoint<BS, true>(a, C, S, nxt, r3n, fq, bucket, BS);
    }
}

/* Second half of a pull round (SSSP): every pull-list entry whose edges
 * found an offer (pbest, complete after the grid barrier that follows the
 * expansion) makes one atomicMin on its vertex's distance; an improvement
 * below thr joins the next round's near queue (once, by round stamp), one
 * at or above it the far pile fq.  A streaming pass over the list, PE
 * entries per thread in flight; block-uniform, with the same checkpoints as
 * split_pile (the caller publishes the last stage). */
template <int BS>
__device__ __forceinline__ void pull_apply(const Args &a, Ctrl &C, const Stage &S, const uint32_t *qv, uint32_t nitems,
                                           uint32_t thr, uint32_t round, uint32_t nxt, uint32_t r3n, uint32_t fq,
                                           uint32_t bucket) {
    const uint32_t tid = threadIdx.x;
    constexpr uint32_t PE = STAGE_BATCH;
    const uint64_t gstep = (uint64_t)gridDim.x * BS * PE;
    for (uint64_t base = (uint64_t)blockIdx.x * BS * PE; base < nitems; base += gstep) {
        uint32_t v[PE], b[PE], old[PE];
#pragma unroll
        for (uint32_t q = 0; q < PE; ++q) {
            const uint64_t i = base + q * BS + tid;
            v[q] = i < nitems ? __ldcg(qv + i) : 0u;
            b[q] = i < nitems ? __ldcg(a.pbest + i) : NONE;
        }
#pragma unroll
        for (uint32_t q = 0; q < PE; ++q) old[q] = b[q] != NONE ? atomicMin(a.dist + v[q], b[q]) : 0u;
#pragma unroll
        for (uint32_t q = 0; q < PE; ++q) {
            if (b[q] == NONE || b[q] >= old[q]) continue;
            const uint32_t vq = v[q];
            if (b[q] < thr) {
                if (atomicExch(a.stamp + vq, round + 1) != round + 1) stage_near(a, C, S.sv, vq);
            } else {
                atomicMin(&C.fmin, b[q]);
                const uint32_t bit = 1u << (vq & 31);
                if (!(atomicOr(a.farbits + (vq >> 5), bit) & bit)) stage_far(a, C, S.sf, vq);
            }
        }
        checkpoint<BS, true>(a, C, S, nxt, r3n, fq, bucket, BS);
    }
}

/* Unit boundaries of an entry list written directly (one thread). */
__device__ __forceinline__ void put_one(const Args &a, uint32_t i, uint32_t o, uint32_t v, uint32_t b, uint32_t d,
                                        uint32_t *qv, uint32_t *qo, uint32_t *qb, uint32_t *uf) {
    qv[i] = v;
    qo[i] = o;
    qb[i] = b;
    for (uint64_t k = ((uint64_t)o + a.unit - 1) / a.unit; k * a.unit < (uint64_t)o + d && k < a.ucap; ++k) uf[k] = i;
}

template <int BS, bool SSSP>
__global__ void __launch_bounds__(BS, BS >= 1024 ? 1 : (BS >= 512 ? 2 : 4)) k_frontier(Args a) {
    extern __shared__ uint32_t dyn[];
    __shared__ Ctrl C;

    FrontierCtl *ctl = a.ctl;
    const uint32_t tid = threadIdx.x;
    const uint64_t gtid = (uint64_t)blockIdx.x * BS + tid, gthreads = (uint64_t)gridDim.x * BS;
    const uint32_t U = a.unit, SC = a.scap;
    const bool lh = SSSP && a.light != nullptr;
    uint32_t *t_o = dyn, *t_b = dyn + (U + 1), *t_du = dyn + 2 * (U + 1);
    uint32_t *stage = dyn + (SSSP ? 4u : 2u) * (U + 1);
    Stage S;
    S.sv = stage;
    S.sf = stage + SC;
    uint32_t gen = 0;
    unsigned long long relaxed = 0;

    /* ---- initialisation: dist = MYINFINITY, bitmaps and stamps cleared */
    for (uint64_t i = gtid; i < a.n; i += gthreads) {
        a.dist[i] = GGA_INFINITY;
        if (SSSP) a.stamp[i] = 0;
        if (lh) a.hstamp[i] = 0;
    }
    const uint32_t nwords = (a.n + 31) / 32;
    for (uint64_t i = gtid; i < nwords; i += gthreads) {
        if (SSSP) a.farbits[i] = 0;
        else a.bits[i] = 0;
    }
    if (tid == 0) {
        C.nn = 0;
        C.fn = 0;
        C.fmin = NONE;
        C.full = 0;
        if (blockIdx.x == 0) {
            ctl->far_min[0] = NONE;
            ctl->far_min[1] = NONE;
            ctl->far_min[2] = NONE;
        }
    }
    if (!grid_barrier(&ctl->bar, &ctl->err, a.nblocks, gen, a.timeout_ns)) return;

    /* ---- the source: original vertex src -> its parent split id and pieces
     * (bfs_sssp.cu:301-318 zeroes the parent and its children) */
    if (blockIdx.x == 0 && tid == 0) {
        const uint32_t s0 = a.first ? a.first[a.src] : a.src;
        const uint32_t cnt = a.cc ? a.cc[s0] + 1 : 1;
        for (uint32_t k = 0; k < cnt; ++k) a.dist[s0 + k] = 0;
        if (!SSSP) a.bits[s0 >> 5] |= 1u << (s0 & 31);
        uint32_t b, d;
        item_range(a, s0, b, d);
        const uint32_t dl = lh ? a.light[s0] : d;
        if (dl) {
            ctl->qctr[0] = (1ull << 32) | dl;
            put_one(a, 0, 0, s0, b, dl, a.qv0, a.qo0, a.qb0, a.uf0);
        }
        if (lh && d > dl) {
            a.hstamp[s0] = 1; /* bucket 0 */
            ctl->hctr[0] = (1ull << 32) | (d - dl);
            put_one(a, 0, 0, s0, b + dl, d - dl, a.hv0, a.ho0, a.hb0, a.huf0);
        }
    }
    if (!grid_barrier(&ctl->bar, &ctl->err, a.nblocks, gen, a.timeout_ns)) return;

    uint32_t thr = SSSP ? (a.delta ? a.delta : NONE) : 0;
    uint32_t fp = 0;
    uint32_t round = 0;
    uint32_t bucket = 0;          /* SSSP: far passes so far (same value in every block) */
    bool heavy_done = false;      /* this bucket's heavy list was expanded (or pulled) */
    bool pulling = false;         /* this round's queue is a pull list */
    bool tail = false;            /* SSSP: buckets ended, label-correcting from here */
    uint32_t fpeak = 0;           /* SSSP: largest far pile seen at a round start */
    uint64_t hsettled = 0;        /* heavy edges of the closed buckets' vertices */
    bool bottom_up = false;       /* BFS direction of the current round */
    uint64_t unexplored = a.m;    /* edges of vertices not yet reached (same value in every block) */
    unsigned long long busy = 0;  /* thread 0: cycles from round start to the barrier */
    long long t_round = 0;
    /* Each block reads a round's counters once (thread 0) and shares them, and
     * those counters are not written during the round (pushes go to the next
     * slot or list; when the near queue is empty nothing joins a heavy list,
     * and nothing relaxes during a far pass's reads).  All blocks therefore
     * take the same branches and meet the same barriers, and all threads of a
     * block the same __syncthreads. */
    for (;; ++round) {
        const uint32_t r3 = round % 3, r3n = (round + 1) % 3, cur = round & 1, nxt = cur ^ 1;
        const uint32_t hl = bucket % 3;
        if (tid == 0) {
            const unsigned long long qc = ld_relaxed_u64(&ctl->qctr[r3]);
            /* an overflowing push sets the error word, so an over-full queue
             * is never consumed; the clamps only keep reads in bounds */
            const uint32_t ni = min((uint32_t)(qc >> 32), a.cap);
            C.nitems = ni;
            C.total = ni ? (uint32_t)qc : 0u;
            C.fc = SSSP ? min(ld_relaxed_u32(&ctl->far_count[fp]), a.cap) : 0u;
            C.fm = SSSP ? ld_relaxed_u32(&ctl->far_min[fp]) : NONE;
            if (lh) {
                const unsigned long long hc = ld_relaxed_u64(&ctl->hctr[hl]);
                const uint32_t hn = min((uint32_t)(hc >> 32), a.cap);
                C.hn = hn;
                C.htot = hn ? (uint32_t)hc : 0u;
            } else {
                C.hn = 0;
                C.htot = 0;
            }
        }
        __syncthreads();
        const uint32_t nitems = C.nitems, total = C.total, fc = C.fc, fm = C.fm, hn = C.hn, htot = C.htot;
        fpeak = max(fpeak, fc);
        const uint32_t units = min((uint32_t)(((uint64_t)total + U - 1) / U), a.ucap);
        const uint32_t hunits = min((uint32_t)(((uint64_t)htot + U - 1) / U), a.ucap);
        __syncthreads(); /* C is rewritten below */
        if (a.trace && tid == 0) t_round = clock64();
        trace_time(a, round);
        if (round >= a.max_rounds) { /* safety net; every block stops in the same round */
            if (blockIdx.x == 0 && tid == 0) set_err(ctl, GGA_DEV_ROUND_LIMIT);
            break;
        }
        if (blockIdx.x == 0 && tid == 0) {
            ctl->qctr[(round + 2) % 3] = 0;
        }
        /* Next bucket (SSSP): the threshold rises by delta (to `lowest` +
         * delta), a new pile takes the far entries, and the lists and piles
         * that rotate out are cleared.  Block 0 clears the pile after fq (read
         * by the previous far pass, a barrier ago; written by the next, a
         * barrier ahead) and the heavy list after the new bucket's (expanded
         * two buckets ago). */
        auto open_bucket = [&](uint32_t lowest) -> uint32_t {
            thr = lowest > NONE - a.delta ? NONE : lowest + a.delta;
            if (!tail && fc <= a.tail_at && fc < fpeak) {
                /* the pile is small and shrinking (opening buckets now drains
                 * it faster than relaxations fill it): no more buckets.  Every
                 * later improvement joins the near queue and expands its whole
                 * row, so no heavy list is needed (C.full is read after the
                 * next barrier).  On R-MAT the vertices left are low-degree and
                 * mostly final already, so the label-correcting rounds redo
                 * almost nothing while the tail's ~5 rounds per bucket go. */
                tail = true;
                thr = NONE;
                if (tid == 0) C.full = 1;
            }
            ++bucket;
            heavy_done = false;
            const uint32_t fq = fp == 2 ? 0 : fp + 1;
            if (blockIdx.x == 0 && tid == 0) {
                const uint32_t dead = fq == 2 ? 0 : fq + 1;
                ctl->far_count[dead] = 0;
                ctl->far_min[dead] = NONE;
                ctl->far_phases++;
                ctl->hctr[(bucket + 1) % 3] = 0;
            }
            return fq;
        };
        /* end of a round that wrote far pushes and pile entries to pile fq */
        auto publish_far = [&](uint32_t fq) {
            checkpoint<BS, SSSP>(a, C, S, nxt, r3n, fq, bucket, 1);
            if (SSSP && tid == 0 && C.fmin != NONE) {
                atomicMin(&ctl->far_min[fq], C.fmin);
                C.fmin = NONE;
            }
        };
        if (units == 0) {
            pulling = false;
            if (lh && !heavy_done && hunits > 0) {
                /* ---- bucket closes: its vertices' distances are final, so
                 * their heavy edges (w >= delta, results >= thr) are relaxed
                 * once */
                heavy_done = true;
                hsettled += htot;
                /* by pull when the unsettled vertices' heavy edges (plus a
                 * scan of every vertex) are far fewer than the bucket's: the
                 * same relaxations seen from the other end (edge (u, v, w)
                 * is also (v, u, w)), done in this round's scan and the next
                 * round's expansion */
                const uint64_t hleft = a.heavy_edges > hsettled ? a.heavy_edges - hsettled : 0;
                if (a.pull == 2 || (a.pull == 1 && (uint64_t)htot > 2 * hleft + a.n / 2)) {
                    trace_round(a, round, 4, hn, htot, fc);
                    pull_scan<BS>(a, thr, nxt, r3n);
                    pulling = true;
                    if (a.trace && tid == 0) busy += clock64() - t_round;
                    if (!grid_barrier(&ctl->bar, &ctl->err, a.nblocks, gen, a.timeout_ns)) break;
                    continue;
                }
                /* pushed, in the same round as the far pass that opens the
                 * next bucket: results below the new threshold join its
                 * near queue, the rest the new pile */
                trace_round(a, round, 3, hn, htot, fc);
                const uint32_t thr_old = thr, hl_old = hl;
                const uint32_t fq = open_bucket(thr);
                expand_units<BS, SSSP>(a, C, S, t_o, t_b, t_du, sel3(hl_old, a.hv0, a.hv1, a.hv2),
                                       sel3(hl_old, a.ho0, a.ho1, a.ho2), sel3(hl_old, a.hb0, a.hb1, a.hb2),
                                       sel3(hl_old, a.huf0, a.huf1, a.huf2), hn, htot, hunits, round, thr, 0u, nxt,
                                       r3n, fq, bucket, relaxed);
                split_pile<BS>(a, C, S, fp, fq, fc, thr, thr_old, round, nxt, r3n, bucket);
                publish_far(fq);
                if (a.trace && tid == 0) busy += clock64() - t_round;
                if (!grid_barrier(&ctl->bar, &ctl->err, a.nblocks, gen, a.timeout_ns)) break;
                fp = fq;
                continue;
            }
            if (!SSSP || fc == 0) break;
            /* ---- near queue drained and nothing left to close: open the
             * next bucket at the lowest piled distance and split the pile */
            const uint32_t thr_old = thr;
            const uint32_t fq = open_bucket(max(thr, fm));
            trace_round(a, round, 2, fc, 0, fc);
            split_pile<BS>(a, C, S, fp, fq, fc, thr, thr_old, round, nxt, r3n, bucket);
            publish_far(fq);
            if (a.trace && tid == 0) busy += clock64() - t_round;
            if (!grid_barrier(&ctl->bar, &ctl->err, a.nblocks, gen, a.timeout_ns)) break;
            fp = fq;
            continue;
        }
        if (!SSSP && a.bu) {
            /* direction rule from this round's counters (identical in every block) */
            unexplored = unexplored > total ? unexplored - total : 0;
            if (!bottom_up) bottom_up = (uint64_t)total * a.alpha > unexplored;
            else bottom_up = (uint64_t)nitems * a.beta >= a.n;
            if (bottom_up) {
                trace_round(a, round, 1, nitems, total, 0);
                bottom_up_round<BS>(a, round, nxt, r3n, relaxed);
                if (a.trace && tid == 0) busy += clock64() - t_round;
                if (!grid_barrier(&ctl->bar, &ctl->err, a.nblocks, gen, a.timeout_ns)) break;
                continue;
            }
        }
        if (SSSP && pulling) {
            /* ---- second half of a pulling bucket close, in the same round
             * as the far pass that opens the next bucket: offers from
             * vertices settled below the old threshold, results below the
             * new one to its near queue, the rest to the new pile */
            pulling = false;
            trace_round(a, round, 5, nitems, total, fc);
            const uint32_t thr_old = thr;
            const uint32_t fq = open_bucket(thr);
            expand_units<BS, SSSP, true>(a, C, S, t_o, t_b, t_du, sel(cur, a.qv0, a.qv1), sel(cur, a.qo0, a.qo1),
                                         sel(cur, a.qb0, a.qb1), sel(cur, a.uf0, a.uf1), nitems, total, units, round,
                                         thr, thr_old, nxt, r3n, fq, bucket, relaxed);
            /* every unit's offers are in the pbest words before any is applied */
            if (!grid_barrier(&ctl->bar, &ctl->err, a.nblocks, gen, a.timeout_ns)) break;
            pull_apply<BS>(a, C, S, sel(cur, a.qv0, a.qv1), nitems, thr, round, nxt, r3n, fq, bucket);
            split_pile<BS>(a, C, S, fp, fq, fc, thr, thr_old, round, nxt, r3n, bucket);
            publish_far(fq);
            if (a.trace && tid == 0) busy += clock64() - t_round;
            if (!grid_barrier(&ctl->bar, &ctl->err, a.nblocks, gen, a.timeout_ns)) break;
            fp = fq;
            continue;
        }
        trace_round(a, round, 0, nitems, total, fc);
        expand_units<BS, SSSP>(a, C, S, t_o, t_b, t_du, sel(cur, a.qv0, a.qv1), sel(cur, a.qo0, a.qo1),
                               sel(cur, a.qb0, a.qb1), sel(cur, a.uf0, a.uf1), nitems, total, units, round, thr, 0u,
                               nxt, r3n, fp, bucket, relaxed);
        publish_far(fp);
        if (a.trace && tid == 0) busy += clock64() - t_round;
        if (!grid_barrier(&ctl->bar, &ctl->err, a.nblocks, gen, a.timeout_ns)) break;
    }
    trace_time(a, round < TRACE_ROUNDS ? round + 1 : TRACE_ROUNDS);
    if (a.trace && tid == 0 && blockIdx.x < TRACE_MAX_CTAS)
        a.trace[(size_t)(TRACE_ROUNDS + 1) * TRACE_REC + blockIdx.x] = (uint32_t)min(busy / 1000ull, 0xffffffffull);
    /* every thread of every block leaves the round loop at the same point */
    for (int d = 16; d > 0; d >>= 1) relaxed += __shfl_down_sync(0xffffffffu, relaxed, d);
    if ((tid & 31u) == 0 && relaxed) atomicAdd(&ctl->edges_relaxed, relaxed);
    if (blockIdx.x == 0 && tid == 0) ctl->rounds = round;
}

template <int BS, bool SSSP>
size_t dyn_smem(uint32_t unit, uint32_t scap) {
    return ((size_t)(unit + 1) * (SSSP ? 4 : 2) + (size_t)scap * (SSSP ? 2 : 1)) * sizeof(uint32_t);
}

/* Resident CTAs per SM for this instance and shared-memory size; the first
 * call per size also raises the instance's dynamic shared-memory limit, so
 * later launches make no driver calls before the launch itself (the time
 * between the start event and the kernel is host time). */
template <int BS, bool SSSP>
int occupancy(size_t smem) {
    constexpr int SLOTS = 16, DEVS = 64;
    static int occ[SLOTS], occ_dev[SLOTS];
    static size_t occ_smem[SLOTS];
    static size_t attr[DEVS]; /* the limit set on each device (it only grows) */
    static int used = 0;
    static std::mutex mu;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= DEVS) return 0;
    std::lock_guard<std::mutex> lk(mu);
    if (smem > attr[dev]) {
        if (cudaFuncSetAttribute(k_frontier<BS, SSSP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
            return 0;
        attr[dev] = smem;
    }
    for (int i = 0; i < used; ++i)
        if (occ_smem[i] == smem && occ_dev[i] == dev) return occ[i];
    int v = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_frontier<BS, SSSP>, BS, smem) != cudaSuccess) v = 0;
    if (used < SLOTS && v > 0) { /* a full cache only costs the calls above again */
        occ[used] = v;
        occ_dev[used] = dev;
        occ_smem[used] = smem;
        ++used;
    }
    return v;
}

template <int BS, bool SSSP>
gga_status launch(Args &a, const gga_params &p, int sms, cudaStream_t st) {
    const size_t smem = dyn_smem<BS, SSSP>(a.unit, a.scap);
    int occ = occupancy<BS, SSSP>(smem);
    if (occ <= 0) return gga_fail(GGA_ERR_CUDA, "frontier kernel: zero occupancy (unit %u)", a.unit);
    int per_sm = p.blocks_per_sm ? (int)p.blocks_per_sm : occ;
    if (per_sm > occ) per_sm = occ;
    a.nblocks = (uint32_t)(sms * per_sm);
    void *args[] = {&a};
    GGA_CK(cudaLaunchCooperativeKernel((const void *)k_frontier<BS, SSSP>, dim3(a.nblocks), dim3(BS), args, smem, st));
    return GGA_OK;
}

} // namespace

static gga_status alloc_u32(uint32_t **p, size_t n) {
    GGA_CK(cudaMalloc((void **)p, (n ? n : 1) * sizeof(uint32_t)));
    return GGA_OK;
}

void frontier_scratch_free(FrontierScratch *s) {
    cudaFree(s->dist); cudaFree(s->bits); cudaFree(s->farbits); cudaFree(s->stamp);
    cudaFree(s->qv0); cudaFree(s->qv1); cudaFree(s->qo0); cudaFree(s->qo1); cudaFree(s->qb0); cudaFree(s->qb1);
    cudaFree(s->uf0); cudaFree(s->uf1);
    cudaFree(s->far0); cudaFree(s->far1); cudaFree(s->far2);
    cudaFree(s->out); cudaFree(s->ctl); cudaFree(s->trace); cudaFree(s->hstamp); cudaFree(s->pbest);
    for (int i = 0; i < 3; ++i) {
        cudaFree(s->hv[i]); cudaFree(s->ho[i]); cudaFree(s->hb[i]); cudaFree(s->huf[i]);
    }
    if (s->hctl) cudaFreeHost(s->hctl);
    memset(s, 0, sizeof *s);
}

gga_status frontier_scratch_ensure(FrontierScratch *s, uint32_t n, uint32_t m) {
    const uint32_t ucap = m / MIN_UNIT + 4;
    if (s->cap >= n && s->ucap >= ucap && s->ctl) return GGA_OK;
    frontier_scratch_free(s);
    const uint32_t cap = n < 1024 ? 1024 : n;
    const size_t words = (cap + 31) / 32 + 1;
    gga_status st;
    if ((st = alloc_u32(&s->dist, cap)) || (st = alloc_u32(&s->bits, words)) ||
        (st = alloc_u32(&s->farbits, words)) || (st = alloc_u32(&s->stamp, cap)) ||
        (st = alloc_u32(&s->qv0, cap)) || (st = alloc_u32(&s->qv1, cap)) || (st = alloc_u32(&s->qo0, cap)) ||
        (st = alloc_u32(&s->qo1, cap)) || (st = alloc_u32(&s->qb0, cap)) || (st = alloc_u32(&s->qb1, cap)) ||
        (st = alloc_u32(&s->uf0, ucap)) || (st = alloc_u32(&s->uf1, ucap)) ||
        (st = alloc_u32(&s->far0, cap)) || (st = alloc_u32(&s->far1, cap)) || (st = alloc_u32(&s->far2, cap)) ||
        (st = alloc_u32(&s->out, cap)) || (st = alloc_u32(&s->hstamp, cap)) || (st = alloc_u32(&s->pbest, cap)) ||
        (st = alloc_u32(&s->hv[0], cap)) || (st = alloc_u32(&s->hv[1], cap)) || (st = alloc_u32(&s->hv[2], cap)) ||
        (st = alloc_u32(&s->ho[0], cap)) || (st = alloc_u32(&s->ho[1], cap)) || (st = alloc_u32(&s->ho[2], cap)) ||
        (st = alloc_u32(&s->hb[0], cap)) || (st = alloc_u32(&s->hb[1], cap)) || (st = alloc_u32(&s->hb[2], cap)) ||
        (st = alloc_u32(&s->huf[0], ucap)) || (st = alloc_u32(&s->huf[1], ucap)) || (st = alloc_u32(&s->huf[2], ucap))) {
        frontier_scratch_free(s);
        return st;
    }
    cudaError_t e = cudaMalloc((void **)&s->ctl, sizeof(FrontierCtl));
    if (e == cudaSuccess) e = cudaMallocHost((void **)&s->hctl, sizeof(FrontierCtl));
    if (e != cudaSuccess) {
        frontier_scratch_free(s);
        return gga_fail(GGA_ERR_CUDA, "frontier control block: %s", cudaGetErrorString(e));
    }
    s->cap = cap;
    s->ucap = ucap;
    return GGA_OK;
}

gga_status frontier_run(FrontierScratch *s, const GraphView &view, const uint32_t *first, uint32_t src,
                        bool sssp, const gga_params &p, int sms, cudaStream_t st, cudaEvent_t ev0,
                        cudaEvent_t ev1, FrontierResult *res, bool trace, const LightHeavy &lh,
                        FrontierCtl *hctl_async) {
    Args a;
    memset(&a, 0, sizeof a);
    if (trace) {
        if (!s->trace) GGA_CK(cudaMalloc((void **)&s->trace, TRACE_WORDS * sizeof(uint32_t)));
        GGA_CK(cudaMemsetAsync(s->trace, 0, TRACE_WORDS * sizeof(uint32_t), st));
        a.trace = s->trace;
    }
    a.off = view.off; a.col = view.col; a.wt = view.wt; a.cc = view.cc;
    a.first = first;
    a.n = view.n;
    a.m = view.m;
    a.dist = s->dist; a.bits = s->bits; a.farbits = s->farbits; a.stamp = s->stamp;
    a.qv0 = s->qv0; a.qv1 = s->qv1; a.qo0 = s->qo0; a.qo1 = s->qo1; a.qb0 = s->qb0; a.qb1 = s->qb1;
    a.uf0 = s->uf0; a.uf1 = s->uf1;
    a.far0 = s->far0; a.far1 = s->far1; a.far2 = s->far2;
    a.ctl = s->ctl;
    a.cap = s->cap;
    a.ucap = s->ucap;
    a.src = src;
    const uint32_t bs = p.block_threads ? p.block_threads : 256;
    /* measured on R-MAT 22 (GB300): BFS is fastest with the largest units
     * (4096 edges), SSSP with 1024-edge units (one batch of edges per
     * thread per unit) */
    a.iters = p.unit_iters ? p.unit_iters : (sssp ? 4 : MAX_UNIT / bs);
    if (a.iters < 2 || a.iters > 16)
        return gga_fail(GGA_ERR_INVALID_ARG, "unit_iters must be in [2, 16] (got %u)", a.iters);
    a.unit = bs * a.iters;
    if (a.unit < MIN_UNIT || a.unit > MAX_UNIT)
        return gga_fail(GGA_ERR_INVALID_ARG, "block_threads x unit_iters = %u edges per unit, need %u..%u", a.unit,
                        MIN_UNIT, MAX_UNIT);
    a.scap = bs * (STAGE_BATCH + 1); /* < BS staged after a checkpoint, + one batch */
    a.delta = p.sssp_delta;
    /* the tail by default only where vertices average 8+ edges: on R-MAT the
     * vertices left are low-degree and mostly final (SSSP 2.27 -> 1.40 ms at
     * R-MAT 22), but on a 4096^2 grid the label-correcting rounds redo whole
     * wavefronts (9.2 -> 18.1 ms); it starts once the far pile is below n / 2
     * (measured against n / 4 on R-MAT 18-22: as fast or faster at every
     * bucket width, R-MAT 22 with its best width 1.23 -> 1.19 ms) */
    if (sssp && a.delta && p.sssp_tail != 1) {
        if (p.sssp_tail) a.tail_at = view.n / p.sssp_tail;
        else if ((uint64_t)view.m >= 8ull * view.n) a.tail_at = view.n / 2u;
    }
    a.bu = !sssp && view.cc == nullptr && view.symmetric && p.bfs_direction == 0;
    if (sssp && lh.light && a.delta) {
        a.light = lh.light;
        a.pull = lh.pull;
        a.pbest = s->pbest;
        a.cw = lh.cw;
        a.heavy_edges = lh.heavy_edges;
        a.hstamp = s->hstamp;
        a.hv0 = s->hv[0]; a.hv1 = s->hv[1]; a.hv2 = s->hv[2];
        a.ho0 = s->ho[0]; a.ho1 = s->ho[1]; a.ho2 = s->ho[2];
        a.hb0 = s->hb[0]; a.hb1 = s->hb[1]; a.hb2 = s->hb[2];
        a.huf0 = s->huf[0]; a.huf1 = s->huf[1]; a.huf2 = s->huf[2];
    }
    /* Beamer's alpha is 15; with four bitmap words per bottom-up warp step a
     * later switch pays (R-MAT 22 on GB300: 0.225 ms at 15, 0.219 at 6-10) */
    a.alpha = p.bfs_alpha ? p.bfs_alpha : 8;
    a.beta = p.bfs_beta ? p.bfs_beta : 18;
    /* BFS needs at most n levels; near-far SSSP at most a level per
     * improvement, which the bound below leaves ample room for */
    a.max_rounds = view.n > 0x3fffffffu ? 0xffffffffu : 4u * view.n + 4096u;
    a.timeout_ns = 4000000000ull;
    GGA_CK(cudaMemsetAsync(s->ctl, 0, sizeof(FrontierCtl), st));
    if (ev0) GGA_CK(cudaEventRecord(ev0, st));
    gga_status r;
    switch (bs) {
    case 256: r = sssp ? launch<256, true>(a, p, sms, st) : launch<256, false>(a, p, sms, st); break;
    case 512: r = sssp ? launch<512, true>(a, p, sms, st) : launch<512, false>(a, p, sms, st); break;
    case 1024: r = sssp ? launch<1024, true>(a, p, sms, st) : launch<1024, false>(a, p, sms, st); break;
    default: return gga_fail(GGA_ERR_INVALID_ARG, "block_threads must be 256, 512 or 1024 (got %u)", bs);
    }
    if (r) return r;
    if (ev1) GGA_CK(cudaEventRecord(ev1, st));
    if (res) {
        res->launches = 1;
        res->nblocks = a.nblocks;
    }
    if (hctl_async) { /* the caller waits, then calls frontier_verdict */
        GGA_CK(cudaMemcpyAsync(hctl_async, s->ctl, sizeof(FrontierCtl), cudaMemcpyDeviceToHost, st));
        return GGA_OK;
    }
    GGA_CK(cudaMemcpyAsync(s->hctl, s->ctl, sizeof(FrontierCtl), cudaMemcpyDeviceToHost, st));
    gga_status w = dev_wait(st, 60.0);
    if (w) return w;
    if ((w = frontier_verdict(*s->hctl))) return w;
    if (res) {
        res->rounds = s->hctl->rounds;
        res->edges_relaxed = s->hctl->edges_relaxed;
        res->kernel_ms = 0;
        if (ev0 && ev1) cudaEventElapsedTime(&res->kernel_ms, ev0, ev1);
    }
    return GGA_OK;
}

gga_status frontier_verdict(const FrontierCtl &h) {
    if (h.err == GGA_DEV_TIMEOUT)
        return gga_fail(GGA_ERR_TIMEOUT, "frontier grid barrier timed out after %u rounds", h.rounds);
    if (h.err == GGA_DEV_OVERFLOW) return gga_fail(GGA_ERR_CUDA, "frontier queue overflow (internal error)");
    if (h.err == GGA_DEV_ROUND_LIMIT) return gga_fail(GGA_ERR_CUDA, "frontier round limit reached (internal error)");
    if (h.err == GGA_DEV_BAD_TARGET) return gga_fail(GGA_ERR_FORMAT, "malformed CSR: an edge target is >= n");
    if (h.err == GGA_DEV_OVERFLOW_UNITS) return gga_fail(GGA_ERR_CUDA, "frontier unit table overflow (internal error)");
    if (h.err == GGA_DEV_OVERFLOW_FAR) return gga_fail(GGA_ERR_CUDA, "frontier far pile overflow (internal error)");
    if (h.err == GGA_DEV_BAD_EDGE)
        return gga_fail(GGA_ERR_CUDA,
                        "frontier unit mapping self-check failed: round %u unit %u e %u jj %u cnt %u i0 %u t_o[jj] %u "
                        "t_b[jj] %u total %u nitems %u t_o[0] %u t_o[jj+1] %u units %u uf[k] %u uf[k+1] %u ei %u",
                        h.diag[0], h.diag[1], h.diag[2], h.diag[3], h.diag[4], h.diag[5], h.diag[6], h.diag[7],
                        h.diag[8], h.diag[9], h.diag[10], h.diag[11], h.diag[12], h.diag[13], h.diag[14], h.diag[15]);
    if (h.err != GGA_DEV_OK) return gga_fail(GGA_ERR_CUDA, "frontier kernel error %u", h.err);
    return GGA_OK;
}

/* ------------------------------------------------------------------------
 * Allocation-free BFS entry point.
 *
 * Some callers cannot allocate GPU memory when they run a traversal: code
 * that runs inside a memory pool or arena another framework owns (calling
 * cudaMalloc there fragments or oversubscribes that pool), real-time or
 * latency-critical paths where an allocation may synchronise the device or
 * take unbounded time, and processes whose device memory is fully reserved
 * up front.  gga_bfs_noalloc serves them: it runs the same frontier BFS
 * kernel as gga_bfs, but all of its working memory (queues, visited bitmap,
 * control block) lives in the fixed array below, which the library
 * reserves on every GPU where it is loaded and keeps until the process
 * exits.  The caller provides the graph and the output in device memory.
 *
 * Limits: at most NOALLOC_MAX_NODES vertices and NOALLOC_MAX_EDGES edges;
 * larger graphs are rejected with GGA_ERR_TOO_LARGE.  All calls share the
 * one array, so calls whose work overlaps on the GPU (different host
 * threads, or different streams without ordering between them) race and
 * corrupt each other's results; serialise them.  Each call is synchronous
 * (it waits for the traversal on `stream` and reads its status back), so it
 * must not be made while any stream of the device is being captured into a
 * CUDA graph; the first call on a device also looks up the array's device
 * address (cudaGetSymbolAddress).  The
 * caller's CSR is not validated on the host (it is device memory): a column
 * id >= n is caught in the kernel, which skips that edge and makes the call
 * return GGA_ERR_FORMAT.
 * ------------------------------------------------------------------------ */


#define NOALLOC_MAX_NODES (1u << 18) /* 262,144 vertices */
#define NOALLOC_MAX_EDGES (1u << 23) /* 8,388,608 directed edges */

namespace {
constexpr size_t NA_CTL_WORDS = (sizeof(FrontierCtl) + 255) / 256 * 64; /* control block, 256-byte rounded */
constexpr size_t NA_BITS_WORDS = NOALLOC_MAX_NODES / 32 + 64;
constexpr size_t NA_UCAP = NOALLOC_MAX_EDGES / MIN_UNIT + 4;
constexpr size_t NA_WORDS = NA_CTL_WORDS + NA_BITS_WORDS + 6 * (size_t)NOALLOC_MAX_NODES + 2 * NA_UCAP;
} // namespace

/* Fixed working memory of gga_bfs_noalloc (about 6.2 MiB per GPU). */
static __device__ __align__(256) uint32_t g_noalloc_scratch[NA_WORDS];

static std::mutex g_noalloc_mu;
static uint32_t *g_noalloc_ptr[64]; /* device address of the array, per device */
static int g_noalloc_sms[64];

extern "C" gga_status gga_bfs_noalloc(const uint32_t *d_offsets, const uint32_t *d_cols, uint32_t n, uint32_t m,
                                      uint32_t src, uint32_t *d_dist, void *stream) {
    if (!d_offsets || !d_dist || (m && !d_cols))
        return gga_fail(GGA_ERR_INVALID_ARG, "gga_bfs_noalloc: NULL device pointer");
    if (n == 0 || src >= n) return gga_fail(GGA_ERR_INVALID_ARG, "gga_bfs_noalloc: source %u of %u vertices", src, n);
    if (n > NOALLOC_MAX_NODES || m > NOALLOC_MAX_EDGES)
        return gga_fail(GGA_ERR_TOO_LARGE,
                        "gga_bfs_noalloc: %u vertices / %u edges exceed its fixed working memory "
                        "(at most %u vertices and %u edges); use gga_bfs",
                        n, m, NOALLOC_MAX_NODES, NOALLOC_MAX_EDGES);
    int dev = 0;
    GGA_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return gga_fail(GGA_ERR_INVALID_ARG, "gga_bfs_noalloc: device %d", dev);
    uint32_t *base;
    int sms;
    {
        /* once per device, with that device current: host code cannot use the
         * array's name as a device address, so ask the runtime for it */
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        if (!g_noalloc_ptr[dev]) {
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess)
                return gga_fail(GGA_ERR_CUDA, "gga_bfs_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
            int s = 0;
            e = cudaDeviceGetAttribute(&s, cudaDevAttrMultiProcessorCount, dev);
            if (e != cudaSuccess)
                return gga_fail(GGA_ERR_CUDA, "gga_bfs_noalloc: SM count: %s", cudaGetErrorString(e));
            g_noalloc_sms[dev] = s;
            g_noalloc_ptr[dev] = (uint32_t *)p;
        }
        base = g_noalloc_ptr[dev];
        sms = g_noalloc_sms[dev];
    }
    cudaStream_t st = (cudaStream_t)stream;
    FrontierCtl *ctl = (FrontierCtl *)base;
    uint32_t *w = base + NA_CTL_WORDS;
    Args a;
    memset(&a, 0, sizeof a);
    a.off = d_offsets;
    a.col = d_cols;
    a.n = n;
    a.m = m;
    a.dist = d_dist;
    a.bits = w;
    w += NA_BITS_WORDS;
    a.qv0 = w; a.qv1 = w + NOALLOC_MAX_NODES; a.qo0 = w + 2 * NOALLOC_MAX_NODES; a.qo1 = w + 3 * NOALLOC_MAX_NODES;
    a.qb0 = w + 4 * NOALLOC_MAX_NODES; a.qb1 = w + 5 * NOALLOC_MAX_NODES;
    w += 6 * (size_t)NOALLOC_MAX_NODES;
    a.uf0 = w;
    a.uf1 = w + NA_UCAP;
    a.ctl = ctl;
    a.cap = NOALLOC_MAX_NODES;
    a.ucap = (uint32_t)NA_UCAP;
    a.src = src;
    a.iters = 8;
    a.unit = 256 * a.iters;
    a.scap = 256 * (a.iters + 1);
    a.max_rounds = 4u * n + 4096u;
    a.timeout_ns = 4000000000ull;
    /* the control block must start at zero; the kernel clears the bitmap */
    GGA_CK(cudaMemsetAsync(ctl, 0, sizeof(FrontierCtl), st));
    gga_params p;
    memset(&p, 0, sizeof p);
    gga_status s = launch<256, false>(a, p, sms, st);
    if (s) return s;
    s = dev_wait(st, 60.0); /* bounded wait for the kernel */
    if (s) return s;
    uint32_t err = 0;
    GGA_CK(cudaMemcpyAsync(&err, &ctl->err, sizeof err, cudaMemcpyDeviceToHost, st));
    GGA_CK(cudaStreamSynchronize(st));
    if (err == GGA_DEV_TIMEOUT) return gga_fail(GGA_ERR_TIMEOUT, "gga_bfs_noalloc: grid barrier timed out");
    if (err == GGA_DEV_BAD_TARGET)
        return gga_fail(GGA_ERR_FORMAT, "gga_bfs_noalloc: malformed CSR: an edge target is >= n (%u)", n);
    if (err != GGA_DEV_OK) return gga_fail(GGA_ERR_CUDA, "gga_bfs_noalloc: kernel error %u", err);
    return GGA_OK;
}
