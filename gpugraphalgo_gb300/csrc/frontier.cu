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
 *   - a CTA takes 256..1024 frontier vertices, scans their degrees and walks
 *     the concatenated edge lists with all its threads, so consecutive lanes
 *     read consecutive edges (coalesced) whatever the degree skew;
 *   - vertices above `huge_degree` are cut into fixed edge chunks that any
 *     CTA can take, so the 10^5-degree hubs of R-MAT do not serialise a CTA;
 *   - work units are handed out by an atomic ticket (dynamic balancing);
 *   - pushes are warp-aggregated (__ballot_sync/__popc, one atomic per warp)
 *     and deduplicated: BFS by a visited bitmap, SSSP by a per-vertex round
 *     stamp (near queue) and a "far pile" bitmap;
 *   - relaxation is atomicMin on uint32 distances, as the reference does;
 *   - rounds are separated by a bounded grid barrier (no host round trip);
 *     a barrier that waits past its limit sets an error word and the kernel
 *     returns, so the host gets GGA_ERR_TIMEOUT instead of a hung GPU.
 * On a node-split graph (graph.h:415-522) the engine walks the split view:
 * edges target parents, and reaching a parent reaches its children too
 * (their distances mirror the parent's, cudaKernels.h:326-330), each child
 * being expanded as its own work item over its slice of the edges.
 */
#include <stdio.h>

#include "frontier.cuh"

namespace {

constexpr uint32_t FULL = 0xffffffffu;
constexpr uint32_t NONE = 0xffffffffu;

struct Args {
    const uint32_t *off, *col, *wt, *cc;
    const uint32_t *first; /* split view: original -> parent split id */
    uint32_t n;
    uint32_t *dist, *bits, *farbits, *stamp;
    uint32_t *q0, *q1, *hq0, *hq1, *hqb0, *hqb1, *far0, *far1, *far2;
    FrontierCtl *ctl;
    uint32_t cap, hcap;
    uint32_t src;
    uint32_t huge_degree, chunk_edges;
    uint32_t delta;
    uint32_t nblocks;
    unsigned long long timeout_ns;
};

__device__ __forceinline__ uint32_t *sel(uint32_t p, uint32_t *a, uint32_t *b) { return p ? b : a; }
__device__ __forceinline__ uint32_t *sel3(uint32_t p, uint32_t *a, uint32_t *b, uint32_t *c) {
    return p == 0 ? a : (p == 1 ? b : c);
}

__device__ __forceinline__ void set_err(FrontierCtl *c, uint32_t code) { atomicCAS(&c->err, GGA_DEV_OK, code); }

/* Queue the pieces of vertex v (v itself plus its split children) for the
 * next round.  Must be called by all 32 lanes of a warp (want may differ). */
__device__ __forceinline__ void push_near(const Args &a, uint32_t v, bool want, uint32_t nxt, uint32_t r3n) {
    bool simple = false;
    uint32_t pieces = 1;
    if (want) {
        if (a.cc) pieces = a.cc[v] + 1;
        if (pieces == 1) {
            const uint32_t d = __ldg(a.off + v + 1) - __ldg(a.off + v);
            simple = d != 0 && d <= a.huge_degree;
            if (d == 0) want = false; /* nothing to expand */
        }
    }
    const uint32_t mask = __ballot_sync(FULL, simple);
    if (mask) {
        const uint32_t leader = __ffs(mask) - 1;
        uint32_t base = 0;
        if (lane_id() == leader) base = atomicAdd(&a.ctl->qcount[r3n], (uint32_t)__popc(mask));
        base = __shfl_sync(FULL, base, leader);
        if (simple) {
            const uint32_t idx = base + __popc(mask & lanemask_lt());
            if (idx < a.cap) sel(nxt, a.q0, a.q1)[idx] = v;
            else set_err(a.ctl, GGA_DEV_OVERFLOW);
        }
    }
    if (want && !simple) {
        for (uint32_t k = 0; k < pieces; ++k) {
            const uint32_t w = v + k;
            const uint32_t b = __ldg(a.off + w), d = __ldg(a.off + w + 1) - b;
            if (d == 0) continue;
            if (d <= a.huge_degree) {
                const uint32_t idx = atomicAdd(&a.ctl->qcount[r3n], 1u);
                if (idx < a.cap) sel(nxt, a.q0, a.q1)[idx] = w;
                else set_err(a.ctl, GGA_DEV_OVERFLOW);
            } else {
                const uint32_t nch = (d + a.chunk_edges - 1) / a.chunk_edges;
                const unsigned long long old = atomicAdd(&a.ctl->huge[r3n], (1ull << 32) | nch);
                const uint32_t it = (uint32_t)(old >> 32);
                if (it < a.hcap) {
                    sel(nxt, a.hq0, a.hq1)[it] = w;
                    sel(nxt, a.hqb0, a.hqb1)[it] = (uint32_t)old;
                } else {
                    set_err(a.ctl, GGA_DEV_OVERFLOW);
                }
            }
        }
    }
}

/* Add v to the far pile `fp` (warp-uniform call). */
__device__ __forceinline__ void push_far(const Args &a, uint32_t v, bool want, uint32_t fp) {
    const uint32_t mask = __ballot_sync(FULL, want);
    if (!mask) return;
    const uint32_t leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (lane_id() == leader) base = atomicAdd(&a.ctl->far_count[fp], (uint32_t)__popc(mask));
    base = __shfl_sync(FULL, base, leader);
    if (want) {
        const uint32_t idx = base + __popc(mask & lanemask_lt());
        if (idx < a.cap) sel3(fp, a.far0, a.far1, a.far2)[idx] = v;
        else set_err(a.ctl, GGA_DEV_OVERFLOW);
    }
}

/* Relax one edge to v with candidate distance alt; returns through the
 * out-parameters whether v goes to the near queue or the far pile.
 * Called under warp-uniform control flow; `active` masks idle lanes. */
template <bool SSSP>
__device__ __forceinline__ void relax(const Args &a, bool active, uint32_t v, uint32_t alt, uint32_t round,
                                      uint32_t thr, uint32_t fp, uint32_t nxt, uint32_t r3n) {
    bool near = false, far = false;
    uint32_t farval = NONE;
    if (active) {
        if (!SSSP) {
            const uint32_t bit = 1u << (v & 31);
            if (!(__ldcg(a.bits + (v >> 5)) & bit)) {
                const uint32_t old = atomicOr(a.bits + (v >> 5), bit);
                if (!(old & bit)) {
                    a.dist[v] = alt;
                    if (a.cc) {
                        const uint32_t c = a.cc[v];
                        for (uint32_t k = 1; k <= c; ++k) a.dist[v + k] = alt;
                    }
                    near = true;
                }
            }
        } else if (alt < __ldcg(a.dist + v)) {
            const uint32_t old = atomicMin(a.dist + v, alt);
            if (alt < old) {
                if (a.cc) {
                    const uint32_t c = a.cc[v];
                    for (uint32_t k = 1; k <= c; ++k) atomicMin(a.dist + v + k, alt);
                }
                if (alt < thr) {
                    near = atomicExch(a.stamp + v, round + 1) != round + 1;
                } else {
                    farval = alt;
                    const uint32_t bit = 1u << (v & 31);
                    far = !(atomicOr(a.farbits + (v >> 5), bit) & bit);
                }
            }
        }
    }
    push_near(a, v, near, nxt, r3n);
    if (SSSP) {
        const uint32_t wmin = __reduce_min_sync(FULL, farval);
        if (wmin != NONE && lane_id() == __ffs(__ballot_sync(FULL, farval == wmin)) - 1)
            atomicMin(&a.ctl->far_min[fp], wmin);
        push_far(a, v, far, fp);
    }
}

template <int BS, bool SSSP>
__global__ void __launch_bounds__(BS) k_frontier(Args a) {
    __shared__ uint32_t s_incl[BS];
    __shared__ uint32_t s_adj[BS];
    __shared__ uint32_t s_du[SSSP ? BS : 1];
    __shared__ uint32_t s_ws[32];
    __shared__ uint32_t s_unit, s_hstart, s_hcnt, s_hdu;

    FrontierCtl *ctl = a.ctl;
    const uint32_t tid = threadIdx.x;
    const uint64_t gtid = (uint64_t)blockIdx.x * BS + tid, gthreads = (uint64_t)gridDim.x * BS;
    uint32_t gen = 0;
    unsigned long long relaxed = 0;

    /* ---- initialisation: dist = MYINFINITY, bitmaps and stamps cleared */
    for (uint64_t i = gtid; i < a.n; i += gthreads) {
        a.dist[i] = GGA_INFINITY;
        if (SSSP) a.stamp[i] = 0;
    }
    const uint32_t nwords = (a.n + 31) / 32;
    for (uint64_t i = gtid; i < nwords; i += gthreads) {
        if (SSSP) a.farbits[i] = 0;
        else a.bits[i] = 0;
    }
    if (blockIdx.x == 0 && tid == 0) {
        ctl->far_min[0] = NONE;
        ctl->far_min[1] = NONE;
        ctl->far_min[2] = NONE;
    }
    if (!grid_barrier(&ctl->bar, &ctl->err, a.nblocks, gen, a.timeout_ns)) return;

    /* ---- the source: original vertex src -> its parent split id and pieces
     * (bfs_sssp.cu:301-318 zeroes the parent and its children) */
    if (blockIdx.x == 0 && tid < 32) {
        const uint32_t s0 = a.first ? a.first[a.src] : a.src;
        const uint32_t cnt = a.cc ? a.cc[s0] + 1 : 1;
        for (uint32_t k = tid; k < cnt; k += 32) a.dist[s0 + k] = 0;
        if (tid == 0) {
            if (!SSSP) a.bits[s0 >> 5] |= 1u << (s0 & 31);
            else a.stamp[s0] = 0;
        }
        __syncwarp();
        push_near(a, s0, tid == 0, 0, 0);
    }
    if (!grid_barrier(&ctl->bar, &ctl->err, a.nblocks, gen, a.timeout_ns)) return;

    uint32_t thr = SSSP ? (a.delta ? a.delta : NONE) : 0;
    uint32_t fp = 0;
    uint32_t round = 0;
    /* Every decision below reads only counters that no block writes during
     * the current round: the round's input queue (pushes go to the next
     * slot) and, when that queue is empty, the far pile (nothing relaxes).
     * So all blocks take the same branch and meet the same barriers. */
    for (;; ++round) {
        const uint32_t r3 = round % 3, r3n = (round + 1) % 3, cur = round & 1, nxt = cur ^ 1;
        /* an overflowing push sets the error word, so a queue past its
         * capacity is never consumed; the clamps only keep reads in bounds */
        const uint32_t qn = min(ld_relaxed_u32(&ctl->qcount[r3]), a.cap);
        const unsigned long long hh = ld_relaxed_u64(&ctl->huge[r3]);
        const uint32_t hitems = min((uint32_t)(hh >> 32), a.hcap), hchunks = hitems ? (uint32_t)hh : 0u;
        const uint32_t nchunks = (qn + BS - 1) / BS;
        const uint32_t units = nchunks + hchunks;
        const uint32_t *qin = sel(cur, a.q0, a.q1);
        const uint32_t *hqin = sel(cur, a.hq0, a.hq1);
        const uint32_t *hqbin = sel(cur, a.hqb0, a.hqb1);
        if (blockIdx.x == 0 && tid == 0) {
            const uint32_t r3nn = (round + 2) % 3;
            ctl->qcount[r3nn] = 0;
            ctl->work[r3nn] = 0;
            ctl->huge[r3nn] = 0;
        }
        if (units == 0) {
            if (!SSSP) break;
            const uint32_t fc = min(ld_relaxed_u32(&ctl->far_count[fp]), a.cap);
            if (fc == 0) break;
            /* ---- near queue drained: raise the threshold and split the far
             * pile into the next round's near queue and the other pile */
            const uint32_t fmin = ld_relaxed_u32(&ctl->far_min[fp]);
            const uint32_t thr_old = thr;
            const uint32_t lowest = max(thr, fmin);
            thr = lowest > NONE - a.delta ? NONE : lowest + a.delta;
            const uint32_t fq = fp == 2 ? 0 : fp + 1; /* pile that keeps the far items */
            if (blockIdx.x == 0 && tid == 0) {
                /* three piles rotate: the one after fq was read by the
                 * previous far pass (a barrier ago) and is written by the
                 * next one (a barrier ahead), so it can be cleared now */
                const uint32_t dead = fq == 2 ? 0 : fq + 1;
                ctl->far_count[dead] = 0;
                ctl->far_min[dead] = NONE;
                ctl->far_phases++;
            }
            const uint32_t *fin = sel3(fp, a.far0, a.far1, a.far2);
            for (uint64_t base = (uint64_t)blockIdx.x * BS; base < fc; base += gthreads) {
                const uint64_t i = base + tid;
                bool to_near = false, keep = false;
                uint32_t v = 0, d = NONE;
                if (i < fc) {
                    v = __ldcg(fin + i);
                    d = __ldcg(a.dist + v);
                    if (d >= thr) {
                        keep = true;
                    } else {
                        atomicAnd(a.farbits + (v >> 5), ~(1u << (v & 31)));
                        if (d >= thr_old) to_near = atomicExch(a.stamp + v, round + 1) != round + 1;
                    }
                }
                push_near(a, v, to_near, nxt, r3n);
                const uint32_t kmin = __reduce_min_sync(FULL, keep ? d : NONE);
                if (kmin != NONE && lane_id() == __ffs(__ballot_sync(FULL, keep && d == kmin)) - 1)
                    atomicMin(&ctl->far_min[fq], kmin);
                push_far(a, v, keep, fq);
            }
            if (!grid_barrier(&ctl->bar, &ctl->err, a.nblocks, gen, a.timeout_ns)) break;
            fp = fq;
            continue;
        }
        for (;;) {
            if (tid == 0) s_unit = atomicAdd(&ctl->work[r3], 1u);
            __syncthreads();
            const uint32_t unit = s_unit;
            if (unit >= units) break;
            if (unit < nchunks) {
                /* a tile of BS frontier vertices, expanded by the whole CTA */
                const uint32_t idx = unit * BS + tid;
                uint32_t beg = 0, deg = 0, du = 0;
                if (idx < qn) {
                    const uint32_t v = __ldcg(qin + idx);
                    beg = __ldg(a.off + v);
                    deg = __ldg(a.off + v + 1) - beg;
                    if (SSSP) du = __ldcg(a.dist + v);
                }
                uint32_t total;
                const uint32_t pos = block_exclusive_scan(deg, s_ws, &total);
                s_incl[tid] = pos + deg;
                s_adj[tid] = beg - pos;
                if (SSSP) s_du[tid] = du;
                __syncthreads();
                for (uint32_t base = 0; base < total; base += BS) {
                    const uint32_t e = base + tid;
                    const bool act = e < total;
                    uint32_t v = 0, alt = 0;
                    if (act) {
                        uint32_t lo = 0, hi = BS - 1; /* first o with s_incl[o] > e */
                        while (lo < hi) {
                            const uint32_t mid = (lo + hi) >> 1;
                            if (s_incl[mid] > e) hi = mid; else lo = mid + 1;
                        }
                        const uint32_t ei = e + s_adj[lo];
                        v = __ldg(a.col + ei);
                        alt = SSSP ? s_du[lo] + __ldg(a.wt + ei) : round + 1;
                    }
                    relax<SSSP>(a, act, v, alt, round, thr, fp, nxt, r3n);
                }
                if (tid == 0) relaxed += total;
            } else {
                /* one chunk of a huge vertex's edge list */
                if (tid == 0) {
                    const uint32_t c = unit - nchunks;
                    uint32_t lo = 0, hi = hitems; /* last item whose first chunk <= c */
                    while (hi - lo > 1) {
                        const uint32_t mid = (lo + hi) >> 1;
                        if (__ldcg(hqbin + mid) <= c) lo = mid; else hi = mid;
                    }
                    const uint32_t v = __ldcg(hqin + lo);
                    const uint32_t b = __ldg(a.off + v), d = __ldg(a.off + v + 1) - b;
                    const uint32_t start = (c - __ldcg(hqbin + lo)) * a.chunk_edges;
                    s_hstart = b + start;
                    s_hcnt = start < d ? min(a.chunk_edges, d - start) : 0u;
                    s_hdu = SSSP ? __ldcg(a.dist + v) : 0;
                }
                __syncthreads();
                const uint32_t hs = s_hstart, hc = s_hcnt, hdu = s_hdu;
                for (uint32_t base = 0; base < hc; base += BS) {
                    const uint32_t e = base + tid;
                    const bool act = e < hc;
                    uint32_t v = 0, alt = 0;
                    if (act) {
                        v = __ldg(a.col + hs + e);
                        alt = SSSP ? hdu + __ldg(a.wt + hs + e) : round + 1;
                    }
                    relax<SSSP>(a, act, v, alt, round, thr, fp, nxt, r3n);
                }
                if (tid == 0) relaxed += hc;
            }
            __syncthreads();
        }
        if (!grid_barrier(&ctl->bar, &ctl->err, a.nblocks, gen, a.timeout_ns)) break;
    }
    if (tid == 0 && relaxed) atomicAdd(&ctl->edges_relaxed, relaxed);
    if (blockIdx.x == 0 && tid == 0) ctl->rounds = round;
}

template <int BS, bool SSSP>
int occupancy() {
    static int occ = -1;
    if (occ < 0) {
        int v = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_frontier<BS, SSSP>, BS, 0) != cudaSuccess) v = 0;
        occ = v;
    }
    return occ;
}

template <int BS, bool SSSP>
gga_status launch(Args &a, const gga_params &p, int sms, cudaStream_t st) {
    int occ = occupancy<BS, SSSP>();
    if (occ <= 0) return gga_fail(GGA_ERR_CUDA, "frontier kernel: zero occupancy");
    int per_sm = p.blocks_per_sm ? (int)p.blocks_per_sm : occ;
    if (per_sm > occ) per_sm = occ;
    a.nblocks = (uint32_t)(sms * per_sm);
    void *args[] = {&a};
    GGA_CK(cudaLaunchCooperativeKernel((const void *)k_frontier<BS, SSSP>, dim3(a.nblocks), dim3(BS), args, 0, st));
    return GGA_OK;
}

} // namespace

static gga_status alloc_u32(uint32_t **p, size_t n) {
    GGA_CK(cudaMalloc((void **)p, (n ? n : 1) * sizeof(uint32_t)));
    return GGA_OK;
}

void frontier_scratch_free(FrontierScratch *s) {
    cudaFree(s->dist); cudaFree(s->bits); cudaFree(s->farbits); cudaFree(s->stamp);
    cudaFree(s->q0); cudaFree(s->q1); cudaFree(s->hq0); cudaFree(s->hq1);
    cudaFree(s->hqb0); cudaFree(s->hqb1); cudaFree(s->far0); cudaFree(s->far1); cudaFree(s->far2);
    cudaFree(s->out); cudaFree(s->ctl);
    memset(s, 0, sizeof *s);
}

gga_status frontier_scratch_ensure(FrontierScratch *s, uint32_t n, uint32_t m) {
    (void)m;
    if (s->cap >= n && s->ctl) return GGA_OK;
    frontier_scratch_free(s);
    const uint32_t cap = n < 1024 ? 1024 : n;
    const size_t words = (cap + 31) / 32 + 1;
    gga_status st;
    if ((st = alloc_u32(&s->dist, cap)) || (st = alloc_u32(&s->bits, words)) ||
        (st = alloc_u32(&s->farbits, words)) || (st = alloc_u32(&s->stamp, cap)) ||
        (st = alloc_u32(&s->q0, cap)) || (st = alloc_u32(&s->q1, cap)) || (st = alloc_u32(&s->hq0, cap)) ||
        (st = alloc_u32(&s->hq1, cap)) || (st = alloc_u32(&s->hqb0, cap)) || (st = alloc_u32(&s->hqb1, cap)) ||
        (st = alloc_u32(&s->far0, cap)) || (st = alloc_u32(&s->far1, cap)) || (st = alloc_u32(&s->far2, cap)) ||
        (st = alloc_u32(&s->out, cap))) {
        frontier_scratch_free(s);
        return st;
    }
    cudaError_t e = cudaMalloc((void **)&s->ctl, sizeof(FrontierCtl));
    if (e != cudaSuccess) {
        frontier_scratch_free(s);
        return gga_fail(GGA_ERR_CUDA, "frontier control block: %s", cudaGetErrorString(e));
    }
    s->cap = cap;
    s->hcap = cap;
    return GGA_OK;
}

gga_status frontier_run(FrontierScratch *s, const GraphView &view, const uint32_t *first, uint32_t src,
                        bool sssp, const gga_params &p, int sms, cudaStream_t st, cudaEvent_t ev0,
                        cudaEvent_t ev1, FrontierResult *res) {
    Args a;
    memset(&a, 0, sizeof a);
    a.off = view.off; a.col = view.col; a.wt = view.wt; a.cc = view.cc;
    a.first = first;
    a.n = view.n;
    a.dist = s->dist; a.bits = s->bits; a.farbits = s->farbits; a.stamp = s->stamp;
    a.q0 = s->q0; a.q1 = s->q1; a.hq0 = s->hq0; a.hq1 = s->hq1; a.hqb0 = s->hqb0; a.hqb1 = s->hqb1;
    a.far0 = s->far0; a.far1 = s->far1; a.far2 = s->far2;
    a.ctl = s->ctl;
    a.cap = s->cap;
    a.hcap = s->hcap;
    a.src = src;
    a.huge_degree = p.huge_degree ? p.huge_degree : 4096;
    a.delta = p.sssp_delta;
    a.timeout_ns = 4000000000ull;
    const uint32_t bs = p.block_threads ? p.block_threads : 256;
    a.chunk_edges = bs * 16;
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
    FrontierCtl h;
    GGA_CK(cudaMemcpyAsync(&h, s->ctl, sizeof h, cudaMemcpyDeviceToHost, st));
    GGA_CK(cudaStreamSynchronize(st));
    if (h.err == GGA_DEV_TIMEOUT)
        return gga_fail(GGA_ERR_TIMEOUT, "frontier grid barrier timed out after %u rounds", h.rounds);
    if (h.err == GGA_DEV_OVERFLOW) return gga_fail(GGA_ERR_CUDA, "frontier queue overflow (internal error)");
    if (h.err != GGA_DEV_OK) return gga_fail(GGA_ERR_CUDA, "frontier kernel error %u", h.err);
    if (res) {
        res->rounds = h.rounds;
        res->launches = 1;
        res->edges_relaxed = h.edges_relaxed;
        res->kernel_ms = 0;
        if (ev0 && ev1) cudaEventElapsedTime(&res->kernel_ms, ev0, ev1);
    }
    return GGA_OK;
}
