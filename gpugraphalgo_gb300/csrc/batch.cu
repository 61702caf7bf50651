/*
 * Batched queries: many BFS / SSSP queries, over any mix of resident graphs,
 * in ONE persistent cooperative launch.
 *
 * The reference answers one source per process run (bfs_sssp.cu:103-539).
 * Here every queue entry carries its query id, so the edge-balanced units of
 * the frontier engine (frontier.cu) are cut from the concatenated frontiers
 * of all queries at once: a tiny query and an R-MAT hub share the same work
 * pool, and a round costs one grid barrier for the whole batch instead of one
 * host round trip per query.  Answers are identical to single-query runs:
 * BFS levels are recomputed per query (round - start round), SSSP uses the
 * improved-vertex frontier (Bellman-Ford order, per-query round stamps), and
 * both converge to the unique distances.
 *
 * The same engine runs in supersteps for the server (serve.cu): a launch
 * processes at most `max_rounds` rounds and stops; between launches new
 * queries are initialised and injected into the next round's queue and
 * finished ones retired (continuous batching).
 *
 * Device memory of a batch (MqEngine): the query table, per-query distance
 * and visited/stamp arrays (pooled by the caller), and queue arrays shared by
 * all queries (entry = query, vertex, edge offset, first edge).
 */
#include <algorithm>
#include <string.h>
#include <vector>

#include "batch.cuh"

namespace {

constexpr uint32_t NONE = 0xffffffffu;
constexpr uint32_t MQ_BS = 256;
constexpr uint32_t MQ_ITERS = 4;
constexpr uint32_t MQ_UNIT = MQ_BS * MQ_ITERS;       /* edges per unit */
constexpr uint32_t MQ_BATCH = 4;                     /* edges per thread between staging checkpoints */
constexpr uint32_t MQ_SCAP = MQ_BS * (MQ_BATCH + 1); /* staging slots per CTA */
constexpr uint32_t MQ_FCH = MQ_BS * 4;               /* far-pile items per split chunk */
static_assert(MQ_MAXQ <= MQ_BS, "one query per thread in the round-start scan");

struct MqArgs {
    const MqQuery *__restrict__ qt;
    MqQstate *qs;
    uint32_t nq;      /* table slots in use */
    uint32_t nearfar; /* SSSP queries run near-far buckets (nq <= MQ_MAXQ) */
    uint32_t *qq0, *qq1, *qv0, *qv1, *qo0, *qo1, *qb0, *qb1, *uf0, *uf1;
    MqCtl *ctl;
    uint32_t cap, ucap;
    uint32_t nblocks;
    uint32_t max_rounds; /* rounds this launch may run */
    unsigned long long timeout_ns;
    /* near-far mode: stop at the start of the first round in which at least
     * this many of the queries that had work when the launch started have
     * finished (0: never) */
    uint32_t stop_on_finish;
    /* NULL, or (zeroed by the caller) per table slot: queue entries and far
     * items the slot has when the launch stops (0: its answer is final) */
    uint32_t *active;
};

__device__ __forceinline__ uint32_t *sel(uint32_t p, uint32_t *a, uint32_t *b) { return p ? b : a; }
__device__ __forceinline__ void set_err(MqCtl *c, uint32_t code) { atomicCAS(&c->err, GGA_DEV_OK, code); }

/* Shared control of one CTA.  The per-query arrays hold this round's view of
 * each query (near-far mode): threshold, the previous threshold (a far split
 * re-queues only items the previous buckets did not expand), the pile far
 * pushes go to, the prefix of far-split work, and flush histograms. */
struct MqCtrl {
    uint32_t nn, fn;
    uint32_t base_i, base_e;
    uint32_t unit, i0, cnt;
    uint32_t nitems, total;
    uint32_t ftot, fany;
    uint32_t nact; /* near-far mode: queries with queue entries or far items this round */
    uint32_t fchunk; /* far-split ticket: its own field, because threads may still
                      * be reading `unit` for the expansion loop's exit test */
    uint32_t ws[32];
    uint32_t thr[MQ_MAXQ], old[MQ_MAXQ], tgt[MQ_MAXQ], pre[MQ_MAXQ + 1];
    uint32_t hist[MQ_MAXQ], base[MQ_MAXQ], fmin[MQ_MAXQ];
};

/* Write queue entry i and the unit boundaries inside its edge range. */
__device__ __forceinline__ void mq_put(const MqArgs &a, uint32_t buf, uint32_t i, uint32_t o, uint32_t q, uint32_t v,
                                       uint32_t b, uint32_t d) {
    if (i >= a.cap) {
        set_err(a.ctl, GGA_DEV_OVERFLOW);
        return;
    }
    sel(buf, a.qq0, a.qq1)[i] = q;
    sel(buf, a.qv0, a.qv1)[i] = v;
    sel(buf, a.qo0, a.qo1)[i] = o;
    sel(buf, a.qb0, a.qb1)[i] = b;
    uint32_t *uf = sel(buf, a.uf0, a.uf1);
    for (uint64_t k = ((uint64_t)o + MQ_UNIT - 1) / MQ_UNIT; k * MQ_UNIT < (uint64_t)o + d; ++k) {
        if (k < a.ucap) uf[k] = i;
        else set_err(a.ctl, GGA_DEV_OVERFLOW_UNITS);
    }
}

struct MqStage {
    uint32_t *sq, *sv, *sb, *sd; /* near: query, vertex, first edge, degree */
    uint32_t *fq, *fv;           /* far: query (| rank << 8 during a flush), vertex */
};

__device__ __forceinline__ void mq_stage(const MqArgs &a, MqCtrl &C, const MqStage &S, uint32_t q, uint32_t v,
                                         uint32_t b, uint32_t d) {
    const uint32_t k = atomicAdd(&C.nn, 1u);
    if (k < MQ_SCAP) {
        S.sq[k] = q;
        S.sv[k] = v;
        S.sb[k] = b;
        S.sd[k] = d;
    } else {
        set_err(a.ctl, GGA_DEV_OVERFLOW);
    }
}

__device__ __forceinline__ void mq_stage_far(const MqArgs &a, MqCtrl &C, const MqStage &S, uint32_t q, uint32_t v) {
    const uint32_t k = atomicAdd(&C.fn, 1u);
    if (k < MQ_SCAP) {
        S.fq[k] = q;
        S.fv[k] = v;
    } else {
        set_err(a.ctl, GGA_DEV_OVERFLOW_FAR);
    }
}

/* Publish the CTA's staged queue entries (block-uniform call, see
 * frontier.cu); in near-far mode also count them per query for round + 1. */
__device__ __forceinline__ void mq_flush(const MqArgs &a, MqCtrl &C, const MqStage &S, uint32_t nn, uint32_t nxt,
                                         uint32_t r3n) {
    if (nn == 0) return;
    const uint32_t tid = threadIdx.x;
    uint32_t *sq = S.sq, *sv = S.sv, *sb = S.sb, *sd = S.sd;
    const uint32_t chunk = (nn + MQ_BS - 1) / MQ_BS;
    const uint32_t j0 = min(tid * chunk, nn), j1 = min(j0 + chunk, nn);
    uint32_t local = 0;
    for (uint32_t j = j0; j < j1; ++j) {
        local += sd[j];
        if (a.nearfar) atomicAdd(&C.hist[sq[j]], 1u);
    }
    uint32_t tot;
    uint32_t run = block_exclusive_scan(local, C.ws, &tot);
    for (uint32_t j = j0; j < j1; ++j) {
        const uint32_t d = sd[j];
        sd[j] = run;
        run += d;
    }
    if (tid == 0) {
        const unsigned long long old =
            atomicAdd(&a.ctl->qctr[r3n], ((unsigned long long)nn << 32) | (unsigned long long)tot);
        C.base_i = (uint32_t)(old >> 32);
        C.base_e = (uint32_t)old;
    }
    if (a.nearfar && tid < a.nq && C.hist[tid]) { /* the scan's barriers ordered the histogram */
        atomicAdd(&a.qs[tid].nr[r3n], C.hist[tid]);
        C.hist[tid] = 0;
    }
    __syncthreads();
    const uint32_t bi = C.base_i, be = C.base_e;
    for (uint32_t j = tid; j < nn; j += MQ_BS) {
        const uint32_t i = bi + j;
        if (i < a.cap) {
            sel(nxt, a.qq0, a.qq1)[i] = sq[j];
            sel(nxt, a.qv0, a.qv1)[i] = sv[j];
            sel(nxt, a.qo0, a.qo1)[i] = be + sd[j];
            sel(nxt, a.qb0, a.qb1)[i] = sb[j];
        } else {
            set_err(a.ctl, GGA_DEV_OVERFLOW);
        }
    }
    uint32_t *uf = sel(nxt, a.uf0, a.uf1);
    const uint64_t k0 = ((uint64_t)be + MQ_UNIT - 1) / MQ_UNIT, k1 = ((uint64_t)be + tot + MQ_UNIT - 1) / MQ_UNIT;
    for (uint64_t k = k0 + tid; k < k1; k += MQ_BS) {
        const uint32_t rel = (uint32_t)(k * MQ_UNIT - be);
        uint32_t lo = 0, hi = nn;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (sd[mid] <= rel) lo = mid; else hi = mid;
        }
        if (k < a.ucap) uf[k] = bi + lo;
        else set_err(a.ctl, GGA_DEV_OVERFLOW_UNITS);
    }
    __syncthreads();
    if (tid == 0) C.nn = 0;
    __syncthreads();
}

/* Publish staged far-pile items: a shared histogram gives each item its rank
 * within its query and the query's smallest distance, then one atomicAdd per
 * query allocates room in the pile the query fills this round. */
__device__ __forceinline__ void mq_flush_far(const MqArgs &a, MqCtrl &C, const MqStage &S, uint32_t nf) {
    if (nf == 0) return;
    const uint32_t tid = threadIdx.x;
    for (uint32_t j = tid; j < nf; j += MQ_BS) {
        const uint32_t q = S.fq[j];
        const uint32_t r = atomicAdd(&C.hist[q], 1u);
        atomicMin(&C.fmin[q], __ldcg(a.qt[q].dist + S.fv[j]));
        S.fq[j] = q | (r << 8);
    }
    __syncthreads();
    if (tid < a.nq && C.hist[tid]) {
        MqQstate *st = a.qs + tid;
        const uint32_t t = C.tgt[tid];
        C.base[tid] = atomicAdd(&st->fc[t], C.hist[tid]);
        atomicMin(&st->fmin[t], C.fmin[tid]);
        C.hist[tid] = 0;
        C.fmin[tid] = NONE;
    }
    __syncthreads();
    for (uint32_t j = tid; j < nf; j += MQ_BS) {
        const uint32_t q = S.fq[j] & 0xffu, r = S.fq[j] >> 8;
        const MqQuery &Q = a.qt[q];
        const uint32_t pos = C.base[q] + r;
        if (pos < Q.n) (C.tgt[q] ? Q.pile1 : Q.pile0)[pos] = S.fv[j];
        else set_err(a.ctl, GGA_DEV_OVERFLOW_FAR);
    }
    __syncthreads();
    if (tid == 0) C.fn = 0;
    __syncthreads();
}

__device__ __forceinline__ void mq_checkpoint(const MqArgs &a, MqCtrl &C, const MqStage &S, uint32_t nxt,
                                              uint32_t r3n, uint32_t limit) {
    __syncthreads();
    const uint32_t nn = C.nn, nf = C.fn;
    __syncthreads();
    if (nn >= limit) mq_flush(a, C, S, nn, nxt, r3n);
    if (nf >= limit) mq_flush_far(a, C, S, nf);
}

/* The batch kernel.  Rounds continue from ctl->round; the launch stops when
 * no query has work left or after a.max_rounds rounds and records where it
 * stopped, so the next launch (after injecting new queries) picks up there.
 *
 * SSSP in near-far mode, per query q (the single-source engine's buckets,
 * frontier.cu, run independently per query inside shared rounds): an
 * improvement below q's threshold joins the next round's queue, one at or
 * above it joins q's far pile.  A round in which q has no queue entries
 * (and q did not split a pile in the previous round) splits q's pile with
 * the threshold raised by q's delta: items below it join the next round's
 * queue, the rest the other pile.  Such a query has no expansion work in
 * that round, so its split runs beside the other queries' expansions without
 * a barrier between them.  Every answer equals the single-source one. */
__global__ void __launch_bounds__(MQ_BS, 4) k_mq(MqArgs a) {
    extern __shared__ uint32_t dyn[];
    __shared__ MqCtrl C;
    MqCtl *ctl = a.ctl;
    const uint32_t tid = threadIdx.x;
    uint32_t *t_o = dyn, *t_b = dyn + (MQ_UNIT + 1), *t_q = dyn + 2 * (MQ_UNIT + 1), *t_a = dyn + 3 * (MQ_UNIT + 1);
    uint32_t *stage = dyn + 4 * (MQ_UNIT + 1);
    MqStage S;
    S.sq = stage;
    S.sv = stage + MQ_SCAP;
    S.sb = stage + 2 * MQ_SCAP;
    S.sd = stage + 3 * MQ_SCAP;
    S.fq = stage + 4 * MQ_SCAP;
    S.fv = stage + 5 * MQ_SCAP;
    uint32_t gen = 0;
    unsigned long long relaxed = 0;
    if (tid == 0) {
        C.nn = 0;
        C.fn = 0;
    }
    if (tid < MQ_MAXQ) {
        C.hist[tid] = 0;
        C.fmin[tid] = NONE;
        C.thr[tid] = NONE;
        C.tgt[tid] = 0;
    }
    __syncthreads();
    uint32_t round = ld_relaxed_u32(&ctl->round); /* fixed before launch */
    uint32_t done = 0, nact0 = 0;
    for (;; ++round, ++done) {
        const uint32_t r3 = round % 3, r3n = (round + 1) % 3, cur = round & 1, nxt = cur ^ 1;
        if (tid == 0) {
            const unsigned long long qc = ld_relaxed_u64(&ctl->qctr[r3]);
            const uint32_t ni = min((uint32_t)(qc >> 32), a.cap);
            C.nitems = ni;
            C.total = ni ? (uint32_t)qc : 0u;
            C.fany = 0;
            C.nact = 0;
        }
        __syncthreads();
        /* ---- this round's view of every query (near-far mode): one thread
         * per table slot; block 0 also writes the next round's bucket state */
        uint32_t fcount = 0;
        if (a.nearfar && tid < a.nq) {
            const MqQuery &Q = a.qt[tid];
            MqQstate *st = a.qs + tid;
            uint32_t thr = NONE, old = NONE, tgt = 0;
            const uint32_t nr = ld_relaxed_u32(&st->nr[r3]);
            bool act = nr != 0;
            if (Q.algo == GGA_SSSP) {
                const uint32_t par = round & 1;
                thr = ld_relaxed_u32(&st->thr[par]);
                const uint32_t fp = ld_relaxed_u32(&st->fp[par]) & 1u, cool = ld_relaxed_u32(&st->cool[par]);
                const uint32_t fc = min(ld_relaxed_u32(&st->fc[fp]), Q.n);
                const uint32_t fm = ld_relaxed_u32(&st->fmin[fp]);
                const uint32_t fpk = ld_relaxed_u32(&st->fpeak[par]);
                old = thr;
                const bool split = nr == 0 && fc > 0 && !cool;
                if (split) {
                    const uint32_t lowest = max(thr, fm);
                    thr = lowest > NONE - Q.delta ? NONE : lowest + Q.delta;
                    /* a small and shrinking pile: no more buckets */
                    if (fc <= Q.tail_at && fc < fpk) thr = NONE;
                    fcount = fc;
                }
                tgt = split ? fp ^ 1u : fp;
                if (fc) atomicAdd(&C.fany, 1u);
                act = act || fc != 0;
                if (blockIdx.x == 0) {
                    st->thr[par ^ 1] = thr;
                    st->fp[par ^ 1] = tgt;
                    st->cool[par ^ 1] = split ? 1u : 0u;
                    st->fpeak[par ^ 1] = max(fpk, fc);
                    if (cool) { /* the pile split last round is free again */
                        st->fc[fp ^ 1] = 0;
                        st->fmin[fp ^ 1] = NONE;
                    }
                }
            }
            /* every query's round counter: read two rounds ago, counted from next round */
            if (blockIdx.x == 0) st->nr[(round + 2) % 3] = 0;
            if (act) atomicAdd(&C.nact, 1u);
            C.thr[tid] = thr;
            C.old[tid] = old;
            C.tgt[tid] = tgt;
        }
        uint32_t ftot = 0;
        if (a.nearfar) { /* prefix of the far-split work (block-uniform) */
            uint32_t t;
            const uint32_t p = block_exclusive_scan(fcount, C.ws, &t);
            if (tid < a.nq) C.pre[tid] = p;
            if (tid == 0) {
                C.pre[a.nq] = t;
                C.ftot = t;
            }
            __syncthreads();
            ftot = C.ftot;
        }
        const uint32_t nitems = C.nitems, total = C.total, fany = a.nearfar ? C.fany : 0u;
        const uint32_t nact = a.nearfar ? C.nact : 0u;
        const uint32_t units = min((uint32_t)(((uint64_t)total + MQ_UNIT - 1) / MQ_UNIT), a.ucap);
        __syncthreads();
        if (done == 0) nact0 = nact;
        /* same decision in every block: the counters are the same everywhere */
        if (done >= a.max_rounds || (units == 0 && fany == 0) ||
            (a.stop_on_finish && a.nearfar && nact + a.stop_on_finish <= nact0))
            break;
        if (blockIdx.x == 0 && tid == 0) {
            ctl->qctr[(round + 2) % 3] = 0;
            ctl->work[(round + 2) % 3] = 0;
            ctl->fwork[(round + 2) % 3] = 0;
        }
        const uint32_t *qq = sel(cur, a.qq0, a.qq1), *qv = sel(cur, a.qv0, a.qv1);
        const uint32_t *qo = sel(cur, a.qo0, a.qo1), *qb = sel(cur, a.qb0, a.qb1);
        const uint32_t *uf = sel(cur, a.uf0, a.uf1);
        /* ---- expansion of the round's queue */
        for (;;) {
            if (tid == 0) {
                const uint32_t k = atomicAdd(&ctl->work[r3], 1u);
                C.unit = k;
                if (k < units) {
                    const uint32_t i0 = min(__ldcg(uf + k), nitems - 1);
                    const uint32_t i1 = k + 1 < units ? min(__ldcg(uf + k + 1), nitems - 1) : nitems - 1;
                    C.i0 = i0;
                    C.cnt = i1 >= i0 ? min(i1 - i0 + 1, MQ_UNIT + 1) : 1u;
                }
            }
            __syncthreads();
            const uint32_t k = C.unit;
            if (k >= units) break;
            const uint32_t i0 = C.i0, cnt = C.cnt;
            const uint32_t ebase = k * MQ_UNIT, eend = min(ebase + MQ_UNIT, total);
            for (uint32_t j = tid; j < cnt; j += MQ_BS) {
                const uint32_t i = i0 + j;
                const uint32_t q = __ldcg(qq + i);
                t_o[j] = __ldcg(qo + i);
                t_b[j] = __ldcg(qb + i);
                t_q[j] = q;
                const MqQuery &Q = a.qt[q];
                /* source distance (SSSP) or the level this round assigns (BFS) */
                t_a[j] = Q.algo == GGA_SSSP ? __ldcg(Q.dist + __ldcg(qv + i)) : round + 1 - Q.start_round;
            }
            __syncthreads();
            for (uint32_t it0 = 0; it0 < MQ_ITERS; it0 += MQ_BATCH) {
                if (it0) mq_checkpoint(a, C, S, nxt, r3n, MQ_BS);
#pragma unroll
                for (uint32_t s = 0; s < MQ_BATCH; ++s) {
                    const uint32_t e = ebase + (it0 + s) * MQ_BS + tid;
                    if (it0 + s >= MQ_ITERS || e >= eend) continue;
                    uint32_t lo = 0, hi = cnt;
                    while (hi - lo > 1) {
                        const uint32_t mid = (lo + hi) >> 1;
                        if (t_o[mid] <= e) lo = mid; else hi = mid;
                    }
                    const uint32_t q = t_q[lo];
                    const MqQuery &Q = a.qt[q];
                    const uint32_t ei = t_b[lo] + (e - t_o[lo]);
                    if (ei >= Q.m) {
                        set_err(ctl, GGA_DEV_BAD_EDGE);
                        continue;
                    }
                    const uint32_t v = __ldg(Q.col + ei);
                    uint32_t *dist = Q.dist;
                    uint32_t *aux = Q.aux;
                    bool push = false;
                    if (Q.algo == GGA_SSSP) {
                        const uint32_t alt = t_a[lo] + __ldg(Q.wt + ei);
                        /* an offer that beats the probe: fire-and-forget min, and v
                         * is queued by its stamp without waiting for the old value
                         * (its expansion reads the distance then) */
                        if (alt < __ldcg(dist + v)) {
                            red_min_u32(dist + v, alt);
                            const uint32_t thr = a.nearfar ? C.thr[q] : NONE;
                            if (alt < thr) {
                                push = atomicExch(aux + v, round + 1) != round + 1;
                            } else {
                                const uint32_t bit = 1u << (v & 31);
                                if (!(atomicOr(Q.fbits + (v >> 5), bit) & bit)) mq_stage_far(a, C, S, q, v);
                            }
                        }
                    } else {
                        const uint32_t bit = 1u << (v & 31);
                        if (!(__ldcg(aux + (v >> 5)) & bit) && !(atomicOr(aux + (v >> 5), bit) & bit)) {
                            dist[v] = t_a[lo];
                            push = true;
                        }
                    }
                    if (push) {
                        const uint32_t *off = Q.off;
                        const uint32_t b = __ldg(off + v), d = __ldg(off + v + 1) - b;
                        if (d) mq_stage(a, C, S, q, v, b, d);
                    }
                }
            }
            if (tid == 0) relaxed += eend - ebase;
            mq_checkpoint(a, C, S, nxt, r3n, MQ_BS);
        }
        /* ---- far-pile splits of the queries that had no queue entries */
        if (ftot) {
            for (;;) {
                if (tid == 0) C.fchunk = atomicAdd(&ctl->fwork[r3], 1u);
                __syncthreads();
                const uint64_t c0 = (uint64_t)C.fchunk * MQ_FCH;
                if (c0 >= ftot) break;
                const uint32_t c1 = (uint32_t)min((uint64_t)ftot, c0 + MQ_FCH);
                for (uint32_t i = (uint32_t)c0 + tid; i < c1; i += MQ_BS) {
                    uint32_t lo = 0, hi = a.nq; /* last q with pre[q] <= i */
                    while (hi - lo > 1) {
                        const uint32_t mid = (lo + hi) >> 1;
                        if (C.pre[mid] <= i) lo = mid; else hi = mid;
                    }
                    const uint32_t q = lo;
                    const MqQuery &Q = a.qt[q];
                    const uint32_t *pile = C.tgt[q] ? Q.pile0 : Q.pile1; /* splitting: the pile not being filled */
                    const uint32_t v = __ldcg(pile + (i - C.pre[q]));
                    const uint32_t d = __ldcg(Q.dist + v);
                    if (d >= C.thr[q]) {
                        mq_stage_far(a, C, S, q, v); /* stays far, in the other pile */
                    } else {
                        atomicAnd(Q.fbits + (v >> 5), ~(1u << (v & 31)));
                        if (d >= C.old[q] && atomicExch(Q.aux + v, round + 1) != round + 1) {
                            const uint32_t b = __ldg(Q.off + v), dg = __ldg(Q.off + v + 1) - b;
                            if (dg) mq_stage(a, C, S, q, v, b, dg);
                        }
                    }
                }
                mq_checkpoint(a, C, S, nxt, r3n, MQ_BS);
            }
        }
        mq_checkpoint(a, C, S, nxt, r3n, 1);
        if (!grid_barrier(&ctl->bar, &ctl->err, a.nblocks, gen, a.timeout_ns)) break;
    }
    if (tid == 0 && relaxed) atomicAdd(&ctl->edges_relaxed, relaxed);
    /* what each slot still has when round `round` starts (k_mq_count's
     * figures, without a second launch): that round's queue is complete, and
     * the piles' counters are those round `round` reads */
    if (a.active) {
        const unsigned long long qc = ld_relaxed_u64(&ctl->qctr[round % 3]);
        const uint32_t ni = min((uint32_t)(qc >> 32), a.cap);
        const uint32_t *qq = sel(round & 1, a.qq0, a.qq1);
        for (uint64_t i = (uint64_t)blockIdx.x * MQ_BS + tid; i < ni; i += (uint64_t)gridDim.x * MQ_BS)
            atomicAdd(a.active + __ldcg(qq + i), 1u);
        if (a.nearfar && blockIdx.x == 0)
            for (uint32_t q = tid; q < a.nq; q += MQ_BS) {
                const MqQstate &st = a.qs[q];
                const uint32_t fc = ld_relaxed_u32(&st.fc[ld_relaxed_u32(&st.fp[round & 1]) & 1u]);
                if (fc) atomicAdd(a.active + q, fc);
            }
    }
    if (blockIdx.x == 0 && tid == 0) {
        ctl->round = round;
        ctl->rounds_done += done;
    }
}

/* Copies each staged record to its table slot and sets the query's state
 * before its first round: dist = MYINFINITY, visited bits / stamps and the
 * far bitmap cleared.  Block row y handles queries y, y + gridDim.y, ... */
__global__ void k_mq_init(MqQuery *qt, const MqQuery *stage, const uint32_t *list, uint32_t nlist) {
    for (uint32_t t = blockIdx.y; t < nlist; t += gridDim.y) {
        const MqQuery Q = stage[t];
        if (blockIdx.x == 0 && threadIdx.x == 0) qt[list[t]] = Q;
        const uint32_t naux = Q.algo == GGA_SSSP ? Q.n : (Q.n + 31) / 32;
        const uint32_t nfb = Q.algo == GGA_SSSP ? (Q.n + 31) / 32 : 0;
        for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < Q.n; i += gridDim.x * blockDim.x)
            Q.dist[i] = GGA_INFINITY;
        for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < naux; i += gridDim.x * blockDim.x) Q.aux[i] = 0;
        for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nfb; i += gridDim.x * blockDim.x) Q.fbits[i] = 0;
    }
}

/* Puts each listed query's source into the queue of round ctl->round and
 * sets its counters and bucket state (one thread, a few queries per call:
 * appends are serialised on purpose). */
__global__ void k_mq_inject(MqArgs a, MqQuery *qt, const uint32_t *list, uint32_t nlist) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    MqCtl *ctl = a.ctl;
    const uint32_t round = ctl->round, par = round & 1;
    for (uint32_t t = 0; t < nlist; ++t) {
        const uint32_t q = list[t];
        MqQuery *Q = qt + q;
        const uint32_t s = Q->src;
        Q->start_round = round;
        Q->dist[s] = 0;
        if (Q->algo == GGA_SSSP) Q->aux[s] = round;
        else Q->aux[s >> 5] |= 1u << (s & 31);
        const uint32_t b = Q->off[s], d = Q->off[s + 1] - b;
        if (a.qs) {
            MqQstate *st = a.qs + q;
            for (int k = 0; k < 3; ++k) st->nr[k] = 0;
            for (int k = 0; k < 2; ++k) {
                st->fc[k] = 0;
                st->fmin[k] = NONE;
            }
            st->thr[par] = Q->algo == GGA_SSSP && Q->delta ? Q->delta : NONE;
            st->fp[par] = 0;
            st->cool[par] = 0;
            st->fpeak[0] = st->fpeak[1] = 0;
            st->nr[round % 3] = d ? 1u : 0u;
        }
        if (!d) continue;
        const unsigned long long old = atomicAdd(&ctl->qctr[round % 3], (1ull << 32) | d);
        mq_put(a, round & 1, (uint32_t)(old >> 32), (uint32_t)old, q, s, b, d);
    }
}

/* active[q] = queue entries and far-pile items query q still has when round
 * ctl->round starts (0: its distances are final). */
__global__ void k_mq_count(MqArgs a, uint32_t *active) {
    const MqCtl *ctl = a.ctl;
    const uint32_t round = ctl->round;
    const unsigned long long qc = ctl->qctr[round % 3];
    const uint32_t ni = min((uint32_t)(qc >> 32), a.cap);
    const uint32_t *qq = sel(round & 1, a.qq0, a.qq1);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < ni; i += gridDim.x * blockDim.x)
        atomicAdd(active + qq[i], 1u);
    if (a.nearfar)
        for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < a.nq; q += gridDim.x * blockDim.x) {
            const MqQstate &st = a.qs[q];
            const uint32_t fc = st.fc[st.fp[round & 1] & 1u];
            if (fc) atomicAdd(active + q, fc);
        }
}

/* Reached vertices and their out-edges summed over the listed queries. */
__global__ void k_mq_reached(const MqQuery *qt, uint32_t nq, unsigned long long *acc) {
    unsigned long long vr = 0, er = 0;
    for (uint32_t t = blockIdx.y; t < nq; t += gridDim.y) {
        const MqQuery &Q = qt[t];
        for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < Q.n; i += gridDim.x * blockDim.x)
            if (Q.dist[i] < GGA_INFINITY) {
                vr++;
                er += Q.off[i + 1] - Q.off[i];
            }
    }
    for (int d = 16; d > 0; d >>= 1) {
        vr += __shfl_down_sync(0xffffffffu, vr, d);
        er += __shfl_down_sync(0xffffffffu, er, d);
    }
    if ((threadIdx.x & 31) == 0 && (vr || er)) {
        atomicAdd(acc, vr);
        atomicAdd(acc + 1, er);
    }
}

} // namespace

/* ------------------------------------------------------------ engine */

namespace {

size_t mq_smem() { return ((size_t)4 * (MQ_UNIT + 1) + (size_t)6 * MQ_SCAP) * sizeof(uint32_t); }

template <typename T> gga_status grow(T **p, uint32_t *have, uint32_t want, const char *what) {
    if (*have >= want) return GGA_OK;
    cudaFree(*p);
    *p = nullptr;
    *have = 0;
    cudaError_t e = cudaMalloc((void **)p, (size_t)want * sizeof(T));
    if (e != cudaSuccess) {
        cudaGetLastError();
        return gga_fail(GGA_ERR_CUDA, "batch %s (%u entries): %s", what, want, cudaGetErrorString(e));
    }
    *have = want;
    return GGA_OK;
}

/* Table slots a launch scans: the caller's nslots, else every slot. */
uint32_t mq_slots(const MqEngine *e) { return e->nslots ? std::min(e->nslots, e->qcap) : e->qcap; }

MqArgs mq_args(const MqEngine *e) {
    MqArgs a;
    memset(&a, 0, sizeof a);
    a.qt = e->qt;
    a.qs = e->qs;
    a.nq = mq_slots(e);
    a.nearfar = a.nq <= MQ_MAXQ ? 1u : 0u;
    a.qq0 = e->qq[0]; a.qq1 = e->qq[1];
    a.qv0 = e->qv[0]; a.qv1 = e->qv[1];
    a.qo0 = e->qo[0]; a.qo1 = e->qo[1];
    a.qb0 = e->qb[0]; a.qb1 = e->qb[1];
    a.uf0 = e->uf[0]; a.uf1 = e->uf[1];
    a.ctl = e->ctl;
    a.cap = e->cap;
    a.ucap = e->ucap;
    a.nblocks = (uint32_t)e->nblocks;
    a.timeout_ns = 4000000000ull;
    return a;
}

} // namespace

gga_status mq_engine_reserve(MqEngine *e, int device, uint32_t cap, uint64_t edges, uint32_t qcap) {
    if (e->device != device) {
        mq_engine_free(e);
        e->device = device;
    }
    if (edges + 2ull * MQ_UNIT > 0xFFFFFFFFull)
        return gga_fail(GGA_ERR_TOO_LARGE, "batch holds %llu edges; one batch is limited to %u",
                        (unsigned long long)edges, 0xFFFFFFFFu - 2 * MQ_UNIT);
    if (cap == 0) cap = 1;
    if (qcap == 0) qcap = 1;
    const uint32_t ucap = (uint32_t)(edges / MQ_UNIT + 4);
    gga_status s;
    for (int b = 0; b < 2; ++b) {
        uint32_t h;
        h = e->cap; if ((s = grow(&e->qq[b], &h, cap, "queue"))) return s;
        h = e->cap; if ((s = grow(&e->qv[b], &h, cap, "queue"))) return s;
        h = e->cap; if ((s = grow(&e->qo[b], &h, cap, "queue"))) return s;
        h = e->cap; if ((s = grow(&e->qb[b], &h, cap, "queue"))) return s;
        h = e->ucap; if ((s = grow(&e->uf[b], &h, ucap, "unit table"))) return s;
    }
    if (e->cap < cap) e->cap = cap;
    if (e->ucap < ucap) e->ucap = ucap;
    if (e->qcap < qcap) {
        uint32_t h = e->qcap;
        if ((s = grow(&e->qt, &h, qcap, "query table"))) return s;
        h = e->qcap; if ((s = grow(&e->qstage, &h, qcap, "query staging"))) return s;
        h = e->qcap; if ((s = grow(&e->qs, &h, qcap, "query counters"))) return s;
        GGA_CK(cudaMemset(e->qt, 0, (size_t)qcap * sizeof(MqQuery)));
        GGA_CK(cudaMemset(e->qs, 0, (size_t)qcap * sizeof(MqQstate)));
        h = e->qcap; if ((s = grow(&e->list, &h, qcap, "query list"))) return s;
        h = e->qcap; if ((s = grow(&e->active, &h, qcap, "query counts"))) return s;
        cudaFreeHost(e->hactive);
        e->hactive = nullptr;
        GGA_CK(cudaMallocHost((void **)&e->hactive, (size_t)qcap * sizeof(uint32_t)));
        e->qcap = qcap;
    }
    if (!e->ctl) {
        GGA_CK(cudaMalloc((void **)&e->ctl, sizeof(MqCtl)));
        GGA_CK(cudaMallocHost((void **)&e->hctl, sizeof(MqCtl)));
    }
    if (!e->nblocks) {
        const size_t smem = mq_smem();
        GGA_CK(cudaFuncSetAttribute(k_mq, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int occ = 0, sms = 0;
        GGA_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_mq, MQ_BS, smem));
        GGA_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
        if (occ <= 0) return gga_fail(GGA_ERR_CUDA, "batch kernel: zero occupancy");
        e->nblocks = occ * sms;
    }
    return GGA_OK;
}

void mq_engine_free(MqEngine *e) {
    for (int b = 0; b < 2; ++b) {
        cudaFree(e->qq[b]);
        cudaFree(e->qv[b]);
        cudaFree(e->qo[b]);
        cudaFree(e->qb[b]);
        cudaFree(e->uf[b]);
    }
    cudaFree(e->qt);
    cudaFree(e->qs);
    cudaFree(e->qstage);
    cudaFree(e->list);
    cudaFree(e->active);
    cudaFree(e->ctl);
    cudaFreeHost(e->hctl);
    cudaFreeHost(e->hactive);
    *e = MqEngine();
}

gga_status mq_engine_reset(MqEngine *e, cudaStream_t st) {
    GGA_CK(cudaMemsetAsync(e->ctl, 0, sizeof(MqCtl), st));
    if (e->qs) GGA_CK(cudaMemsetAsync(e->qs, 0, (size_t)e->qcap * sizeof(MqQstate), st));
    e->rounds_done = 0;
    e->edges_relaxed = 0;
    return GGA_OK;
}

gga_status mq_engine_admit(MqEngine *e, const MqQuery *host_q, const uint32_t *slots, uint32_t n, cudaStream_t st) {
    if (n == 0) return GGA_OK;
    if (n > e->qcap) return gga_fail(GGA_ERR_INVALID_ARG, "admitting %u queries into %u slots", n, e->qcap);
    for (uint32_t i = 0; i < n; ++i)
        if (slots[i] >= e->qcap) return gga_fail(GGA_ERR_INVALID_ARG, "slot %u of %u", slots[i], e->qcap);
    GGA_CK(cudaMemcpyAsync(e->qstage, host_q, (size_t)n * sizeof(MqQuery), cudaMemcpyHostToDevice, st));
    GGA_CK(cudaMemcpyAsync(e->list, slots, (size_t)n * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    uint32_t maxn = 1;
    for (uint32_t i = 0; i < n; ++i) maxn = std::max(maxn, host_q[i].n);
    const uint32_t gx = std::min<uint32_t>((maxn + 255) / 256, 64);
    const uint32_t gy = std::min<uint32_t>(n, 1024);
    k_mq_init<<<dim3(gx, gy), 256, 0, st>>>(e->qt, e->qstage, e->list, n);
    GGA_CK(cudaGetLastError());
    MqArgs a = mq_args(e);
    k_mq_inject<<<1, 1, 0, st>>>(a, e->qt, e->list, n);
    GGA_CK(cudaGetLastError());
    return GGA_OK;
}

gga_status mq_engine_run(MqEngine *e, uint32_t max_rounds, cudaStream_t st, cudaEvent_t ev0, cudaEvent_t ev1,
                         uint32_t *rounds_run, float *ms, uint32_t superstep) {
    MqArgs a = mq_args(e);
    a.max_rounds = max_rounds;
    const uint32_t ns = mq_slots(e); /* a.nq: every slot the launch scans gets a count */
    if (superstep) {
        a.stop_on_finish = superstep;
        a.active = e->active;
        GGA_CK(cudaMemsetAsync(e->active, 0, (size_t)(ns ? ns : 1) * sizeof(uint32_t), st));
    }
    GGA_CK(cudaMemsetAsync(&e->ctl->bar, 0, sizeof(GridBarrier), st));
    if (ev0) GGA_CK(cudaEventRecord(ev0, st));
    void *args[] = {&a};
    GGA_CK(cudaLaunchCooperativeKernel((const void *)k_mq, dim3(a.nblocks), dim3(MQ_BS), args, mq_smem(), st));
    if (ev1) GGA_CK(cudaEventRecord(ev1, st));
    GGA_CK(cudaMemcpyAsync(e->hctl, e->ctl, sizeof(MqCtl), cudaMemcpyDeviceToHost, st));
    if (superstep && ns)
        GGA_CK(cudaMemcpyAsync(e->hactive, e->active, (size_t)ns * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    gga_status s = dev_wait(st, 60.0);
    if (s) return s;
    const MqCtl &h = *e->hctl;
    if (rounds_run) *rounds_run = h.rounds_done - e->rounds_done;
    e->rounds_done = h.rounds_done;
    e->edges_relaxed = h.edges_relaxed;
    if (ms) {
        *ms = 0;
        if (ev0 && ev1) GGA_CK(cudaEventElapsedTime(ms, ev0, ev1));
    }
    switch (h.err) {
    case GGA_DEV_OK: return GGA_OK;
    case GGA_DEV_TIMEOUT: return gga_fail(GGA_ERR_TIMEOUT, "batch grid barrier timed out at round %u", h.round);
    case GGA_DEV_OVERFLOW: return gga_fail(GGA_ERR_CUDA, "batch queue overflow (internal error)");
    case GGA_DEV_OVERFLOW_UNITS: return gga_fail(GGA_ERR_CUDA, "batch unit table overflow (internal error)");
    case GGA_DEV_BAD_EDGE: return gga_fail(GGA_ERR_CUDA, "batch edge index out of range (internal error)");
    default: return gga_fail(GGA_ERR_CUDA, "batch kernel error %u", h.err);
    }
}

gga_status mq_engine_count(MqEngine *e, uint32_t nslots, cudaStream_t st) {
    if (nslots > e->qcap) nslots = e->qcap;
    if (nslots == 0) return GGA_OK;
    GGA_CK(cudaMemsetAsync(e->active, 0, (size_t)nslots * sizeof(uint32_t), st));
    MqArgs a = mq_args(e);
    k_mq_count<<<std::max(1, e->nblocks), 256, 0, st>>>(a, e->active);
    GGA_CK(cudaGetLastError());
    GGA_CK(cudaMemcpyAsync(e->hactive, e->active, (size_t)nslots * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    return dev_wait(st, 60.0);
}

/* ------------------------------------------------------------ scratch */

static size_t r64(size_t w) { return (w + 63) & ~(size_t)63; }

size_t mq_state_words(uint32_t n, uint32_t algo) {
    if (algo == GGA_SSSP) /* dist, stamps, far bitmap, two far piles */
        return r64(n) + r64(n) + r64(((size_t)n + 31) / 32) + 2 * r64(n);
    return r64(n) + r64(((size_t)n + 31) / 32); /* levels, visited bitmap */
}

void mq_state_layout(MqQuery *q, uint32_t *base) {
    const size_t n = q->n;
    q->dist = base;
    q->aux = base + r64(n);
    q->fbits = q->pile0 = q->pile1 = nullptr;
    if (q->algo == GGA_SSSP) {
        q->fbits = q->aux + r64(n);
        q->pile0 = q->fbits + r64((n + 31) / 32);
        q->pile1 = q->pile0 + r64(n);
    }
}

BatchScratch *ctx_batch(gga_ctx *c) {
    if (!c->batch) c->batch = new (std::nothrow) BatchScratch();
    return c->batch;
}

gga_status batch_pool_reserve(BatchScratch *b, size_t words) {
    if (b->pool_words >= words) return GGA_OK;
    cudaFree(b->pool);
    b->pool = nullptr;
    b->pool_words = 0;
    cudaError_t e = cudaMalloc((void **)&b->pool, words * sizeof(uint32_t));
    if (e != cudaSuccess) {
        cudaGetLastError();
        return gga_fail(GGA_ERR_CUDA, "batch state (%zu MiB): %s", (words * 4) >> 20, cudaGetErrorString(e));
    }
    b->pool_words = words;
    return GGA_OK;
}

void ctx_batch_release(gga_ctx *c) {
    if (!c->batch) return;
    mq_engine_free(&c->batch->eng);
    cudaFree(c->batch->pool);
    msbfs_scratch_free(c->batch->ms);
    su_scratch_free(c->batch->su);
    delete c->batch;
    c->batch = nullptr;
}

/* ------------------------------------------------------------ API */

gga_status gga_multi_solve(gga_ctx *c, uint32_t nq, const gga_query *queries, gga_stats *stats) {
    const double t0 = gga_now_ms();
    if (!c || (nq && !queries)) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    gga_stats st;
    memset(&st, 0, sizeof st);
    if (nq == 0) {
        if (stats) *stats = st;
        return GGA_OK;
    }
    gga_status s;
    for (uint32_t i = 0; i < nq; ++i) {
        const gga_query &q = queries[i];
        if (!q.graph || !q.dist_out) return gga_fail(GGA_ERR_INVALID_ARG, "query %u: NULL graph or dist_out", i);
        if ((s = ctx_validate_solve(q.graph, (gga_algo)q.algo, q.src))) return s;
    }
    std::lock_guard<std::mutex> lk(c->mu);
    if ((s = ctx_activate(c))) return s;
    BatchScratch *b = ctx_batch(c);
    if (!b) return gga_fail(GGA_ERR_NO_MEMORY, "batch scratch");
    uint64_t cap = 0, edges = 0;
    size_t words = 0;
    uint32_t maxn = 0;
    for (uint32_t i = 0; i < nq; ++i) {
        gga_graph *g = queries[i].graph;
        if ((s = dev_graph_ensure(g, c->device, c->st))) return s;
        cap += g->n;
        edges += g->m;
        words += mq_state_words(g->n, queries[i].algo);
        maxn = std::max(maxn, g->n);
    }
    if (cap > 0xFFFFFFF0ull) return gga_fail(GGA_ERR_TOO_LARGE, "batch holds %llu vertices", (unsigned long long)cap);
    if ((s = batch_pool_reserve(b, words))) return s;
    if ((s = mq_engine_reserve(&b->eng, c->device, (uint32_t)cap, edges, nq))) return s;
    std::vector<MqQuery> hq(nq);
    std::vector<uint32_t> slots(nq);
    size_t at = 0;
    for (uint32_t i = 0; i < nq; ++i) {
        const gga_query &q = queries[i];
        const DevGraph *d = dev_graph_of(q.graph);
        MqQuery &r = hq[i];
        memset(&r, 0, sizeof r);
        r.off = d->off;
        r.col = d->col;
        r.wt = d->wt;
        r.n = d->n;
        r.m = d->m;
        r.algo = q.algo;
        r.src = q.src;
        r.delta = q.algo == GGA_SSSP ? ctx_batch_delta(q.graph) : 0;
        r.tail_at = r.delta && (uint64_t)d->m >= 8ull * d->n ? d->n / 4 : 0; /* graphs averaging 8+ edges per vertex */
        mq_state_layout(&r, b->pool + at);
        at += mq_state_words(d->n, q.algo);
        slots[i] = i;
    }
    MqEngine *e = &b->eng;
    e->nslots = nq;
    if ((s = mq_engine_reset(e, c->st))) return s;
    if ((s = mq_engine_admit(e, hq.data(), slots.data(), nq, c->st))) return s;
    uint32_t rounds = 0;
    float ms = 0;
    const uint32_t max_rounds = maxn > 0x3fffffffu ? 0xffffffffu : 4u * maxn + 4096u;
    if ((s = mq_engine_run(e, max_rounds, c->st, c->ev[0], c->ev[1], &rounds, &ms))) return s;
    if (rounds >= max_rounds)
        return gga_fail(GGA_ERR_CUDA, "batch did not converge in %u rounds (internal error)", rounds);
    st.iterations = rounds;
    st.kernel_launches = 3;
    st.edges_relaxed = e->edges_relaxed;
    st.kernel_ms = ms;
    for (uint32_t i = 0; i < nq; ++i) {
        const gga_query &q = queries[i];
        GGA_CK(cudaMemcpyAsync(q.dist_out, hq[i].dist, (size_t)hq[i].n * sizeof(uint32_t),
                               ptr_is_device(q.dist_out) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c->st));
    }
    if (stats) {
        unsigned long long *acc = (unsigned long long *)(c->dflag + 32);
        GGA_CK(cudaMemsetAsync(acc, 0, 2 * sizeof(unsigned long long), c->st));
        const uint32_t gx = std::min<uint32_t>((maxn + 255) / 256, 64);
        k_mq_reached<<<dim3(gx, std::min<uint32_t>(nq, 1024)), 256, 0, c->st>>>(e->qt, nq, acc);
        GGA_CK(cudaGetLastError());
        GGA_CK(cudaMemcpyAsync(c->hflag + 32, acc, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->st));
        st.kernel_launches++;
    }
    if ((s = dev_wait(c->st, 60.0))) return s;
    if (stats) {
        const unsigned long long *h = (const unsigned long long *)(c->hflag + 32);
        st.vertices_reached = h[0];
        st.edges_reached = h[1];
        st.total_ms = gga_now_ms() - t0;
        *stats = st;
    }
    return GGA_OK;
}

