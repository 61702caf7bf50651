/*
 * Batch engine interface (batch.cu): many queries in one persistent launch.
 */
#pragma once
#include <vector>

#include "ctx.cuh"

/* Queries per launch for which SSSP runs near-far buckets (per-query shared
 * memory in the kernel); larger batches run SSSP in Bellman-Ford order. */
constexpr uint32_t MQ_MAXQ = 256;

/* One query as the batch kernel sees it (device memory). */
struct MqQuery {
    const uint32_t *off, *col, *wt; /* the graph's unsplit CSR (device) */
    uint32_t *dist;                 /* n distances / levels */
    uint32_t *aux;                  /* BFS: visited bitmap (n/32 words); SSSP: round stamps (n) */
    uint32_t *fbits;                /* SSSP: "in a far pile" bitmap (n/32 words) */
    uint32_t *pile0, *pile1;        /* SSSP: far piles (n each) */
    uint32_t n, m;
    uint32_t algo;        /* gga_algo */
    uint32_t src;
    uint32_t start_round; /* round in which the source is expanded */
    uint32_t delta;       /* SSSP bucket width (0: Bellman-Ford order) */
    /* SSSP: once the query's near queue drains with at most this many far-pile
     * entries, below the largest pile it has had, its buckets end and the
     * rest runs label-correcting (threshold infinity); 0 = never */
    uint32_t tail_at;
    uint32_t pad;
};

/* Per-query counters and bucket state of the batch kernel.  Counters are
 * updated with atomics; the bucket state is double-buffered by round parity
 * (round r reads entry r & 1, block 0 writes entry (r + 1) & 1). */
struct MqQstate {
    uint32_t nr[3];   /* queue entries for the round with this index mod 3 */
    uint32_t fc[2];   /* far pile sizes */
    uint32_t fmin[2]; /* smallest distance in each pile (a lower bound) */
    uint32_t thr[2];  /* near threshold */
    uint32_t fp[2];   /* pile that far pushes go to */
    uint32_t cool[2]; /* 1: split a pile in the previous round */
    uint32_t fpeak[2]; /* largest far pile seen */
};

/* Control block of the batch kernel; persists across superstep launches
 * (only the barrier is reset before each launch). */
struct MqCtl {
    GridBarrier bar;
    uint32_t err;
    uint32_t round;       /* next round to run */
    uint32_t rounds_done; /* rounds run so far */
    uint32_t pad0;
    unsigned long long qctr[3]; /* (entries << 32) | edges, rotating by round */
    uint32_t work[3];
    uint32_t fwork[3];          /* far-split chunk tickets, rotating by round */
    unsigned long long edges_relaxed;
};

/* Device buffers of one batch engine. */
struct MqEngine {
    int device = -1;
    uint32_t cap = 0;  /* queue entries (>= sum of admitted queries' n) */
    uint32_t ucap = 0; /* unit boundaries (>= sum of m / unit + 4) */
    uint32_t qcap = 0; /* query-table slots */
    uint32_t *qq[2] = {}, *qv[2] = {}, *qo[2] = {}, *qb[2] = {}, *uf[2] = {};
    MqQuery *qt = nullptr;    /* device query table */
    MqQstate *qs = nullptr;   /* device per-query counters (qcap) */
    uint32_t nslots = 0;      /* table slots the kernel scans (set by the caller) */
    MqQuery *qstage = nullptr; /* device staging for admitted records (qcap) */
    uint32_t *list = nullptr; /* device index list for init / inject (qcap) */
    uint32_t *active = nullptr; /* device per-query entry counts (qcap) */
    MqCtl *ctl = nullptr;
    MqCtl *hctl = nullptr;    /* pinned mirror */
    uint32_t *hactive = nullptr; /* pinned mirror of active */
    int nblocks = 0;
    uint32_t rounds_done = 0;          /* rounds run since the last reset */
    unsigned long long edges_relaxed = 0;
};

gga_status mq_engine_reserve(MqEngine *e, int device, uint32_t cap, uint64_t edges, uint32_t qcap);
void mq_engine_free(MqEngine *e);
/* Zeroes the control block (round 0, empty queues). */
gga_status mq_engine_reset(MqEngine *e, cudaStream_t st);
/* Uploads the n query records `host_q` into table slots `slots`, initialises
 * their distance / visited state and injects their sources into the queue of
 * the next round. */
gga_status mq_engine_admit(MqEngine *e, const MqQuery *host_q, const uint32_t *slots, uint32_t n, cudaStream_t st);
/* Runs at most max_rounds rounds (UINT32_MAX: until the queue drains) and
 * waits for them; *rounds_run receives the rounds this launch ran.  With
 * superstep = k > 0 (near-far mode, at most MQ_MAXQ slots) the launch also
 * stops at the first round in which k of its queries have finished, and
 * fills e->hactive with what each slot still has then (as mq_engine_count
 * does). */
gga_status mq_engine_run(MqEngine *e, uint32_t max_rounds, cudaStream_t st, cudaEvent_t ev0, cudaEvent_t ev1,
                         uint32_t *rounds_run, float *ms, uint32_t superstep = 0);
/* Fills e->hactive[slot] with the queue entries each slot still has. */
gga_status mq_engine_count(MqEngine *e, uint32_t nslots, cudaStream_t st);

struct MsbfsScratch;
struct SuScratch;

/* Batch state owned by a context (created on first batched call). */
struct BatchScratch {
    MqEngine eng;
    uint32_t *pool = nullptr; /* per-query dist + visited / stamp words */
    size_t pool_words = 0;
    MsbfsScratch *ms = nullptr;
    SuScratch *su = nullptr;
};

BatchScratch *ctx_batch(gga_ctx *c);
gga_status batch_pool_reserve(BatchScratch *b, size_t words);
void msbfs_scratch_free(MsbfsScratch *m);
void su_scratch_free(SuScratch *s);
/* Words of device state one query needs (dist + visited bits or stamps),
 * each part rounded up to 64 words. */
size_t mq_state_words(uint32_t n, uint32_t algo);
/* Lays one query's state out at `base` (dist, aux, and for SSSP the far
 * bitmap and piles). */
void mq_state_layout(MqQuery *q, uint32_t *base);
