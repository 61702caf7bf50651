/*
 * Frontier engine interface (frontier.cu).
 */
#pragma once
#include "gga_device.cuh"

/* Control block of one persistent frontier launch (zeroed before launch). */
struct FrontierCtl {
    GridBarrier bar;
    uint32_t err;
    uint32_t rounds;
    unsigned long long qctr[3];   /* near queue: (entries << 32) | edges, rotating by round */
    uint32_t far_count[3];        /* three far piles rotate across far passes */
    uint32_t far_min[3];
    uint32_t far_phases;
    unsigned long long hctr[3];   /* SSSP heavy lists: (entries << 32) | edges, rotating by bucket */
    uint32_t overflow_at;
    unsigned long long edges_relaxed;
    uint32_t diag[16];            /* first failed self-check: where and what */
};

/* Per-context device scratch of the frontier engine, sized by vertices. */
struct FrontierScratch {
    uint32_t cap;        /* vertex capacity */
    uint32_t ucap;       /* unit-boundary capacity */
    uint32_t *dist;      /* cap */
    uint32_t *bits;      /* cap/32: BFS visited / SSSP unused */
    uint32_t *farbits;   /* cap/32: SSSP "in far pile" */
    uint32_t *stamp;     /* cap: SSSP last round a vertex was queued */
    uint32_t *qv0, *qv1; /* near queues: vertex */
    uint32_t *qo0, *qo1; /* exclusive edge offset of each entry in the round */
    uint32_t *qb0, *qb1; /* first edge of each entry in the CSR */
    uint32_t *uf0, *uf1; /* unit k's first entry */
    uint32_t *far0, *far1, *far2;
    uint32_t *out;       /* cap: gathered original-order output */
    uint32_t *trace;     /* (TRACE_ROUNDS + 1) round records + per-CTA busy kilocycles */
    uint32_t *hstamp;    /* cap: SSSP light/heavy mode, bucket a vertex last joined a heavy list */
    uint32_t *pbest;     /* cap: SSSP pull rounds, the best offer per pull-list entry */
    uint32_t *hv[3], *ho[3], *hb[3], *huf[3]; /* heavy lists (cap, cap, cap, ucap) */
    FrontierCtl *ctl;
    FrontierCtl *hctl;   /* pinned host mirror (keeps the read-back asynchronous) */
};

struct FrontierResult {
    uint32_t rounds;
    uint32_t launches;
    unsigned long long edges_relaxed;
    float kernel_ms;
    uint32_t nblocks; /* CTAs of the launch */
};

constexpr uint32_t TRACE_ROUNDS = 65536;
constexpr uint32_t TRACE_MAX_CTAS = 8192;
constexpr uint32_t TRACE_REC = 8; /* words per round: kind, items, edges, far, start time (2 words), - */
constexpr size_t TRACE_WORDS = (size_t)(TRACE_ROUNDS + 1) * TRACE_REC + TRACE_MAX_CTAS;

gga_status frontier_scratch_ensure(FrontierScratch *s, uint32_t n, uint32_t m);
void frontier_scratch_free(FrontierScratch *s);

/* SSSP light/heavy edge classes of an unsplit graph (light == NULL: off). */
struct LightHeavy {
    const uint32_t *light = nullptr; /* n: light edges per row, rows in light-first order */
    uint32_t heavy_edges = 0;        /* edges with w >= delta */
    uint32_t pull = 0;               /* bucket closes by pull: 0 never, 1 by the cost rule, 2 always (every
                                      * edge's reverse must have its weight) */
    uint32_t cw = 0;                 /* width of the heavy-edge weight classes of the rows (0: not ordered) */
};

/* Runs one single-source BFS (sssp=false) or SSSP over `view`.  `first`
 * (split view) maps the original source to its split parent id; NULL for the
 * unsplit view.  `lh.light` (SSSP, unsplit, delta > 0): light edges per row,
 * with view.col / view.wt in light-first row order; turns on
 * delta-stepping's light/heavy edge classes.  Distances land in s->dist
 * (view ids).  With hctl_async the call only queues the launch and the copy
 * of its control block into *hctl_async (pinned) on `st`: the caller waits
 * for the stream, checks the block with frontier_verdict and reads rounds
 * and edges_relaxed from it (res gets launches and nblocks only). */
gga_status frontier_run(FrontierScratch *s, const GraphView &view, const uint32_t *first, uint32_t src,
                        bool sssp, const gga_params &p, int sms, cudaStream_t st, cudaEvent_t ev0,
                        cudaEvent_t ev1, FrontierResult *res, bool trace = false, const LightHeavy &lh = {},
                        FrontierCtl *hctl_async = nullptr);
/* GGA_OK, or the error a finished launch's control block records. */
gga_status frontier_verdict(const FrontierCtl &h);
