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
    uint32_t qcount[3];           /* near-queue counts, rotating by round */
    uint32_t work[3];             /* work-unit tickets, rotating by round */
    unsigned long long huge[3];   /* (items << 32) | edge chunks, rotating */
    uint32_t far_count[3];        /* three far piles rotate across far passes */
    uint32_t far_min[3];
    uint32_t far_phases;
    uint32_t overflow_at;
    unsigned long long edges_relaxed;
    unsigned long long pad[4];
};

/* Per-context device scratch of the frontier engine, sized by vertices. */
struct FrontierScratch {
    uint32_t cap;        /* vertex capacity */
    uint32_t hcap;       /* huge-queue capacity */
    uint32_t *dist;      /* cap */
    uint32_t *bits;      /* cap/32: BFS visited / SSSP unused */
    uint32_t *farbits;   /* cap/32: SSSP "in far pile" */
    uint32_t *stamp;     /* cap: SSSP last round a vertex was queued */
    uint32_t *q0, *q1;   /* near queues */
    uint32_t *hq0, *hq1, *hqb0, *hqb1; /* huge items and their first chunk */
    uint32_t *far0, *far1, *far2;
    uint32_t *out;       /* cap: gathered original-order output */
    FrontierCtl *ctl;
};

struct FrontierResult {
    uint32_t rounds;
    uint32_t launches;
    unsigned long long edges_relaxed;
    float kernel_ms;
};

gga_status frontier_scratch_ensure(FrontierScratch *s, uint32_t n, uint32_t m);
void frontier_scratch_free(FrontierScratch *s);

/* Runs one single-source BFS (sssp=false) or SSSP over `view`.  `first`
 * (split view) maps the original source to its split parent id; NULL for the
 * unsplit view.  Distances land in s->dist (view ids). */
gga_status frontier_run(FrontierScratch *s, const GraphView &view, const uint32_t *first, uint32_t src,
                        bool sssp, const gga_params &p, int sms, cudaStream_t st, cudaEvent_t ev0,
                        cudaEvent_t ev1, FrontierResult *res);
