/*
 * The device context behind gga_ctx (one per host thread).
 */
#pragma once
#include <mutex>
#include <string>
#include <vector>

#include "frontier.cuh"

struct BatchScratch;

/* Working state of gga_solve_many (created on first use): a ring of result
 * buffers, so a finished traversal's distances are copied to the host on a
 * second stream while the next traversal runs. */
struct ManyScratch {
    static constexpr int RING = 3;
    cudaStream_t copy = nullptr;
    uint32_t *buf[RING] = {};
    size_t buf_words = 0;
    cudaEvent_t ready[RING] = {}, copied[RING] = {};
    std::vector<cudaEvent_t> ev;      /* two per source: kernel start and end */
    FrontierCtl *hctl = nullptr;      /* pinned: each launch's control block */
    unsigned long long *acc = nullptr; /* device: reached vertices and edges, two per source */
    unsigned long long *hacc = nullptr; /* pinned mirror */
    uint32_t cap = 0;                 /* sources hctl / acc hold */
};

struct gga_ctx {
    int device = 0;
    int sms = 0;
    size_t l2_bytes = 0;
    char name[256] = {0};
    cudaStream_t st = nullptr;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    cudaEvent_t user_ev[8] = {};
    gga_params params;
    bool params_set = false;
    FrontierScratch fs = {};
    uint32_t *dflag = nullptr; /* 64 words of device flags / counters */
    uint32_t *hflag = nullptr; /* pinned mirror */
    uint32_t *heavy = nullptr; /* CDP heavy-vertex list */
    uint32_t heavy_cap = 0;
    BatchScratch *batch = nullptr;
    ManyScratch many;
    bool trace_on = false;
    std::vector<uint32_t> trace_rounds; /* 5 words per round of the last traced solve */
    std::vector<uint32_t> trace_cta;    /* busy kilocycles per CTA */
    std::string tune_report;            /* JSON of the last gga_autotune's trials */
    void *stage = nullptr;              /* pinned staging for large host<->device copies (mesh refinement) */
    size_t stage_bytes = 0;
    void *dmr_state = nullptr;          /* pinned host copy of the mesh refinement's round state */
    std::mutex mu;
};

gga_status ctx_activate(gga_ctx *c);
gga_params ctx_default_params(const gga_graph *g);
/* SSSP bucket width from g's degree profile (never 0): the batch engines'
 * width, whose rounds are shared by many queries. */
uint32_t ctx_profile_delta(const gga_graph *g);
/* SSSP bucket width of g's queries in the batch engine (autotuned, else the
 * profile width). */
uint32_t ctx_batch_delta(const gga_graph *g);
gga_status ctx_validate_solve(const gga_graph *g, gga_algo algo, uint32_t src);
gga_status ctx_finish_output(gga_ctx *c, const DevGraph *d, const uint32_t *dev_out, uint32_t *dist_out,
                             gga_stats *stats);
unsigned ctx_grid(const gga_ctx *c, uint64_t items, unsigned bs);
bool ptr_is_device(const void *p);
void ctx_batch_release(gga_ctx *c);
