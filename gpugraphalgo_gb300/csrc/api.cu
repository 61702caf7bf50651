/*
 * C ABI: device contexts and single-source solves.
 *
 * The reference's driver (bfs_sssp.cu:103-539) reads the graph, splits it,
 * copies eight arrays to the device, initialises dist on the host, loops the
 * relax kernel with two synchronous memcpys per iteration and copies dist
 * back.  Here a context owns a stream, events and reusable device scratch; a
 * solve is: upload once (cached) -> one persistent launch (frontier engine)
 * or the reference's host loop (TOPO/CDP variants) -> gather the parents'
 * distances in original order -> one copy to the caller's buffer.
 */
#include <algorithm>
#include <mutex>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ctx.cuh"

/* ------------------------------------------------------------ context */

gga_status ctx_activate(gga_ctx *c) {
    GGA_CK(cudaSetDevice(c->device));
    return GGA_OK;
}

gga_status gga_ctx_create(int device, gga_ctx **out) {
    if (!out) return gga_fail(GGA_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0)
        return gga_fail(GGA_ERR_NO_DEVICE, "no CUDA device (%s)", e == cudaSuccess ? "count 0" : cudaGetErrorString(e));
    if (device < 0 || device >= count) return gga_fail(GGA_ERR_INVALID_ARG, "device %d of %d", device, count);
    GGA_CK(cudaSetDevice(device));
    gga_ctx *c = new (std::nothrow) gga_ctx();
    if (!c) return gga_fail(GGA_ERR_NO_MEMORY, "context");
    c->device = device;
    cudaDeviceProp p;
    e = cudaGetDeviceProperties(&p, device);
    if (e != cudaSuccess) { delete c; return gga_fail(GGA_ERR_CUDA, "device properties: %s", cudaGetErrorString(e)); }
    c->sms = p.multiProcessorCount;
    c->l2_bytes = (size_t)p.l2CacheSize;
    snprintf(c->name, sizeof c->name, "%s", p.name);
    e = cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking);
    for (int i = 0; i < 4 && e == cudaSuccess; ++i) e = cudaEventCreate(&c->ev[i]);
    for (int i = 0; i < 8 && e == cudaSuccess; ++i) e = cudaEventCreate(&c->user_ev[i]);
    if (e == cudaSuccess) e = cudaMalloc((void **)&c->dflag, 64 * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMallocHost((void **)&c->hflag, 64 * sizeof(uint32_t));
    if (e == cudaSuccess) {
        /* keep up to 4 GiB (GGA_POOL_KEEP_GIB) of freed stream-ordered
         * memory in this process's pool, so the working buffers of
         * back-to-back calls (a refinement's plan records, a re-uploaded
         * graph, scan temporaries) are not unmapped and mapped again */
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
            uint64_t keep = 4ull << 30, cur = 0;
            const char *env = getenv("GGA_POOL_KEEP_GIB");
            if (env && *env) {
                const long gib = strtol(env, nullptr, 10);
                if (gib >= 0 && gib <= 1024) keep = (uint64_t)gib << 30;
            }
            cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &cur);
            if (cur < keep) cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
    }
    if (e != cudaSuccess) {
        gga_ctx_destroy(c);
        return gga_fail(GGA_ERR_CUDA, "context setup: %s", cudaGetErrorString(e));
    }
    memset(&c->params, 0, sizeof c->params);
    *out = c;
    return GGA_OK;
}

void gga_ctx_destroy(gga_ctx *c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->st) cudaStreamSynchronize(c->st);
    ctx_batch_release(c);
    ManyScratch &m = c->many;
    if (m.copy) cudaStreamSynchronize(m.copy);
    for (int i = 0; i < ManyScratch::RING; ++i) {
        cudaFree(m.buf[i]);
        if (m.ready[i]) cudaEventDestroy(m.ready[i]);
        if (m.copied[i]) cudaEventDestroy(m.copied[i]);
    }
    for (cudaEvent_t e : m.ev) cudaEventDestroy(e);
    cudaFreeHost(m.hctl);
    cudaFree(m.acc);
    cudaFreeHost(m.hacc);
    if (m.copy) cudaStreamDestroy(m.copy);
    frontier_scratch_free(&c->fs);
    if (c->stage) cudaFreeHost(c->stage);
    if (c->dmr_state) cudaFreeHost(c->dmr_state);
    cudaFree(c->dflag);
    cudaFreeHost(c->hflag);
    cudaFree(c->heavy);
    for (int i = 0; i < 4; ++i)
        if (c->ev[i]) cudaEventDestroy(c->ev[i]);
    for (int i = 0; i < 8; ++i)
        if (c->user_ev[i]) cudaEventDestroy(c->user_ev[i]);
    if (c->st) cudaStreamDestroy(c->st);
    delete c;
}

gga_status gga_ctx_device_info(gga_ctx *c, int *sm_count, char *name, size_t name_len) {
    if (!c) return gga_fail(GGA_ERR_INVALID_ARG, "NULL context");
    if (sm_count) *sm_count = c->sms;
    if (name && name_len) {
        strncpy(name, c->name, name_len - 1);
        name[name_len - 1] = 0;
    }
    return GGA_OK;
}

gga_status gga_ctx_mark(gga_ctx *c, int slot) {
    if (!c || slot < 0 || slot >= 8) return gga_fail(GGA_ERR_INVALID_ARG, "bad context or slot");
    GGA_CK(cudaSetDevice(c->device));
    GGA_CK(cudaEventRecord(c->user_ev[slot], c->st));
    return GGA_OK;
}

gga_status gga_ctx_elapsed(gga_ctx *c, int a, int b, double *ms) {
    if (!c || !ms || a < 0 || a >= 8 || b < 0 || b >= 8) return gga_fail(GGA_ERR_INVALID_ARG, "bad context or slot");
    GGA_CK(cudaSetDevice(c->device));
    GGA_CK(cudaEventSynchronize(c->user_ev[b]));
    float f = 0;
    GGA_CK(cudaEventElapsedTime(&f, c->user_ev[a], c->user_ev[b]));
    *ms = f;
    return GGA_OK;
}

gga_status gga_ctx_synchronize(gga_ctx *c) {
    if (!c) return gga_fail(GGA_ERR_INVALID_ARG, "NULL context");
    GGA_CK(cudaSetDevice(c->device));
    GGA_CK(cudaStreamSynchronize(c->st));
    return GGA_OK;
}

gga_status gga_graph_pin(gga_graph *g, int pin) {
    if (!g) return gga_fail(GGA_ERR_INVALID_ARG, "NULL graph");
    uint32_t *arr[3] = {g->off, g->col, g->wt};
    size_t len[3] = {((size_t)g->n + 1) * 4, ((size_t)g->m + 1) * 4, ((size_t)g->m + 1) * 4};
    for (int i = 0; i < 3; ++i) {
        cudaError_t e = pin ? cudaHostRegister(arr[i], len[i], cudaHostRegisterDefault) : cudaHostUnregister(arr[i]);
        if (e != cudaSuccess && e != cudaErrorHostMemoryAlreadyRegistered && e != cudaErrorHostMemoryNotRegistered)
            return gga_fail(GGA_ERR_CUDA, "host register: %s", cudaGetErrorString(e));
        cudaGetLastError();
    }
    return GGA_OK;
}

gga_status gga_graph_release_device(gga_graph *g) {
    if (!g) return gga_fail(GGA_ERR_INVALID_ARG, "NULL graph");
    pthread_mutex_lock(&g->lock);
    if (g->dev && gga_dev_graph_release_hook) gga_dev_graph_release_hook(g);
    g->split_level = 0;
    g->ns = g->mda = g->parents_with_children = 0;
    pthread_mutex_unlock(&g->lock);
    return GGA_OK;
}

gga_status gga_graph_upload(gga_ctx *c, gga_graph *g) {
    if (!c || !g) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    gga_status s = ctx_activate(c);
    if (s) return s;
    return dev_graph_ensure(g, c->device, c->st);
}

/* ------------------------------------------------------------ split */

gga_status dev_node_split(gga_graph *g, int32_t level, int32_t buckets, cudaStream_t st);
gga_status dev_split_maps(gga_graph *g, uint32_t *psrc, uint32_t *noutgoing, uint32_t *edgessrcdst,
                          uint32_t *child_count, uint32_t *is_parent, uint32_t *parent_node, cudaStream_t st);
gga_status dev_child_index(gga_graph *g, uint32_t *count, uint32_t *cidx, uint32_t *ccnt, cudaStream_t st);

gga_status gga_node_split(gga_ctx *c, gga_graph *g, int32_t level, int32_t buckets) {
    if (!c || !g) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(c->mu);
    gga_status s = ctx_activate(c);
    if (!s) s = dev_graph_ensure(g, c->device, c->st);
    if (!s) s = dev_node_split(g, level, buckets, c->st);
    return s;
}

gga_status gga_graph_split_maps(gga_ctx *c, const gga_graph *g, uint32_t *psrc, uint32_t *noutgoing,
                                uint32_t *edgessrcdst, uint32_t *child_count, uint32_t *is_parent,
                                uint32_t *parent_node) {
    if (!c || !g) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(c->mu);
    gga_status s = ctx_activate(c);
    if (!s) s = dev_graph_ensure((gga_graph *)g, c->device, c->st);
    if (!s) s = dev_split_maps((gga_graph *)g, psrc, noutgoing, edgessrcdst, child_count, is_parent, parent_node, c->st);
    return s;
}

gga_status gga_child_index(gga_ctx *c, const gga_graph *g, uint32_t *count, uint32_t *cidx, uint32_t *ccnt) {
    if (!c || !g || !count) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(c->mu);
    gga_status s = ctx_activate(c);
    if (!s) s = dev_graph_ensure((gga_graph *)g, c->device, c->st);
    if (!s) s = dev_child_index((gga_graph *)g, count, cidx, ccnt, c->st);
    return s;
}

/* ------------------------------------------------------------ params */

gga_status gga_set_params(gga_ctx *c, const gga_params *p) {
    if (!c) return gga_fail(GGA_ERR_INVALID_ARG, "NULL context");
    if (!p) {
        c->params_set = false;
        memset(&c->params, 0, sizeof c->params);
        return GGA_OK;
    }
    if (p->block_threads && p->block_threads != 256 && p->block_threads != 512 && p->block_threads != 1024)
        return gga_fail(GGA_ERR_INVALID_ARG, "block_threads must be 256, 512 or 1024");
    if (p->cdp_mode > 2) return gga_fail(GGA_ERR_INVALID_ARG, "cdp_mode must be 0, 1 or 2");
    if (p->sssp_pull > 2) return gga_fail(GGA_ERR_INVALID_ARG, "sssp_pull must be 0, 1 or 2");
    c->params = *p;
    c->params_set = true;
    return GGA_OK;
}

gga_status gga_get_params(gga_ctx *c, gga_params *p) {
    if (!c || !p) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    *p = c->params;
    return GGA_OK;
}

/* Bucket width from the degree profile: a few average weights over the
 * average degree. */
uint32_t ctx_profile_delta(const gga_graph *g) {
    const double wavg = g->wavg > 0 ? g->wavg : 1.0; /* computed once when the graph is built */
    const double davg = g->n ? (double)g->m / g->n : 1.0;
    const double delta = wavg * 8.0 / (davg > 1.0 ? davg : 1.0);
    return delta < 1.0 ? 1u : (uint32_t)delta;
}

/* Degree-profile defaults (gga_autotune refines them with timed trials). */
gga_params ctx_default_params(const gga_graph *g) {
    gga_params p;
    memset(&p, 0, sizeof p);
    p.block_threads = 256;
    p.unit_iters = 0; /* per algorithm: 4096 edges per unit for BFS, 4 per thread for SSSP */
    /* graphs under 4M edges take the plain improved-vertex frontier (delta
     * 0), whose few latency-bound rounds beat buckets there (measured on
     * GB300: R-MAT 10-16 and grids to 1024^2 with long-range edges run
     * 1.2-2x faster; R-MAT 18 and up keep buckets) */
    p.sssp_delta = g->m < (1u << 22) ? 0u : ctx_profile_delta(g);
    /* edge-balanced units need no split; the unsplit CSR also allows
     * bottom-up BFS and light/heavy SSSP (R-MAT 22 split at the histogram
     * rule: BFS 1.25 -> 0.21 ms, SSSP 3.7 -> 1.25 ms walking it unsplit) */
    p.use_split = 0;
    p.cdp_level = 1;
    p.cdp_buckets = 10;
    p.expansion = 0;
    p.split_level = 0;
    p.split_buckets = 10;
    p.batch_delta = 0xFFFFFFFFu;
    return p;
}

/* Bucket width of g's queries in the batch engine: the autotuner's pick, else
 * the degree-profile width. */
uint32_t ctx_batch_delta(const gga_graph *g) {
    if (g->has_tuned && g->tuned.batch_delta != 0xFFFFFFFFu) return g->tuned.batch_delta;
    return ctx_profile_delta(g);
}

static gga_params effective_params(gga_ctx *c, const gga_graph *g) {
    gga_params d = g->has_tuned ? g->tuned : ctx_default_params(g);
    if (!c->params_set) return d;
    gga_params p = c->params;
    if (!p.block_threads) p.block_threads = d.block_threads;
    if (!p.unit_iters) p.unit_iters = d.unit_iters;
    if (!p.cdp_buckets) p.cdp_buckets = d.cdp_buckets;
    if (!p.cdp_level) p.cdp_level = d.cdp_level;
    return p;
}

/* ------------------------------------------------------------ solve */

__global__ void k_gather_parents(const uint32_t *dist, const uint32_t *first, uint32_t n, uint32_t *out) {
    for (uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; u < n; u += (uint64_t)gridDim.x * blockDim.x)
        out[u] = dist[first[u]];
}

__global__ void k_reached(const uint32_t *dist, const uint32_t *off, uint32_t n, unsigned long long *acc) {
    unsigned long long vr = 0, er = 0;
    for (uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; u < n; u += (uint64_t)gridDim.x * blockDim.x)
        if (dist[u] < GGA_INFINITY) {
            vr++;
            er += off[u + 1] - off[u];
        }
    vr = __reduce_add_sync(0xffffffffu, (uint32_t)vr);
    for (int d = 16; d > 0; d >>= 1) er += __shfl_down_sync(0xffffffffu, er, d);
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(acc, vr);
        atomicAdd(acc + 1, er);
    }
}

bool ptr_is_device(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

unsigned ctx_grid(const gga_ctx *c, uint64_t items, unsigned bs) {
    uint64_t b = (items + bs - 1) / bs;
    uint64_t cap = (uint64_t)c->sms * 32;
    if (b > cap) b = cap;
    return b ? (unsigned)b : 1;
}

/* Copies the original-order result (device) to the caller and fills the
 * reached-vertex statistics. */
gga_status ctx_finish_output(gga_ctx *c, const DevGraph *d, const uint32_t *dev_out, uint32_t *dist_out,
                             gga_stats *stats) {
    const size_t bytes = (size_t)d->n * sizeof(uint32_t);
    if (dist_out && dev_out != dist_out)
        GGA_CK(cudaMemcpyAsync(dist_out, dev_out, bytes,
                               ptr_is_device(dist_out) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c->st));
    if (stats) {
        unsigned long long *acc = (unsigned long long *)(c->dflag + 32);
        GGA_CK(cudaMemsetAsync(acc, 0, 2 * sizeof(unsigned long long), c->st));
        k_reached<<<ctx_grid(c, d->n, 256), 256, 0, c->st>>>(dev_out, d->off, d->n, acc);
        GGA_CK(cudaMemcpyAsync(c->hflag + 32, acc, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->st));
    }
    gga_status w = dev_wait(c->st, 60.0);
    if (w) return w;
    if (stats) {
        const unsigned long long *h = (const unsigned long long *)(c->hflag + 32);
        stats->vertices_reached = h[0];
        stats->edges_reached = h[1];
    }
    return GGA_OK;
}

struct TopoResult {
    uint32_t iterations, launches, cdp_children, cdp_fallbacks;
    float ktime, sktime;
};
gga_status topo_run(const DevGraph *d, bool split, gga_variant variant, bool sssp, uint32_t src,
                    uint32_t max_allowed, uint32_t cdp_mode, uint32_t *dist, uint32_t *scratch_heavy,
                    uint32_t *dflag, uint32_t *hflag, int sms, cudaStream_t st, cudaEvent_t *ev,
                    TopoResult *res, ConvHook *conv);

/* Set by gga_convergence around its gga_solve call (same thread). */
static thread_local ConvHook *tl_conv = nullptr;

gga_status ctx_validate_solve(const gga_graph *g, gga_algo algo, uint32_t src) {
    if (algo != GGA_BFS && algo != GGA_SSSP) return gga_fail(GGA_ERR_INVALID_ARG, "unknown algorithm %d", (int)algo);
    if (src >= g->n) return gga_fail(GGA_ERR_INVALID_ARG, "source %u >= %u vertices", src, g->n);
    if (algo == GGA_SSSP && g->maxw > GGA_MAX_WEIGHT)
        return gga_fail(GGA_ERR_INVALID_ARG, "edge weight %u > %u: dist + weight would wrap in uint32", g->maxw,
                        GGA_MAX_WEIGHT);
    return GGA_OK;
}

/* What the frontier engine walks for one solve: the split or unsplit view,
 * SSSP's light-first rows, and whether bucket closes may pull.  Runs the
 * once-per-graph device checks and builds the light/heavy order on first
 * use; sizes the scratch. */
struct FrontierPlan {
    GraphView v;
    LightHeavy lh;
    bool use_split = false;
};

static gga_status frontier_plan(gga_ctx *c, gga_graph *g, const gga_params &p, bool sssp, FrontierPlan *out) {
    const DevGraph *d = dev_graph_of(g);
    gga_status s;
    out->use_split = d->level != 0 && p.use_split;
    if (!sssp && !out->use_split && p.bfs_direction == 0 && d->symmetric == 0 &&
        (s = dev_graph_check_symmetric(g, c->dflag + 40, c->hflag + 40, c->st)))
        return s;
    out->v = dev_graph_view(d, out->use_split);
    if (sssp && !out->use_split && p.sssp_delta && p.sssp_light_heavy == 0) {
        if ((s = dev_graph_light_heavy(g, p.sssp_delta, c->st))) return s;
        /* pulling bucket closes need every edge's reverse with its weight */
        if (p.sssp_pull != 1 && (d->symmetric == 0 || d->wsymmetric == 0) &&
            (s = dev_graph_check_symmetric(g, c->dflag + 40, c->hflag + 40, c->st)))
            return s;
        out->v.col = d->lcol;
        out->v.wt = d->lwt;
        out->lh.light = d->light;
        out->lh.heavy_edges = d->lh_heavy;
        out->lh.cw = d->lh_cw;
        out->lh.pull = p.sssp_pull == 1 || d->wsymmetric <= 0 ? 0u : (p.sssp_pull == 2 ? 2u : 1u);
    }
    return frontier_scratch_ensure(&c->fs, out->v.n > d->n ? out->v.n : d->n, d->m);
}

gga_status gga_graph_prepare(gga_ctx *c, gga_graph *g, gga_algo algo) {
    if (!c || !g) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    if (algo != GGA_BFS && algo != GGA_SSSP) return gga_fail(GGA_ERR_INVALID_ARG, "unknown algorithm %d", (int)algo);
    std::lock_guard<std::mutex> lk(c->mu);
    gga_status s = ctx_activate(c);
    if (!s) s = dev_graph_ensure(g, c->device, c->st);
    FrontierPlan fp;
    gga_params p = effective_params(c, g);
    if (p.expansion == 1) p.use_split = 1;
    if (!s) s = frontier_plan(c, g, p, algo == GGA_SSSP, &fp);
    if (!s) s = dev_wait(c->st, 60.0);
    return s;
}

gga_status gga_solve(gga_ctx *c, gga_graph *g, gga_algo algo, uint32_t src, gga_variant variant,
                     uint32_t *dist_out, gga_stats *stats) {
    const double t0 = gga_now_ms();
    if (!c || !g) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    gga_status s = ctx_validate_solve(g, algo, src);
    if (s) return s;
    if ((int)variant < GGA_VARIANT_AUTO || (int)variant > GGA_VARIANT_CDP_PLAIN)
        return gga_fail(GGA_ERR_INVALID_ARG, "unknown variant %d", (int)variant);
    std::lock_guard<std::mutex> lk(c->mu);
    if ((s = ctx_activate(c))) return s;
    if ((s = dev_graph_ensure(g, c->device, c->st))) return s;
    const DevGraph *d = dev_graph_of(g);
    gga_params p = effective_params(c, g);
    if (variant == GGA_VARIANT_AUTO && p.expansion == 2) { /* the autotuner picked the CDP variant */
        variant = GGA_VARIANT_CDP_ATOMIC;
        p.cdp_level = p.split_level ? p.split_level : 1;
        p.cdp_buckets = p.split_buckets ? p.split_buckets : 10;
    } else if (variant == GGA_VARIANT_AUTO && p.expansion == 1) { /* edge units over the split CSR */
        p.use_split = 1;
    }
    const bool sssp = algo == GGA_SSSP;
    const bool split = d->level != 0;
    gga_stats st;
    memset(&st, 0, sizeof st);

    if (variant == GGA_VARIANT_AUTO || variant == GGA_VARIANT_FRONTIER) {
        FrontierPlan fp;
        if ((s = frontier_plan(c, g, p, sssp, &fp))) return s;
        const bool use_split = fp.use_split;
        FrontierResult r;
        s = frontier_run(&c->fs, fp.v, use_split ? d->first : nullptr, src, sssp, p, c->sms, c->st, c->ev[0], c->ev[1],
                         &r, c->trace_on, fp.lh);
        if (s) return s;
        if (c->trace_on) {
            const uint32_t nr = r.rounds < TRACE_ROUNDS ? r.rounds : TRACE_ROUNDS;
            const uint32_t nb = r.nblocks < TRACE_MAX_CTAS ? r.nblocks : TRACE_MAX_CTAS;
            std::vector<uint32_t> raw((size_t)(nr + 1) * TRACE_REC);
            c->trace_cta.assign(nb, 0);
            GGA_CK(cudaMemcpyAsync(raw.data(), c->fs.trace, raw.size() * 4, cudaMemcpyDeviceToHost, c->st));
            if (nb)
                GGA_CK(cudaMemcpyAsync(c->trace_cta.data(), c->fs.trace + (size_t)(TRACE_ROUNDS + 1) * TRACE_REC,
                                       (size_t)nb * 4, cudaMemcpyDeviceToHost, c->st));
            GGA_CK(cudaStreamSynchronize(c->st));
            /* 5 words per round: the record and its duration (start of the next round - start) */
            c->trace_rounds.assign((size_t)nr * 5, 0);
            for (uint32_t i = 0; i < nr; ++i) {
                const uint32_t *r = raw.data() + (size_t)i * TRACE_REC, *q = r + TRACE_REC;
                const unsigned long long t0 = r[4] | ((unsigned long long)r[5] << 32);
                const unsigned long long t1 = q[4] | ((unsigned long long)q[5] << 32);
                for (int k = 0; k < 4; ++k) c->trace_rounds[(size_t)i * 5 + k] = r[k];
                const unsigned long long dt = t1 > t0 ? t1 - t0 : 0;
                c->trace_rounds[(size_t)i * 5 + 4] = (uint32_t)(dt < 0xffffffffull ? dt : 0xffffffffull);
            }
        }
        st.iterations = r.rounds;
        st.kernel_launches = r.launches;
        st.edges_relaxed = r.edges_relaxed;
        st.kernel_ms = r.kernel_ms;
        const uint32_t *res = c->fs.dist;
        if (use_split) {
            k_gather_parents<<<ctx_grid(c, d->n, 256), 256, 0, c->st>>>(c->fs.dist, d->first, d->n, c->fs.out);
            st.kernel_launches++;
            res = c->fs.out;
        }
        if ((s = ctx_finish_output(c, d, res, dist_out, stats && !p.skip_reached ? &st : nullptr))) return s;
    } else {
        const bool cdp = variant == GGA_VARIANT_CDP_ATOMIC || variant == GGA_VARIANT_CDP_PLAIN;
        uint32_t max_allowed = d->maxdeg;
        if (cdp) {
            /* bfs_sssp.cu:224-236: histogram rule for a negative level, else ceil(maxdeg/level) */
            if (p.cdp_level < 0) {
                if ((s = gga_max_allowed_out_degree(g, p.cdp_buckets, &max_allowed))) return s;
            } else {
                const uint32_t lv = p.cdp_level > 0 ? (uint32_t)p.cdp_level : 1u;
                max_allowed = (uint32_t)(((uint64_t)d->maxdeg + lv - 1) / lv);
            }
            if (c->heavy_cap < d->n) {
                cudaFree(c->heavy);
                c->heavy = nullptr;
                c->heavy_cap = 0;
                GGA_CK(cudaMalloc((void **)&c->heavy, (size_t)d->n * sizeof(uint32_t)));
                c->heavy_cap = d->n;
            }
            if (p.cdp_pending_limit)
                GGA_CK(cudaDeviceSetLimit(cudaLimitDevRuntimePendingLaunchCount, p.cdp_pending_limit));
        }
        const GraphView v = dev_graph_view(d, split && !cdp);
        if ((s = frontier_scratch_ensure(&c->fs, v.n > d->n ? v.n : d->n, d->m))) return s;
        TopoResult r;
        s = topo_run(d, split, variant, sssp, src, max_allowed, p.cdp_mode, c->fs.dist, c->heavy, c->dflag, c->hflag,
                     c->sms, c->st, c->ev, &r, tl_conv);
        if (s) return s;
        st.iterations = r.iterations;
        st.kernel_launches = r.launches;
        st.kernel_ms = r.ktime;
        st.aux_ms = r.sktime;
        st.cdp_children = r.cdp_children;
        st.cdp_fallbacks = r.cdp_fallbacks;
        const uint32_t *res = c->fs.dist;
        if (split && !cdp) {
            k_gather_parents<<<ctx_grid(c, d->n, 256), 256, 0, c->st>>>(c->fs.dist, d->first, d->n, c->fs.out);
            st.kernel_launches++;
            res = c->fs.out;
        }
        if ((s = ctx_finish_output(c, d, res, dist_out, stats && !p.skip_reached ? &st : nullptr))) return s;
    }
    st.total_ms = gga_now_ms() - t0;
    if (stats) *stats = st;
    return GGA_OK;
}

gga_status gga_convergence(gga_ctx *c, gga_graph *g, gga_algo algo, uint32_t src, gga_variant variant,
                           const uint32_t *final_dist, gga_conv_record *records, uint32_t cap, uint32_t *nrec,
                           uint32_t *dist_out) {
    if (!c || !g || !final_dist || !nrec || (cap && !records)) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    if (variant != GGA_VARIANT_TOPO_ATOMIC && variant != GGA_VARIANT_TOPO_PLAIN && variant != GGA_VARIANT_CDP_ATOMIC &&
        variant != GGA_VARIANT_CDP_PLAIN)
        return gga_fail(GGA_ERR_INVALID_ARG, "convergence logs need a topology-driven variant (got %d)", (int)variant);
    gga_status s = ctx_validate_solve(g, algo, src);
    if (s) return s;
    uint32_t *fin = nullptr;
    unsigned long long *acc = nullptr;
    uint32_t *tmp = nullptr;
    {
        std::lock_guard<std::mutex> lk(c->mu);
        if ((s = ctx_activate(c))) return s;
        cudaError_t e = cudaMalloc((void **)&fin, (size_t)g->n * sizeof(uint32_t));
        if (e == cudaSuccess) e = cudaMalloc((void **)&acc, 2 * sizeof(unsigned long long));
        if (e == cudaSuccess && !dist_out) e = cudaMalloc((void **)&tmp, (size_t)g->n * sizeof(uint32_t));
        if (e == cudaSuccess) e = cudaMemcpy(fin, final_dist, (size_t)g->n * sizeof(uint32_t), cudaMemcpyDefault);
        if (e != cudaSuccess) {
            cudaGetLastError();
            cudaFree(fin);
            cudaFree(acc);
            cudaFree(tmp);
            return gga_fail(GGA_ERR_CUDA, "convergence buffers: %s", cudaGetErrorString(e));
        }
    }
    ConvHook h;
    h.fin = fin;
    h.cnt = acc;
    h.norm = acc + 1;
    h.rec = records;
    h.cap = cap;
    h.n = 0;
    tl_conv = &h;
    s = gga_solve(c, g, algo, src, variant, dist_out ? dist_out : tmp, nullptr);
    tl_conv = nullptr;
    cudaFree(fin);
    cudaFree(acc);
    cudaFree(tmp);
    *nrec = h.n;
    return s;
}

/* Buffers of gga_solve_many for n sources of `words`-vertex results. */
static gga_status many_reserve(gga_ctx *c, size_t words, uint32_t n) {
    ManyScratch &m = c->many;
    if (!m.copy) {
        GGA_CK(cudaStreamCreateWithFlags(&m.copy, cudaStreamNonBlocking));
        for (int i = 0; i < ManyScratch::RING; ++i) {
            GGA_CK(cudaEventCreateWithFlags(&m.ready[i], cudaEventDisableTiming));
            GGA_CK(cudaEventCreateWithFlags(&m.copied[i], cudaEventDisableTiming));
        }
    }
    if (m.buf_words < words) {
        for (int i = 0; i < ManyScratch::RING; ++i) {
            cudaFree(m.buf[i]);
            m.buf[i] = nullptr;
        }
        m.buf_words = 0;
        for (int i = 0; i < ManyScratch::RING; ++i) GGA_CK(cudaMalloc((void **)&m.buf[i], words * sizeof(uint32_t)));
        m.buf_words = words;
    }
    if (m.cap < n) {
        cudaFreeHost(m.hctl);
        cudaFree(m.acc);
        cudaFreeHost(m.hacc);
        m.hctl = nullptr;
        m.acc = m.hacc = nullptr;
        m.cap = 0;
        GGA_CK(cudaMallocHost((void **)&m.hctl, (size_t)n * sizeof(FrontierCtl)));
        GGA_CK(cudaMalloc((void **)&m.acc, (size_t)n * 2 * sizeof(unsigned long long)));
        GGA_CK(cudaMallocHost((void **)&m.hacc, (size_t)n * 2 * sizeof(unsigned long long)));
        m.cap = n;
    }
    while (m.ev.size() < 2 * (size_t)n) {
        cudaEvent_t e;
        GGA_CK(cudaEventCreate(&e));
        m.ev.push_back(e);
    }
    return GGA_OK;
}

gga_status gga_solve_many(gga_ctx *c, gga_graph *g, gga_algo algo, uint32_t n, const uint32_t *srcs,
                          uint32_t *dist_out, gga_stats *stats) {
    const double t0 = gga_now_ms();
    if (!c || !g || (n && (!srcs || !dist_out))) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    gga_status s;
    for (uint32_t i = 0; i < n; ++i)
        if ((s = ctx_validate_solve(g, algo, srcs[i]))) return s;
    if (n == 0) return GGA_OK;
    std::lock_guard<std::mutex> lk(c->mu);
    if ((s = ctx_activate(c))) return s;
    if ((s = dev_graph_ensure(g, c->device, c->st))) return s;
    const DevGraph *d = dev_graph_of(g);
    gga_params p = effective_params(c, g);
    if (p.expansion == 1) p.use_split = 1; /* the autotuner's split view */
    const bool sssp = algo == GGA_SSSP;
    FrontierPlan fp;
    if ((s = frontier_plan(c, g, p, sssp, &fp))) return s;
    if ((s = many_reserve(c, d->n ? d->n : 1, n))) return s;
    ManyScratch &m = c->many;
    const bool reached = stats && !p.skip_reached;
    const size_t bytes = (size_t)d->n * sizeof(uint32_t);
    if (reached) GGA_CK(cudaMemsetAsync(m.acc, 0, (size_t)n * 2 * sizeof(unsigned long long), c->st));
    std::vector<FrontierResult> r(n);
    for (uint32_t i = 0; i < n && s == GGA_OK; ++i) {
        const int slot = (int)(i % ManyScratch::RING);
        /* the slot's previous result has reached the host */
        if (i >= (uint32_t)ManyScratch::RING && (s = gga_cuda_check(cudaStreamWaitEvent(c->st, m.copied[slot], 0))))
            break;
        s = frontier_run(&c->fs, fp.v, fp.use_split ? d->first : nullptr, srcs[i], sssp, p, c->sms, c->st,
                         m.ev[2 * i], m.ev[2 * i + 1], &r[i], false, fp.lh, &m.hctl[i]);
        if (s) break;
        uint32_t *res = m.buf[slot];
        if (fp.use_split) k_gather_parents<<<ctx_grid(c, d->n, 256), 256, 0, c->st>>>(c->fs.dist, d->first, d->n, res);
        else if (bytes) s = gga_cuda_check(cudaMemcpyAsync(res, c->fs.dist, bytes, cudaMemcpyDeviceToDevice, c->st));
        if (reached && s == GGA_OK) k_reached<<<ctx_grid(c, d->n, 256), 256, 0, c->st>>>(res, d->off, d->n, m.acc + 2 * i);
        if (s == GGA_OK) s = gga_cuda_check(cudaGetLastError());
        if (s == GGA_OK) s = gga_cuda_check(cudaEventRecord(m.ready[slot], c->st));
        if (s == GGA_OK) s = gga_cuda_check(cudaStreamWaitEvent(m.copy, m.ready[slot], 0));
        if (s == GGA_OK && bytes)
            s = gga_cuda_check(cudaMemcpyAsync(dist_out + (size_t)i * d->n, res, bytes, cudaMemcpyDefault, m.copy));
        if (s == GGA_OK) s = gga_cuda_check(cudaEventRecord(m.copied[slot], m.copy));
    }
    if (s == GGA_OK && reached)
        s = gga_cuda_check(cudaMemcpyAsync(m.hacc, m.acc, (size_t)n * 2 * sizeof(unsigned long long),
                                           cudaMemcpyDeviceToHost, c->st));
    /* drain both streams even after an error, so no copy outlives the call */
    gga_status w = dev_wait(c->st, 60.0 + n);
    gga_status w2 = dev_wait(m.copy, 60.0);
    if (s) return s;
    if (w) return w;
    if (w2) return w2;
    for (uint32_t i = 0; i < n; ++i)
        if ((s = frontier_verdict(m.hctl[i]))) return s;
    if (stats) {
        const double each = (gga_now_ms() - t0) / n;
        for (uint32_t i = 0; i < n; ++i) {
            gga_stats &st = stats[i];
            memset(&st, 0, sizeof st);
            st.iterations = m.hctl[i].rounds;
            st.kernel_launches = r[i].launches + (fp.use_split ? 1 : 0) + (reached ? 1 : 0);
            st.edges_relaxed = m.hctl[i].edges_relaxed;
            float ms = 0;
            cudaEventElapsedTime(&ms, m.ev[2 * i], m.ev[2 * i + 1]);
            st.kernel_ms = ms;
            if (reached) {
                st.vertices_reached = m.hacc[2 * i];
                st.edges_reached = m.hacc[2 * i + 1];
            }
            st.total_ms = each;
        }
    }
    return GGA_OK;
}

gga_status gga_host_alloc(size_t bytes, void **out) {
    if (!out) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    GGA_CK(cudaMallocHost(out, bytes ? bytes : 1));
    return GGA_OK;
}

void gga_host_free(void *p) {
    if (p) cudaFreeHost(p);
}

gga_status gga_bfs(gga_ctx *c, gga_graph *g, uint32_t src, gga_variant variant, uint32_t *dist_out, gga_stats *stats) {
    return gga_solve(c, g, GGA_BFS, src, variant, dist_out, stats);
}

gga_status gga_sssp(gga_ctx *c, gga_graph *g, uint32_t src, gga_variant variant, uint32_t *dist_out, gga_stats *stats) {
    return gga_solve(c, g, GGA_SSSP, src, variant, dist_out, stats);
}

/* ------------------------------------------------------------ instrumentation */

gga_status gga_trace_enable(gga_ctx *c, int enable) {
    if (!c) return gga_fail(GGA_ERR_INVALID_ARG, "NULL context");
    std::lock_guard<std::mutex> lk(c->mu);
    c->trace_on = enable != 0;
    return GGA_OK;
}

gga_status gga_trace_get(gga_ctx *c, gga_round_trace *rounds, uint32_t cap, uint32_t *nrounds,
                         uint32_t *cta_kcycles, uint32_t cta_cap, uint32_t *ncta) {
    if (!c) return gga_fail(GGA_ERR_INVALID_ARG, "NULL context");
    std::lock_guard<std::mutex> lk(c->mu);
    const uint32_t nr = (uint32_t)(c->trace_rounds.size() / 5), nb = (uint32_t)c->trace_cta.size();
    if (nrounds) *nrounds = nr;
    if (ncta) *ncta = nb;
    if (rounds)
        for (uint32_t i = 0; i < nr && i < cap; ++i) {
            rounds[i].kind = c->trace_rounds[5 * (size_t)i];
            rounds[i].items = c->trace_rounds[5 * (size_t)i + 1];
            rounds[i].edges = c->trace_rounds[5 * (size_t)i + 2];
            rounds[i].far_items = c->trace_rounds[5 * (size_t)i + 3];
            rounds[i].ns = c->trace_rounds[5 * (size_t)i + 4];
        }
    if (cta_kcycles)
        for (uint32_t i = 0; i < nb && i < cta_cap; ++i) cta_kcycles[i] = c->trace_cta[i];
    return GGA_OK;
}

/* ------------------------------------------------------------ autotune */

namespace {

/* Timed trials of one candidate parameter set: kernel time (CUDA events) of
 * solving `algo` from each source, `trials` times, on `variant`. */
struct Tuner {
    gga_ctx *c;
    gga_graph *g;
    uint32_t trials;
    uint32_t srcs[2];
    uint32_t nsrc;
    uint32_t *tmp;
    std::string log;

    double time(const gga_params &p, gga_algo algo, gga_variant variant) {
        c->params = p;
        c->params_set = true;
        double t = 0;
        for (uint32_t k = 0; k < trials; ++k)
            for (uint32_t i = 0; i < nsrc; ++i) {
                gga_stats st;
                if (gga_solve(c, g, algo, srcs[i], variant, tmp, &st)) return 1e30;
                t += st.kernel_ms + st.aux_ms;
            }
        return t / trials;
    }
    void note(const char *key, double ms) {
        char b[96];
        snprintf(b, sizeof b, "%s\"%s\": %.4f", log.size() > 1 ? ", " : "", key, ms < 1e29 ? ms : -1.0);
        log += b;
    }
};

} // namespace

gga_status gga_autotune(gga_ctx *c, gga_graph *g, uint32_t trials, gga_params *chosen) {
    if (!c || !g) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    gga_params best = ctx_default_params(g);
    if (c->params_set) {
        best.cdp_mode = c->params.cdp_mode;
        best.cdp_level = c->params.cdp_level ? c->params.cdp_level : best.cdp_level;
        best.cdp_buckets = c->params.cdp_buckets ? c->params.cdp_buckets : best.cdp_buckets;
    }
    std::string report = "{";
    if (trials) {
        /* two sources: the highest-degree vertex and the vertex of median
         * degree among those with edges */
        Tuner T;
        T.c = c;
        T.g = g;
        T.trials = trials;
        T.nsrc = 0;
        T.tmp = nullptr;
        T.log = "{";
        uint32_t md = 0, top = 0;
        std::vector<uint32_t> degs;
        degs.reserve(g->n);
        for (uint32_t u = 0; u < g->n; ++u) {
            const uint32_t dgr = g->off[u + 1] - g->off[u];
            if (dgr > md) { md = dgr; top = u; }
            if (dgr) degs.push_back(dgr);
        }
        T.srcs[T.nsrc++] = top;
        if (!degs.empty()) {
            std::nth_element(degs.begin(), degs.begin() + degs.size() / 2, degs.end());
            const uint32_t med = degs[degs.size() / 2];
            for (uint32_t u = 0; u < g->n; ++u)
                if (u != top && g->off[u + 1] - g->off[u] == med) {
                    T.srcs[T.nsrc++] = u;
                    break;
                }
        }
        const bool sssp_ok = g->maxw <= GGA_MAX_WEIGHT;
        const int32_t level0 = g->split_level, buckets0 = g->split_buckets;
        {
            std::lock_guard<std::mutex> lk(c->mu);
            gga_status s = ctx_activate(c);
            if (!s) s = dev_graph_ensure(g, c->device, c->st);
            if (s) return s;
            GGA_CK(cudaMalloc((void **)&T.tmp, (size_t)g->n * sizeof(uint32_t)));
        }
        const gga_params saved = c->params;
        const bool saved_set = c->params_set;
        char key[64];
        /* 1. CTA size and SSSP bucket width (edge units, unsplit CSR) */
        const uint32_t base = ctx_profile_delta(g);
        const uint32_t deltas[] = {base / 4 ? base / 4 : 1,         base * 3 / 8 ? base * 3 / 8 : 1,
                                   base / 2 ? base / 2 : 1,         base * 3 / 4 ? base * 3 / 4 : 1,
                                   base, base * 3 / 2, base * 2, base * 4, 0};
        double best_s = 1e30;
        for (uint32_t bs : {256u, 512u})
            for (uint32_t dl : deltas) {
                gga_params p = best;
                p.block_threads = bs;
                p.sssp_delta = dl;
                const double t = T.time(p, sssp_ok ? GGA_SSSP : GGA_BFS, GGA_VARIANT_FRONTIER);
                snprintf(key, sizeof key, "sssp_bs%u_delta%u", bs, dl);
                T.note(key, t);
                if (t < best_s) {
                    best_s = t;
                    best = p;
                }
            }
        /* 2. BFS direction thresholds (bottom-up rounds need a symmetric graph) */
        double best_b = T.time(best, GGA_BFS, GGA_VARIANT_FRONTIER);
        T.note("bfs_alpha8_beta18", best_b);
        const DevGraph *dg = dev_graph_of(g);
        if (dg && dg->symmetric > 0) {
            const uint32_t ab[][2] = {{4, 18}, {15, 18}, {30, 18}, {8, 12}, {8, 24}, {8, 48}};
            for (const auto &x : ab) {
                gga_params p = best;
                p.bfs_alpha = x[0];
                p.bfs_beta = x[1];
                const double t = T.time(p, GGA_BFS, GGA_VARIANT_FRONTIER);
                snprintf(key, sizeof key, "bfs_alpha%u_beta%u", x[0], x[1]);
                T.note(key, t);
                if (t < best_b) {
                    best_b = t;
                    best = p;
                }
            }
        }
        /* 3. expansion strategy: BFS + SSSP time of edge units over the
         * unsplit CSR, of the same units over the node-split CSR (histogram
         * rule, ceil(maxdeg / level) for a few levels), and of the
         * reference's CDP variant on small graphs */
        double best_x = best_b + (sssp_ok ? best_s : 0.0);
        T.note("expansion_edges_unsplit", best_x);
        struct Split { int32_t level, buckets; };
        std::vector<Split> splits;
        uint32_t mda = 0;
        if (md + 1 >= 10 && gga_max_allowed_out_degree(g, 10, &mda) == GGA_OK && mda) splits.push_back({-1, 10});
        for (int32_t lv : {4, 16, 64})
            if (md >= (uint32_t)lv * 2) splits.push_back({lv, 10});
        int32_t split_pick = 0, split_pick_b = 10;
        uint32_t x_pick = 0;
        for (const Split &sp : splits) {
            if (gga_node_split(c, g, sp.level, sp.buckets)) continue;
            gga_params p = best;
            p.use_split = 1;
            const double t = T.time(p, GGA_BFS, GGA_VARIANT_FRONTIER) +
                             (sssp_ok ? T.time(p, GGA_SSSP, GGA_VARIANT_FRONTIER) : 0.0);
            snprintf(key, sizeof key, "expansion_edges_split_level%d", sp.level);
            T.note(key, t);
            if (t < best_x) {
                best_x = t;
                x_pick = 1;
                split_pick = sp.level;
                split_pick_b = sp.buckets;
            }
        }
        if (g->m <= (1u << 21)) {
            gga_node_split(c, g, 0, 10); /* CDP walks the unsplit graph */
            for (int32_t lv : {-1, 1, 8}) {
                if (lv < 0 && !(md + 1 >= 10)) continue;
                gga_params p = best;
                p.cdp_level = lv;
                p.cdp_buckets = 10;
                p.cdp_mode = 0;
                const double t = T.time(p, GGA_BFS, GGA_VARIANT_CDP_ATOMIC) +
                                 (sssp_ok ? T.time(p, GGA_SSSP, GGA_VARIANT_CDP_ATOMIC) : 0.0);
                snprintf(key, sizeof key, "expansion_cdp_level%d", lv);
                T.note(key, t);
                if (t < best_x) {
                    best_x = t;
                    x_pick = 2;
                    split_pick = lv;
                    split_pick_b = 10;
                }
            }
        }
        best.expansion = x_pick;
        best.split_level = x_pick ? split_pick : 0;
        best.split_buckets = split_pick_b;
        best.use_split = x_pick == 1 ? 1u : 0u;
        /* leave the graph split as the pick needs it, else as it was */
        if (x_pick == 1) gga_node_split(c, g, split_pick, split_pick_b);
        else gga_node_split(c, g, level0, buckets0 ? buckets0 : 10);
        c->params = saved;
        c->params_set = saved_set;
        /* 4. the batch engine's bucket width: eight SSSP queries of this graph
         * in one gga_multi_solve launch per candidate */
        if (sssp_ok) {
            const uint32_t nq = 8;
            std::vector<uint32_t *> outs(nq, nullptr);
            bool ok = true;
            for (uint32_t i = 0; i < nq && ok; ++i)
                ok = cudaMalloc((void **)&outs[i], (size_t)g->n * sizeof(uint32_t)) == cudaSuccess;
            if (ok) {
                std::vector<gga_query> qs(nq);
                for (uint32_t i = 0; i < nq; ++i) {
                    qs[i].graph = g;
                    qs[i].algo = GGA_SSSP;
                    qs[i].src = (uint32_t)(((uint64_t)i * 2654435761u) % g->n);
                    qs[i].dist_out = outs[i];
                }
                double bt = 1e30;
                uint32_t bpick = 0xFFFFFFFFu;
                const int had = g->has_tuned;
                const gga_params had_p = g->tuned;
                for (uint32_t dl : {0u, base / 2 ? base / 2 : 1u, base, base * 2}) {
                    g->tuned = best;
                    g->tuned.batch_delta = dl;
                    g->has_tuned = 1;
                    double t = 0;
                    for (uint32_t k = 0; k < trials; ++k) {
                        gga_stats st;
                        if (gga_multi_solve(c, nq, qs.data(), &st)) {
                            t = 1e30;
                            break;
                        }
                        t += st.kernel_ms;
                    }
                    snprintf(key, sizeof key, "batch_sssp8_delta%u", dl);
                    T.note(key, t / trials);
                    if (t < bt) {
                        bt = t;
                        bpick = dl;
                    }
                }
                g->tuned = had_p;
                g->has_tuned = had;
                best.batch_delta = bpick;
            }
            cudaGetLastError();
            for (uint32_t *o : outs) cudaFree(o);
        }
        cudaFree(T.tmp);
        report = T.log;
    }
    report += "}";
    g->tuned = best;
    g->has_tuned = 1;
    c->params = best;
    c->params_set = true;
    c->tune_report = report;
    if (chosen) *chosen = best;
    return GGA_OK;
}

gga_status gga_autotune_report(gga_ctx *c, char *buf, size_t len) {
    if (!c || !buf || !len) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    snprintf(buf, len, "%s", c->tune_report.empty() ? "{}" : c->tune_report.c_str());
    return GGA_OK;
}
