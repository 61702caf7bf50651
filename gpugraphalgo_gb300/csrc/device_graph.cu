/*
 * Device residency of a graph (Graph::cudaCopy, graph.h:683-699) and the
 * device-side node-split builder (Graph::NodeSplit, graph.h:415-522, with the
 * INT_SPLIT slicing of bfs_sssp.cu:60 and the child-index lists of
 * bfs_sssp.cu:256-283).
 *
 * Split on the device, in five launches over HBM-resident arrays:
 *   1. degree histogram -> MDA (getMaxAllowedOutDegree, graph.h:359-385) when
 *      the level is negative; ceil(maxdeg/level) otherwise (graph.h:390);
 *   2. pieces[u] = max(1, ceil(deg/MDA))                     (graph.h:401-410);
 *   3. exclusive scan of pieces -> first[u] = u + presum[u]  (graph.h:429-456);
 *   4. one thread per split id fills psrc/noutgoing slices, childCount,
 *      IsParent and parentNode                               (graph.h:458-495);
 *   5. edge targets remapped, dst' = first[dst]              (graph.h:500-502).
 * The arrays are identical to the reference's (tests compare them element by
 * element); only psrc is stored 0-based.
 */
#include <stdlib.h>
#include <string.h>

#include <algorithm>

#include "gga_device.cuh"

#include <time.h>
#include <unistd.h>

gga_status dev_wait(cudaStream_t st, double limit_s) {
    const double t0 = gga_now_ms();
    for (;;) {
        cudaError_t e = cudaStreamQuery(st);
        if (e == cudaSuccess) return GGA_OK;
        if (e != cudaErrorNotReady) return gga_fail(GGA_ERR_CUDA, "stream: %s", cudaGetErrorString(e));
        const double el = gga_now_ms() - t0;
        if (el > limit_s * 1e3)
            return gga_fail(GGA_ERR_TIMEOUT, "device work still running after %.0f s; end the process to free the GPU",
                            limit_s);
        if (el > 5.0) usleep(50);
    }
}

/* ------------------------------------------------------------------ scan */

static constexpr uint32_t SCAN_BS = 1024, SCAN_ITEMS = 4;
static constexpr uint32_t SCAN_TILE = SCAN_BS * SCAN_ITEMS;

__global__ void __launch_bounds__(SCAN_BS) k_tile_sums(const uint32_t *in, uint32_t count, uint32_t *sums) {
    __shared__ uint32_t ws[32];
    uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_ITEMS;
    uint32_t s = 0;
#pragma unroll
    for (uint32_t i = 0; i < SCAN_ITEMS; ++i)
        if (base + i < count) s += in[base + i];
    uint32_t tot;
    block_exclusive_scan(s, ws, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(SCAN_BS) k_tile_scan(const uint32_t *in, uint32_t count,
                                                      const uint32_t *tile_base, uint32_t *out) {
    __shared__ uint32_t ws[32];
    uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS], s = 0;
#pragma unroll
    for (uint32_t i = 0; i < SCAN_ITEMS; ++i) {
        v[i] = base + i < count ? in[base + i] : 0;
        s += v[i];
    }
    uint32_t tot;
    uint32_t p = block_exclusive_scan(s, ws, &tot) + tile_base[blockIdx.x];
#pragma unroll
    for (uint32_t i = 0; i < SCAN_ITEMS; ++i) {
        if (base + i < count) out[base + i] = p;
        p += v[i];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) out[count] = p;
}

/* out[0..count] = exclusive prefix sums of in[0..count-1]; out[count] = total.
 * `in` and `out` may alias only if identical. */
gga_status dev_exclusive_scan(const uint32_t *in, uint32_t *out, uint32_t count, cudaStream_t st) {
    if (count == 0) {
        GGA_CK(cudaMemsetAsync(out, 0, sizeof(uint32_t), st));
        return GGA_OK;
    }
    uint32_t tiles = (count + SCAN_TILE - 1) / SCAN_TILE;
    uint32_t *sums = nullptr;
    GGA_CK(cudaMallocAsync((void **)&sums, ((size_t)tiles + 1) * 2 * sizeof(uint32_t), st));
    uint32_t *scanned = sums + tiles + 1;
    k_tile_sums<<<tiles, SCAN_BS, 0, st>>>(in, count, sums);
    gga_status s = GGA_OK;
    if (tiles > 1) {
        s = dev_exclusive_scan(sums, scanned, tiles, st);
    } else {
        cudaMemsetAsync(scanned, 0, sizeof(uint32_t), st);
    }
    if (s == GGA_OK) k_tile_scan<<<tiles, SCAN_BS, 0, st>>>(in, count, scanned, out);
    cudaFreeAsync(sums, st);
    GGA_CK(cudaGetLastError());
    return s;
}

/* ------------------------------------------------------------ residency */

static void dev_free_split(DevGraph *d) {
    cudaFree(d->s_off); cudaFree(d->s_col); cudaFree(d->s_cc); cudaFree(d->s_isp);
    cudaFree(d->s_par); cudaFree(d->first); cudaFree(d->cidx); cudaFree(d->ccnt);
    d->s_off = d->s_col = d->s_cc = d->s_isp = d->s_par = d->first = d->cidx = d->ccnt = nullptr;
    d->level = 0;
    d->ns = d->mda = d->npar = 0;
}

/* The base arrays and the light/heavy order come from the device's
 * stream-ordered pool (the context keeps up to 4 GiB of it mapped), so a
 * graph released and uploaded again reuses the same memory instead of
 * mapping fresh pages.  Released after a device synchronize, as cudaFree
 * would: no launch on any stream still reads them. */
static void pool_release(void *p) {
    if (p) cudaFreeAsync(p, 0);
}

static void dev_graph_release(gga_graph *g) {
    DevGraph *d = (DevGraph *)g->dev;
    if (!d) return;
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(d->device);
    dev_free_split(d);
    cudaDeviceSynchronize();
    pool_release(d->off); pool_release(d->col); pool_release(d->wt);
    pool_release(d->lcol); pool_release(d->lwt); pool_release(d->light);
    cudaStreamSynchronize(0);
    if (prev >= 0) cudaSetDevice(prev);
    free(d);
    g->dev = nullptr;
    g->dev_device = -1;
}

DevGraph *dev_graph_of(gga_graph *g) { return (DevGraph *)g->dev; }

GraphView dev_graph_view(const DevGraph *d, bool split) {
    GraphView v;
    if (split && d->level != 0) {
        v.off = d->s_off; v.col = d->s_col; v.wt = d->wt; v.cc = d->s_cc; v.n = d->ns; v.m = d->m;
        v.symmetric = 0;
    } else {
        v.off = d->off; v.col = d->col; v.wt = d->wt; v.cc = nullptr; v.n = d->n; v.m = d->m;
        v.symmetric = d->symmetric > 0;
    }
    return v;
}

/* ------------------------------------------------------------ light / heavy */

static unsigned grid_for(uint64_t items, unsigned bs);

/* Light-first, class-ordered rows for bucket width delta (delta-stepping's
 * edge classes, Meyer & Sanders, refined): within each row the edges with
 * w < delta come first (class 0), then the heavy edges in LH_CLASSES weight
 * classes of width cw = ceil((maxw - delta + 1) / LH_CLASSES), class
 * c >= 1 holding delta + (c-1) cw <= w < delta + c cw, each class in its
 * original order; light[u] counts class 0.  So the class of the heavy edges
 * never falls along a row, and a pulling bucket close can cut a vertex's
 * heavy range where the classes become too heavy to lower its distance.  A
 * stable multi-way partition per row:
 *   k_lh_rows: one warp per row of at most LH_WARP_MAX edges: a first pass
 *     counts each class (one ballot per class per 32 edges), a second
 *     writes each edge at its class start plus its rank in the class
 *     (ballot + popc); longer rows are listed in `big` for
 *   k_lh_big: one CTA per long row, the same passes with CTA-wide ranks
 *     (per-warp ballot counts in shared memory) per 32 x warps edges.
 * Loop bounds are warp- (CTA-) uniform; every collective is reached by the
 * whole warp (CTA).  nlight accumulates the light edges of the graph. */
constexpr uint32_t LH_WARP_MAX = 4096;
constexpr unsigned LH_BIG_BS = 1024;
constexpr uint32_t LH_NCLS = LH_CLASSES + 1; /* class 0 light, 1..LH_CLASSES heavy */

__device__ __forceinline__ uint32_t lh_class(uint32_t w, uint32_t delta, uint32_t cw) {
    return w < delta ? 0u : 1u + min((w - delta) / cw, LH_CLASSES - 1);
}

__global__ void k_lh_rows(const uint32_t *off, const uint32_t *col, const uint32_t *wt, uint32_t n, uint32_t delta,
                          uint32_t cw, uint32_t *lcol, uint32_t *lwt, uint32_t *light, uint32_t *big, uint32_t *nbig,
                          unsigned long long *nlight) {
    constexpr unsigned FULL = 0xffffffffu;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lt = (1u << lane) - 1u;
    const uint64_t w0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    unsigned long long mine = 0;
    for (uint64_t u = w0; u < n; u += nw) {
        const uint32_t b = off[u], e = off[u + 1];
        if (e - b > LH_WARP_MAX) {
            if (lane == 0) big[atomicAdd(nbig, 1u)] = (uint32_t)u;
            continue;
        }
        uint32_t pos[LH_NCLS]; /* class counts, then class write cursors (the same in every lane) */
#pragma unroll
        for (uint32_t c = 0; c < LH_NCLS; ++c) pos[c] = 0;
        for (uint64_t k0 = b; k0 < e; k0 += 32) { /* 64-bit: no wrap near 2^32 edges */
            const uint64_t k = k0 + lane;
            const uint32_t cls = k < e ? lh_class(wt[k], delta, cw) : LH_NCLS;
#pragma unroll
            for (uint32_t c = 0; c < LH_NCLS; ++c) pos[c] += __popc(__ballot_sync(FULL, cls == c));
        }
        const uint32_t nl = pos[0];
        uint32_t run = b;
#pragma unroll
        for (uint32_t c = 0; c < LH_NCLS; ++c) {
            const uint32_t cnt = pos[c];
            pos[c] = run;
            run += cnt;
        }
        for (uint64_t k0 = b; k0 < e; k0 += 32) {
            const uint64_t k = k0 + lane;
            const bool in = k < e;
            const uint32_t w = in ? wt[k] : 0u, cv = in ? col[k] : 0u;
            const uint32_t cls = in ? lh_class(w, delta, cw) : LH_NCLS;
            uint32_t p = 0;
#pragma unroll
            for (uint32_t c = 0; c < LH_NCLS; ++c) {
                const uint32_t m = __ballot_sync(FULL, cls == c);
                if (cls == c) p = pos[c] + __popc(m & lt);
                pos[c] += __popc(m);
            }
            if (in) {
                lcol[p] = cv;
                lwt[p] = w;
            }
        }
        if (lane == 0) {
            light[u] = nl;
            mine += nl;
        }
    }
    if (lane == 0 && mine) atomicAdd(nlight, mine);
}

__global__ void __launch_bounds__(LH_BIG_BS) k_lh_big(const uint32_t *off, const uint32_t *col, const uint32_t *wt,
                                                      uint32_t delta, uint32_t cw, const uint32_t *big,
                                                      const uint32_t *nbig, uint32_t *lcol, uint32_t *lwt,
                                                      uint32_t *light, unsigned long long *nlight) {
    constexpr unsigned FULL = 0xffffffffu;
    constexpr uint32_t NWARP = LH_BIG_BS / 32;
    __shared__ uint32_t s_cnt[LH_NCLS][NWARP]; /* per class, per warp: edges of the chunk */
    __shared__ uint32_t s_pos[LH_NCLS];        /* per class: row total, then write cursor */
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t lt = (1u << lane) - 1u;
    const uint32_t rows = *nbig;
    for (uint32_t r = blockIdx.x; r < rows; r += gridDim.x) {
        const uint32_t u = big[r], b = off[u], e = off[u + 1];
        if (threadIdx.x < LH_NCLS) s_pos[threadIdx.x] = 0;
        __syncthreads();
        for (uint64_t k0 = b; k0 < e; k0 += LH_BIG_BS) { /* pass 1: class totals */
            const uint64_t k = k0 + threadIdx.x;
            const uint32_t cls = k < e ? lh_class(wt[k], delta, cw) : LH_NCLS;
            for (uint32_t c = 0; c < LH_NCLS; ++c) {
                const uint32_t m = __ballot_sync(FULL, cls == c);
                if (lane == 0 && m) atomicAdd(&s_pos[c], (uint32_t)__popc(m));
            }
        }
        __syncthreads();
        const uint32_t nl = s_pos[0];
        __syncthreads();
        if (threadIdx.x == 0) { /* totals -> class starts */
            uint32_t run = b;
            for (uint32_t c = 0; c < LH_NCLS; ++c) {
                const uint32_t cnt = s_pos[c];
                s_pos[c] = run;
                run += cnt;
            }
        }
        __syncthreads();
        for (uint64_t k0 = b; k0 < e; k0 += LH_BIG_BS) { /* pass 2: ranks within class across warps */
            const uint64_t k = k0 + threadIdx.x;
            const bool in = k < e;
            const uint32_t w = in ? wt[k] : 0u, cv = in ? col[k] : 0u;
            const uint32_t cls = in ? lh_class(w, delta, cw) : LH_NCLS;
            uint32_t mine = 0;
            for (uint32_t c = 0; c < LH_NCLS; ++c) {
                const uint32_t m = __ballot_sync(FULL, cls == c);
                if (lane == 0) s_cnt[c][warp] = __popc(m);
                if (cls == c) mine = __popc(m & lt);
            }
            __syncthreads();
            if (in) {
                uint32_t before = 0; /* edges of my class in earlier warps of this chunk */
                for (uint32_t q = 0; q < warp; ++q) before += s_cnt[cls][q];
                const uint32_t p = s_pos[cls] + before + mine;
                lcol[p] = cv;
                lwt[p] = w;
            }
            __syncthreads();
            if (threadIdx.x < LH_NCLS) { /* advance the cursors past this chunk */
                uint32_t t = 0;
                for (uint32_t q = 0; q < NWARP; ++q) t += s_cnt[threadIdx.x][q];
                s_pos[threadIdx.x] += t;
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            light[u] = nl;
            atomicAdd(nlight, (unsigned long long)nl);
        }
        __syncthreads(); /* s_pos is reset by the next row */
    }
}

gga_status dev_graph_light_heavy(gga_graph *g, uint32_t delta, cudaStream_t st) {
    DevGraph *d = dev_graph_of(g);
    if (!d) return gga_fail(GGA_ERR_INVALID_ARG, "graph not resident");
    if (d->lcol && d->lh_delta == delta) return GGA_OK;
    const size_t mpad = ((size_t)d->m + 4) & ~(size_t)3;
    cudaError_t e = cudaSuccess;
    if (!d->lcol) {
        e = cudaMallocAsync((void **)&d->lcol, mpad * sizeof(uint32_t), st);
        if (e == cudaSuccess) e = cudaMallocAsync((void **)&d->lwt, mpad * sizeof(uint32_t), st);
        if (e == cudaSuccess) e = cudaMallocAsync((void **)&d->light, ((size_t)d->n + 1) * sizeof(uint32_t), st);
        if (e != cudaSuccess) {
            cudaGetLastError();
            cudaStreamSynchronize(st);
            pool_release(d->lcol); pool_release(d->lwt); pool_release(d->light);
            d->lcol = d->lwt = d->light = nullptr;
            return gga_fail(GGA_ERR_CUDA, "light/heavy order (%u edges): %s", d->m, cudaGetErrorString(e));
        }
        GGA_CK(cudaMemsetAsync(d->lcol + d->m, 0, (mpad - d->m) * sizeof(uint32_t), st));
        GGA_CK(cudaMemsetAsync(d->lwt + d->m, 0, (mpad - d->m) * sizeof(uint32_t), st));
    }
    d->lh_delta = 0;
    /* heavy class width: maxw < delta + LH_CLASSES * cw */
    const uint32_t cw = g->maxw >= delta ? (uint32_t)(((uint64_t)g->maxw - delta + LH_CLASSES) / LH_CLASSES) : 1u;
    /* scratch: the long-row list (at most m / LH_WARP_MAX rows), its count and the light total */
    const size_t nbig_cap = (size_t)d->m / LH_WARP_MAX + 1;
    uint32_t *scr = nullptr;
    GGA_CK(cudaMallocAsync((void **)&scr, (nbig_cap + 4) * sizeof(uint32_t), st));
    uint32_t *nbig = scr, *big = scr + 4;
    unsigned long long *nlight = (unsigned long long *)(scr + 2);
    gga_status s = gga_cuda_check(cudaMemsetAsync(scr, 0, 4 * sizeof(uint32_t), st));
    if (s == GGA_OK && d->n) {
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d->device);
        const uint64_t want_warps = d->n;
        const unsigned grid = (unsigned)std::min<uint64_t>((want_warps + 7) / 8, (uint64_t)(sms > 0 ? sms : 1) * 16);
        k_lh_rows<<<grid ? grid : 1, 256, 0, st>>>(d->off, d->col, d->wt, d->n, delta, cw, d->lcol, d->lwt, d->light,
                                                    big, nbig, nlight);
        k_lh_big<<<(sms > 0 ? sms : 1) * 2, LH_BIG_BS, 0, st>>>(d->off, d->col, d->wt, delta, cw, big, nbig, d->lcol,
                                                                 d->lwt, d->light, nlight);
        s = gga_cuda_check(cudaGetLastError());
    }
    unsigned long long hl = 0;
    if (s == GGA_OK) s = gga_cuda_check(cudaMemcpyAsync(&hl, nlight, sizeof hl, cudaMemcpyDeviceToHost, st));
    cudaFreeAsync(scr, st);
    if (s) return s;
    if ((s = dev_wait(st, 60.0))) return s;
    d->lh_delta = delta;
    d->lh_cw = cw;
    d->lh_heavy = d->m - (uint32_t)hl;
    return GGA_OK;
}

/* flag bit 0: a row is not sorted; bit 1: an edge (u, v) has no (v, u);
 * bit 2: the (v, u) found has another weight.  One thread per edge: its row
 * by binary search over the offsets, its reverse by binary search in the
 * target's (sorted) row. */
__global__ void k_check_symmetric(const uint32_t *off, const uint32_t *col, const uint32_t *wt, uint32_t n, uint32_t m,
                                  uint32_t *flag) {
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = n; /* largest u with off[u] <= e */
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (off[mid] <= e) lo = mid; else hi = mid;
        }
        const uint32_t u = lo, v = col[e];
        if (e + 1 < off[u + 1] && col[e + 1] < v) atomicOr(flag, 1u);
        uint32_t b = off[v], t = off[v + 1];
        const uint32_t end = t;
        while (b < t) {
            const uint32_t mid = b + ((t - b) >> 1);
            if (col[mid] < u) b = mid + 1; else t = mid;
        }
        if (b >= end || col[b] != u) atomicOr(flag, 2u);
        else if (wt[b] != wt[e]) atomicOr(flag, 4u);
    }
}

gga_status dev_graph_check_symmetric(gga_graph *g, uint32_t *dflag, uint32_t *hflag, cudaStream_t st) {
    DevGraph *d = dev_graph_of(g);
    if (!d) return gga_fail(GGA_ERR_INVALID_ARG, "graph not resident");
    if (d->symmetric != 0 && d->wsymmetric != 0) return GGA_OK;
    GGA_CK(cudaMemsetAsync(dflag, 0, sizeof(uint32_t), st));
    if (d->m) {
        int sms = 0;
        GGA_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d->device));
        const uint64_t want = ((uint64_t)d->m + 255) / 256;
        const unsigned grid = (unsigned)(want < (uint64_t)sms * 16 ? want : (uint64_t)sms * 16);
        k_check_symmetric<<<grid, 256, 0, st>>>(d->off, d->col, d->wt, d->n, d->m, dflag);
        GGA_CK(cudaGetLastError());
    }
    GGA_CK(cudaMemcpyAsync(hflag, dflag, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    gga_status s = dev_wait(st, 60.0);
    if (s) return s;
    d->symmetric = (*hflag & 3u) ? -1 : 1;
    d->wsymmetric = *hflag ? -1 : 1;
    g->symmetric = d->symmetric;
    g->wsymmetric = d->wsymmetric;
    return GGA_OK;
}

/* Uploads g to `device` once; later calls return at once (cudaCopy,
 * graph.h:683-699 copies eight arrays; the relaxation needs three). */
gga_status dev_graph_ensure(gga_graph *g, int device, cudaStream_t st) {
    if (g->dev) {
        if (g->dev_device != device)
            return gga_fail(GGA_ERR_INVALID_ARG, "graph is resident on device %d, context uses %d",
                            g->dev_device, device);
        return GGA_OK;
    }
    pthread_mutex_lock(&g->lock);
    gga_status s = GGA_OK;
    if (!g->dev) {
        gga_dev_graph_release_hook = dev_graph_release;
        DevGraph *d = (DevGraph *)calloc(1, sizeof *d);
        if (!d) {
            pthread_mutex_unlock(&g->lock);
            return gga_fail(GGA_ERR_NO_MEMORY, "DevGraph");
        }
        d->device = device;
        d->n = g->n;
        d->m = g->m;
        d->maxdeg = g->maxdeg;
        d->symmetric = g->symmetric;
        d->wsymmetric = g->wsymmetric;
        size_t mpad = ((size_t)g->m + 4) & ~(size_t)3; /* room for 16-byte vector loads */
        cudaError_t e = cudaMallocAsync((void **)&d->off, ((size_t)g->n + 1) * sizeof(uint32_t), st);
        if (e == cudaSuccess) e = cudaMallocAsync((void **)&d->col, mpad * sizeof(uint32_t), st);
        if (e == cudaSuccess) e = cudaMallocAsync((void **)&d->wt, mpad * sizeof(uint32_t), st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d->off, g->off, ((size_t)g->n + 1) * sizeof(uint32_t),
                                cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess && g->m)
            e = cudaMemcpyAsync(d->col, g->col, (size_t)g->m * sizeof(uint32_t), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess && g->m)
            e = cudaMemcpyAsync(d->wt, g->wt, (size_t)g->m * sizeof(uint32_t), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(d->col + g->m, 0, (mpad - g->m) * sizeof(uint32_t), st);
        if (e == cudaSuccess) e = cudaMemsetAsync(d->wt + g->m, 0, (mpad - g->m) * sizeof(uint32_t), st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            const cudaError_t e0 = e;
            cudaGetLastError();
            cudaStreamSynchronize(st);
            pool_release(d->off); pool_release(d->col); pool_release(d->wt);
            cudaStreamSynchronize(0);
            e = e0;
            free(d);
            s = gga_fail(GGA_ERR_CUDA, "graph upload (%u vertices, %u edges): %s", g->n, g->m,
                         cudaGetErrorString(e));
        } else {
            g->dev = d;
            g->dev_device = device;
        }
    }
    pthread_mutex_unlock(&g->lock);
    return s;
}

/* ------------------------------------------------------------ split */

__global__ void k_max_degree(const uint32_t *off, uint32_t n, uint32_t *out) {
    uint32_t best = 0;
    for (uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; u < n;
         u += (uint64_t)gridDim.x * blockDim.x)
        best = max(best, off[u + 1] - off[u]);
    best = __reduce_max_sync(0xffffffffu, best);
    if ((threadIdx.x & 31) == 0) atomicMax(out, best);
}

/* Bucket = (int)((deg / (float)(maxdeg+1)) * buckets) in round-to-nearest
 * single precision, as graph.h:365 computes it on the host. */
__global__ void k_degree_histogram(const uint32_t *off, uint32_t n, const uint32_t *maxdeg,
                                   int32_t buckets, uint32_t *histo) {
    extern __shared__ uint32_t sh[];
    const bool use_smem = buckets <= 8192;
    if (use_smem)
        for (int32_t i = threadIdx.x; i < buckets; i += blockDim.x) sh[i] = 0;
    __syncthreads();
    const float fm = (float)(int32_t)(*maxdeg + 1u), fb = (float)buckets;
    for (uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; u < n;
         u += (uint64_t)gridDim.x * blockDim.x) {
        float q = __fdiv_rn((float)(off[u + 1] - off[u]), fm);
        int32_t idx = (int32_t)__fmul_rn(q, fb);
        if (idx >= buckets) idx = buckets - 1;
        atomicAdd(use_smem ? &sh[idx] : &histo[idx], 1u);
    }
    __syncthreads();
    if (use_smem)
        for (int32_t i = threadIdx.x; i < buckets; i += blockDim.x)
            if (sh[i]) atomicAdd(&histo[i], sh[i]);
}

/* MAX_EDGES_ALLOWED from the split level or the histogram (first maximum). */
__global__ void k_split_limit(const uint32_t *histo, int32_t buckets, int32_t level,
                              const uint32_t *maxdeg, uint32_t *mda) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    uint32_t md = *maxdeg;
    if (level > 0) {
        *mda = (uint32_t)(((uint64_t)md + (uint32_t)level - 1) / (uint32_t)level);
        return;
    }
    int32_t best = -1, bi = -1;
    for (int32_t i = 0; i < buckets; ++i)
        if ((int32_t)histo[i] > best) { best = (int32_t)histo[i]; bi = i; }
    int32_t maxdeg1 = (int32_t)md + 1;
    *mda = (uint32_t)((maxdeg1 / buckets) * (bi + 1));
}

__global__ void k_pieces(const uint32_t *off, uint32_t n, const uint32_t *mda, uint32_t *pieces,
                         uint32_t *err) {
    const uint32_t lim = *mda;
    for (uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; u < n;
         u += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t d = off[u + 1] - off[u];
        uint32_t p = 1;
        if (d) {
            if (lim == 0) {
                atomicExch(err, GGA_DEV_SPLIT_RULE);
                p = 1;
            } else {
                p = (uint32_t)(((uint64_t)d + lim - 1) / lim);
            }
        }
        pieces[u] = p;
    }
}

/* One thread per split id k: owner u has first[u] <= k < first[u+1]. */
__global__ void k_split_fill(const uint32_t *off, uint32_t n, uint32_t m, const uint32_t *first,
                             uint32_t ns, uint32_t *s_off, uint32_t *s_cc, uint32_t *s_isp,
                             uint32_t *s_par) {
    for (uint64_t k64 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k64 < ns;
         k64 += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t k = (uint32_t)k64;
        uint32_t lo = 0, hi = n; /* last u with first[u] <= k */
        while (hi - lo > 1) {
            uint32_t mid = (lo + hi) >> 1;
            if (first[mid] <= k) lo = mid; else hi = mid;
        }
        uint32_t u = lo;
        uint32_t j = k - first[u];
        uint32_t pieces = first[u + 1] - first[u];
        uint32_t deg = off[u + 1] - off[u];
        uint32_t local = deg ? (deg + pieces - 1) / pieces : 0; /* INT_SPLIT, graph.h:462 */
        s_off[k] = off[u] + j * local;
        s_cc[k] = j == 0 ? pieces - 1 : 0;
        s_isp[k] = j == 0 ? 1u : 0u;
        s_par[k] = u;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) s_off[ns] = m;
}

__global__ void k_remap_targets(const uint32_t *col, uint32_t m, const uint32_t *first, uint32_t *s_col) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m;
         e += (uint64_t)gridDim.x * blockDim.x)
        s_col[e] = first[col[e]];
}

__global__ void k_flag_parents(const uint32_t *s_cc, uint32_t ns, uint32_t *flags) {
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < ns;
         k += (uint64_t)gridDim.x * blockDim.x)
        flags[k] = s_cc[k] ? 1u : 0u;
}

__global__ void k_compact_parents(const uint32_t *s_cc, uint32_t ns, const uint32_t *pos,
                                  uint32_t *cidx, uint32_t *ccnt) {
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < ns;
         k += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t c = s_cc[k];
        if (c) {
            cidx[pos[k]] = (uint32_t)k;
            ccnt[pos[k]] = c;
        }
    }
}

static unsigned grid_for(uint64_t items, unsigned bs) {
    uint64_t b = (items + bs - 1) / bs;
    if (b < 1) b = 1;
    if (b > 152u * 64u) b = 152u * 64u;
    return (unsigned)b;
}

/* Builds the split for `level`/`buckets` on the device (ctx stream `st`). */
gga_status dev_node_split(gga_graph *g, int32_t level, int32_t buckets, cudaStream_t st) {
    DevGraph *d = (DevGraph *)g->dev;
    if (!d) return gga_fail(GGA_ERR_INVALID_ARG, "graph not resident");
    dev_free_split(d);
    g->split_level = 0;
    g->ns = g->mda = g->parents_with_children = 0;
    if (level == 0) return GGA_OK;
    if (level < 0 && buckets <= 0)
        return gga_fail(GGA_ERR_INVALID_ARG, "buckets must be positive (got %d)", buckets);

    const uint32_t n = d->n, m = d->m;
    uint32_t *scal = nullptr; /* [0]=maxdeg [1]=mda [2]=err */
    uint32_t *histo = nullptr, *pieces = nullptr;
    gga_status s = GGA_OK;
    uint32_t hs[3];
    int32_t nb = level < 0 ? buckets : 1;
    GGA_CK(cudaMallocAsync((void **)&scal, 4 * sizeof(uint32_t), st));
    GGA_CK(cudaMallocAsync((void **)&histo, (size_t)nb * sizeof(uint32_t), st));
    GGA_CK(cudaMallocAsync((void **)&pieces, ((size_t)n + 1) * sizeof(uint32_t), st));
    cudaMemsetAsync(scal, 0, 4 * sizeof(uint32_t), st);
    cudaMemsetAsync(histo, 0, (size_t)nb * sizeof(uint32_t), st);
    k_max_degree<<<grid_for(n, 256), 256, 0, st>>>(d->off, n, scal);
    if (level < 0) {
        size_t sm = buckets <= 8192 ? (size_t)buckets * sizeof(uint32_t) : 0;
        k_degree_histogram<<<grid_for(n, 256), 256, sm, st>>>(d->off, n, scal, buckets, histo);
    }
    k_split_limit<<<1, 32, 0, st>>>(histo, nb, level, scal, scal + 1);
    k_pieces<<<grid_for(n, 256), 256, 0, st>>>(d->off, n, scal + 1, pieces, scal + 2);
    cudaError_t e = cudaMemcpyAsync(hs, scal, 3 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        s = gga_fail(GGA_ERR_CUDA, "split limit: %s", cudaGetErrorString(e));
        goto done;
    }
    if (hs[2] == GGA_DEV_SPLIT_RULE) {
        s = gga_fail(GGA_ERR_SPLIT_RULE,
                     "edge limit is 0 (maxdeg %u, level %d, buckets %d): the reference divides by zero",
                     hs[0], level, buckets);
        goto done;
    }
    GGA_CK(cudaMalloc((void **)&d->first, ((size_t)n + 1) * sizeof(uint32_t)));
    s = dev_exclusive_scan(pieces, d->first, n, st);
    if (s) goto done;
    {
        uint32_t ns = 0;
        e = cudaMemcpyAsync(&ns, d->first + n, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) { s = gga_fail(GGA_ERR_CUDA, "split size: %s", cudaGetErrorString(e)); goto done; }
        if (ns > GGA_MAX_NODES) { s = gga_fail(GGA_ERR_TOO_LARGE, "split gives %u vertices", ns); goto done; }
        size_t mpad = ((size_t)m + 4) & ~(size_t)3;
        e = cudaMalloc((void **)&d->s_off, ((size_t)ns + 1) * sizeof(uint32_t));
        if (e == cudaSuccess) e = cudaMalloc((void **)&d->s_cc, (size_t)ns * sizeof(uint32_t));
        if (e == cudaSuccess) e = cudaMalloc((void **)&d->s_isp, (size_t)ns * sizeof(uint32_t));
        if (e == cudaSuccess) e = cudaMalloc((void **)&d->s_par, (size_t)ns * sizeof(uint32_t));
        if (e == cudaSuccess) e = cudaMalloc((void **)&d->s_col, mpad * sizeof(uint32_t));
        if (e != cudaSuccess) { s = gga_fail(GGA_ERR_CUDA, "split arrays: %s", cudaGetErrorString(e)); goto done; }
        cudaMemsetAsync(d->s_col + m, 0, (mpad - m) * sizeof(uint32_t), st);
        k_split_fill<<<grid_for(ns, 256), 256, 0, st>>>(d->off, n, m, d->first, ns, d->s_off, d->s_cc,
                                                        d->s_isp, d->s_par);
        k_remap_targets<<<grid_for(m, 256), 256, 0, st>>>(d->col, m, d->first, d->s_col);
        /* child index lists: reuse `pieces` as flags when large enough */
        uint32_t *flags = nullptr, *pos = nullptr;
        GGA_CK(cudaMallocAsync((void **)&flags, ((size_t)ns + 1) * 2 * sizeof(uint32_t), st));
        pos = flags + ns + 1;
        k_flag_parents<<<grid_for(ns, 256), 256, 0, st>>>(d->s_cc, ns, flags);
        s = dev_exclusive_scan(flags, pos, ns, st);
        uint32_t npar = 0;
        if (s == GGA_OK) {
            e = cudaMemcpyAsync(&npar, pos + ns, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e == cudaSuccess) e = cudaMalloc((void **)&d->cidx, ((size_t)npar + 1) * sizeof(uint32_t));
            if (e == cudaSuccess) e = cudaMalloc((void **)&d->ccnt, ((size_t)npar + 1) * sizeof(uint32_t));
            if (e == cudaSuccess)
                k_compact_parents<<<grid_for(ns, 256), 256, 0, st>>>(d->s_cc, ns, pos, d->cidx, d->ccnt);
            if (e == cudaSuccess) e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) s = gga_fail(GGA_ERR_CUDA, "child index: %s", cudaGetErrorString(e));
        }
        cudaFreeAsync(flags, st);
        if (s) goto done;
        d->level = level;
        d->buckets = buckets;
        d->ns = ns;
        d->mda = hs[1];
        d->npar = npar;
        d->maxdeg = hs[0];
        g->split_level = level;
        g->split_buckets = buckets;
        g->ns = ns;
        g->mda = hs[1];
        g->parents_with_children = npar;
    }
done:
    cudaFreeAsync(scal, st);
    cudaFreeAsync(histo, st);
    cudaFreeAsync(pieces, st);
    if (s) dev_free_split(d);
    cudaStreamSynchronize(st);
    return s;
}

/* Reference-layout export of the (split) graph. */
__global__ void k_export_psrc(const uint32_t *s_off, uint32_t ns, uint32_t m, uint32_t *psrc,
                              uint32_t *nout) {
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k <= ns;
         k += (uint64_t)gridDim.x * blockDim.x) {
        if (k < ns) {
            if (psrc) psrc[k] = s_off[k] + 1;
            if (nout) nout[k] = s_off[k + 1] - s_off[k];
        } else if (psrc) {
            psrc[ns] = m; /* graph.h:498 */
        }
    }
}

gga_status dev_split_maps(gga_graph *g, uint32_t *psrc, uint32_t *noutgoing, uint32_t *edgessrcdst,
                          uint32_t *child_count, uint32_t *is_parent, uint32_t *parent_node,
                          cudaStream_t st) {
    DevGraph *d = (DevGraph *)g->dev;
    const bool split = d->level != 0;
    const uint32_t n = split ? d->ns : d->n, m = d->m;
    uint32_t *tmp = nullptr;
    GGA_CK(cudaMallocAsync((void **)&tmp, ((size_t)n + 1) * 2 * sizeof(uint32_t), st));
    uint32_t *t_psrc = tmp, *t_nout = tmp + n + 1;
    k_export_psrc<<<grid_for(n + 1, 256), 256, 0, st>>>(split ? d->s_off : d->off, n, m, t_psrc, t_nout);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && psrc)
        e = cudaMemcpyAsync(psrc, t_psrc, ((size_t)n + 1) * 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && noutgoing)
        e = cudaMemcpyAsync(noutgoing, t_nout, (size_t)n * 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && edgessrcdst) {
        edgessrcdst[0] = 0; /* null slot; left uninitialised by the reference */
        if (m)
            e = cudaMemcpyAsync(edgessrcdst + 1, split ? d->s_col : d->col, (size_t)m * 4,
                                cudaMemcpyDeviceToHost, st);
    }
    if (split) {
        if (e == cudaSuccess && child_count)
            e = cudaMemcpyAsync(child_count, d->s_cc, (size_t)n * 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess && is_parent)
            e = cudaMemcpyAsync(is_parent, d->s_isp, (size_t)n * 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess && parent_node)
            e = cudaMemcpyAsync(parent_node, d->s_par, (size_t)n * 4, cudaMemcpyDeviceToHost, st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFreeAsync(tmp, st);
    cudaStreamSynchronize(st);
    if (e != cudaSuccess) return gga_fail(GGA_ERR_CUDA, "split export: %s", cudaGetErrorString(e));
    if (!split) {
        for (uint32_t i = 0; i < n; ++i) {
            if (child_count) child_count[i] = 0;
            if (is_parent) is_parent[i] = 1;
            if (parent_node) parent_node[i] = i;
        }
    }
    return GGA_OK;
}

gga_status dev_child_index(gga_graph *g, uint32_t *count, uint32_t *cidx, uint32_t *ccnt, cudaStream_t st) {
    DevGraph *d = (DevGraph *)g->dev;
    uint32_t np = d->level ? d->npar : 0;
    if (*count < np || (np && (!cidx || !ccnt))) {
        *count = np;
        return gga_fail(GGA_ERR_INVALID_ARG, "child index needs capacity %u", np);
    }
    *count = np;
    if (np) {
        GGA_CK(cudaMemcpyAsync(cidx, d->cidx, (size_t)np * 4, cudaMemcpyDeviceToHost, st));
        GGA_CK(cudaMemcpyAsync(ccnt, d->ccnt, (size_t)np * 4, cudaMemcpyDeviceToHost, st));
        GGA_CK(cudaStreamSynchronize(st));
    }
    return GGA_OK;
}
