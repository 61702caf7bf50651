/*
 * Reference-semantics engines: the topology-driven fixed point of the
 * reference's four builds, re-expressed over the 0-based device CSR.
 *
 *   na_  (GGA_VARIANT_TOPO_ATOMIC): M_my_drelax, cudaKernels.h:285-344.
 *        One thread per (split) vertex relaxes all its out-edges with
 *        atomicMin and mirrors an improvement into the target's children.
 *   n_   (GGA_VARIANT_TOPO_PLAIN): my_updateDist (cudaKernels.h:129-141)
 *        then my_drelax_no_atomic (cudaKernels.h:161-220), plain stores.
 *   da_/d_ (GGA_VARIANT_CDP_*): my_drelax_dynamicP (cudaKernels.h:438-520)
 *        on the unsplit graph.  Vertices above maxAllowed are not relaxed by
 *        their thread.  In the default mode they are appended to a heavy list
 *        and the last CTA of the grid makes ONE CDP2 tail launch
 *        (cudaStreamTailLaunch) that relaxes all heavy edge lists, one CTA
 *        per vertex; in the reference's own shape (cdp_mode 1) every heavy
 *        vertex's thread launches a fire-and-forget <<<1,32>>> child, the
 *        dynamicP_relax_coal grid of cudaKernels.h:347-377.  A failed device
 *        launch falls back to relaxing inline, as cudaKernels.h:483-512 do.
 * The host loop is the reference's (bfs_sssp.cu:372-468): clear `changed`,
 * launch, read `changed`, repeat; launch shape BLOCKSIZE=1024 threads x
 * #SMs x FACTOR blocks (bfs_sssp.cu:145,333-334).
 */
#include <algorithm>
#include <math.h>

#include "gga_device.cuh"

namespace {

constexpr uint32_t TOPO_BS = 1024; /* BLOCKSIZE, bfs_sssp.cu:50 */

struct CdpState {
    uint32_t heavy_count;
    uint32_t ticket;
    uint32_t children;   /* device launches that succeeded */
    uint32_t fallbacks;  /* launches that failed -> inline */
};

template <bool SSSP, bool ATOMIC>
__device__ __forceinline__ void relax_vertex(const GraphView g, uint32_t *dist, uint32_t u, bool &any) {
    const uint32_t start = g.off[u], end = g.off[u + 1];
    for (uint32_t ii = start; ii < end; ++ii) {
        const uint32_t v = g.col[ii];
        const uint32_t wt = SSSP ? g.wt[ii] : 1u;
        const uint32_t alt = dist[u] + wt;
        if (alt < dist[v]) {
            if (ATOMIC) atomicMin(dist + v, alt);
            else dist[v] = alt;
            if (g.cc) {
                const uint32_t c = g.cc[v];
                for (uint32_t k = 1; k <= c; ++k) {
                    if (ATOMIC) atomicMin(dist + v + k, alt);
                    else dist[v + k] = alt;
                }
            }
            any = true;
        }
    }
}

template <bool SSSP, bool ATOMIC>
__global__ void __launch_bounds__(TOPO_BS) k_topo_relax(const GraphView g, uint32_t *dist, uint32_t *changed) {
    const uint32_t u = blockIdx.x * blockDim.x + threadIdx.x;
    bool any = false;
    if (u < g.n) relax_vertex<SSSP, ATOMIC>(g, dist, u, any);
    if (any) *changed = 1;
}

/* my_updateDist: copy each parent's distance into its children. */
__global__ void __launch_bounds__(TOPO_BS) k_update_children(uint32_t *dist, const uint32_t *cidx,
                                                              const uint32_t *ccnt, uint32_t npar) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < npar) {
        const uint32_t p = cidx[i], c = ccnt[i];
        const uint32_t d = dist[p];
        for (uint32_t k = 1; k <= c; ++k) dist[p + k] = d;
    }
}

/* dist = MYINFINITY except the source's parent and children (bfs_sssp.cu:301-318). */
__global__ void k_topo_init(uint32_t *dist, uint32_t n, const uint32_t *first, const uint32_t *cc, uint32_t src) {
    const uint32_t s0 = first ? first[src] : src;
    const uint32_t cnt = cc ? cc[s0] + 1 : 1;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        dist[i] = (i >= s0 && i < (uint64_t)s0 + cnt) ? 0u : GGA_INFINITY;
}

/* dynamicP_relax_coal: grid-stride over one vertex's edges. */
template <bool SSSP, bool ATOMIC>
__global__ void k_cdp_child(const GraphView g, uint32_t *dist, uint32_t *changed, uint32_t u) {
    const uint32_t nthreads = blockDim.x * gridDim.x;
    const uint32_t start = g.off[u], end = g.off[u + 1];
    const uint32_t du = dist[u];
    bool flag = false;
    for (uint32_t ii = start + threadIdx.x + blockDim.x * blockIdx.x; ii < end; ii += nthreads) {
        const uint32_t v = g.col[ii];
        const uint32_t alt = du + (SSSP ? g.wt[ii] : 1u);
        if (alt < dist[v]) {
            if (ATOMIC) atomicMin(dist + v, alt);
            else dist[v] = alt;
            flag = true;
        }
    }
    if (flag) *changed = 1;
}

/* Tail-launched: one CTA per heavy vertex. */
template <bool SSSP, bool ATOMIC>
__global__ void k_cdp_heavy(const GraphView g, uint32_t *dist, uint32_t *changed, const uint32_t *heavy) {
    const uint32_t u = heavy[blockIdx.x];
    const uint32_t start = g.off[u], end = g.off[u + 1];
    const uint32_t du = dist[u];
    bool flag = false;
    for (uint32_t ii = start + threadIdx.x; ii < end; ii += blockDim.x) {
        const uint32_t v = g.col[ii];
        const uint32_t alt = du + (SSSP ? g.wt[ii] : 1u);
        if (alt < dist[v]) {
            if (ATOMIC) atomicMin(dist + v, alt);
            else dist[v] = alt;
            flag = true;
        }
    }
    if (flag) *changed = 1;
}

template <bool SSSP, bool ATOMIC>
__global__ void __launch_bounds__(TOPO_BS) k_cdp_relax(const GraphView g, uint32_t *dist, uint32_t *changed,
                                                        uint32_t max_allowed, uint32_t *heavy, CdpState *cs,
                                                        uint32_t mode) {
    const uint32_t u = blockIdx.x * blockDim.x + threadIdx.x;
    bool any = false;
    if (u < g.n) {
        const uint32_t nout = g.off[u + 1] - g.off[u];
        bool inline_relax = true;
        if (nout > max_allowed && mode != 2) {
            if (mode == 1) {
                /* the reference's shape: one <<<1,32>>> child per heavy vertex */
                k_cdp_child<SSSP, ATOMIC><<<1, 32, 0, cudaStreamFireAndForget>>>(g, dist, changed, u);
                if (cudaGetLastError() == cudaSuccess) {
                    atomicAdd(&cs->children, 1u);
                    inline_relax = false;
                } else {
                    atomicAdd(&cs->fallbacks, 1u);
                }
            } else {
                heavy[atomicAdd(&cs->heavy_count, 1u)] = u;
                inline_relax = false;
            }
        }
        if (inline_relax) relax_vertex<SSSP, ATOMIC>(g, dist, u, any);
    }
    if (any) *changed = 1;
    if (mode != 0) return;

    /* last CTA to finish makes the single tail launch over the heavy list */
    __shared__ uint32_t s_last, s_fallback, s_hc;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(&cs->ticket, 1u) == gridDim.x - 1;
        s_fallback = 0;
        s_hc = 0;
        if (s_last) {
            __threadfence();
            const uint32_t hc = atomicAdd(&cs->heavy_count, 0u);
            s_hc = hc;
            if (hc) {
                k_cdp_heavy<SSSP, ATOMIC><<<hc, 256, 0, cudaStreamTailLaunch>>>(g, dist, changed, heavy);
                if (cudaGetLastError() == cudaSuccess) {
                    atomicAdd(&cs->children, 1u);
                } else {
                    atomicAdd(&cs->fallbacks, 1u);
                    s_fallback = 1;
                }
            }
        }
    }
    __syncthreads();
    if (s_fallback) {
        bool f = false;
        for (uint32_t i = threadIdx.x; i < s_hc; i += blockDim.x)
            relax_vertex<SSSP, ATOMIC>(g, dist, heavy[i], f);
        if (f) *changed = 1;
    }
}

} // namespace

struct TopoResult {
    uint32_t iterations, launches, cdp_children, cdp_fallbacks;
    float ktime, sktime;
};

/* printConv_rtime (convergence.h:100-159) on the device: over the original
 * vertices u, the current distance of u's parent against fin[u]; the count
 * of differences and the sum of (fs - fi)^2 taken in 32-bit unsigned
 * arithmetic, as the reference's foru expression computes it.  Every term is
 * below 2^32 and there are fewer than 2^32 of them, so the sum is exact in a
 * 64-bit integer whatever order the atomics land in; the host converts it to
 * double once, which equals the reference's sequential double sum wherever
 * that sum is exact (below 2^53). */
__global__ void k_conv_compare(const uint32_t *dist, const uint32_t *first, const uint32_t *fin, uint32_t n,
                               unsigned long long *cnt, unsigned long long *norm) {
    unsigned long long c = 0, sum = 0;
    for (uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; u < n; u += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t fi = dist[first ? first[u] : u], fs = fin[u];
        const uint32_t d = fs - fi;
        sum += (uint32_t)(d * d);
        c += fs != fi;
    }
    for (int o = 16; o > 0; o >>= 1) {
        c += __shfl_down_sync(0xffffffffu, c, o);
        sum += __shfl_down_sync(0xffffffffu, sum, o);
    }
    if ((threadIdx.x & 31) == 0 && c) {
        atomicAdd(cnt, c);
        atomicAdd(norm, sum);
    }
}

/* Runs a reference-semantics variant; distances land in `dist` (view ids). */
gga_status topo_run(const DevGraph *d, bool split, gga_variant variant, bool sssp, uint32_t src,
                    uint32_t max_allowed, uint32_t cdp_mode, uint32_t *dist, uint32_t *scratch_heavy,
                    uint32_t *dflag, uint32_t *hflag, int sms, cudaStream_t st, cudaEvent_t *ev,
                    TopoResult *res, ConvHook *conv) {
    const bool cdp = variant == GGA_VARIANT_CDP_ATOMIC || variant == GGA_VARIANT_CDP_PLAIN;
    const bool atomic = variant == GGA_VARIANT_TOPO_ATOMIC || variant == GGA_VARIANT_CDP_ATOMIC;
    const GraphView g = dev_graph_view(d, split && !cdp);
    const uint32_t factor = (g.n + TOPO_BS * sms - 1) / (TOPO_BS * sms);
    const uint32_t nblocks = sms * (factor ? factor : 1);
    const bool children = !cdp && split && d->level != 0 && d->npar != 0 && !atomic;
    const uint32_t dist_factor = children ? (d->npar + TOPO_BS * sms - 1) / (TOPO_BS * sms) : 0;
    CdpState *cs = (CdpState *)(dflag + 4);
    memset(res, 0, sizeof *res);
    k_topo_init<<<nblocks, TOPO_BS, 0, st>>>(dist, g.n, split && !cdp && d->level ? d->first : nullptr, g.cc, src);
    res->launches++;
    const uint32_t max_iter = g.n + 2; /* Bellman-Ford needs at most n passes */
    float t;
    for (;;) {
        if (res->iterations >= max_iter)
            return gga_fail(GGA_ERR_CUDA, "fixed point not reached after %u iterations", res->iterations);
        ++res->iterations;
        GGA_CK(cudaMemsetAsync(dflag, 0, 4 * sizeof(uint32_t) + sizeof(CdpState), st));
        if (children) {
            cudaEventRecord(ev[2], st);
            k_update_children<<<sms * dist_factor, TOPO_BS, 0, st>>>(dist, d->cidx, d->ccnt, d->npar);
            cudaEventRecord(ev[3], st);
            res->launches++;
        }
        cudaEventRecord(ev[0], st);
        if (cdp) {
            if (sssp) {
                if (atomic) k_cdp_relax<true, true><<<nblocks, TOPO_BS, 0, st>>>(g, dist, dflag, max_allowed, scratch_heavy, cs, cdp_mode);
                else k_cdp_relax<true, false><<<nblocks, TOPO_BS, 0, st>>>(g, dist, dflag, max_allowed, scratch_heavy, cs, cdp_mode);
            } else {
                if (atomic) k_cdp_relax<false, true><<<nblocks, TOPO_BS, 0, st>>>(g, dist, dflag, max_allowed, scratch_heavy, cs, cdp_mode);
                else k_cdp_relax<false, false><<<nblocks, TOPO_BS, 0, st>>>(g, dist, dflag, max_allowed, scratch_heavy, cs, cdp_mode);
            }
        } else if (sssp) {
            if (atomic) k_topo_relax<true, true><<<nblocks, TOPO_BS, 0, st>>>(g, dist, dflag);
            else k_topo_relax<true, false><<<nblocks, TOPO_BS, 0, st>>>(g, dist, dflag);
        } else {
            if (atomic) k_topo_relax<false, true><<<nblocks, TOPO_BS, 0, st>>>(g, dist, dflag);
            else k_topo_relax<false, false><<<nblocks, TOPO_BS, 0, st>>>(g, dist, dflag);
        }
        cudaEventRecord(ev[1], st);
        res->launches++;
        GGA_CK(cudaGetLastError());
        if (conv) {
            GGA_CK(cudaMemsetAsync(conv->cnt, 0, sizeof(unsigned long long), st));
            GGA_CK(cudaMemsetAsync(conv->norm, 0, sizeof(unsigned long long), st));
            const uint32_t cb = std::min<uint32_t>((d->n + 255) / 256, (uint32_t)sms * 8);
            k_conv_compare<<<cb ? cb : 1, 256, 0, st>>>(dist, split && !cdp ? d->first : nullptr, conv->fin, d->n,
                                                        conv->cnt, conv->norm);
            GGA_CK(cudaGetLastError());
            res->launches++;
        }
        GGA_CK(cudaMemcpyAsync(hflag, dflag, 4 * sizeof(uint32_t) + sizeof(CdpState), cudaMemcpyDeviceToHost, st));
        gga_status w = dev_wait(st, 60.0);
        if (w) return w;
        if (conv) {
            unsigned long long hc = 0, hn = 0;
            GGA_CK(cudaMemcpy(&hc, conv->cnt, sizeof hc, cudaMemcpyDeviceToHost));
            GGA_CK(cudaMemcpy(&hn, conv->norm, sizeof hn, cudaMemcpyDeviceToHost));
            if (conv->n < conv->cap) {
                gga_conv_record &r = conv->rec[conv->n];
                r.iteration = res->iterations;
                r.pad = 0;
                r.diff_count = hc;
                r.norm2 = sqrt((double)hn);
            }
            conv->n++;
        }
        cudaEventElapsedTime(&t, ev[0], ev[1]);
        res->ktime += t;
        if (children) {
            cudaEventElapsedTime(&t, ev[2], ev[3]);
            res->sktime += t;
        }
        const CdpState *hc = (const CdpState *)(hflag + 4);
        res->cdp_children += hc->children;
        res->cdp_fallbacks += hc->fallbacks;
        if (!hflag[0]) break;
    }
    return GGA_OK;
}
