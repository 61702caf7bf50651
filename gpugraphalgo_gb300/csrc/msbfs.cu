/*
 * Bit-packed multi-source BFS: up to 64 BFS traversals of one graph in one
 * persistent cooperative launch.
 *
 * Each vertex holds two 64-bit masks, one bit per source: `seen` (sources that
 * have reached it) and `nxt` (sources reaching it in the level being built).
 * A level is two grid-wide phases separated by grid barriers:
 *
 *   settle(L): every candidate vertex v (nxt[v] became non-zero during the
 *     previous expand) takes its new bits f = nxt[v] & ~seen[v], records level
 *     L for each set bit (vertex-major, the vertex's levels in one short span,
 *     written by the whole warp; one tiled transpose gives the source-major
 *     output), folds f into seen[v] and, if it has out-edges, is appended to
 *     the expansion list with its frontier mask f and an exclusive edge offset
 *     (a block scan and one 64-bit atomicAdd of (entries << 32 | edges) per
 *     block, so entry index and edge offset grow together).
 *   expand(L): the expansion list's edges are cut into fixed units of
 *     MB_UNIT edges; CTAs take units by ticket, load the unit's entries into
 *     shared memory and give one edge to each thread: for the edge (u, v) the
 *     new sources are f_u & ~seen[v]; they are OR-ed into nxt[v] and the thread
 *     whose OR found nxt[v] == 0 appends v to the next candidate list (staged
 *     in shared memory, published at block-uniform checkpoints).
 *
 * One edge read serves every source whose frontier contains u, so a vertex
 * reached by all 64 sources in the same level is expanded once instead of 64
 * times.
 *
 * On symmetric graphs a level whose frontier edges exceed m / 4 expands
 * bottom-up instead (the multi-source form of Beamer's rule; measured on
 * GB300 with 64 sources, R-MAT 22: 7.98 -> 4.92 ms, R-MAT 20: 1.65 -> 1.52
 * ms, while m / 16 was several times slower, since a vertex stops only once
 * it has every source's bit): every vertex
 * not yet seen by all sources ORs its neighbours' `seen` masks until it has
 * every source, and the bits it lacked are exactly the sources reaching it
 * at level L + 1 (a neighbour seen by source s at level <= L means level
 * L + 1, as the vertex was not reached by level L).  `seen` is only written
 * in settle, so the masks read are those of level L.  Levels equal those of 64 single-source BFS runs (the reference's
 * BFS levels, K/graph.h:115-149 serial and K/cudaKernels.h:285-344 device),
 * on the unsplit graph: splitting a vertex does not change any level.
 */
#include <algorithm>
#include <string.h>
#include <vector>

#include "batch.cuh"

namespace {

constexpr uint32_t MB_BS = 256;
constexpr uint32_t MB_ITERS = 4; /* 1024-edge units (measured: 2048 0.53 ms, 1024 0.50, 512 0.52 for 64 sources on R-MAT 20) */
constexpr uint32_t MB_UNIT = MB_BS * MB_ITERS;
constexpr uint32_t MB_BATCH = 4;
constexpr uint32_t MB_SCAP = MB_BS * (MB_BATCH + 1);
constexpr unsigned FULL = 0xffffffffu;
constexpr uint32_t NONE = 0xffffffffu;

struct MsCtl {
    GridBarrier bar;
    uint32_t err;
    uint32_t levels;
    uint32_t cand[2];               /* candidate counts, by level parity */
    unsigned long long xctr[2];     /* (entries << 32) | edges of the expansion list, by parity */
    uint32_t work[2];               /* unit tickets, by parity */
    unsigned long long edges_relaxed;
};

struct MsArgs {
    const uint32_t *off, *col;
    uint32_t n, m;
    unsigned long long *seen, *nxt; /* n each */
    uint32_t *cand;                 /* n */
    uint32_t *xv, *xo, *xb;         /* n each: vertex, edge offset, first edge */
    unsigned long long *xf;         /* n: frontier mask of the entry */
    uint32_t *uf;                   /* ucap: first entry of each unit */
    uint32_t *dist;                 /* n * ns, vertex-major: levels of vertex v at dist[v * ns ...] */
    uint32_t ns;                    /* sources (row stride of dist) */
    MsCtl *ctl;
    uint32_t ucap, nblocks, max_levels;
    unsigned long long timeout_ns;
    uint32_t bu;              /* symmetric graph: bottom-up levels allowed */
    unsigned long long all;   /* the mask of every source */
};

struct MsCtrl {
    uint32_t nn, base, unit, i0, cnt, ncand, nitems, total;
    unsigned long long xbase;  /* settle: the block's slice of the expansion list */
    unsigned long long ws64[32];
};

__device__ __forceinline__ void ms_err(MsCtl *c, uint32_t code) { atomicCAS(&c->err, GGA_DEV_OK, code); }

__device__ __forceinline__ void ms_checkpoint(const MsArgs &a, MsCtrl &C, uint32_t *sc, uint32_t np,
                                              uint32_t limit) {
    __syncthreads();
    const uint32_t nn = C.nn;
    __syncthreads();
    if (nn < limit || nn == 0) return;
    if (threadIdx.x == 0) C.base = atomicAdd(&a.ctl->cand[np], nn);
    __syncthreads();
    const uint32_t base = C.base;
    for (uint32_t j = threadIdx.x; j < nn; j += MB_BS) {
        if (base + j < a.n) a.cand[base + j] = sc[j];
        else ms_err(a.ctl, GGA_DEV_OVERFLOW);
    }
    __syncthreads();
    if (threadIdx.x == 0) C.nn = 0;
    __syncthreads();
}

/* One bottom-up expansion of level L: a warp takes 2 x 32 consecutive
 * vertices per step (lane i vertices 64w + i and 64w + 32 + i), each lane
 * ORs its vertices' neighbours' seen masks, 4 per vertex per step, until the
 * vertex has every source; vertices that gained bits get them in nxt (this
 * lane is their only writer this level) and join the next candidate list
 * through one warp-aggregated atomicAdd.  A vertex with more than MS_HEAVY
 * neighbours is scanned by the whole warp instead, 32 x NB neighbours a step
 * with the masks OR-reduced across the warp, so one lane's long row does not
 * hold its warp, block and the level's grid barrier (on R-MAT 20 the blocks
 * waited 44% of the kernel at that barrier).  Either scan stops once the
 * vertex has every source, and then acc & ~seen is the same whichever
 * neighbours were read.  Trip counts are warp-uniform; the per-lane scans
 * reconverge before the ballots. */
constexpr uint32_t MS_HEAVY = 64;

__device__ __forceinline__ unsigned long long warp_or64(unsigned long long x) {
    for (int d = 16; d > 0; d >>= 1) x |= __shfl_down_sync(FULL, x, d);
    return __shfl_sync(FULL, x, 0);
}

__device__ __forceinline__ void ms_bottom_up(const MsArgs &a, uint32_t np, unsigned long long &relaxed) {
    constexpr uint32_t NV = 2, NB = 4;
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t gw = ((uint64_t)blockIdx.x * MB_BS + threadIdx.x) >> 5, nw = ((uint64_t)gridDim.x * MB_BS) >> 5;
    const uint64_t steps = ((uint64_t)a.n + 32 * NV - 1) / (32 * NV);
    for (uint64_t w = gw; w < steps; w += nw) {
        uint32_t v[NV], cur[NV], e1[NV];
        unsigned long long sv[NV], acc[NV];
        bool open[NV], heavy[NV];
#pragma unroll
        for (uint32_t k = 0; k < NV; ++k) {
            const uint64_t vk = w * 32 * NV + 32 * k + lane;
            v[k] = (uint32_t)vk;
            sv[k] = vk < a.n ? __ldcg(a.seen + vk) : a.all;
            acc[k] = 0;
            open[k] = sv[k] != a.all;
            cur[k] = e1[k] = 0;
            if (open[k]) {
                cur[k] = __ldg(a.off + vk);
                e1[k] = __ldg(a.off + vk + 1);
            }
            heavy[k] = open[k] && e1[k] - cur[k] > MS_HEAVY;
        }
        for (;;) {
            bool act[NV], any = false;
#pragma unroll
            for (uint32_t k = 0; k < NV; ++k) {
                act[k] = open[k] && !heavy[k] && cur[k] < e1[k] && (acc[k] | sv[k]) != a.all;
                any |= act[k];
            }
            if (!any) break;
            uint32_t u[NV][NB];
#pragma unroll
            for (uint32_t k = 0; k < NV; ++k)
#pragma unroll
                for (uint32_t q = 0; q < NB; ++q) u[k][q] = act[k] && cur[k] + q < e1[k] ? __ldg(a.col + cur[k] + q) : NONE;
#pragma unroll
            for (uint32_t k = 0; k < NV; ++k) {
#pragma unroll
                for (uint32_t q = 0; q < NB; ++q)
                    if (u[k][q] != NONE) acc[k] |= __ldcg(a.seen + u[k][q]);
                if (act[k]) {
                    relaxed += min(NB, e1[k] - cur[k]);
                    cur[k] += NB;
                }
            }
        }
        /* the heavy rows, one at a time by the whole warp */
#pragma unroll
        for (uint32_t k = 0; k < NV; ++k) {
            for (unsigned hm = __ballot_sync(FULL, heavy[k]); hm; hm &= hm - 1) {
                const int owner = __ffs(hm) - 1;
                const uint32_t hb = __shfl_sync(FULL, cur[k], owner), he = __shfl_sync(FULL, e1[k], owner);
                const unsigned long long hs = __shfl_sync(FULL, sv[k], owner);
                unsigned long long hacc = 0;
                uint64_t hend = hb;
                for (uint64_t base = hb; base < he; base += 32 * NB) { /* warp-uniform; 64-bit: no wrap near 2^32 edges */
                    uint32_t u[NB];
#pragma unroll
                    for (uint32_t q = 0; q < NB; ++q) {
                        const uint64_t j = base + q * 32 + lane;
                        u[q] = j < he ? __ldg(a.col + j) : NONE;
                    }
#pragma unroll
                    for (uint32_t q = 0; q < NB; ++q)
                        if (u[q] != NONE) hacc |= __ldcg(a.seen + u[q]);
                    hacc = warp_or64(hacc);
                    hend = min(base + 32 * NB, (uint64_t)he);
                    if ((hacc | hs) == a.all) break;
                }
                if (lane == (uint32_t)owner) {
                    acc[k] = hacc;
                    relaxed += hend - hb;
                }
            }
        }
        uint32_t fm[NV], cnt = 0;
#pragma unroll
        for (uint32_t k = 0; k < NV; ++k) {
            const bool found = open[k] && (acc[k] & ~sv[k]) != 0;
            if (found) a.nxt[v[k]] = acc[k] & ~sv[k];
            fm[k] = __ballot_sync(FULL, found);
            cnt += (uint32_t)__popc(fm[k]);
        }
        if (cnt == 0) continue; /* warp-uniform */
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(&a.ctl->cand[np], cnt);
        base = __shfl_sync(FULL, base, 0);
#pragma unroll
        for (uint32_t k = 0, before = 0; k < NV; before += (uint32_t)__popc(fm[k]), ++k)
            if ((fm[k] >> lane) & 1u) {
                const uint32_t idx = base + before + (uint32_t)__popc(fm[k] & lanemask_lt());
                if (idx < a.n) a.cand[idx] = v[k];
                else ms_err(a.ctl, GGA_DEV_OVERFLOW);
            }
    }
}

__global__ void __launch_bounds__(MB_BS, 4) k_msbfs(MsArgs a) {
    extern __shared__ unsigned long long dyn64[];
    __shared__ MsCtrl C;
    unsigned long long *t_f = dyn64;
    uint32_t *t_o = (uint32_t *)(t_f + MB_UNIT + 1);
    uint32_t *t_b = t_o + MB_UNIT + 1;
    uint32_t *sc = t_b + MB_UNIT + 1;
    MsCtl *ctl = a.ctl;
    const uint32_t tid = threadIdx.x, lane = tid & 31;
    const uint64_t gthreads = (uint64_t)gridDim.x * MB_BS;
    uint32_t gen = 0;
    unsigned long long relaxed = 0;
    if (tid == 0) C.nn = 0;
    __syncthreads();
    uint32_t L = 0;
    for (;; ++L) {
        const uint32_t p = L & 1, np = p ^ 1;
        /* ---------------- settle(L) */
        if (tid == 0) C.ncand = min(ld_relaxed_u32(&ctl->cand[p]), a.n);
        __syncthreads();
        const uint32_t ncand = C.ncand;
        __syncthreads();
        if (ncand == 0) break; /* same decision in every block */
        if (L >= a.max_levels) {
            if (blockIdx.x == 0 && tid == 0) ms_err(ctl, GGA_DEV_ROUND_LIMIT);
            break;
        }
        if (blockIdx.x == 0 && tid == 0) ctl->work[p] = 0;
        /* block-uniform trip count: every thread of a block runs each iteration */
        for (uint64_t base = (uint64_t)blockIdx.x * MB_BS; base < ncand; base += gthreads) {
            const uint64_t i = base + tid;
            uint32_t v = 0, b = 0, d = 0;
            unsigned long long f = 0;
            if (i < ncand) {
                v = __ldcg(a.cand + i);
                const unsigned long long s0 = __ldcg(a.seen + v);
                f = __ldcg(a.nxt + v) & ~s0;
                a.nxt[v] = 0;
                a.seen[v] = s0 | f;
                b = __ldg(a.off + v);
                d = f ? __ldg(a.off + v + 1) - b : 0u;
            }
            /* the new levels, one vertex at a time by the whole warp: lane j
             * writes sources j and j + 32 of the vertex's span (two coalesced
             * masked stores), not one lane looping over its vertex's bits */
            for (unsigned lm = __ballot_sync(FULL, f != 0); lm; lm &= lm - 1) {
                const int src = __ffs(lm) - 1;
                const uint32_t vv = __shfl_sync(FULL, v, src);
                const unsigned long long ff = __shfl_sync(FULL, f, src);
                uint32_t *lv = a.dist + (size_t)vv * a.ns;
                if (lane < a.ns && ((ff >> lane) & 1ull)) lv[lane] = L;
                if (lane + 32 < a.ns && ((ff >> (lane + 32)) & 1ull)) lv[lane + 32] = L;
            }
            /* one list allocation per block: a block scan of (entries << 32 | edges)
             * and one atomicAdd, not one per warp on the same counter */
            unsigned long long tot;
            const unsigned long long run = block_exclusive_scan64(d > 0 ? (1ull << 32) | d : 0ull, C.ws64, &tot);
            if (tid == 0) C.xbase = tot ? atomicAdd(&ctl->xctr[p], tot) : 0ull;
            __syncthreads(); /* read before the next iteration's scan lets thread 0 write it again */
            const unsigned long long old = C.xbase;
            if (d > 0) {
                const uint32_t idx = (uint32_t)(old >> 32) + (uint32_t)(run >> 32);
                const uint32_t o = (uint32_t)old + (uint32_t)run;
                if (idx < a.n) {
                    a.xv[idx] = v;
                    a.xo[idx] = o;
                    a.xb[idx] = b;
                    a.xf[idx] = f;
                    for (uint64_t k = ((uint64_t)o + MB_UNIT - 1) / MB_UNIT; k * MB_UNIT < (uint64_t)o + d; ++k) {
                        if (k < a.ucap) a.uf[k] = idx;
                        else ms_err(ctl, GGA_DEV_OVERFLOW_UNITS);
                    }
                } else {
                    ms_err(ctl, GGA_DEV_OVERFLOW);
                }
            }
        }
        if (!grid_barrier(&ctl->bar, &ctl->err, a.nblocks, gen, a.timeout_ns)) break;

        /* ---------------- expand(L) */
        if (tid == 0) {
            const unsigned long long qc = ld_relaxed_u64(&ctl->xctr[p]);
            const uint32_t ni = min((uint32_t)(qc >> 32), a.n);
            C.nitems = ni;
            C.total = ni ? (uint32_t)qc : 0u;
        }
        __syncthreads();
        const uint32_t nitems = C.nitems, total = C.total;
        const uint32_t units = min((uint32_t)(((uint64_t)total + MB_UNIT - 1) / MB_UNIT), a.ucap);
        __syncthreads();
        if (blockIdx.x == 0 && tid == 0) {
            ctl->cand[p] = 0;  /* read at the start of settle(L), appended in expand(L+1) */
            ctl->xctr[np] = 0; /* read in expand(L-1), appended in settle(L+1) */
        }
        /* direction of this level, from counters every block read alike */
        if (a.bu && (uint64_t)total * 4 > a.m) {
            ms_bottom_up(a, np, relaxed);
            if (!grid_barrier(&ctl->bar, &ctl->err, a.nblocks, gen, a.timeout_ns)) break;
            continue;
        }
        for (;;) {
            if (tid == 0) {
                const uint32_t k = atomicAdd(&ctl->work[p], 1u);
                C.unit = k;
                if (k < units) {
                    const uint32_t i0 = min(__ldcg(a.uf + k), nitems - 1);
                    const uint32_t i1 = k + 1 < units ? min(__ldcg(a.uf + k + 1), nitems - 1) : nitems - 1;
                    C.i0 = i0;
                    C.cnt = i1 >= i0 ? min(i1 - i0 + 1, MB_UNIT + 1) : 1u;
                }
            }
            __syncthreads();
            const uint32_t k = C.unit;
            if (k >= units) break;
            const uint32_t i0 = C.i0, cnt = C.cnt;
            const uint32_t ebase = k * MB_UNIT, eend = min(ebase + MB_UNIT, total);
            for (uint32_t j = tid; j < cnt; j += MB_BS) {
                t_o[j] = __ldcg(a.xo + i0 + j);
                t_b[j] = __ldcg(a.xb + i0 + j);
                t_f[j] = __ldcg(a.xf + i0 + j);
            }
            __syncthreads();
            for (uint32_t it0 = 0; it0 < MB_ITERS; it0 += MB_BATCH) {
                if (it0) ms_checkpoint(a, C, sc, np, MB_BS);
                /* MB_BATCH edges per thread: table lookups and edge loads,
                 * then the seen/nxt probes, then the updates */
                uint32_t v[MB_BATCH];
                unsigned long long f[MB_BATCH], sn[MB_BATCH], nx[MB_BATCH];
#pragma unroll
                for (uint32_t s = 0; s < MB_BATCH; ++s) {
                    const uint32_t e = ebase + (it0 + s) * MB_BS + tid;
                    f[s] = 0;
                    v[s] = 0;
                    if (e >= eend) continue;
                    uint32_t lo = 0, hi = cnt;
                    while (hi - lo > 1) {
                        const uint32_t mid = (lo + hi) >> 1;
                        if (t_o[mid] <= e) lo = mid; else hi = mid;
                    }
                    const uint32_t ei = t_b[lo] + (e - t_o[lo]);
                    if (ei >= a.m) {
                        ms_err(ctl, GGA_DEV_BAD_EDGE);
                        continue;
                    }
                    v[s] = __ldg(a.col + ei);
                    f[s] = t_f[lo];
                }
#pragma unroll
                for (uint32_t s = 0; s < MB_BATCH; ++s) {
                    sn[s] = f[s] ? __ldcg(a.seen + v[s]) : 0ull;
                    nx[s] = f[s] ? __ldcg(a.nxt + v[s]) : 0ull;
                }
#pragma unroll
                for (uint32_t s = 0; s < MB_BATCH; ++s) {
                    const unsigned long long nb = f[s] & ~sn[s];
                    if (nb && (nb & ~nx[s]) && atomicOr(a.nxt + v[s], nb) == 0) {
                        const uint32_t slot = atomicAdd(&C.nn, 1u);
                        if (slot < MB_SCAP) sc[slot] = v[s];
                        else ms_err(ctl, GGA_DEV_OVERFLOW);
                    }
                }
            }
            if (tid == 0) relaxed += eend - ebase;
            ms_checkpoint(a, C, sc, np, MB_BS);
        }
        ms_checkpoint(a, C, sc, np, 1);
        if (!grid_barrier(&ctl->bar, &ctl->err, a.nblocks, gen, a.timeout_ns)) break;
    }
    /* every thread of every block leaves the level loop at the same point;
     * top-down counts sit in thread 0, bottom-up counts in every lane */
    for (int d = 16; d > 0; d >>= 1) relaxed += __shfl_down_sync(FULL, relaxed, d);
    if (lane == 0 && relaxed) atomicAdd(&ctl->edges_relaxed, relaxed);
    if (blockIdx.x == 0 && tid == 0) ctl->levels = L;
}

/* Source-major output: out[s * n + v] = lvl[v * ns + s] where source s
 * reached v (bit s of seen[v]) and MYINFINITY elsewhere, through a shared
 * tile of 32 vertices x ns sources (coalesced reads and writes).  Settle
 * writes each reached (vertex, source) level exactly once, so the level array
 * needs no fill before the launch: the entries of unreached pairs are never
 * read. */
__global__ void k_ms_transpose(const uint32_t *lvl, const unsigned long long *seen, uint32_t n, uint32_t ns,
                               uint32_t *out) {
    __shared__ uint32_t tile[32][65];
    const uint32_t tx = threadIdx.x & 31, ty = threadIdx.x >> 5; /* 32 x 8 threads */
    for (uint64_t v0 = (uint64_t)blockIdx.x * 32; v0 < n; v0 += (uint64_t)gridDim.x * 32) {
        const uint32_t nv = (uint32_t)min((uint64_t)32, n - v0);
        for (uint32_t k = threadIdx.x; k < nv * ns; k += blockDim.x) {
            const uint32_t vv = k / ns, s = k % ns;
            tile[vv][s] = (seen[v0 + vv] >> s) & 1ull ? lvl[v0 * ns + k] : GGA_INFINITY;
        }
        __syncthreads();
        for (uint32_t s = ty; s < ns; s += 8)
            if (tx < nv) out[(size_t)s * n + v0 + tx] = tile[tx][s];
        __syncthreads();
    }
}

/* Level-0 candidates: each distinct source vertex once, carrying the bits of
 * every source index that names it. */
__global__ void k_ms_sources(MsArgs a, const uint32_t *srcs, uint32_t nsrc) {
    const uint32_t s = threadIdx.x;
    if (s >= nsrc) return;
    const uint32_t v = srcs[s];
    if (atomicOr(a.nxt + v, 1ull << s) == 0) {
        const uint32_t idx = atomicAdd(&a.ctl->cand[0], 1u);
        a.cand[idx] = v;
    }
}

/* vertices_reached / edges_reached summed over the sources: popcount(seen). */
__global__ void k_ms_reached(const unsigned long long *seen, const uint32_t *off, uint32_t n,
                             unsigned long long *acc) {
    unsigned long long vr = 0, er = 0;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const uint32_t c = (uint32_t)__popcll(seen[v]);
        vr += c;
        er += (unsigned long long)c * (off[v + 1] - off[v]);
    }
    for (int d = 16; d > 0; d >>= 1) {
        vr += __shfl_down_sync(FULL, vr, d);
        er += __shfl_down_sync(FULL, er, d);
    }
    if ((threadIdx.x & 31) == 0 && (vr || er)) {
        atomicAdd(acc, vr);
        atomicAdd(acc + 1, er);
    }
}

size_t ms_smem() { return (size_t)(MB_UNIT + 1) * 16 + (size_t)MB_SCAP * 4; }

} // namespace

struct MsbfsScratch {
    int device = -1;
    uint32_t ncap = 0, ucap = 0;
    size_t dcap = 0, ocap = 0;
    uint32_t *out = nullptr; /* source-major levels for host output */
    unsigned long long *seen = nullptr, *nxt = nullptr, *xf = nullptr;
    uint32_t *cand = nullptr, *xv = nullptr, *xo = nullptr, *xb = nullptr, *uf = nullptr;
    uint32_t *dist = nullptr, *srcs = nullptr;
    MsCtl *ctl = nullptr, *hctl = nullptr;
    int nblocks = 0;
};

void msbfs_scratch_free(MsbfsScratch *m) {
    if (!m) return;
    cudaFree(m->seen);
    cudaFree(m->nxt);
    cudaFree(m->xf);
    cudaFree(m->cand);
    cudaFree(m->xv);
    cudaFree(m->xo);
    cudaFree(m->xb);
    cudaFree(m->uf);
    cudaFree(m->dist);
    cudaFree(m->out);
    cudaFree(m->srcs);
    cudaFree(m->ctl);
    cudaFreeHost(m->hctl);
    delete m;
}

static gga_status ms_reserve(MsbfsScratch *m, uint32_t n, uint32_t edges, size_t dist_words, size_t out_words) {
    cudaError_t e = cudaSuccess;
    if (m->ncap < n) {
        cudaFree(m->seen); cudaFree(m->nxt); cudaFree(m->xf);
        cudaFree(m->cand); cudaFree(m->xv); cudaFree(m->xo); cudaFree(m->xb);
        m->seen = m->nxt = m->xf = nullptr;
        m->cand = m->xv = m->xo = m->xb = nullptr;
        m->ncap = 0;
        e = cudaMalloc((void **)&m->seen, (size_t)n * 8);
        if (e == cudaSuccess) e = cudaMalloc((void **)&m->nxt, (size_t)n * 8);
        if (e == cudaSuccess) e = cudaMalloc((void **)&m->xf, (size_t)n * 8);
        if (e == cudaSuccess) e = cudaMalloc((void **)&m->cand, (size_t)n * 4);
        if (e == cudaSuccess) e = cudaMalloc((void **)&m->xv, (size_t)n * 4);
        if (e == cudaSuccess) e = cudaMalloc((void **)&m->xo, (size_t)n * 4);
        if (e == cudaSuccess) e = cudaMalloc((void **)&m->xb, (size_t)n * 4);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return gga_fail(GGA_ERR_CUDA, "msbfs scratch (%u vertices): %s", n, cudaGetErrorString(e));
        }
        m->ncap = n;
    }
    const uint32_t ucap = edges / MB_UNIT + 4;
    if (m->ucap < ucap) {
        cudaFree(m->uf);
        m->uf = nullptr;
        m->ucap = 0;
        GGA_CK(cudaMalloc((void **)&m->uf, (size_t)ucap * 4));
        m->ucap = ucap;
    }
    if (m->dcap < dist_words) {
        cudaFree(m->dist);
        m->dist = nullptr;
        m->dcap = 0;
        e = cudaMalloc((void **)&m->dist, dist_words * 4);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return gga_fail(GGA_ERR_CUDA, "msbfs levels (%zu MiB): %s", (dist_words * 4) >> 20,
                            cudaGetErrorString(e));
        }
        m->dcap = dist_words;
    }
    if (m->ocap < out_words) {
        cudaFree(m->out);
        m->out = nullptr;
        m->ocap = 0;
        e = cudaMalloc((void **)&m->out, out_words * 4);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return gga_fail(GGA_ERR_CUDA, "msbfs output (%zu MiB): %s", (out_words * 4) >> 20, cudaGetErrorString(e));
        }
        m->ocap = out_words;
    }
    if (!m->ctl) {
        GGA_CK(cudaMalloc((void **)&m->ctl, sizeof(MsCtl)));
        GGA_CK(cudaMallocHost((void **)&m->hctl, sizeof(MsCtl)));
        GGA_CK(cudaMalloc((void **)&m->srcs, 64 * sizeof(uint32_t)));
    }
    if (!m->nblocks) {
        const size_t smem = ms_smem();
        GGA_CK(cudaFuncSetAttribute(k_msbfs, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int occ = 0, sms = 0;
        GGA_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_msbfs, MB_BS, smem));
        GGA_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, m->device));
        if (occ <= 0) return gga_fail(GGA_ERR_CUDA, "msbfs kernel: zero occupancy");
        m->nblocks = occ * sms;
    }
    return GGA_OK;
}

gga_status gga_msbfs(gga_ctx *c, gga_graph *g, uint32_t nsrc, const uint32_t *srcs, uint32_t *dist_out,
                     gga_stats *stats) {
    const double t0 = gga_now_ms();
    if (!c || !g || !srcs || !dist_out) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    if (nsrc == 0 || nsrc > 64) return gga_fail(GGA_ERR_INVALID_ARG, "nsrc %u (1..64)", nsrc);
    for (uint32_t i = 0; i < nsrc; ++i)
        if (srcs[i] >= g->n) return gga_fail(GGA_ERR_INVALID_ARG, "source %u >= %u vertices", srcs[i], g->n);
    std::lock_guard<std::mutex> lk(c->mu);
    gga_status s;
    if ((s = ctx_activate(c))) return s;
    if ((s = dev_graph_ensure(g, c->device, c->st))) return s;
    const DevGraph *d = dev_graph_of(g);
    /* bottom-up levels need every edge's reverse (checked once per graph) */
    if (d->symmetric == 0 && (s = dev_graph_check_symmetric(g, c->dflag + 40, c->hflag + 40, c->st))) return s;
    BatchScratch *b = ctx_batch(c);
    if (!b) return gga_fail(GGA_ERR_NO_MEMORY, "batch scratch");
    if (!b->ms) {
        b->ms = new (std::nothrow) MsbfsScratch();
        if (!b->ms) return gga_fail(GGA_ERR_NO_MEMORY, "msbfs scratch");
        b->ms->device = c->device;
    }
    MsbfsScratch *m = b->ms;
    const bool dev_out = ptr_is_device(dist_out);
    const size_t words = (size_t)nsrc * d->n;
    if ((s = ms_reserve(m, d->n, d->m, words, dev_out ? 0 : words))) return s;
    uint32_t *levels = m->dist;                      /* vertex-major */
    uint32_t *out = dev_out ? dist_out : m->out;     /* source-major */

    MsArgs a;
    memset(&a, 0, sizeof a);
    a.off = d->off;
    a.col = d->col;
    a.n = d->n;
    a.m = d->m;
    a.seen = m->seen;
    a.nxt = m->nxt;
    a.cand = m->cand;
    a.xv = m->xv;
    a.xo = m->xo;
    a.xb = m->xb;
    a.xf = m->xf;
    a.uf = m->uf;
    a.dist = levels;
    a.ns = nsrc;
    a.ctl = m->ctl;
    a.ucap = m->ucap;
    a.nblocks = (uint32_t)m->nblocks;
    a.max_levels = d->n + 1;
    a.timeout_ns = 4000000000ull;
    a.bu = d->symmetric > 0 ? 1u : 0u;
    a.all = nsrc == 64 ? ~0ull : (1ull << nsrc) - 1;

    GGA_CK(cudaMemsetAsync(m->ctl, 0, sizeof(MsCtl), c->st));
    GGA_CK(cudaMemsetAsync(m->seen, 0, (size_t)d->n * 8, c->st));
    GGA_CK(cudaMemsetAsync(m->nxt, 0, (size_t)d->n * 8, c->st));
    GGA_CK(cudaMemcpyAsync(m->srcs, srcs, nsrc * sizeof(uint32_t), cudaMemcpyHostToDevice, c->st));
    k_ms_sources<<<1, 64, 0, c->st>>>(a, m->srcs, nsrc);
    GGA_CK(cudaGetLastError());
    GGA_CK(cudaEventRecord(c->ev[0], c->st));
    void *args[] = {&a};
    GGA_CK(cudaLaunchCooperativeKernel((const void *)k_msbfs, dim3(a.nblocks), dim3(MB_BS), args, ms_smem(), c->st));
    GGA_CK(cudaEventRecord(c->ev[1], c->st));
    GGA_CK(cudaMemcpyAsync(m->hctl, m->ctl, sizeof(MsCtl), cudaMemcpyDeviceToHost, c->st));
    k_ms_transpose<<<ctx_grid(c, ((uint64_t)d->n + 31) / 32 * 256, 256), 256, 0, c->st>>>(levels, m->seen, d->n, nsrc,
                                                                                       out);
    GGA_CK(cudaGetLastError());
    uint32_t launches = 3; /* the sources, the traversal, the transpose */
    if (!dev_out) GGA_CK(cudaMemcpyAsync(dist_out, out, words * 4, cudaMemcpyDeviceToHost, c->st));
    if (stats) {
        unsigned long long *acc = (unsigned long long *)(c->dflag + 32);
        GGA_CK(cudaMemsetAsync(acc, 0, 2 * sizeof(unsigned long long), c->st));
        k_ms_reached<<<ctx_grid(c, d->n, 256), 256, 0, c->st>>>(m->seen, d->off, d->n, acc);
        GGA_CK(cudaGetLastError());
        GGA_CK(cudaMemcpyAsync(c->hflag + 32, acc, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->st));
        launches++;
    }
    if ((s = dev_wait(c->st, 60.0))) return s;
    const MsCtl &h = *m->hctl;
    switch (h.err) {
    case GGA_DEV_OK: break;
    case GGA_DEV_TIMEOUT: return gga_fail(GGA_ERR_TIMEOUT, "msbfs grid barrier timed out");
    case GGA_DEV_OVERFLOW: return gga_fail(GGA_ERR_CUDA, "msbfs list overflow (internal error)");
    case GGA_DEV_OVERFLOW_UNITS: return gga_fail(GGA_ERR_CUDA, "msbfs unit table overflow (internal error)");
    case GGA_DEV_BAD_EDGE: return gga_fail(GGA_ERR_CUDA, "msbfs edge index out of range (internal error)");
    case GGA_DEV_ROUND_LIMIT: return gga_fail(GGA_ERR_CUDA, "msbfs level limit reached (internal error)");
    default: return gga_fail(GGA_ERR_CUDA, "msbfs kernel error %u", h.err);
    }
    if (stats) {
        gga_stats st;
        memset(&st, 0, sizeof st);
        float ms = 0;
        GGA_CK(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
        const unsigned long long *hr = (const unsigned long long *)(c->hflag + 32);
        st.iterations = h.levels;
        st.kernel_launches = launches;
        st.edges_relaxed = h.edges_relaxed;
        st.vertices_reached = hr[0];
        st.edges_reached = hr[1];
        st.kernel_ms = ms;
        st.total_ms = gga_now_ms() - t0;
        *stats = st;
    }
    return GGA_OK;
}
