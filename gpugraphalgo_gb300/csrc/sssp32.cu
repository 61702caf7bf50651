/*
 * 32-source SSSP in one persistent launch, one warp lane per source.
 *
 * Distances are vertex-major: D[v * 32 + s] for source s, so the 32
 * distances of a vertex are one 128-byte line and a warp reads or updates
 * them in one coalesced access.  A queue entry is a vertex u whose distance
 * improved for some sources in the previous round, with the mask of those
 * sources; for each edge (u, v, w) of a warp step (SU_EB of them in flight)
 * lane s relaxes D[v][s] from D[u][s] + w when bit s of u's mask is set (a
 * min on uint32, as M_my_drelax's atomicMin is, cudaKernels.h:323-330, sent
 * as a fire-and-forget red.min once it beats the probed D[v][s]).  The
 * improved lanes' bits are OR-ed into v's mask for the next round, one edge's
 * OR per lane; the lane whose OR found the mask empty enqueues v.  So one
 * read of an edge serves every source whose
 * frontier holds its tail, where 32 single-source runs read it up to 32
 * times.  Per source this is the improved-vertex frontier (Bellman-Ford
 * order), which converges to the unique shortest distances: every answer
 * equals the single-source one.
 *
 * Queue entries carry exclusive edge offsets and the edge list is cut into
 * units of SU_UNIT edges exactly as in the frontier engine (frontier.cu);
 * pushes are staged per CTA and published at block-uniform checkpoints.
 * Masks rotate over three arrays: round r reads M[r % 3], ORs into
 * M[(r + 1) % 3] and clears M[(r + 2) % 3] at the vertices of round r - 1's
 * queue (three vertex queues rotate for that).
 */
#include <algorithm>
#include <string.h>
#include <vector>

#include "batch.cuh"

namespace {

constexpr uint32_t SU_BS = 256;
constexpr uint32_t SU_WARPS = SU_BS / 32;
constexpr uint32_t SU_UNIT = 1024;              /* edges per unit */
constexpr uint32_t SU_EPW = SU_UNIT / SU_WARPS; /* edges per warp per unit */
constexpr uint32_t SU_SCAP = SU_BS * 5;         /* staging slots (the bound below) */
constexpr uint32_t SU_CHECK = SU_EPW;           /* warp-edges per warp between checkpoints: one per unit */
constexpr uint32_t SU_EB = 16;                  /* edges per warp in flight (measured: 4 -> 8 -> 16 with one checkpoint per unit, 14.1 -> 9.6 ms for 32 sources on R-MAT 20) */
constexpr unsigned FULL = 0xffffffffu;
/* staged pushes between checkpoints: fewer than SU_BS left after one, at most one per warp-edge */
static_assert(SU_SCAP >= SU_WARPS * SU_CHECK + SU_BS - 1, "staging too small");

struct SuCtl {
    GridBarrier bar;
    uint32_t err;
    uint32_t rounds;
    unsigned long long qctr[3]; /* (entries << 32) | edges, rotating by round */
    uint32_t work[3];
    uint32_t pad;
    unsigned long long edges_relaxed;
};

struct SuArgs {
    const uint32_t *off, *col, *wt;
    uint32_t n, m;
    uint32_t *D;                       /* n * 32 */
    uint32_t *M0, *M1, *M2;            /* n each */
    uint32_t *qv0, *qv1, *qv2;         /* n each */
    uint32_t *qo0, *qo1, *qb0, *qb1;   /* n each */
    uint32_t *uf0, *uf1;               /* ucap */
    SuCtl *ctl;
    uint32_t ucap, nblocks, max_rounds;
    unsigned long long timeout_ns;
};

struct SuCtrl {
    uint32_t nn, base_i, base_e, unit, i0, cnt, nitems, total;
    uint32_t ws[32];
};

__device__ __forceinline__ uint32_t *sel2(uint32_t p, uint32_t *a, uint32_t *b) { return p ? b : a; }
__device__ __forceinline__ uint32_t *sel3(uint32_t p, uint32_t *a, uint32_t *b, uint32_t *c) {
    return p == 0 ? a : (p == 1 ? b : c);
}
__device__ __forceinline__ void su_err(SuCtl *c, uint32_t code) { atomicCAS(&c->err, GGA_DEV_OK, code); }

/* Publish staged entries (vertex, first edge, degree): block scan of the
 * degrees, one packed atomicAdd, coalesced writes, unit boundaries. */
__device__ __forceinline__ void su_flush(const SuArgs &a, SuCtrl &C, uint32_t *sv, uint32_t *sb, uint32_t *sd,
                                         uint32_t nn, uint32_t r3n, uint32_t nb) {
    const uint32_t tid = threadIdx.x;
    const uint32_t chunk = (nn + SU_BS - 1) / SU_BS;
    const uint32_t j0 = min(tid * chunk, nn), j1 = min(j0 + chunk, nn);
    uint32_t local = 0;
    for (uint32_t j = j0; j < j1; ++j) local += sd[j];
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
    __syncthreads();
    const uint32_t bi = C.base_i, be = C.base_e;
    /* qv rotates over three buffers (r3n), qo / qb / uf alternate by parity (nb) */
    uint32_t *qv = sel3(r3n, a.qv0, a.qv1, a.qv2);
    for (uint32_t j = tid; j < nn; j += SU_BS) {
        const uint32_t i = bi + j;
        if (i < a.n) {
            qv[i] = sv[j];
            sel2(nb, a.qo0, a.qo1)[i] = be + sd[j];
            sel2(nb, a.qb0, a.qb1)[i] = sb[j];
        } else {
            su_err(a.ctl, GGA_DEV_OVERFLOW);
        }
    }
    uint32_t *uf = sel2(nb, a.uf0, a.uf1);
    const uint64_t k0 = ((uint64_t)be + SU_UNIT - 1) / SU_UNIT, k1 = ((uint64_t)be + tot + SU_UNIT - 1) / SU_UNIT;
    for (uint64_t k = k0 + tid; k < k1; k += SU_BS) {
        const uint32_t rel = (uint32_t)(k * SU_UNIT - be);
        uint32_t lo = 0, hi = nn;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (sd[mid] <= rel) lo = mid; else hi = mid;
        }
        if (k < a.ucap) uf[k] = bi + lo;
        else su_err(a.ctl, GGA_DEV_OVERFLOW_UNITS);
    }
    __syncthreads();
    if (tid == 0) C.nn = 0;
    __syncthreads();
}

__device__ __forceinline__ void su_checkpoint(const SuArgs &a, SuCtrl &C, uint32_t *sv, uint32_t *sb, uint32_t *sd,
                                              uint32_t r3n, uint32_t nb, uint32_t limit) {
    __syncthreads();
    const uint32_t nn = C.nn;
    __syncthreads();
    if (nn >= limit && nn > 0) su_flush(a, C, sv, sb, sd, nn, r3n, nb);
}

__global__ void __launch_bounds__(SU_BS, 4) k_sssp32(SuArgs a) {
    extern __shared__ uint32_t dyn[];
    __shared__ SuCtrl C;
    uint32_t *t_o = dyn, *t_b = dyn + (SU_UNIT + 1), *t_u = dyn + 2 * (SU_UNIT + 1), *t_m = dyn + 3 * (SU_UNIT + 1);
    uint32_t *sv = dyn + 4 * (SU_UNIT + 1), *sb = sv + SU_SCAP, *sd = sb + SU_SCAP;
    SuCtl *ctl = a.ctl;
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint64_t gtid = (uint64_t)blockIdx.x * SU_BS + tid, gthreads = (uint64_t)gridDim.x * SU_BS;
    uint32_t gen = 0, prev_items = 0;
    unsigned long long relaxed = 0;
    if (tid == 0) C.nn = 0;
    __syncthreads();
    uint32_t round = 0;
    for (;; ++round) {
        const uint32_t r3 = round % 3, r3n = (round + 1) % 3, r3p = (round + 2) % 3, cur = round & 1, nb = cur ^ 1;
        if (tid == 0) {
            const unsigned long long qc = ld_relaxed_u64(&ctl->qctr[r3]);
            const uint32_t ni = min((uint32_t)(qc >> 32), a.n);
            C.nitems = ni;
            C.total = ni ? (uint32_t)qc : 0u;
        }
        __syncthreads();
        const uint32_t nitems = C.nitems, total = C.total;
        const uint32_t units = min((uint32_t)(((uint64_t)total + SU_UNIT - 1) / SU_UNIT), a.ucap);
        __syncthreads();
        if (units == 0) break;
        if (round >= a.max_rounds) {
            if (blockIdx.x == 0 && tid == 0) su_err(ctl, GGA_DEV_ROUND_LIMIT);
            break;
        }
        if (blockIdx.x == 0 && tid == 0) {
            ctl->qctr[r3p] = 0;
            ctl->work[r3p] = 0;
        }
        /* masks of round - 1's queue are done with: clear them for round + 1 */
        {
            const uint32_t *qp = sel3(r3p, a.qv0, a.qv1, a.qv2);
            uint32_t *Mp = sel3(r3p, a.M0, a.M1, a.M2);
            for (uint64_t i = gtid; i < prev_items; i += gthreads) Mp[__ldcg(qp + i)] = 0;
        }
        prev_items = nitems;
        const uint32_t *qv = sel3(r3, a.qv0, a.qv1, a.qv2);
        const uint32_t *qo = sel2(cur, a.qo0, a.qo1), *qb = sel2(cur, a.qb0, a.qb1), *uf = sel2(cur, a.uf0, a.uf1);
        const uint32_t *Mc = sel3(r3, a.M0, a.M1, a.M2);
        uint32_t *Mn = sel3(r3n, a.M0, a.M1, a.M2);
        for (;;) {
            if (tid == 0) {
                const uint32_t k = atomicAdd(&ctl->work[r3], 1u);
                C.unit = k;
                if (k < units) {
                    const uint32_t i0 = min(__ldcg(uf + k), nitems - 1);
                    const uint32_t i1 = k + 1 < units ? min(__ldcg(uf + k + 1), nitems - 1) : nitems - 1;
                    C.i0 = i0;
                    C.cnt = i1 >= i0 ? min(i1 - i0 + 1, SU_UNIT + 1) : 1u;
                }
            }
            __syncthreads();
            const uint32_t k = C.unit;
            if (k >= units) break;
            const uint32_t i0 = C.i0, cnt = C.cnt;
            const uint32_t ebase = k * SU_UNIT, eend = min(ebase + SU_UNIT, total);
            for (uint32_t j = tid; j < cnt; j += SU_BS) {
                const uint32_t i = i0 + j;
                const uint32_t u = __ldcg(qv + i);
                t_o[j] = __ldcg(qo + i);
                t_b[j] = __ldcg(qb + i);
                t_u[j] = u;
                t_m[j] = __ldcg(Mc + u);
            }
            __syncthreads();
            /* warp w takes edges ebase + w, + SU_WARPS, ...; a checkpoint
             * every SU_CHECK edges bounds the staging (one push per
             * warp-edge).  SU_EB edges per step: lanes 0..SU_EB-1 each look
             * one up and broadcast it, then every lane issues all its
             * distance loads before any update (SU_EB independent chains). */
            for (uint32_t c0 = 0; c0 < SU_EPW; c0 += SU_CHECK) {
                if (c0) su_checkpoint(a, C, sv, sb, sd, r3n, nb, SU_BS);
                for (uint32_t c = c0; c < c0 + SU_CHECK; c += SU_EB) { /* warp-uniform */
                    uint32_t my_u = 0, my_m = 0, my_v = 0, my_w = 0;
                    if (lane < SU_EB) {
                        const uint32_t e = ebase + (c + lane) * SU_WARPS + warp;
                        if (e < eend) {
                            uint32_t lo = 0, hi = cnt;
                            while (hi - lo > 1) {
                                const uint32_t mid = (lo + hi) >> 1;
                                if (t_o[mid] <= e) lo = mid; else hi = mid;
                            }
                            const uint32_t ei = t_b[lo] + (e - t_o[lo]);
                            if (ei < a.m) {
                                my_u = t_u[lo];
                                my_m = t_m[lo];
                                my_v = __ldg(a.col + ei);
                                my_w = __ldg(a.wt + ei);
                            } else {
                                su_err(ctl, GGA_DEV_BAD_EDGE);
                            }
                        }
                    }
                    uint32_t u[SU_EB], m[SU_EB], v[SU_EB], w[SU_EB], du[SU_EB], dv[SU_EB];
#pragma unroll
                    for (uint32_t q = 0; q < SU_EB; ++q) {
                        u[q] = __shfl_sync(FULL, my_u, q);
                        m[q] = __shfl_sync(FULL, my_m, q); /* 0 for a missing edge */
                        v[q] = __shfl_sync(FULL, my_v, q);
                        w[q] = __shfl_sync(FULL, my_w, q);
                    }
#pragma unroll
                    for (uint32_t q = 0; q < SU_EB; ++q) {
                        const bool on = (m[q] >> lane) & 1u;
                        du[q] = on ? __ldcg(a.D + (size_t)u[q] * 32 + lane) : 0u;
                        dv[q] = on ? __ldcg(a.D + (size_t)v[q] * 32 + lane) : 0u;
                    }
                    /* an offer that beats the probed distance goes out as a
                     * fire-and-forget red.min and marks v for the next round
                     * without waiting for the old value: if a concurrent offer
                     * landed lower, v's expansion next round reads that value,
                     * so the mark costs at most a redundant relaxation */
                    uint32_t imq[SU_EB];
#pragma unroll
                    for (uint32_t q = 0; q < SU_EB; ++q) {
                        bool imp = false;
                        if ((m[q] >> lane) & 1u) {
                            const uint32_t alt = du[q] + w[q];
                            if (alt < dv[q]) {
                                red_min_u32(a.D + (size_t)v[q] * 32 + lane, alt);
                                imp = true;
                            }
                        }
                        imq[q] = __ballot_sync(FULL, imp);
                    }
                    /* lane q ORs edge q's improved lanes into v's next mask, so the
                     * step's SU_EB atomics are in flight together; the lane whose
                     * OR found the mask empty stages v */
                    uint32_t mim = 0, mv = 0;
#pragma unroll
                    for (uint32_t q = 0; q < SU_EB; ++q)
                        if (lane == q) {
                            mim = imq[q];
                            mv = v[q];
                        }
                    if (mim && atomicOr(Mn + mv, mim) == 0) {
                        const uint32_t b = __ldg(a.off + mv), d = __ldg(a.off + mv + 1) - b;
                        if (d) {
                            const uint32_t slot = atomicAdd(&C.nn, 1u);
                            if (slot < SU_SCAP) {
                                sv[slot] = mv;
                                sb[slot] = b;
                                sd[slot] = d;
                            } else {
                                su_err(ctl, GGA_DEV_OVERFLOW);
                            }
                        }
                    }
                }
            }
            if (tid == 0) relaxed += eend - ebase;
            su_checkpoint(a, C, sv, sb, sd, r3n, nb, SU_BS);
        }
        su_checkpoint(a, C, sv, sb, sd, r3n, nb, 1);
        if (!grid_barrier(&ctl->bar, &ctl->err, a.nblocks, gen, a.timeout_ns)) break;
    }
    if (tid == 0 && relaxed) atomicAdd(&ctl->edges_relaxed, relaxed);
    if (blockIdx.x == 0 && tid == 0) ctl->rounds = round;
}

/* D = MYINFINITY except D[src_s][s] = 0; the masks and the level-0 queue. */
__global__ void k_su_sources(SuArgs a, const uint32_t *srcs, uint32_t nsrc) {
    const uint32_t s = threadIdx.x;
    if (s >= nsrc) return;
    const uint32_t v = srcs[s];
    a.D[(size_t)v * 32 + s] = 0;
    if (atomicOr(a.M0 + v, 1u << s) == 0) {
        const uint32_t b = a.off[v], d = a.off[v + 1] - b;
        if (!d) return;
        const unsigned long long old = atomicAdd(&a.ctl->qctr[0], (1ull << 32) | d);
        const uint32_t i = (uint32_t)(old >> 32), o = (uint32_t)old;
        a.qv0[i] = v;
        a.qo0[i] = o;
        a.qb0[i] = b;
        for (uint64_t k = ((uint64_t)o + SU_UNIT - 1) / SU_UNIT; k * SU_UNIT < (uint64_t)o + d; ++k)
            if (k < a.ucap) a.uf0[k] = i;
    }
}

/* Source-major output: out[s * n + v] = D[v * 32 + s] through a 32 x 32
 * shared tile (coalesced on both sides). */
__global__ void k_su_transpose(const uint32_t *D, uint32_t n, uint32_t nsrc, uint32_t *out) {
    __shared__ uint32_t tile[32][33];
    const uint32_t tx = threadIdx.x & 31, ty = threadIdx.x >> 5; /* 32 x 8 threads */
    for (uint64_t v0 = (uint64_t)blockIdx.x * 32; v0 < n; v0 += (uint64_t)gridDim.x * 32) {
        for (uint32_t r = ty; r < 32; r += 8) {
            const uint64_t v = v0 + r;
            tile[r][tx] = v < n ? D[v * 32 + tx] : 0u;
        }
        __syncthreads();
        for (uint32_t s = ty; s < nsrc; s += 8) {
            const uint64_t v = v0 + tx;
            if (v < n) out[(size_t)s * n + v] = tile[tx][s];
        }
        __syncthreads();
    }
}

__global__ void k_su_fill(uint32_t *p, size_t count, uint32_t value) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
        p[i] = value;
}

/* reached (vertex, source) pairs and their out-edges */
__global__ void k_su_reached(const uint32_t *D, const uint32_t *off, uint32_t n, uint32_t nsrc,
                             unsigned long long *acc) {
    unsigned long long vr = 0, er = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < (size_t)n * 32; i += (size_t)gridDim.x * blockDim.x) {
        const uint32_t v = (uint32_t)(i >> 5), s = (uint32_t)(i & 31);
        if (s < nsrc && D[i] < GGA_INFINITY) {
            vr++;
            er += off[v + 1] - off[v];
        }
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

size_t su_smem() { return ((size_t)4 * (SU_UNIT + 1) + (size_t)3 * SU_SCAP) * sizeof(uint32_t); }

} // namespace

struct SuScratch {
    int device = -1;
    uint32_t ncap = 0, ucap = 0;
    size_t ocap = 0;
    uint32_t *D = nullptr, *M[3] = {}, *qv[3] = {}, *qo[2] = {}, *qb[2] = {}, *uf[2] = {};
    uint32_t *out = nullptr, *srcs = nullptr;
    SuCtl *ctl = nullptr, *hctl = nullptr;
    int nblocks = 0;
};

void su_scratch_free(SuScratch *s) {
    if (!s) return;
    cudaFree(s->D);
    for (int i = 0; i < 3; ++i) {
        cudaFree(s->M[i]);
        cudaFree(s->qv[i]);
    }
    for (int i = 0; i < 2; ++i) {
        cudaFree(s->qo[i]);
        cudaFree(s->qb[i]);
        cudaFree(s->uf[i]);
    }
    cudaFree(s->out);
    cudaFree(s->srcs);
    cudaFree(s->ctl);
    cudaFreeHost(s->hctl);
    delete s;
}

static gga_status su_reserve(SuScratch *s, uint32_t n, uint32_t m, size_t out_words) {
    cudaError_t e = cudaSuccess;
    if (s->ncap < n) {
        cudaFree(s->D);
        s->D = nullptr;
        for (int i = 0; i < 3; ++i) {
            cudaFree(s->M[i]); cudaFree(s->qv[i]);
            s->M[i] = s->qv[i] = nullptr;
        }
        for (int i = 0; i < 2; ++i) {
            cudaFree(s->qo[i]); cudaFree(s->qb[i]);
            s->qo[i] = s->qb[i] = nullptr;
        }
        s->ncap = 0;
        e = cudaMalloc((void **)&s->D, (size_t)n * 32 * 4);
        for (int i = 0; i < 3 && e == cudaSuccess; ++i) e = cudaMalloc((void **)&s->M[i], (size_t)n * 4);
        for (int i = 0; i < 3 && e == cudaSuccess; ++i) e = cudaMalloc((void **)&s->qv[i], (size_t)n * 4);
        for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = cudaMalloc((void **)&s->qo[i], (size_t)n * 4);
        for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = cudaMalloc((void **)&s->qb[i], (size_t)n * 4);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return gga_fail(GGA_ERR_CUDA, "sssp batch scratch (%u vertices): %s", n, cudaGetErrorString(e));
        }
        s->ncap = n;
    }
    const uint32_t ucap = m / SU_UNIT + 4;
    if (s->ucap < ucap) {
        for (int i = 0; i < 2; ++i) {
            cudaFree(s->uf[i]);
            s->uf[i] = nullptr;
        }
        s->ucap = 0;
        for (int i = 0; i < 2; ++i) GGA_CK(cudaMalloc((void **)&s->uf[i], (size_t)ucap * 4));
        s->ucap = ucap;
    }
    if (s->ocap < out_words) {
        cudaFree(s->out);
        s->out = nullptr;
        s->ocap = 0;
        GGA_CK(cudaMalloc((void **)&s->out, out_words * 4));
        s->ocap = out_words;
    }
    if (!s->ctl) {
        GGA_CK(cudaMalloc((void **)&s->ctl, sizeof(SuCtl)));
        GGA_CK(cudaMallocHost((void **)&s->hctl, sizeof(SuCtl)));
        GGA_CK(cudaMalloc((void **)&s->srcs, 32 * sizeof(uint32_t)));
    }
    if (!s->nblocks) {
        const size_t smem = su_smem();
        GGA_CK(cudaFuncSetAttribute(k_sssp32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int occ = 0, sms = 0;
        GGA_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_sssp32, SU_BS, smem));
        GGA_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device));
        if (occ <= 0) return gga_fail(GGA_ERR_CUDA, "sssp batch kernel: zero occupancy");
        s->nblocks = occ * sms;
    }
    return GGA_OK;
}

gga_status gga_sssp_batch(gga_ctx *c, gga_graph *g, uint32_t nsrc, const uint32_t *srcs, uint32_t *dist_out,
                          gga_stats *stats) {
    const double t0 = gga_now_ms();
    if (!c || !g || !srcs || !dist_out) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    if (nsrc == 0 || nsrc > 32) return gga_fail(GGA_ERR_INVALID_ARG, "nsrc %u (1..32)", nsrc);
    gga_status s;
    for (uint32_t i = 0; i < nsrc; ++i)
        if ((s = ctx_validate_solve(g, GGA_SSSP, srcs[i]))) return s;
    std::lock_guard<std::mutex> lk(c->mu);
    if ((s = ctx_activate(c))) return s;
    if ((s = dev_graph_ensure(g, c->device, c->st))) return s;
    const DevGraph *d = dev_graph_of(g);
    BatchScratch *b = ctx_batch(c);
    if (!b) return gga_fail(GGA_ERR_NO_MEMORY, "batch scratch");
    if (!b->su) {
        b->su = new (std::nothrow) SuScratch();
        if (!b->su) return gga_fail(GGA_ERR_NO_MEMORY, "sssp batch scratch");
        b->su->device = c->device;
    }
    SuScratch *sc = b->su;
    const bool dev_out = ptr_is_device(dist_out);
    const size_t words = (size_t)nsrc * d->n;
    if ((s = su_reserve(sc, d->n, d->m, dev_out ? 0 : words))) return s;
    uint32_t *out = dev_out ? dist_out : sc->out;

    SuArgs a;
    memset(&a, 0, sizeof a);
    a.off = d->off;
    a.col = d->col;
    a.wt = d->wt;
    a.n = d->n;
    a.m = d->m;
    a.D = sc->D;
    a.M0 = sc->M[0]; a.M1 = sc->M[1]; a.M2 = sc->M[2];
    a.qv0 = sc->qv[0]; a.qv1 = sc->qv[1]; a.qv2 = sc->qv[2];
    a.qo0 = sc->qo[0]; a.qo1 = sc->qo[1];
    a.qb0 = sc->qb[0]; a.qb1 = sc->qb[1];
    a.uf0 = sc->uf[0]; a.uf1 = sc->uf[1];
    a.ctl = sc->ctl;
    a.ucap = sc->ucap;
    a.nblocks = (uint32_t)sc->nblocks;
    a.max_rounds = d->n + 2;
    a.timeout_ns = 4000000000ull;

    GGA_CK(cudaMemsetAsync(sc->ctl, 0, sizeof(SuCtl), c->st));
    for (int i = 0; i < 3; ++i) GGA_CK(cudaMemsetAsync(sc->M[i], 0, (size_t)d->n * 4, c->st));
    GGA_CK(cudaMemcpyAsync(sc->srcs, srcs, nsrc * sizeof(uint32_t), cudaMemcpyHostToDevice, c->st));
    k_su_fill<<<ctx_grid(c, (uint64_t)d->n * 32, 256), 256, 0, c->st>>>(sc->D, (size_t)d->n * 32, GGA_INFINITY);
    k_su_sources<<<1, 32, 0, c->st>>>(a, sc->srcs, nsrc);
    GGA_CK(cudaGetLastError());
    GGA_CK(cudaEventRecord(c->ev[0], c->st));
    void *args[] = {&a};
    GGA_CK(cudaLaunchCooperativeKernel((const void *)k_sssp32, dim3(a.nblocks), dim3(SU_BS), args, su_smem(), c->st));
    GGA_CK(cudaEventRecord(c->ev[1], c->st));
    GGA_CK(cudaMemcpyAsync(sc->hctl, sc->ctl, sizeof(SuCtl), cudaMemcpyDeviceToHost, c->st));
    k_su_transpose<<<ctx_grid(c, ((uint64_t)d->n + 31) / 32 * 256, 256), 256, 0, c->st>>>(sc->D, d->n, nsrc, out);
    GGA_CK(cudaGetLastError());
    uint32_t launches = 4;
    if (!dev_out) GGA_CK(cudaMemcpyAsync(dist_out, out, words * 4, cudaMemcpyDeviceToHost, c->st));
    if (stats) {
        unsigned long long *acc = (unsigned long long *)(c->dflag + 32);
        GGA_CK(cudaMemsetAsync(acc, 0, 2 * sizeof(unsigned long long), c->st));
        k_su_reached<<<ctx_grid(c, (uint64_t)d->n * 32, 256), 256, 0, c->st>>>(sc->D, d->off, d->n, nsrc, acc);
        GGA_CK(cudaGetLastError());
        GGA_CK(cudaMemcpyAsync(c->hflag + 32, acc, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->st));
        launches++;
    }
    if ((s = dev_wait(c->st, 60.0))) return s;
    const SuCtl &h = *sc->hctl;
    switch (h.err) {
    case GGA_DEV_OK: break;
    case GGA_DEV_TIMEOUT: return gga_fail(GGA_ERR_TIMEOUT, "sssp batch grid barrier timed out");
    case GGA_DEV_OVERFLOW: return gga_fail(GGA_ERR_CUDA, "sssp batch queue overflow (internal error)");
    case GGA_DEV_OVERFLOW_UNITS: return gga_fail(GGA_ERR_CUDA, "sssp batch unit table overflow (internal error)");
    case GGA_DEV_BAD_EDGE: return gga_fail(GGA_ERR_CUDA, "sssp batch edge index out of range (internal error)");
    case GGA_DEV_ROUND_LIMIT: return gga_fail(GGA_ERR_CUDA, "sssp batch round limit reached (internal error)");
    default: return gga_fail(GGA_ERR_CUDA, "sssp batch kernel error %u", h.err);
    }
    if (stats) {
        gga_stats st;
        memset(&st, 0, sizeof st);
        float ms = 0;
        GGA_CK(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
        const unsigned long long *hr = (const unsigned long long *)(c->hflag + 32);
        st.iterations = h.rounds;
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
