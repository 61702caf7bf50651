/*
 * Device-side declarations shared by the CUDA translation units.
 */
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gga_internal.h"

#define GGA_CK(call)                                                                       \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess)                                                             \
            return gga_fail(GGA_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call,       \
                            cudaGetErrorString(e_));                                       \
    } while (0)

/* GGA_OK, or GGA_ERR_CUDA with the error's text (for code that must not
 * return early). */
static inline gga_status gga_cuda_check(cudaError_t e) {
    return e == cudaSuccess ? GGA_OK : gga_fail(GGA_ERR_CUDA, "%s", cudaGetErrorString(e));
}

/* Device-resident graph (one per gga_graph).  The unsplit CSR is 0-based;
 * the split view is the reference's NodeSplit result re-based to 0
 * (s_off[k] = psrc[k] - 1 for k < ns). */
struct DevGraph {
    int device;
    uint32_t n, m;
    uint32_t *off; /* n+1 */
    uint32_t *col; /* m */
    uint32_t *wt;  /* m */
    uint32_t maxdeg;
    int symmetric; /* 1 yes, -1 no (or rows unsorted), 0 not checked */
    int wsymmetric; /* symmetric with equal weights both ways: 1 yes, -1 no, 0 not checked */

    /* delta-stepping light/heavy order of every row for bucket width lh_delta:
     * edges with w < lh_delta first, then the heavy edges in LH_CLASSES weight
     * classes of width lh_cw (lh_delta + (c-1) lh_cw <= w < lh_delta + c lh_cw),
     * each class in CSR order */
    uint32_t lh_delta;
    uint32_t lh_cw;
    uint32_t *lcol, *lwt; /* m each */
    uint32_t *light;      /* n: light edges of each row */
    uint32_t lh_heavy;    /* edges with w >= lh_delta */

    /* node split (graph.h:415-522) */
    int32_t level, buckets;
    uint32_t ns, mda, npar;
    uint32_t *s_off;   /* ns+1, s_off[ns] = m */
    uint32_t *s_col;   /* m, targets remapped to the parent's split id */
    uint32_t *s_cc;    /* ns, childCount (at parents) */
    uint32_t *s_isp;   /* ns, IsParent */
    uint32_t *s_par;   /* ns, parentNode (original id) */
    uint32_t *first;   /* n+1, split id of each original vertex's parent */
    uint32_t *cidx;    /* npar, myChildIndex */
    uint32_t *ccnt;    /* npar, myChildCount */
};

/* The graph a relaxation engine walks: either the unsplit CSR or the split one. */
/* Convergence log of a topology-driven solve (gga_convergence): after every
 * relax launch the current distances are compared with `fin`. */
struct ConvHook {
    const uint32_t *fin;     /* device: final distances of the original vertices */
    unsigned long long *cnt; /* device: vertices that differ (one launch) */
    unsigned long long *norm; /* device: sum of the squared differences (each < 2^32, so exact in 64 bits) */
    gga_conv_record *rec;    /* host: records, room for cap */
    uint32_t cap, n;         /* n: iterations logged */
};

struct GraphView {
    const uint32_t *off;
    const uint32_t *col;
    const uint32_t *wt;
    const uint32_t *cc; /* child counts (split view) or nullptr */
    uint32_t n;
    uint32_t m;
    int symmetric;      /* every edge has its reverse (unsplit view only) */
};

/* Heavy-edge weight classes of the light/heavy row order (device_graph.cu). */
constexpr uint32_t LH_CLASSES = 15;

/* Error codes written by kernels into their control blocks. */
enum : uint32_t {
    GGA_DEV_OK = 0,
    GGA_DEV_TIMEOUT = 1,
    GGA_DEV_OVERFLOW = 2,
    GGA_DEV_SPLIT_RULE = 3,
    GGA_DEV_OVERFLOW_UNITS = 4,
    GGA_DEV_OVERFLOW_FAR = 5,
    GGA_DEV_BAD_EDGE = 6,
    GGA_DEV_ROUND_LIMIT = 7,
    GGA_DEV_BAD_TARGET = 8 /* an edge's target id is >= n (malformed caller CSR) */
};

/* ---- small device helpers ---------------------------------------------- */

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint32_t ld_relaxed_u32(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
/* Fire-and-forget min (the same relaxed, device-scope semantics as an
 * atomicMin whose old value is not read). */
__device__ __forceinline__ void red_min_u32(uint32_t *p, uint32_t v) {
    asm volatile("red.relaxed.gpu.global.min.u32 [%0], %1;" ::"l"(p), "r"(v));
}
__device__ __forceinline__ void st_release_u32(uint32_t *p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint64_t global_timer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

/* Bounded grid barrier for persistent cooperative launches.  Arrivals add
 * to one monotonic counter with acquire-release atomics; barrier number k is
 * complete once the counter reaches k * nblocks (nothing is ever reset, so
 * no plain store races with an arrival).  A block that waits longer than
 * timeout_ns (or sees the error word set) records GGA_DEV_TIMEOUT and returns
 * false instead of spinning on.  The verdict is broadcast through shared
 * memory so all threads of a block agree.  Every block must call it the
 * same number of times. */
struct GridBarrier {
    uint32_t count;
    uint32_t pad;
};

__device__ __forceinline__ uint32_t atom_add_acq_rel_u32(uint32_t *p, uint32_t v) {
    uint32_t old;
    asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

__device__ __forceinline__ bool grid_barrier(GridBarrier *bar, uint32_t *err, uint32_t nblocks,
                                             uint32_t &gen_local, uint64_t timeout_ns) {
    __shared__ uint32_t s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t target = (gen_local + 1) * nblocks;
        __threadfence();
        atom_add_acq_rel_u32(&bar->count, 1u);
        uint64_t t0 = 0;
        uint32_t spins = 0;
        while (ld_acquire_u32(&bar->count) < target) {
            if ((++spins & 63u) == 0) {
                if (ld_relaxed_u32(err) != GGA_DEV_OK) break;
                const uint64_t now = global_timer_ns();
                if (t0 == 0) t0 = now;
                else if (now - t0 > timeout_ns) {
                    atomicCAS(err, GGA_DEV_OK, GGA_DEV_TIMEOUT);
                    break;
                }
            }
            __nanosleep(32);
        }
        __threadfence();
        gen_local += 1;
        s_ok = ld_relaxed_u32(err) == GGA_DEV_OK;
    }
    __syncthreads();
    const bool ok = s_ok != 0;
    __syncthreads(); /* s_ok is rewritten by the next barrier */
    return ok;
}

/* Exclusive block scan of one uint32 per thread (blockDim.x a multiple of
 * 32, <= 1024).  `warp_sums` needs 32 entries of shared memory.  Returns the
 * exclusive prefix; *total receives the block sum. */
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t x, uint32_t *warp_sums,
                                                         uint32_t *total) {
    const uint32_t lane = lane_id(), wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t v = x;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= (uint32_t)d) v += y;
    }
    if (lane == 31) warp_sums[wid] = v;
    __syncthreads();
    if (wid == 0) {
        uint32_t s = lane < nw ? warp_sums[lane] : 0;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, s, d);
            if (lane >= (uint32_t)d) s += y;
        }
        if (lane < nw) warp_sums[lane] = s; /* inclusive over warps */
    }
    __syncthreads();
    uint32_t base = wid ? warp_sums[wid - 1] : 0;
    *total = warp_sums[nw - 1];
    __syncthreads();
    return base + v - x;
}

/* The same scan for 64-bit values (e.g. (count << 32) | edges pairs). */
__device__ __forceinline__ unsigned long long block_exclusive_scan64(unsigned long long x, unsigned long long *warp_sums,
                                                                    unsigned long long *total) {
    const uint32_t lane = lane_id(), wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    unsigned long long v = x;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= (uint32_t)d) v += y;
    }
    if (lane == 31) warp_sums[wid] = v;
    __syncthreads();
    if (wid == 0) {
        unsigned long long s = lane < nw ? warp_sums[lane] : 0ull;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, s, d);
            if (lane >= (uint32_t)d) s += y;
        }
        if (lane < nw) warp_sums[lane] = s;
    }
    __syncthreads();
    const unsigned long long base = wid ? warp_sums[wid - 1] : 0ull;
    *total = warp_sums[nw - 1];
    __syncthreads();
    return base + v - x;
}

/* ---- host-side entry points implemented in the .cu files ----------------- */

#ifdef __cplusplus
extern "C++" {
#endif
/* device_graph.cu */
/* Waits for `st` like cudaStreamSynchronize, but gives up after limit_s
 * seconds with GGA_ERR_TIMEOUT (a kernel that never finishes then surfaces as
 * an error; only ending the process frees the device). */
gga_status dev_wait(cudaStream_t st, double limit_s);
gga_status dev_graph_ensure(gga_graph *g, int device, cudaStream_t st);
DevGraph *dev_graph_of(gga_graph *g);
gga_status dev_exclusive_scan(const uint32_t *in, uint32_t *out, uint32_t count, cudaStream_t st);
GraphView dev_graph_view(const DevGraph *d, bool split);
/* Builds (or reuses) the light/heavy row order for bucket width delta. */
gga_status dev_graph_light_heavy(gga_graph *g, uint32_t delta, cudaStream_t st);
/* Decides (once per resident graph) whether every edge has its reverse;
 * dflag/hflag: 2 words of device / pinned scratch. */
gga_status dev_graph_check_symmetric(gga_graph *g, uint32_t *dflag, uint32_t *hflag, cudaStream_t st);
#ifdef __cplusplus
}
#endif
