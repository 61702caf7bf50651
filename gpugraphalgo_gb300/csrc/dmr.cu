/*
 * Delaunay mesh refinement on the GPU (the reference's DMR program,
 * Programs/CUDA_src/Kepler_DMR/dmr.cu:54-398 with its refine kernels in
 * m_refine.h), redesigned as rounds of short kernels over a mesh kept
 * resident in HBM, and a one-block kernel for the small last rounds.
 *
 * Round (all state on the device; the host only launches):
 *   k_bad_count / k_bad_gather  worklist = the bad triangles in ascending id
 *                               (two-pass chunked compaction; at most
 *                               batch_cap of them);
 *   k_decide    one warp: done, out of rounds, over to k_tail, or the round's
 *               worklist length;
 *   k_plan      one thread per bad triangle (a lean variant for big rounds, a
 *               prefetching one for rounds of up to pf_max plans; both are
 *               launched, one returns): circumcentre, straight walk to
 *               the triangle that holds it (or to the boundary edge the walk
 *               leaves through), cavity growth by the in-circle test, the
 *               boundary-encroachment rule, and 64-bit atomicMax claims of
 *               its cavity and of its outer ring (the triangles across the
 *               cavity boundary, whose links it rewrites) in two tables, keyed
 *               by (round, pass, a bijection of the triangle id);
 *   k_resolve0  a plan wins the first pass if no higher key claims its cavity
 *               (in either table) or claims its ring as cavity; winners stamp
 *               their cavity and ring in the lock table;
 *   k_reclaim   plans that lost and touch no stamp claim again, higher keys;
 *   k_resolve1  second-pass winners; per-chunk winner and triangle counts;
 *   k_compact   winners listed in worklist order with their point and
 *               triangle slots (chunk prefix + block scan);
 *   k_commit    one thread per winner rewrites its cavity as a fan from the
 *               new point, relinks the outer ring and re-marks the new
 *               triangles;
 *   k_finish    advances the point/triangle counts and the stop word.
 * k_tail       once at most tail_max triangles are bad, one block runs whole
 *              rounds with the same per-plan functions between __syncthreads
 *              and rebuilds the worklist from the triangles a round can change.
 * Two rings may share a triangle (their plans rewrite different edges of it),
 * and then neither plan's new triangles can hold the other's point, so the
 * commits of one round equal some sequential order of insertions.
 * Committed cavities and rings never overlap a cavity, so commits never race;
 * the round structure is the reference's mark / re-mark / retriangulate loop,
 * with its spin barrier (helpers.h:415) replaced by kernel boundaries.
 *
 * The result is a function of the input mesh and the arguments alone: every
 * step is deterministic, new coordinates are IEEE double without fused
 * multiply-adds (this file is compiled with --fmad=false), and every
 * geometric decision equals the all-double one (single-precision filters
 * with proven error bounds, falling back to double), so the result equals
 * the oracle's serial restatement of the same schedule bit for bit.
 *
 * Rounds are issued in groups with no host synchronisation inside a group;
 * once the stop word is set every kernel returns at once, so surplus rounds
 * of the last group cost one launch each.  Every index read from the mesh is
 * bounds-checked (an out-of-range id stops the refinement with an error
 * instead of being used), and every loop is bounded (walk length, cavity
 * size, round count).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <thread>
#include <vector>

#include "ctx.cuh"
#include "gga_device.cuh"

namespace {

constexpr uint32_t NONE = GGA_MESH_NONE;
constexpr uint32_t CAV_MAX = 64;            /* cavity triangles per plan */
constexpr uint32_t FAN_MAX = CAV_MAX + 2;   /* boundary edges of a cavity */
constexpr uint32_t WALK_MAX = 65536;        /* point-location steps */
constexpr uint32_t MAX_ROUNDS = 65536;
constexpr uint32_t PLAN_FAIL = 0, PLAN_INSERT = 1, PLAN_SPLIT = 2;
constexpr uint32_t STOP_NONE = 0, STOP_DONE = 1, STOP_CAPACITY = 2, STOP_STALLED = 3, STOP_ROUNDS = 4,
                   STOP_ERROR = 5;
constexpr uint32_t SCAN_BS = 1024;          /* compaction / commit blocks */
constexpr uint32_t PLAN_BS = 128;
constexpr uint32_t ROUND_GROUP = 8;         /* rounds launched between host checks */
constexpr uint32_t TAIL_BS = 1024;          /* k_tail: one block runs the small rounds */
constexpr uint32_t PF_MAX = 32768;          /* rounds up to this many plans prefetch (k_plan<true>) */
constexpr uint32_t TAIL_SORT = 4096;        /* its worklist capacity (shared-memory sort) */
constexpr uint32_t TAIL_MAX = 2048;         /* bad triangles at which it takes over */

struct DmrState {
    uint32_t npts, ntri, round, nw;
    uint32_t nbad, stop, winners, added;
    uint32_t pcap, tcap, bcap, max_rounds;
    uint32_t err, bad_in, fits, tail; /* tail: the worklist is small enough for k_tail */
    unsigned long long insertions, splits, failed;
    uint32_t pad_s, pad_t; /* host side: the coordinate bound's bits read back */
};

struct DmrArgs {
    double *x, *y;
    float4 *pq;                /* per point (xh, yh, xl, yl): float pairs of the coordinates (predicate filters) */
    uint32_t *tri, *nbr, *bad;
    unsigned long long *owner; /* cavity claims */
    unsigned long long *ring;  /* outer-ring claims */
    uint32_t *lock;            /* round << 2 | 1 (cavity) or 2 (ring) of a first-pass winner */
    uint32_t *work;
    uint32_t *wlist, *wtri;    /* winners in worklist order, their first new triangle */
    uint32_t *p_mode; /* mode | nc << 8 | nf << 16 */
    double *p_px, *p_py;
    uint32_t *p_cav;  /* [CAV_MAX][B] */
    uint4 *p_fan;     /* [FAN_MAX][B]: (a, b, outer, outer's edge | member when outer is NONE) */
    uint32_t *p_win;  /* [B] */
    uint32_t *bsum;   /* [3][G] */
    DmrState *st;
    double cos_bound;
    float cos_bound_f; /* cos_bound rounded to float */
    float S;           /* bound on every point's |x| and |y| (rounded up) */
    uint32_t B, G;
    uint32_t tail_max; /* k_tail takes over at most this many bad triangles (<= B, <= TAIL_SORT) */
    uint32_t pf_max;   /* rounds of at most this many plans use k_plan<true> */
};

__device__ __forceinline__ void set_err(DmrState *st) { atomicCAS(&st->err, 0u, 1u); }

/* Predicates.  Every geometric decision must equal the sign of the all-double
 * expression the oracle evaluates (on the double differences of double
 * coordinates).  Each predicate first evaluates its expression in single
 * precision and returns that sign only when |F| exceeds twice a bound on its
 * distance from the exact value on the double differences.
 *
 * Float inputs.  Every point keeps its coordinates as float pairs (hi =
 * x rounded to float, lo = the rest rounded to float; x = hi + lo within
 * eps^2 |x|, eps = 2^-24), one float4 (xh, yh, xl, yl) per point.  A
 * difference is (hi_a - hi_b) + (lo_a - lo_b) in float: within
 * D = 2.02 eps (L + 3 eps A) of the double difference, L the largest float
 * difference of the test and A a bound on the coordinates' magnitudes
 * (their rounding, eps |d| each for the two float additions, eps^2 terms
 * for the lo parts, 2^-53 |d| for the double subtraction).
 *
 * Bound.  A product of k differences then moves by at most
 * k D (L + D)^(k-1), so the expression moves by the sum over its monomials
 * (orientation: 2 of degree 2, 4 D (L + D); in-circle: 12 of degree 4,
 * 48 D (L + D)^3; the angle test: 8 D (L + D)), plus the float evaluation's
 * own rounding, c eps M, M the float sum of the absolute products.  Past
 * twice that bound the exact value has F's sign with a margin far above the
 * double expression's own error (about 11 2^-53 M), so the double
 * expression has it too.  Otherwise, or when L leaves [1e-9, 1e8] (where
 * float products could underflow or overflow), the double expression
 * decides.  GB300 runs FP64 at 1/64 of FP32; with these filters its FP64
 * pipe is left the new coordinates and the rare undecided cases, and a warp
 * seldom has a lane that needs them. */
constexpr float EPSF = 5.9604644775390625e-08f; /* 2^-24 */
constexpr float LMIN = 1e-9f, LMAX = 1e8f;

__device__ __forceinline__ float fmax4(float a, float b, float c, float d) {
    return fmaxf(fmaxf(fabsf(a), fabsf(b)), fmaxf(fabsf(c), fabsf(d)));
}

/* the point's float pair, and a double point's */
__device__ __forceinline__ float4 fpair(const DmrArgs &a, uint32_t i) { return a.pq[i]; }
__device__ __forceinline__ float4 fpair_of(double x, double y) {
    const float xh = (float)x, yh = (float)y;
    return make_float4(xh, yh, (float)(x - (double)xh), (float)(y - (double)yh));
}
__device__ __forceinline__ float fdx(const float4 &p, const float4 &q) { return (p.x - q.x) + (p.z - q.z); }
__device__ __forceinline__ float fdy(const float4 &p, const float4 &q) { return (p.y - q.y) + (p.w - q.w); }
__device__ __forceinline__ float err_d(float L, float A) { return 2.02f * EPSF * (L + 3.0f * EPSF * A); }

/* sign of the orientation of (p, q, pt): (q - p) x (pt - p); fp, fq are
 * p's and q's float pairs */
__device__ __forceinline__ int orient_sign(const DmrArgs &a, uint32_t p, uint32_t q, const float4 &fp,
                                           const float4 &fq, double px, double py, const float4 &pt, float A) {
    {
        const float u1 = fdx(fq, fp), v1 = fdy(pt, fp), u2 = fdy(fq, fp), v2 = fdx(pt, fp);
        const float a1 = u1 * v1, a2 = u2 * v2, F = a1 - a2;
        const float L = fmax4(u1, v1, u2, v2), D = err_d(L, A);
        const float B = 4.0f * D * (L + D) + 3.0f * EPSF * (fabsf(a1) + fabsf(a2));
        if (L > LMIN && L < LMAX && fabsf(F) > 2.01f * B) return F > 0.0f ? 1 : -1;
    }
    const double xp = a.x[p], yp = a.y[p], xq = a.x[q], yq = a.y[q];
    const double D = (xq - xp) * (py - yp) - (yq - yp) * (px - xp);
    return D > 0 ? 1 : (D < 0 ? -1 : 0);
}

/* sign of the in-circle determinant of the counter-clockwise triangle
 * (i0, i1, i2) and pt: > 0 when the point is strictly inside its circumcircle */
__device__ __forceinline__ int incircle_sign(const DmrArgs &a, uint32_t i0, uint32_t i1, uint32_t i2, double px,
                                             double py, const float4 &pt, float A) {
    {
        const float4 f0 = fpair(a, i0), f1 = fpair(a, i1), f2 = fpair(a, i2);
        const float ax = fdx(f0, pt), ay = fdy(f0, pt), bx = fdx(f1, pt), by = fdy(f1, pt);
        const float cx = fdx(f2, pt), cy = fdy(f2, pt);
        const float ad = ax * ax + ay * ay, bd = bx * bx + by * by, cd = cx * cx + cy * cy;
        const float F = ax * (by * cd - bd * cy) - ay * (bx * cd - bd * cx) + ad * (bx * cy - by * cx);
        const float M = fabsf(ax) * (fabsf(by) * cd + bd * fabsf(cy)) + fabsf(ay) * (fabsf(bx) * cd + bd * fabsf(cx)) +
                        ad * (fabsf(bx * cy) + fabsf(by * cx));
        const float L = fmaxf(fmax4(ax, ay, bx, by), fmaxf(fabsf(cx), fabsf(cy)));
        const float D = err_d(L, A), LD = L + D;
        const float B = 48.0f * D * LD * LD * LD + 12.0f * EPSF * M;
        if (L > LMIN && L < LMAX && fabsf(F) > 2.01f * B) return F > 0.0f ? 1 : -1;
    }
    const double adx = a.x[i0] - px, ady = a.y[i0] - py;
    const double bdx = a.x[i1] - px, bdy = a.y[i1] - py;
    const double cdx = a.x[i2] - px, cdy = a.y[i2] - py;
    const double ad = adx * adx + ady * ady, bd = bdx * bdx + bdy * bdy, cd = cdx * cdx + cdy * cdy;
    const double D = adx * (bdy * cd - bd * cdy) - ady * (bdx * cd - bd * cdx) + ad * (bdx * cdy - bdy * cdx);
    return D > 0 ? 1 : (D < 0 ? -1 : 0);
}

/* the angle between u and w has a cosine above cos(MINANGLE): the float
 * decision (1 or 0) when it is certain, else -1 */
__device__ __forceinline__ int angle_small_f(float ux, float uy, float wx, float wy, float cbf, float A) {
    const float p1 = ux * wx, p2 = uy * wy, dot = p1 + p2;
    const float r = cbf * sqrtf((ux * ux + uy * uy) * (wx * wx + wy * wy)), diff = dot - r;
    const float L = fmax4(ux, uy, wx, wy), D = err_d(L, A);
    const float B = 8.0f * D * (L + D) + 10.0f * EPSF * (fabsf(p1) + fabsf(p2) + r);
    if (L > LMIN && L < LMAX && fabsf(diff) > 2.01f * B) return diff > 0.0f;
    return -1;
}

__device__ __forceinline__ bool angle_small_d(double ux, double uy, double wx, double wy, double cb) {
    const double dot = ux * wx + uy * wy;
    return dot > cb * sqrt((ux * ux + uy * uy) * (wx * wx + wy * wy));
}

/* an angle whose cosine exceeds cos(MINANGLE) (checkbad, helpers.h:147-180);
 * an edge vector from q to p is the negated one from p to q (IEEE
 * subtraction and the float pair sums are antisymmetric), so three
 * differences serve all angles */
__device__ __forceinline__ uint32_t tri_bad(const DmrArgs &a, uint32_t t) {
    const uint32_t v0 = a.tri[3 * t], v1 = a.tri[3 * t + 1], v2 = a.tri[3 * t + 2];
    const float A = 2.0f * a.S;
    const float4 f0 = fpair(a, v0), f1 = fpair(a, v1), f2 = fpair(a, v2);
    const float gx01 = fdx(f1, f0), gy01 = fdy(f1, f0), gx02 = fdx(f2, f0), gy02 = fdy(f2, f0);
    const float gx12 = fdx(f2, f1), gy12 = fdy(f2, f1);
    /* angle at v0: (v1 - v0, v2 - v0); at v1: (v2 - v1, v0 - v1); at v2: (v0 - v2, v1 - v2) */
    const int s0 = angle_small_f(gx01, gy01, gx02, gy02, a.cos_bound_f, A);
    const int s1 = angle_small_f(gx12, gy12, -gx01, -gy01, a.cos_bound_f, A);
    const int s2 = angle_small_f(-gx02, -gy02, -gx12, -gy12, a.cos_bound_f, A);
    if (s0 == 1 || s1 == 1 || s2 == 1) return 1;
    if (s0 == 0 && s1 == 0 && s2 == 0) return 0;
    const double x0 = a.x[v0], y0 = a.y[v0], x1 = a.x[v1], y1 = a.y[v1], x2 = a.x[v2], y2 = a.y[v2];
    const double ex01 = x1 - x0, ey01 = y1 - y0, ex02 = x2 - x0, ey02 = y2 - y0, ex12 = x2 - x1, ey12 = y2 - y1;
    return (s0 < 0 && angle_small_d(ex01, ey01, ex02, ey02, a.cos_bound)) ||
           (s1 < 0 && angle_small_d(ex12, ey12, -ex01, -ey01, a.cos_bound)) ||
           (s2 < 0 && angle_small_d(-ex02, -ey02, -ex12, -ey12, a.cos_bound));
}

__device__ __forceinline__ uint32_t round_prio(uint32_t t, uint32_t round) {
    return (t ^ (round * 0x9E3779B9u)) * 0x85EBCA6Bu; /* a bijection of t */
}

/* pass 0 and 1 keys of a round, above every key of earlier rounds */
__device__ __forceinline__ unsigned long long claim_key(uint32_t t, uint32_t round, uint32_t pass) {
    return ((unsigned long long)(2 * round + pass) << 32) | round_prio(t, round);
}

/* Contiguous chunk of [0, n) for block b of G. */
__device__ __forceinline__ void chunk_of(uint32_t n, uint32_t b, uint32_t G, uint32_t &lo, uint32_t &hi) {
    const uint32_t c = (uint32_t)(((uint64_t)n + G - 1) / G);
    const uint64_t l = (uint64_t)b * c, h = l + c;
    lo = (uint32_t)(l < n ? l : n);
    hi = (uint32_t)(h < n ? h : n);
}

/* Block sum of `v` (one value per thread); result in every thread. */
__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t *ws) {
    uint32_t tot;
    block_exclusive_scan(v, ws, &tot);
    __syncthreads();
    return tot;
}

/* Sum of bsum[row * G + j] for j < upto, across the block. */
__device__ __forceinline__ uint32_t prefix_of(const DmrArgs &a, uint32_t row, uint32_t upto, uint32_t *ws) {
    uint32_t v = 0;
    for (uint32_t j = threadIdx.x; j < upto; j += blockDim.x) v += a.bsum[row * a.G + j];
    return block_sum(v, ws);
}

/* ---------------------------------------------------------------- marking */

/* float pairs of the points, and a bound on every |x|, |y| (rounded up; new
 * points stay inside the input's bounding box) as the bits of a
 * non-negative float, whose integer order is its value order */
__global__ void __launch_bounds__(SCAN_BS) k_shadow(DmrArgs a, uint32_t *sbits) {
    const uint32_t n = a.st->npts;
    float m = 0.0f;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double x = a.x[i], y = a.y[i];
        a.pq[i] = fpair_of(x, y);
        m = fmaxf(m, __double2float_ru(fmax(fabs(x), fabs(y))));
    }
    for (int d = 16; d > 0; d >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, d));
    if ((threadIdx.x & 31) == 0 && m > 0.0f) atomicMax(sbits, __float_as_uint(m));
}

__global__ void __launch_bounds__(SCAN_BS) k_mark_all(DmrArgs a) {
    const uint32_t n = a.st->ntri;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const uint32_t *v = a.tri + 3 * (size_t)t;
        if (v[0] >= a.st->npts || v[1] >= a.st->npts || v[2] >= a.st->npts) {
            set_err(a.st);
            a.bad[t] = 0;
            continue;
        }
        a.bad[t] = tri_bad(a, t);
    }
}

__global__ void __launch_bounds__(SCAN_BS) k_bad_count(DmrArgs a) {
    __shared__ uint32_t ws[32];
    if (a.st->stop != STOP_NONE || a.st->err || a.st->tail) return;
    uint32_t lo, hi, c = 0;
    chunk_of(a.st->ntri, blockIdx.x, a.G, lo, hi);
    for (uint32_t t = lo + threadIdx.x; t < hi; t += blockDim.x) c += a.bad[t];
    c = block_sum(c, ws);
    if (threadIdx.x == 0) a.bsum[blockIdx.x] = c;
}

/* The worklist: the bad triangles in ascending id, at most bcap of them.
 * Writes no state word: every block reads the same stop, tail and err at
 * entry, so a block never splits between returning and entering the scans. */
__global__ void __launch_bounds__(SCAN_BS) k_bad_gather(DmrArgs a) {
    __shared__ uint32_t ws[32];
    const DmrState *st = a.st;
    if (st->stop != STOP_NONE || st->tail || st->err) return;
    uint32_t base = prefix_of(a, 0, blockIdx.x, ws);
    const uint32_t bcap = st->bcap;
    if (base >= bcap) return;
    uint32_t lo, hi;
    chunk_of(st->ntri, blockIdx.x, a.G, lo, hi);
    for (uint32_t t0 = lo; t0 < hi; t0 += blockDim.x) {
        const uint32_t t = t0 + threadIdx.x;
        const uint32_t f = t < hi ? a.bad[t] : 0;
        uint32_t tot;
        const uint32_t pos = base + block_exclusive_scan(f, ws, &tot);
        if (f && pos < bcap) a.work[pos] = t;
        base += tot;
        __syncthreads();
    }
}

/* One warp decides the round from the bad count: done, out of rounds, over to
 * k_tail (which then runs this round and the next ones), or the next round
 * of at most bcap plans. */
__global__ void k_decide(DmrArgs a) {
    DmrState *st = a.st;
    if (st->stop != STOP_NONE || st->tail) return;
    if (st->err) { /* an id out of range: nothing reads the mesh after this */
        if (threadIdx.x == 0) {
            st->nw = 0;
            st->stop = STOP_ERROR;
        }
        return;
    }
    uint32_t total = 0;
    for (uint32_t j = threadIdx.x; j < a.G; j += 32) total += a.bsum[j];
    for (int d = 16; d > 0; d >>= 1) total += __shfl_down_sync(0xffffffffu, total, d);
    if (threadIdx.x != 0) return;
    st->nbad = total;
    if (st->round == 0) st->bad_in = total;
    if (total == 0) {
        st->nw = 0;
        st->stop = STOP_DONE;
    } else if (st->round >= st->max_rounds) {
        st->nw = 0;
        st->stop = STOP_ROUNDS;
    } else if (total <= a.tail_max) {
        st->nw = total;
        st->tail = 1;
    } else {
        st->round += 1;
        st->nw = total < st->bcap ? total : st->bcap;
    }
}

/* ---------------------------------------------------------------- planning */

/* The cavity of (px, py) grown from seed (the oracle's grow_cavity, same
 * visiting order).  Fan entries go to the plan record; cav stays local. */
/* The cavity of (px, py) grown from seed (the oracle's grow_cavity, same
 * visiting order).  Fan entries go to the plan record; cav stays local.
 * With PF (rounds of up to pf_max plans, whose time is the latency of their
 * longest plan) each member's vertex and neighbour ids and its neighbours'
 * vertex and neighbour ids are loaded together before the member's three
 * edges are decided, so a member costs two rounds of dependent loads plus
 * the in-circle tests' coordinates, not three per edge, and the fan's
 * validity test is taken as the entries are made (shape_ok); without it (the
 * big rounds, where registers decide occupancy) ids are loaded as needed and
 * fan_ok tests the entries afterwards.  Both decide alike. */
template <bool PF>
__device__ bool grow_cavity(const DmrArgs &a, uint32_t k, uint32_t ntri, double px, double py, const float4 &pt,
                            float A, uint32_t seed, uint32_t skip_m, uint32_t skip_i, uint32_t *cav, uint32_t &nc,
                            uint32_t &nf, bool &shape_ok, uint32_t *fav) {
    nc = 1;
    nf = 0;
    shape_ok = true;
    cav[0] = seed;
    for (uint32_t q = 0; q < nc; ++q) {
        const uint32_t c = cav[q];
        if constexpr (!PF) { /* ids loaded as each edge needs them */
            for (uint32_t i = 0; i < 3; ++i) {
                const uint32_t o = a.nbr[3 * c + i];
                if (o != NONE) {
                    if (o >= ntri) {
                        set_err(a.st);
                        return false;
                    }
                    bool in = false;
                    for (uint32_t j = 0; j < nc; ++j) in |= cav[j] == o;
                    if (in) continue;
                    if (incircle_sign(a, a.tri[3 * o], a.tri[3 * o + 1], a.tri[3 * o + 2], px, py, pt, A) > 0) {
                        if (nc == CAV_MAX) return false;
                        cav[nc++] = o;
                        continue;
                    }
                }
                if (c == skip_m && i == skip_i) continue;
                if (nf == FAN_MAX) return false;
                uint32_t e = c; /* member id when the edge is on the domain boundary */
                if (o != NONE) {
                    e = 0;
                    while (e < 3 && a.nbr[3 * o + e] != c) ++e;
                    if (e == 3) {
                        set_err(a.st); /* neighbour links not mutual */
                        return false;
                    }
                }
                a.p_fan[(size_t)nf * a.B + k] =
                    make_uint4(a.tri[3 * c + (i + 1) % 3], a.tri[3 * c + (i + 2) % 3], o, e);
                ++nf;
            }
        } else { /* every id of the member and its neighbours in two rounds of loads */
            uint32_t cv[3], cn[3], ov[3][3], on[3][3];
#pragma unroll
            for (uint32_t i = 0; i < 3; ++i) {
                cv[i] = a.tri[3 * c + i];
                cn[i] = a.nbr[3 * c + i];
            }
#pragma unroll
            for (uint32_t i = 0; i < 3; ++i) {
                const bool valid = cn[i] < ntri; /* NONE and out-of-range ids load nothing */
#pragma unroll
                for (uint32_t j = 0; j < 3; ++j) {
                    ov[i][j] = valid ? a.tri[3 * cn[i] + j] : 0u;
                    on[i][j] = valid ? a.nbr[3 * cn[i] + j] : 0u;
                }
            }
            const float4 cp[3] = {fpair(a, cv[0]), fpair(a, cv[1]), fpair(a, cv[2])};
#pragma unroll
            for (uint32_t i = 0; i < 3; ++i) {
                const uint32_t o = cn[i];
                if (o != NONE) {
                    if (o >= ntri) {
                        set_err(a.st);
                        return false;
                    }
                    bool in = false;
                    for (uint32_t j = 0; j < nc; ++j) in |= cav[j] == o;
                    if (in) continue;
                    if (incircle_sign(a, ov[i][0], ov[i][1], ov[i][2], px, py, pt, A) > 0) {
                        if (nc == CAV_MAX) return false;
                        cav[nc++] = o;
                        continue;
                    }
                }
                if (c == skip_m && i == skip_i) continue;
                if (nf == FAN_MAX) return false;
                uint32_t e = c; /* member id when the edge is on the domain boundary */
                if (o != NONE) {
                    e = on[i][0] == c ? 0u : (on[i][1] == c ? 1u : (on[i][2] == c ? 2u : 3u));
                    if (e == 3) {
                        set_err(a.st); /* neighbour links not mutual */
                        return false;
                    }
                }
                const uint32_t i1 = (i + 1) % 3, i2 = (i + 2) % 3;
                if (shape_ok) { /* the fan's validity test as the entries are made */
                    shape_ok = orient_sign(a, cv[i1], cv[i2], cp[i1], cp[i2], px, py, pt, A) > 0;
                    for (uint32_t j = 0; j < nf && shape_ok; ++j) shape_ok = fav[j] != cv[i1];
                }
                fav[nf] = cv[i1];
                a.p_fan[(size_t)nf * a.B + k] = make_uint4(cv[i1], cv[i2], o, e);
                ++nf;
            }
        }
    }
    return true;
}

/* A fan from the point over the cavity boundary is a valid triangulation only
 * if the boundary is one simple cycle the point sees from inside: as many
 * edges as the cavity has triangles plus 2 (plus 1 for a split), each seeing
 * the point on its inner side, no two starting at the same vertex.  PF took
 * the last two tests during growth (shape_ok); otherwise they run here over
 * the plan record. */
template <bool PF>
__device__ bool fan_ok(const DmrArgs &a, uint32_t k, uint32_t mode, uint32_t nc, uint32_t nf, double px, double py,
                       const float4 &pt, float A, bool shape_ok) {
    if (nf != nc + (mode == PLAN_SPLIT ? 1u : 2u)) return false;
    if constexpr (PF) {
        return shape_ok;
    } else {
        for (uint32_t j = 0; j < nf; ++j) {
            const uint4 f = a.p_fan[(size_t)j * a.B + k];
            if (orient_sign(a, f.x, f.y, fpair(a, f.x), fpair(a, f.y), px, py, pt, A) <= 0) return false;
            for (uint32_t i = 0; i < j; ++i)
                if (a.p_fan[(size_t)i * a.B + k].x == f.x) return false;
        }
        return true;
    }
}

/* Plan k (bad triangle t) of a round: the insertion point, its cavity and
 * outer ring in the plan record, and the first-pass claims.  Returns true
 * when the plan failed (no claims made). */
template <bool PF>
__device__ bool plan_one(const DmrArgs &a, uint32_t k, uint32_t t, uint32_t round, uint32_t ntri, uint32_t *cav,
                         uint32_t *fav) {
    DmrState *st = a.st;
    uint32_t mode = PLAN_FAIL, nc = 0, nf = 0;
    const unsigned long long key = claim_key(t, round, 0);
    /* circumcentre (same expression order as the oracle) */
    const uint32_t v0 = a.tri[3 * t], v1 = a.tri[3 * t + 1], v2 = a.tri[3 * t + 2];
    const double bx = a.x[v1] - a.x[v0], by = a.y[v1] - a.y[v0];
    const double cx = a.x[v2] - a.x[v0], cy = a.y[v2] - a.y[v0];
    const double d = 2.0 * (bx * cy - by * cx);
    const double b2 = bx * bx + by * by, c2 = cx * cx + cy * cy;
    double px = a.x[v0] + (cy * b2 - by * c2) / d;
    double py = a.y[v0] + (bx * c2 - cx * b2) / d;
    float4 pt = fpair_of(px, py);
    float A = a.S + fmaxf(a.S, fmaxf(fabsf(pt.x), fabsf(pt.y)));
    uint32_t cur = t, split_m = NONE, split_i = 0, step = 0;
    bool ok = true, shape_ok = true;
    for (; step < WALK_MAX; ++step) {
        uint32_t cross = 3, n;
        if constexpr (PF) { /* the triangle's ids and coordinates in one round of loads */
            const uint32_t w0 = a.tri[3 * cur], w1 = a.tri[3 * cur + 1], w2 = a.tri[3 * cur + 2];
            const uint32_t n0 = a.nbr[3 * cur], n1 = a.nbr[3 * cur + 1], n2 = a.nbr[3 * cur + 2];
            const float4 g0 = fpair(a, w0), g1 = fpair(a, w1), g2 = fpair(a, w2);
            if (orient_sign(a, w1, w2, g1, g2, px, py, pt, A) < 0) cross = 0;
            else if (orient_sign(a, w2, w0, g2, g0, px, py, pt, A) < 0) cross = 1;
            else if (orient_sign(a, w0, w1, g0, g1, px, py, pt, A) < 0) cross = 2;
            n = cross == 0 ? n0 : (cross == 1 ? n1 : n2);
        } else {
            for (uint32_t i = 0; i < 3 && cross == 3; ++i) {
                const uint32_t p = a.tri[3 * cur + (i + 1) % 3], q = a.tri[3 * cur + (i + 2) % 3];
                if (orient_sign(a, p, q, fpair(a, p), fpair(a, q), px, py, pt, A) < 0) cross = i;
            }
            n = cross < 3 ? a.nbr[3 * cur + cross] : NONE;
        }
        if (cross == 3) break;
        if (n == NONE) {
            split_m = cur;
            split_i = cross;
            break;
        }
        if (n >= ntri) {
            set_err(st);
            ok = false;
            break;
        }
        cur = n;
    }
    if (step == WALK_MAX) ok = false;
    if (ok && split_m == NONE) {
        ok = grow_cavity<PF>(a, k, ntri, px, py, pt, A, cur, NONE, 0, cav, nc, nf, shape_ok, fav);
        for (uint32_t j = 0; ok && j < nf && split_m == NONE; ++j) {
            const uint4 f = a.p_fan[(size_t)j * a.B + k];
            if (f.z != NONE) continue;
            if ((px - a.x[f.x]) * (px - a.x[f.y]) + (py - a.y[f.x]) * (py - a.y[f.y]) < 0) {
                split_m = f.w;
                for (uint32_t i = 0; i < 3; ++i)
                    if (a.tri[3 * split_m + (i + 1) % 3] == f.x) split_i = i;
            }
        }
        if (ok && split_m == NONE) {
            mode = fan_ok<PF>(a, k, PLAN_INSERT, nc, nf, px, py, pt, A, shape_ok) ? PLAN_INSERT : PLAN_FAIL;
            ok = false; /* done */
        }
    }
    if (ok) { /* split_m's edge split_i, at its midpoint */
        const uint32_t e0 = a.tri[3 * split_m + (split_i + 1) % 3], e1 = a.tri[3 * split_m + (split_i + 2) % 3];
        px = (a.x[e0] + a.x[e1]) * 0.5;
        py = (a.y[e0] + a.y[e1]) * 0.5;
        pt = fpair_of(px, py);
        A = 2.0f * a.S;
        if (grow_cavity<PF>(a, k, ntri, px, py, pt, A, split_m, split_m, split_i, cav, nc, nf, shape_ok, fav))
            mode = fan_ok<PF>(a, k, PLAN_SPLIT, nc, nf, px, py, pt, A, shape_ok) ? PLAN_SPLIT : PLAN_FAIL;
    }
    a.p_mode[k] = mode | nc << 8 | nf << 16;
    if (mode == PLAN_FAIL) return true;
    a.p_px[k] = px;
    a.p_py[k] = py;
    for (uint32_t j = 0; j < nc; ++j) {
        a.p_cav[(size_t)j * a.B + k] = cav[j];
        atomicMax(a.owner + cav[j], key);
    }
    for (uint32_t j = 0; j < nf; ++j) {
        const uint32_t o = a.p_fan[(size_t)j * a.B + k].z;
        if (o != NONE) atomicMax(a.ring + o, key);
    }
    return false;
}

/* PF: the variant for rounds of up to pf_max plans; both are launched every
 * round and the one that does not fit returns at once. */
template <bool PF>
__global__ void __launch_bounds__(PLAN_BS) k_plan(DmrArgs a) {
    DmrState *st = a.st;
    if (st->stop != STOP_NONE || st->tail) return;
    const uint32_t nw = st->nw, ntri = st->ntri, round = st->round;
    if ((nw <= a.pf_max) != PF) return;
    uint32_t cav[CAV_MAX], fav[FAN_MAX];
    uint32_t fails = 0;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nw; k += gridDim.x * blockDim.x)
        fails += plan_one<PF>(a, k, a.work[k], round, ntri, cav, fav);
    if (fails) atomicAdd(&st->failed, (unsigned long long)fails);
}

/* -------------------------------------------------------- resolve, commit */

/* No higher key on k's cavity (in either table) or on its ring's cavity
 * claims. */
__device__ __forceinline__ bool holds(const DmrArgs &a, uint32_t k, uint32_t nc, uint32_t nf,
                                      unsigned long long key) {
    for (uint32_t j = 0; j < nc; ++j) {
        const uint32_t t = a.p_cav[(size_t)j * a.B + k];
        if (a.owner[t] != key || a.ring[t] >= key) return false;
    }
    for (uint32_t j = 0; j < nf; ++j) {
        const uint32_t o = a.p_fan[(size_t)j * a.B + k].z;
        if (o != NONE && a.owner[o] >= key) return false;
    }
    return true;
}

/* First pass: k wins if it holds every conflicting claim; a winner stamps
 * its cavity (kind 1) and ring (kind 2) in the lock table. */
__device__ __forceinline__ void resolve0_one(const DmrArgs &a, uint32_t k, uint32_t round) {
    const uint32_t pm = a.p_mode[k], nc = (pm >> 8) & 0xFF, nf = pm >> 16, stamp = round << 2;
    const uint32_t win = (pm & 0xFF) != PLAN_FAIL && holds(a, k, nc, nf, claim_key(a.work[k], round, 0));
    a.p_win[k] = win;
    if (!win) return;
    for (uint32_t j = 0; j < nc; ++j) a.lock[a.p_cav[(size_t)j * a.B + k]] = stamp | 1;
    for (uint32_t j = 0; j < nf; ++j) {
        const uint32_t o = a.p_fan[(size_t)j * a.B + k].z;
        if (o != NONE) a.lock[o] = stamp | 2;
    }
}

/* Second pass: a plan that lost and touches no stamp claims again with a
 * higher key; one that touches a stamp is out of the round (p_win = 2). */
__device__ __forceinline__ void reclaim_one(const DmrArgs &a, uint32_t k, uint32_t round) {
    const uint32_t pm = a.p_mode[k], nc = (pm >> 8) & 0xFF, nf = pm >> 16, stamp = round << 2;
    if ((pm & 0xFF) == PLAN_FAIL || a.p_win[k]) return;
    bool blocked = false;
    for (uint32_t j = 0; j < nc && !blocked; ++j) blocked = (a.lock[a.p_cav[(size_t)j * a.B + k]] >> 2) == round;
    for (uint32_t j = 0; j < nf && !blocked; ++j) {
        const uint32_t o = a.p_fan[(size_t)j * a.B + k].z;
        blocked = o != NONE && a.lock[o] == (stamp | 1);
    }
    if (blocked) {
        a.p_win[k] = 2;
        return;
    }
    const unsigned long long key = claim_key(a.work[k], round, 1);
    for (uint32_t j = 0; j < nc; ++j) atomicMax(a.owner + a.p_cav[(size_t)j * a.B + k], key);
    for (uint32_t j = 0; j < nf; ++j) {
        const uint32_t o = a.p_fan[(size_t)j * a.B + k].z;
        if (o != NONE) atomicMax(a.ring + o, key);
    }
}

/* Final verdict of k (1 = commits this round) and the triangles it adds. */
__device__ __forceinline__ uint32_t resolve1_one(const DmrArgs &a, uint32_t k, uint32_t round, uint32_t &need) {
    const uint32_t pm = a.p_mode[k], nc = (pm >> 8) & 0xFF, nf = pm >> 16, w = a.p_win[k];
    const uint32_t win = w == 1 || (w == 0 && (pm & 0xFF) != PLAN_FAIL &&
                                    holds(a, k, nc, nf, claim_key(a.work[k], round, 1)));
    a.p_win[k] = win;
    need = win ? nf - nc : 0;
    return win;
}

__global__ void __launch_bounds__(PLAN_BS) k_resolve0(DmrArgs a) {
    DmrState *st = a.st;
    if (st->stop != STOP_NONE || st->tail) return;
    const uint32_t nw = st->nw, round = st->round;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nw; k += gridDim.x * blockDim.x)
        resolve0_one(a, k, round);
}

__global__ void __launch_bounds__(PLAN_BS) k_reclaim(DmrArgs a) {
    DmrState *st = a.st;
    if (st->stop != STOP_NONE || st->tail) return;
    const uint32_t nw = st->nw, round = st->round;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nw; k += gridDim.x * blockDim.x)
        reclaim_one(a, k, round);
}

__global__ void __launch_bounds__(SCAN_BS) k_resolve1(DmrArgs a) {
    __shared__ uint32_t ws[32];
    DmrState *st = a.st;
    if (st->stop != STOP_NONE || st->tail || st->nw == 0) return;
    const uint32_t round = st->round;
    uint32_t lo, hi, wins = 0, need = 0;
    chunk_of(st->nw, blockIdx.x, a.G, lo, hi);
    for (uint32_t k = lo + threadIdx.x; k < hi; k += blockDim.x) {
        uint32_t nd;
        wins += resolve1_one(a, k, round, nd);
        need += nd;
    }
    wins = block_sum(wins, ws);
    need = block_sum(need, ws);
    if (threadIdx.x == 0) {
        a.bsum[a.G + blockIdx.x] = wins;
        a.bsum[2 * a.G + blockIdx.x] = need;
    }
}

/* Totals of a round's winners and added triangles, and whether they fit. */
__device__ __forceinline__ bool round_fits(const DmrArgs &a, uint32_t *ws, uint32_t &W, uint32_t &A) {
    W = prefix_of(a, 1, a.G, ws);
    A = prefix_of(a, 2, a.G, ws);
    const DmrState *st = a.st;
    return W > 0 && (uint64_t)st->npts + W <= st->pcap && (uint64_t)st->ntri + A <= st->tcap;
}

__global__ void __launch_bounds__(SCAN_BS) k_compact(DmrArgs a) {
    __shared__ uint32_t ws[32];
    DmrState *st = a.st;
    if (st->stop != STOP_NONE || st->tail || st->nw == 0) return;
    uint32_t W, A;
    const bool fits = round_fits(a, ws, W, A);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        st->winners = W;
        st->added = A;
        st->fits = fits;
    }
    if (!fits) return;
    uint32_t wbase = prefix_of(a, 1, blockIdx.x, ws), abase = prefix_of(a, 2, blockIdx.x, ws);
    const uint32_t ntri = st->ntri;
    uint32_t lo, hi;
    chunk_of(st->nw, blockIdx.x, a.G, lo, hi);
    for (uint32_t k0 = lo; k0 < hi; k0 += blockDim.x) {
        const uint32_t k = k0 + threadIdx.x;
        uint32_t win = 0, pm = 0;
        if (k < hi) {
            win = a.p_win[k];
            pm = a.p_mode[k];
        }
        uint32_t wt, at;
        const uint32_t wpre = block_exclusive_scan(win, ws, &wt);
        const uint32_t apre = block_exclusive_scan(win ? (pm >> 16) - ((pm >> 8) & 0xFF) : 0, ws, &at);
        if (win) {
            a.wlist[wbase + wpre] = k;
            a.wtri[wbase + wpre] = ntri + abase + apre;
        }
        wbase += wt;
        abase += at;
    }
}

/* Winner k takes point pid and triangles from tb on: its cavity becomes a
 * fan from the new point, the outer ring is relinked and the new triangles
 * are re-marked.  Returns true for a boundary split. */
__device__ bool commit_one(const DmrArgs &a, uint32_t k, uint32_t pid, uint32_t tb, uint32_t *slot, uint32_t *fa,
                           uint32_t *fb) {
    const uint32_t pm = a.p_mode[k], nc = (pm >> 8) & 0xFF, nf = pm >> 16;
    const double npx = a.p_px[k], npy = a.p_py[k];
    a.x[pid] = npx;
    a.y[pid] = npy;
    a.pq[pid] = fpair_of(npx, npy);
    for (uint32_t j = 0; j < nf; ++j) {
        slot[j] = j < nc ? a.p_cav[(size_t)j * a.B + k] : tb + (j - nc);
        const uint4 f = a.p_fan[(size_t)j * a.B + k];
        fa[j] = f.x;
        fb[j] = f.y;
    }
    for (uint32_t j = 0; j < nf; ++j) {
        const uint4 f = a.p_fan[(size_t)j * a.B + k];
        const uint32_t s = slot[j];
        uint32_t n0 = NONE, n1 = NONE;
        for (uint32_t q = 0; q < nf; ++q) {
            if (fa[q] == fb[j]) n0 = slot[q];
            if (fb[q] == fa[j]) n1 = slot[q];
        }
        a.tri[3 * (size_t)s] = f.x;
        a.tri[3 * (size_t)s + 1] = f.y;
        a.tri[3 * (size_t)s + 2] = pid;
        a.nbr[3 * (size_t)s] = n0;
        a.nbr[3 * (size_t)s + 1] = n1;
        a.nbr[3 * (size_t)s + 2] = f.z;
        if (f.z != NONE) a.nbr[3 * (size_t)f.z + f.w] = s;
    }
    for (uint32_t j = 0; j < nf; ++j) a.bad[slot[j]] = tri_bad(a, slot[j]);
    return (pm & 0xFF) == PLAN_SPLIT;
}

__global__ void __launch_bounds__(PLAN_BS) k_commit(DmrArgs a) {
    DmrState *st = a.st;
    if (st->stop != STOP_NONE || st->tail || st->nw == 0 || !st->fits) return;
    const uint32_t W = st->winners, npts = st->npts;
    uint32_t ins = 0, spl = 0;
    uint32_t slot[FAN_MAX], fa[FAN_MAX], fb[FAN_MAX];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < W; i += gridDim.x * blockDim.x) {
        if (commit_one(a, a.wlist[i], npts + i, a.wtri[i], slot, fa, fb)) ++spl;
        else ++ins;
    }
    if (ins) atomicAdd(&st->insertions, (unsigned long long)ins);
    if (spl) atomicAdd(&st->splits, (unsigned long long)spl);
}

__global__ void k_finish(DmrArgs a) {
    DmrState *st = a.st;
    if (st->stop != STOP_NONE || st->tail) return;
    if (st->err) {
        st->stop = STOP_ERROR;
        return;
    }
    if (st->nw == 0) return;
    if (st->winners == 0) st->stop = STOP_STALLED;
    else if (!st->fits) st->stop = STOP_CAPACITY;
    else {
        st->npts += st->winners;
        st->ntri += st->added;
    }
}

/* ------------------------------------------------------------- the tail */

/* Once at most tail_max triangles are bad, one block runs whole rounds with
 * the same per-plan functions, separated by __syncthreads instead of kernel
 * boundaries, and builds the next worklist from the triangles the round can
 * have changed: the previous worklist (losers and failed plans stay bad),
 * the winners' rewritten cavity slots and the appended ones, each kept if
 * bad, sorted and made unique in shared memory.  That is every bad triangle
 * in ascending id, the same worklist a full compaction gives, so the rounds
 * equal the multi-kernel ones.  When the next worklist would exceed
 * tail_max the block hands back (tail = 0) and the full compaction resumes. */
__global__ void __launch_bounds__(TAIL_BS, 1) k_tail(DmrArgs a) {
    __shared__ uint32_t ws[32];
    __shared__ uint32_t srt[TAIL_SORT];
    __shared__ uint32_t s_cnt;
    DmrState *st = a.st;
    if (st->stop != STOP_NONE || !st->tail) return;
    const uint32_t tid = threadIdx.x, nthr = blockDim.x;
    uint32_t cav[CAV_MAX], slot[FAN_MAX], fa[FAN_MAX], fb[FAN_MAX];
    for (uint32_t guard = 0; guard <= MAX_ROUNDS; ++guard) {
        __syncthreads();
        const uint32_t nw = st->nw, ntri = st->ntri, npts = st->npts, round0 = st->round, err = st->err;
        __syncthreads(); /* every thread has read the state before thread 0 writes it */
        if (err) {
            if (tid == 0) st->stop = STOP_ERROR;
            return;
        }
        if (nw == 0) {
            if (tid == 0) st->stop = STOP_DONE;
            return;
        }
        if (round0 >= st->max_rounds) {
            if (tid == 0) st->stop = STOP_ROUNDS;
            return;
        }
        const uint32_t round = round0 + 1;
        if (tid == 0) st->round = round;
        uint32_t fails = 0;
        for (uint32_t k = tid; k < nw; k += nthr) fails += plan_one<false>(a, k, a.work[k], round, ntri, cav, fa);
        fails = block_sum(fails, ws);
        if (tid == 0 && fails) st->failed += fails;
        for (uint32_t k = tid; k < nw; k += nthr) resolve0_one(a, k, round);
        __syncthreads();
        for (uint32_t k = tid; k < nw; k += nthr) reclaim_one(a, k, round);
        __syncthreads();
        uint32_t W = 0, A = 0;
        for (uint32_t k0 = 0; k0 < nw; k0 += nthr) {
            const uint32_t k = k0 + tid;
            uint32_t win = 0, need = 0, wt, at;
            if (k < nw) win = resolve1_one(a, k, round, need);
            const uint32_t wpre = block_exclusive_scan(win, ws, &wt);
            const uint32_t apre = block_exclusive_scan(need, ws, &at);
            if (win) {
                a.wlist[W + wpre] = k;
                a.wtri[W + wpre] = ntri + A + apre;
            }
            W += wt;
            A += at;
        }
        __syncthreads();
        if (W == 0) {
            if (tid == 0) {
                st->winners = 0;
                st->stop = STOP_STALLED;
            }
            return;
        }
        if ((uint64_t)npts + W > st->pcap || (uint64_t)ntri + A > st->tcap) {
            if (tid == 0) {
                st->winners = W;
                st->added = A;
                st->stop = STOP_CAPACITY;
            }
            return;
        }
        uint32_t ins = 0, spl = 0;
        for (uint32_t i = tid; i < W; i += nthr) {
            if (commit_one(a, a.wlist[i], npts + i, a.wtri[i], slot, fa, fb)) ++spl;
            else ++ins;
        }
        ins = block_sum(ins, ws);
        spl = block_sum(spl, ws);
        /* the next worklist's candidates */
        if (tid == 0) s_cnt = 0;
        __syncthreads();
        for (uint32_t k = tid; k < nw; k += nthr) {
            const uint32_t t = a.work[k];
            if (a.bad[t]) {
                const uint32_t q = atomicAdd(&s_cnt, 1u);
                if (q < TAIL_SORT) srt[q] = t;
            }
        }
        for (uint32_t i = tid; i < W; i += nthr) {
            const uint32_t k = a.wlist[i], nc = (a.p_mode[k] >> 8) & 0xFF;
            for (uint32_t j = 0; j < nc; ++j) {
                const uint32_t t = a.p_cav[(size_t)j * a.B + k];
                if (a.bad[t]) {
                    const uint32_t q = atomicAdd(&s_cnt, 1u);
                    if (q < TAIL_SORT) srt[q] = t;
                }
            }
        }
        for (uint32_t t = ntri + tid; t < ntri + A; t += nthr)
            if (a.bad[t]) {
                const uint32_t q = atomicAdd(&s_cnt, 1u);
                if (q < TAIL_SORT) srt[q] = t;
            }
        __syncthreads();
        const uint32_t c = s_cnt;
        if (tid == 0) {
            st->npts = npts + W;
            st->ntri = ntri + A;
            st->winners = W;
            st->added = A;
            st->insertions += ins;
            st->splits += spl;
        }
        if (c > TAIL_SORT) { /* more than one block sorts: hand back */
            if (tid == 0) st->tail = 0;
            return;
        }
        uint32_t n2 = 1;
        while (n2 < c) n2 <<= 1;
        for (uint32_t i = c + tid; i < n2; i += nthr) srt[i] = NONE;
        __syncthreads();
        for (uint32_t kk = 2; kk <= n2; kk <<= 1) /* bitonic sort, ascending */
            for (uint32_t j = kk >> 1; j > 0; j >>= 1) {
                for (uint32_t i = tid; i < n2; i += nthr) {
                    const uint32_t ij = i ^ j;
                    if (ij > i) {
                        const uint32_t u = srt[i], v = srt[ij];
                        if ((u > v) == ((i & kk) == 0)) {
                            srt[i] = v;
                            srt[ij] = u;
                        }
                    }
                }
                __syncthreads();
            }
        uint32_t nn = 0;
        for (uint32_t i0 = 0; i0 < c; i0 += nthr) { /* unique, into the worklist */
            const uint32_t i = i0 + tid;
            const uint32_t keep = i < c && (i == 0 || srt[i] != srt[i - 1]);
            uint32_t tot;
            const uint32_t pos = block_exclusive_scan(keep, ws, &tot);
            if (keep) a.work[nn + pos] = srt[i];
            nn += tot;
        }
        if (tid == 0) {
            st->nw = nn;
            st->nbad = nn;
            if (nn > a.tail_max) st->tail = 0; /* the full compaction takes it from here */
        }
        if (nn > a.tail_max) return;
    }
}

struct DmrBufs {
    double *x = nullptr, *y = nullptr, *p_px = nullptr, *p_py = nullptr;
    float4 *pq = nullptr;
    uint32_t *tri = nullptr, *nbr = nullptr, *bad = nullptr, *work = nullptr, *p_mode = nullptr, *p_cav = nullptr,
             *p_win = nullptr, *bsum = nullptr, *lock = nullptr, *wlist = nullptr, *wtri = nullptr;
    uint4 *p_fan = nullptr;
    unsigned long long *owner = nullptr, *ring = nullptr;
    DmrState *st = nullptr;
    DmrState *hst = nullptr; /* pinned, owned by the context */
    void free_all(cudaStream_t s) {
        void *p[] = {x, y, pq, p_px, p_py, tri, nbr, bad, work, p_mode, p_cav, p_win, bsum, lock, wlist, wtri, p_fan, owner,
                     ring, st};
        for (void *q : p)
            if (q) cudaFreeAsync(q, s);
        cudaStreamSynchronize(s);
    }
};

/* Large copies between pageable host memory and the device go through two
 * pinned buffers kept in the context (pinned once, reused): host threads copy
 * one chunk while the DMA of the other runs (and take a fresh destination's
 * first-touch page faults in parallel).  The driver's own pageable path
 * ran at 150 GB/s in a fresh process but at about 10 GB/s late in a long one
 * that had page-locked gigabytes, which this path does not depend on. */
constexpr size_t STAGE_CHUNK = 32u << 20;

gga_status stage_ensure(gga_ctx *c) {
    if (c->stage_bytes >= 2 * STAGE_CHUNK) return GGA_OK;
    if (c->stage) cudaFreeHost(c->stage);
    c->stage = nullptr;
    c->stage_bytes = 0;
    GGA_CK(cudaMallocHost(&c->stage, 2 * STAGE_CHUNK));
    c->stage_bytes = 2 * STAGE_CHUNK;
    return GGA_OK;
}

unsigned stage_threads() {
    const unsigned hw = std::thread::hardware_concurrency();
    return std::max(1u, std::min(16u, hw ? hw / 2 : 4u));
}

void par_memcpy(char *to, const char *from, size_t len, unsigned nt) {
    const size_t per = (len + nt - 1) / nt;
    std::vector<std::thread> th;
    for (unsigned t = 1; t < nt && t * per < len; ++t)
        th.emplace_back([=] { memcpy(to + t * per, from + t * per, std::min(per, len - t * per)); });
    memcpy(to, from, std::min(per, len));
    for (auto &x : th) x.join();
}

/* Host-to-device: chunk i is copied into buffer i & 1 once that buffer's
 * previous DMA has finished, then sent.  The last DMAs may still run when
 * this returns; later work on `s` is ordered after them, and the next use of
 * a buffer waits for its event. */
gga_status copy_to_device(gga_ctx *c, cudaStream_t s, void *dst, const void *src, size_t bytes) {
    if (bytes < (8u << 20)) { /* small: the plain path */
        GGA_CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
        return GGA_OK;
    }
    gga_status r = stage_ensure(c);
    if (r) return r;
    cudaEvent_t done[2] = {c->ev[2], c->ev[3]};
    const size_t nchunk = (bytes + STAGE_CHUNK - 1) / STAGE_CHUNK;
    const unsigned nt = stage_threads();
    for (size_t i = 0; i < nchunk; ++i) {
        const size_t off = i * STAGE_CHUNK, len = std::min(STAGE_CHUNK, bytes - off);
        char *buf = (char *)c->stage + (i & 1) * STAGE_CHUNK;
        GGA_CK(cudaEventSynchronize(done[i & 1])); /* the buffer's previous DMA (this call or an earlier one) */
        par_memcpy(buf, (const char *)src + off, len, nt);
        GGA_CK(cudaMemcpyAsync((char *)dst + off, buf, len, cudaMemcpyHostToDevice, s));
        GGA_CK(cudaEventRecord(done[i & 1], s));
    }
    return GGA_OK;
}

/* Device-to-host: the DMA of chunk i + 1 runs while host threads copy chunk
 * i out of its buffer. */
gga_status copy_to_host(gga_ctx *c, cudaStream_t s, void *dst, const void *src, size_t bytes) {
    if (bytes < (8u << 20)) { /* small: the plain path */
        GGA_CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s));
        GGA_CK(cudaStreamSynchronize(s));
        return GGA_OK;
    }
    gga_status r = stage_ensure(c);
    if (r) return r;
    cudaEvent_t done[2] = {c->ev[2], c->ev[3]};
    const size_t nchunk = (bytes + STAGE_CHUNK - 1) / STAGE_CHUNK;
    const unsigned nt = stage_threads();
    auto issue = [&](size_t i) -> cudaError_t {
        const size_t off = i * STAGE_CHUNK, len = std::min(STAGE_CHUNK, bytes - off);
        cudaError_t e = cudaMemcpyAsync((char *)c->stage + (i & 1) * STAGE_CHUNK, (const char *)src + off, len,
                                        cudaMemcpyDeviceToHost, s);
        return e == cudaSuccess ? cudaEventRecord(done[i & 1], s) : e;
    };
    GGA_CK(issue(0));
    for (size_t i = 0; i < nchunk; ++i) {
        GGA_CK(cudaEventSynchronize(done[i & 1]));
        if (i + 1 < nchunk) GGA_CK(issue(i + 1)); /* buffer (i+1)&1 was drained in iteration i-1 */
        const size_t off = i * STAGE_CHUNK, len = std::min(STAGE_CHUNK, bytes - off);
        par_memcpy((char *)dst + off, (const char *)c->stage + (i & 1) * STAGE_CHUNK, len, nt);
    }
    return GGA_OK;
}

template <class T> gga_status dalloc(T **p, size_t n, cudaStream_t s) {
    GGA_CK(cudaMallocAsync((void **)p, (n ? n : 1) * sizeof(T), s));
    return GGA_OK;
}

gga_status refine_run(gga_ctx *c, gga_mesh *m, double cos_bound, uint32_t tcap, uint32_t bcap, uint32_t tail_max,
                      uint32_t pf_max, DmrBufs &b, gga_refine_stats *out) {
    cudaStream_t s = c->st;
    const uint32_t pcap = (uint32_t)(m->npts + (uint64_t)(tcap - m->ntri));
    const uint32_t B = bcap < tcap ? bcap : tcap;
    const uint32_t G = (uint32_t)(c->sms > 0 ? 2 * c->sms : 304);
    gga_status r;
    double tp = gga_now_ms();
    if ((r = dalloc(&b.x, pcap, s)) || (r = dalloc(&b.y, pcap, s)) || (r = dalloc(&b.pq, pcap, s)) || (r = dalloc(&b.tri, 3 * (size_t)tcap, s)) ||
        (r = dalloc(&b.nbr, 3 * (size_t)tcap, s)) || (r = dalloc(&b.bad, tcap, s)) ||
        (r = dalloc(&b.owner, tcap, s)) || (r = dalloc(&b.ring, tcap, s)) || (r = dalloc(&b.lock, tcap, s)) ||
        (r = dalloc(&b.wlist, B, s)) || (r = dalloc(&b.wtri, B, s)) || (r = dalloc(&b.work, B, s)) || (r = dalloc(&b.p_mode, B, s)) ||
        (r = dalloc(&b.p_px, B, s)) || (r = dalloc(&b.p_py, B, s)) || (r = dalloc(&b.p_cav, (size_t)CAV_MAX * B, s)) ||
        (r = dalloc(&b.p_fan, (size_t)FAN_MAX * B, s)) || (r = dalloc(&b.p_win, B, s)) ||
        (r = dalloc(&b.bsum, 3 * (size_t)G, s)) || (r = dalloc(&b.st, 1, s)))
        return r;
    if (!c->dmr_state) GGA_CK(cudaMallocHost(&c->dmr_state, sizeof(DmrState)));
    b.hst = (DmrState *)c->dmr_state;
    memset(b.hst, 0, sizeof(DmrState));
    b.hst->npts = m->npts;
    b.hst->ntri = m->ntri;
    b.hst->pcap = pcap;
    b.hst->tcap = tcap;
    b.hst->bcap = B;
    b.hst->max_rounds = MAX_ROUNDS;
    GGA_CK(cudaMemcpyAsync(b.st, b.hst, sizeof(DmrState), cudaMemcpyHostToDevice, s));
    GGA_CK(cudaMemsetAsync(b.owner, 0, (size_t)tcap * sizeof(unsigned long long), s));
    GGA_CK(cudaMemsetAsync(b.ring, 0, (size_t)tcap * sizeof(unsigned long long), s));
    GGA_CK(cudaMemsetAsync(b.lock, 0, (size_t)tcap * sizeof(uint32_t), s));
    GGA_CK(cudaMemsetAsync(b.bsum, 0, sizeof(uint32_t), s));
    GGA_CK(cudaStreamSynchronize(s));
    out->alloc_ms = gga_now_ms() - tp;
    tp = gga_now_ms();
    if ((r = copy_to_device(c, s, b.x, m->x, (size_t)m->npts * sizeof(double))) ||
        (r = copy_to_device(c, s, b.y, m->y, (size_t)m->npts * sizeof(double))) ||
        (r = copy_to_device(c, s, b.tri, m->tri, (size_t)m->ntri * 3 * sizeof(uint32_t))) ||
        (r = copy_to_device(c, s, b.nbr, m->nbr, (size_t)m->ntri * 3 * sizeof(uint32_t))))
        return r;

    DmrArgs a;
    a.x = b.x;
    a.y = b.y;
    a.pq = b.pq;
    a.tri = b.tri;
    a.nbr = b.nbr;
    a.bad = b.bad;
    a.owner = b.owner;
    a.ring = b.ring;
    a.lock = b.lock;
    a.wlist = b.wlist;
    a.wtri = b.wtri;
    a.work = b.work;
    a.p_mode = b.p_mode;
    a.p_px = b.p_px;
    a.p_py = b.p_py;
    a.p_cav = b.p_cav;
    a.p_fan = b.p_fan;
    a.p_win = b.p_win;
    a.bsum = b.bsum;
    a.st = b.st;
    a.cos_bound = cos_bound;
    a.cos_bound_f = (float)cos_bound;
    a.S = 0.0f; /* set from k_shadow's bound below; no kernel before it reads S */
    a.B = B;
    a.G = G;
    a.tail_max = tail_max == 0xFFFFFFFFu ? 0u : min(min(tail_max ? tail_max : TAIL_MAX, TAIL_SORT), B);
    a.pf_max = pf_max ? pf_max : PF_MAX;
    const unsigned plan_grid = ctx_grid(c, B, PLAN_BS);
    cudaEvent_t e0 = c->ev[0], e1 = c->ev[1];
    /* the float pairs and the coordinate bound S (read back: it is a launch
     * argument of every later kernel) */
    k_shadow<<<G, SCAN_BS, 0, s>>>(a, b.bsum);
    GGA_CK(cudaMemcpyAsync(&b.hst->pad_s, b.bsum, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    GGA_CK(cudaStreamSynchronize(s));
    out->upload_ms = gga_now_ms() - tp;
    {
        float sm;
        memcpy(&sm, &b.hst->pad_s, sizeof sm);
        a.S = sm * (1.0f + 1.0f / 1048576.0f) + 1e-30f;
    }
    GGA_CK(cudaEventRecord(e0, s));
    k_mark_all<<<G, SCAN_BS, 0, s>>>(a);
    for (uint32_t issued = 0;;) {
        for (uint32_t g = 0; g < ROUND_GROUP; ++g) {
            k_bad_count<<<G, SCAN_BS, 0, s>>>(a);
            k_bad_gather<<<G, SCAN_BS, 0, s>>>(a);
            k_decide<<<1, 32, 0, s>>>(a);
            k_plan<false><<<plan_grid, PLAN_BS, 0, s>>>(a);
            k_plan<true><<<plan_grid, PLAN_BS, 0, s>>>(a);
            k_resolve0<<<plan_grid, PLAN_BS, 0, s>>>(a);
            k_reclaim<<<plan_grid, PLAN_BS, 0, s>>>(a);
            k_resolve1<<<G, SCAN_BS, 0, s>>>(a);
            k_compact<<<G, SCAN_BS, 0, s>>>(a);
            k_commit<<<plan_grid, PLAN_BS, 0, s>>>(a);
            k_finish<<<1, 1, 0, s>>>(a);
        }
        GGA_CK(cudaGetLastError());
        issued += ROUND_GROUP;
        GGA_CK(cudaMemcpyAsync(b.hst, b.st, sizeof(DmrState), cudaMemcpyDeviceToHost, s));
        GGA_CK(cudaStreamSynchronize(s));
        if (b.hst->stop == STOP_NONE && b.hst->tail) {
            k_tail<<<1, TAIL_BS, 0, s>>>(a);
            GGA_CK(cudaGetLastError());
            GGA_CK(cudaMemcpyAsync(b.hst, b.st, sizeof(DmrState), cudaMemcpyDeviceToHost, s));
            GGA_CK(cudaStreamSynchronize(s));
        }
        if (b.hst->stop != STOP_NONE || issued > MAX_ROUNDS + ROUND_GROUP) break;
    }
    GGA_CK(cudaEventRecord(e1, s));
    const DmrState h = *b.hst;
    if (h.err || h.stop == STOP_ERROR)
        return gga_fail(GGA_ERR_FORMAT, "mesh refinement: a triangle or neighbour id out of range");
    tp = gga_now_ms();
    if ((r = gga_mesh_resize(m, h.npts, h.ntri))) return r;
    if ((r = copy_to_host(c, s, m->x, b.x, (size_t)h.npts * sizeof(double))) ||
        (r = copy_to_host(c, s, m->y, b.y, (size_t)h.npts * sizeof(double))) ||
        (r = copy_to_host(c, s, m->tri, b.tri, (size_t)h.ntri * 3 * sizeof(uint32_t))) ||
        (r = copy_to_host(c, s, m->nbr, b.nbr, (size_t)h.ntri * 3 * sizeof(uint32_t))))
        return r;
    out->download_ms = gga_now_ms() - tp;
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    out->triangles_out = h.ntri;
    out->points_out = h.npts;
    out->bad_in = h.bad_in;
    out->bad_out = h.nbad;
    out->rounds = h.round;
    out->insertions = h.insertions;
    out->boundary_splits = h.splits;
    out->failed_plans = h.failed;
    out->device_ms = ms;
    switch (h.stop) {
    case STOP_DONE: return GGA_OK;
    case STOP_CAPACITY:
        return gga_fail(GGA_ERR_TOO_LARGE, "mesh refinement: round %u needs more than %u triangles", h.round, tcap);
    case STOP_STALLED:
        return gga_fail(GGA_ERR_NO_PROGRESS, "mesh refinement: every plan of round %u failed (%u bad left)", h.round,
                        h.nbad);
    case STOP_ROUNDS:
        return gga_fail(GGA_ERR_NO_PROGRESS, "mesh refinement: %u rounds, %u bad left", h.round, h.nbad);
    case STOP_ERROR:
        return gga_fail(GGA_ERR_FORMAT, "mesh refinement: a triangle or neighbour id out of range");
    default: return gga_fail(GGA_ERR_NO_PROGRESS, "mesh refinement: round limit");
    }
}

} // namespace

extern "C" gga_status gga_mesh_refine_ex(gga_ctx *c, gga_mesh *m, const gga_refine_params *p,
                                         gga_refine_stats *st) {
    const double t0 = gga_now_ms();
    if (!c || !m || !p) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    double min_angle_deg = p->min_angle_deg;
    if (!(min_angle_deg < 60.0)) return gga_fail(GGA_ERR_INVALID_ARG, "min angle %g (must be below 60)", min_angle_deg);
    if (min_angle_deg <= 0) min_angle_deg = GGA_DMR_MIN_ANGLE;
    const uint32_t max_triangles = p->max_triangles, batch_cap = p->batch_cap;
    const uint64_t dflt = 4ull * m->ntri + 65536;
    const uint64_t tcap64 = max_triangles ? max_triangles : (dflt < 0x3FFFFFFFull ? dflt : 0x3FFFFFFFull);
    if (tcap64 < m->ntri) return gga_fail(GGA_ERR_INVALID_ARG, "max_triangles %u < %u", max_triangles, m->ntri);
    if ((uint64_t)m->npts + (tcap64 - m->ntri) >= NONE)
        return gga_fail(GGA_ERR_TOO_LARGE, "mesh capacity of %llu triangles", (unsigned long long)tcap64);
    gga_refine_stats local;
    gga_refine_stats *out = st ? st : &local;
    memset(out, 0, sizeof *out);
    out->triangles_in = m->ntri;
    std::lock_guard<std::mutex> lk(c->mu);
    gga_status s;
    if ((s = ctx_activate(c))) return s;
    DmrBufs b;
    s = refine_run(c, m, cos(min_angle_deg * (3.14159265358979323846 / 180.0)), (uint32_t)tcap64,
                   batch_cap ? batch_cap : (1u << 20), p->tail_max, p->prefetch_max, b, out);
    b.free_all(c->st);
    out->total_ms = gga_now_ms() - t0;
    return s;
}

extern "C" gga_status gga_mesh_refine(gga_ctx *c, gga_mesh *m, double min_angle_deg, uint32_t max_triangles,
                                      uint32_t batch_cap, gga_refine_stats *st) {
    gga_refine_params p;
    memset(&p, 0, sizeof p);
    p.min_angle_deg = min_angle_deg;
    p.max_triangles = max_triangles;
    p.batch_cap = batch_cap;
    return gga_mesh_refine_ex(c, m, &p, st);
}
