/*
 * CPU emulation of the CUDA constructs the persistent kernels use, so the
 * kernels' own source text can run on the host against the oracle.
 *
 * Every CUDA thread is a std::thread; __syncthreads is a per-block
 * std::barrier that also checks every thread arrived from the same call
 * site; warp collectives (ballot, shuffles) exchange values through a
 * per-warp barrier, so a collective reached by only part of a warp hangs the
 * emulation instead of passing silently.  Shared-memory statics become
 * per-block instances through a BLK template parameter that
 * gen_kernels.py adds to each kernel; dynamic shared memory is a per-block
 * array.  Atomics are sequentially consistent host atomics and grid barriers
 * run on real host threads, so the blocks of a "launch" interleave freely.
 * A watchdog reports the source line each thread waits on if a launch does
 * not finish.
 */
#pragma once
#include <algorithm>
#include <atomic>
#include <cmath>
#include <barrier>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <string>
#include <thread>
#include <vector>
#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __launch_bounds__(...)
#define __restrict__
#define __shared__ static
struct dim3e { uint32_t x = 0, y = 0, z = 0; };
thread_local dim3e threadIdx, blockIdx;
dim3e blockDim, gridDim;
int g_line[8][1024];
#define MARKL(l) (g_line[blockIdx.x][threadIdx.x] = (l))
static std::barrier<> *g_block_bars[8];
struct WarpCtx { std::barrier<> *bar; uint64_t slot[32]; };
static WarpCtx *g_warps[8];
/* Every thread of a block must meet each __syncthreads at the same call
 * site; a thread that reaches another one (a barrier skipped or taken twice
 * on one path) stops the emulation with both source lines.  Slots alternate
 * by barrier phase, so thread 0 cannot overwrite the slot being checked. */
static int g_arrive_line[8][2][1024];
thread_local unsigned g_sync_phase;
inline void sync_threads_impl(int l) {
    MARKL(l);
    const unsigned p = g_sync_phase++ & 1u;
    g_arrive_line[blockIdx.x][p][threadIdx.x] = l;
    g_block_bars[blockIdx.x]->arrive_and_wait();
    const int l0 = g_arrive_line[blockIdx.x][p][0];
    if (l0 != l) {
        printf("BARRIER MISMATCH block %u thread %u at line %d, thread 0 at line %d\n", blockIdx.x, threadIdx.x, l, l0);
        fflush(stdout);
        _exit(4);
    }
    MARKL(-l);
}
#define __syncthreads() sync_threads_impl(__LINE__)
inline WarpCtx &wc() { return g_warps[blockIdx.x][threadIdx.x / 32]; }
template <class T> inline T xchg_all(T v, std::function<T(WarpCtx &, unsigned)> f) {
    WarpCtx &w = wc(); unsigned lane = threadIdx.x & 31;
    uint64_t raw = 0; memcpy(&raw, &v, sizeof(T)); w.slot[lane] = raw;
    w.bar->arrive_and_wait();
    T r = f(w, lane);
    w.bar->arrive_and_wait();
    return r;
}
inline unsigned ballot_impl(unsigned, bool p, int l) {
    MARKL(l);
    return xchg_all<unsigned>(p ? 1u : 0u, [](WarpCtx &w, unsigned) { unsigned m = 0; for (int i = 0; i < 32; ++i) if (w.slot[i]) m |= 1u << i; return m; });
}
template <class T> inline T shfl_impl(unsigned, T v, int src, int l) {
    MARKL(l);
    return xchg_all<T>(v, [src](WarpCtx &w, unsigned) { T r; uint64_t raw = w.slot[src]; memcpy(&r, &raw, sizeof(T)); return r; });
}
template <class T> inline T shfl_up_impl(unsigned, T v, int d, int l) {
    MARKL(l);
    return xchg_all<T>(v, [d](WarpCtx &w, unsigned lane) { int s = (int)lane - d; if (s < 0) s = lane; T r; uint64_t raw = w.slot[s]; memcpy(&r, &raw, sizeof(T)); return r; });
}
template <class T> inline T shfl_down_impl(unsigned, T v, int d, int l) {
    MARKL(l);
    return xchg_all<T>(v, [d](WarpCtx &w, unsigned lane) { int s = (int)lane + d; if (s > 31) s = lane; T r; uint64_t raw = w.slot[s]; memcpy(&r, &raw, sizeof(T)); return r; });
}
#define __ballot_sync(m, p) ballot_impl(m, p, __LINE__)
#define __shfl_sync(m, v, s) shfl_impl(m, v, s, __LINE__)
#define __shfl_up_sync(m, v, d) shfl_up_impl(m, v, d, __LINE__)
#define __shfl_down_sync(m, v, d) shfl_down_impl(m, v, d, __LINE__)
inline int __popc(unsigned x) { return __builtin_popcount(x); }
inline int __popcll(unsigned long long x) { return __builtin_popcountll(x); }
inline int __ffs(unsigned x) { return __builtin_ffs(x); }
inline int __ffsll(long long x) { return __builtin_ffsll(x); }
template <class T> T atomicAdd(T *p, T v) { return __atomic_fetch_add(p, v, __ATOMIC_SEQ_CST); }
inline unsigned atomicOr(unsigned *p, unsigned v) { return __atomic_fetch_or(p, v, __ATOMIC_SEQ_CST); }
inline unsigned long long atomicOr(unsigned long long *p, unsigned long long v) { return __atomic_fetch_or(p, v, __ATOMIC_SEQ_CST); }
inline unsigned atomicAnd(unsigned *p, unsigned v) { return __atomic_fetch_and(p, v, __ATOMIC_SEQ_CST); }
inline unsigned atomicExch(unsigned *p, unsigned v) { return __atomic_exchange_n(p, v, __ATOMIC_SEQ_CST); }
inline unsigned atomicMin(unsigned *p, unsigned v) { unsigned o = __atomic_load_n(p, __ATOMIC_SEQ_CST); while (v < o && !__atomic_compare_exchange_n(p, &o, v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST)) {} return o; }
inline unsigned long long atomicMax(unsigned long long *p, unsigned long long v) { unsigned long long o = __atomic_load_n(p, __ATOMIC_SEQ_CST); while (v > o && !__atomic_compare_exchange_n(p, &o, v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST)) {} return o; }
inline unsigned atomicMax(unsigned *p, unsigned v) { unsigned o = __atomic_load_n(p, __ATOMIC_SEQ_CST); while (v > o && !__atomic_compare_exchange_n(p, &o, v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST)) {} return o; }
inline float __double2float_ru(double x) { float f = (float)x; if ((double)f < x) f = std::nextafter(f, INFINITY); return f; }
inline unsigned __float_as_uint(float f) { unsigned u; memcpy(&u, &f, 4); return u; }
inline float __uint_as_float(unsigned u) { float f; memcpy(&f, &u, 4); return f; }
inline unsigned atomicCAS(unsigned *p, unsigned c, unsigned v) { __atomic_compare_exchange_n(p, &c, v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST); return c; }
template <class T> T __ldg(const T *p) { return *p; }
template <class T> T __ldcg(const T *p) { return __atomic_load_n(p, __ATOMIC_SEQ_CST); }
inline void __threadfence() { __atomic_thread_fence(__ATOMIC_SEQ_CST); }
inline void __nanosleep(unsigned) { std::this_thread::yield(); }
inline long long clock64() { return std::chrono::steady_clock::now().time_since_epoch().count(); }
using std::min; using std::max;
inline uint32_t min(uint32_t a, uint32_t b) { return a < b ? a : b; }
inline uint32_t max(uint32_t a, uint32_t b) { return a > b ? a : b; }
#define GGA_INFINITY 1000000000u
#define GGA_MESH_NONE 0xFFFFFFFFu
struct uint4 { uint32_t x, y, z, w; };
struct float4 { float x, y, z, w; };
inline float4 make_float4(float x, float y, float z, float w) { return float4{x, y, z, w}; }
inline uint4 make_uint4(uint32_t x, uint32_t y, uint32_t z, uint32_t w) { return uint4{x, y, z, w}; }
enum { GGA_BFS = 0, GGA_SSSP = 1 };
inline uint32_t ld_acquire_u32(const uint32_t *p) { return __atomic_load_n(p, __ATOMIC_ACQUIRE); }
inline uint32_t ld_relaxed_u32(const uint32_t *p) { return __atomic_load_n(p, __ATOMIC_RELAXED); }
inline void red_min_u32(uint32_t *p, uint32_t v) { atomicMin(p, v); }
inline unsigned long long ld_relaxed_u64(const unsigned long long *p) { return __atomic_load_n(p, __ATOMIC_RELAXED); }
inline uint64_t global_timer_ns() { return std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now().time_since_epoch()).count(); }
inline uint32_t lane_id() { return threadIdx.x & 31u; }
inline uint32_t lanemask_lt() { return (1u << (threadIdx.x & 31u)) - 1u; }
inline uint32_t atom_add_acq_rel_u32(uint32_t *p, uint32_t v) { return __atomic_fetch_add(p, v, __ATOMIC_ACQ_REL); }
uint32_t g_dyn[8][1 << 16];
constexpr uint32_t LH_CLASSES = 15; /* heavy-edge weight classes of the light/heavy row order */
enum : uint32_t { GGA_DEV_OK = 0, GGA_DEV_TIMEOUT = 1, GGA_DEV_OVERFLOW = 2, GGA_DEV_SPLIT_RULE = 3,
                  GGA_DEV_OVERFLOW_UNITS = 4, GGA_DEV_OVERFLOW_FAR = 5, GGA_DEV_BAD_EDGE = 6, GGA_DEV_ROUND_LIMIT = 7,
                  GGA_DEV_BAD_TARGET = 8 };
struct GridBarrier { uint32_t count; uint32_t pad; };
/* Runs NB blocks of BS threads of fn(block); exits 2 with a per-thread line
 * map if they do not all finish within limit_s. */
template <class F> void run_grid(int NB, int BS, F fn, int limit_s = 600) {
    blockDim.x = BS; gridDim.x = NB;
    for (int b = 0; b < NB; ++b) {
        g_block_bars[b] = new std::barrier<>(BS);
        g_warps[b] = new WarpCtx[BS / 32];
        for (int w = 0; w < BS / 32; ++w) g_warps[b][w].bar = new std::barrier<>(32);
    }
    std::atomic<int> done{0};
    std::vector<std::thread> th;
    for (int b = 0; b < NB; ++b)
        for (int t = 0; t < BS; ++t)
            th.emplace_back([&, t, b] { threadIdx.x = t; blockIdx.x = b; fn(b); done++; });
    auto t0 = std::chrono::steady_clock::now();
    while (done.load() < BS * NB) {
        std::this_thread::sleep_for(std::chrono::milliseconds(20));
        if (std::chrono::steady_clock::now() - t0 > std::chrono::seconds(limit_s)) {
            printf("HANG\n");
            for (int b = 0; b < NB; ++b) { printf("block %d:", b); for (int t = 0; t < BS; t += 8) printf(" %d", g_line[b][t]); printf("\n"); }
            fflush(stdout); _exit(2);
        }
    }
    for (auto &x : th) x.join();
}
static std::vector<uint32_t> rd(const std::string &p) {
    std::ifstream f(p, std::ios::binary); f.seekg(0, std::ios::end); size_t n = f.tellg() / 4; f.seekg(0);
    std::vector<uint32_t> v(n); f.read((char *)v.data(), n * 4); return v;
}
