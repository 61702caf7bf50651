/*
 * gga.h — C ABI of the GB300-native static-graph BFS/SSSP engine.
 *
 * The reference (GPUGraphAlgo, Programs/CUDA_src/Kepler_BFS_SSSP/) exposes no
 * library: its surface is the `Graph` struct (graph.h:23-64), its host methods,
 * the relax kernels (cudaKernels.h) and the fixed-point loop in main()
 * (bfs_sssp.cu:103-539).  Every entry point below names the reference item it
 * replaces.  Conventions that differ from the reference on purpose:
 *   - every call returns a gga_status; nothing calls exit() or abort()
 *     (the reference exits in CudaTest, graph.h:523-533, and aborts on mmap
 *     failure, graph.h:614,627);
 *   - the caller owns output buffers; the library owns graph and device state;
 *   - the source vertex is a parameter (the reference hard-codes original
 *     vertex 0, bfs_sssp.cu:203);
 *   - distance outputs hold one value per ORIGINAL vertex in original order,
 *     which is exactly what Ary2File writes (parents only, myutils.h:51-62).
 * Distances are uint32 with GGA_INFINITY (= MYINFINITY, bfs_sssp.cu:53) for
 * unreachable vertices.  BFS distances are levels (every edge weight taken as 1).
 *
 * Threading: one gga_ctx per host thread; calls on different contexts may run
 * concurrently.  A gga_graph may be shared by contexts on the same device.
 */
#ifndef GGA_H
#define GGA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GGA_INFINITY 1000000000u /* MYINFINITY, bfs_sssp.cu:53 / graph.h:96 */
#define GGA_MSBFS_MAX_SOURCES 64 /* one uint64 lane word per vertex */
#define GGA_SSSP_BATCH_MAX_SOURCES 32 /* one warp lane per source */
/* Largest edge weight for which dist + weight cannot wrap in uint32 while
 * dist <= GGA_INFINITY; heavier weights are rejected (the reference's unsigned
 * arithmetic would wrap, bfs_sssp.cu/cudaKernels.h:323). */
#define GGA_MAX_WEIGHT (0xFFFFFFFFu - GGA_INFINITY)

typedef enum gga_status {
    GGA_OK = 0,
    GGA_ERR_INVALID_ARG = 1, /* bad pointer, size or enum */
    GGA_ERR_IO = 2,          /* open/read/write failed (readFromGR returns 1) */
    GGA_ERR_FORMAT = 3,      /* malformed .gr (bad version, truncated, dst >= n) */
    GGA_ERR_SPLIT_RULE = 4,  /* histogram rule gave MDA 0: the reference divides by zero */
    GGA_ERR_NO_MEMORY = 5,   /* host allocation failed */
    GGA_ERR_CUDA = 6,        /* a CUDA runtime call failed (message via gga_last_error) */
    GGA_ERR_NO_DEVICE = 7,   /* no CUDA device / extension unusable */
    GGA_ERR_TIMEOUT = 8,     /* a bounded device-side wait ran out; context stays usable */
    GGA_ERR_ADMISSION = 9,   /* request exceeds the configured device-memory cap */
    GGA_ERR_TOO_LARGE = 10,  /* graph exceeds the limits: 2^31 vertices, 2^32 - 8192 edges */
    GGA_ERR_NOT_READY = 11,  /* serving ticket not finished yet */
    GGA_ERR_UNSUPPORTED = 12,
    GGA_ERR_NO_PROGRESS = 13 /* mesh refinement: every remaining insertion failed, or the round cap */
} gga_status;

typedef enum gga_algo { GGA_BFS = 0, GGA_SSSP = 1 } gga_algo;

/* Relaxation engine.  All variants return identical distances. */
typedef enum gga_variant {
    GGA_VARIANT_AUTO = 0,        /* frontier engine with autotuned parameters */
    GGA_VARIANT_FRONTIER = 1,    /* data-driven frontier, persistent kernel, CTA-cooperative expansion */
    GGA_VARIANT_TOPO_ATOMIC = 2, /* "na_" build: M_my_drelax, cudaKernels.h:285-344 */
    GGA_VARIANT_TOPO_PLAIN = 3,  /* "n_" build: my_updateDist + my_drelax_no_atomic, cudaKernels.h:129-220 */
    GGA_VARIANT_CDP_ATOMIC = 4,  /* "da_" build: my_drelax_dynamicP, cudaKernels.h:438-520 (CDP2) */
    GGA_VARIANT_CDP_PLAIN = 5    /* "d_" build: as da_ with plain stores */
} gga_variant;

typedef struct gga_graph gga_graph;
typedef struct gga_ctx gga_ctx;

/* Per-call statistics (the reference's SResult, graph.h:66-84, plus work counters). */
typedef struct gga_stats {
    uint32_t iterations;       /* fixed-point iterations / BFS levels / near-far rounds */
    uint32_t kernel_launches;  /* kernels this call launched from the host */
    uint64_t vertices_reached; /* original vertices with dist < GGA_INFINITY */
    uint64_t edges_reached;    /* E_r: sum of out-degrees of reached original vertices */
    uint64_t edges_relaxed;    /* edge visits actually performed (work, >= E_r for SSSP) */
    uint32_t cdp_children;     /* device-side launches made by CDP variants */
    uint32_t cdp_fallbacks;    /* inline relaxations after a failed device launch */
    double kernel_ms;          /* device time of the relax kernels (ktime) by CUDA events */
    double aux_ms;             /* child-distance update time (sktime) */
    double total_ms;           /* whole call, host wall clock, copies included */
} gga_stats;

/* Read-only description of a graph and of its node split. */
typedef struct gga_graph_info {
    uint32_t nnodes;       /* vertices after split (== nodes_orig when not split) */
    uint32_t nodes_orig;   /* vertices before split (nodes_b4_ns) */
    uint32_t nedges;       /* directed edges (unchanged by the split) */
    uint32_t maxdeg;       /* getMaxdeg of the unsplit graph */
    int32_t split_level;   /* 0 = not split */
    int32_t split_buckets; /* histogram buckets used when split_level < 0 */
    uint32_t mda;          /* MAX_EDGES_ALLOWED of the split (0 when not split) */
    uint32_t parents_with_children; /* myParentCount, bfs_sssp.cu:257-262 */
    uint32_t max_weight;
    int32_t symmetric;     /* 1 symmetric (generated, or checked on the device), -1 checked: not
                            * symmetric or rows unsorted, 0 not known yet */
    int32_t wsymmetric;    /* the same, and every edge's reverse has its weight (what a
                            * pulling SSSP bucket close needs) */
} gga_graph_info;

/* ---- errors ----------------------------------------------------------- */
const char *gga_status_string(gga_status s);
/* Message of the last failing call on this host thread (never NULL). */
const char *gga_last_error(void);
/* Library version string. */
const char *gga_version(void);

/* ---- host graph (graph.h: struct Graph, L0) ----------------------------- */

/* Graph::readFromGR, graph.h:599-682.  Galois .gr v1: u64 header
 * {version=1, sizeEdgeTy, n, m}, u64 outIdx[n] (end offsets), u32 outs[m],
 * 4-byte pad when m is odd, u32 edgeData[m] (always read as u32, as the
 * reference does, graph.h:644,672). */
gga_status gga_graph_load_gr(const char *path, gga_graph **out);
/* Writes the same format with 4-byte weights. */
gga_status gga_graph_save_gr(const gga_graph *g, const char *path);
/* Builds a graph from a 0-based CSR: offsets[n+1], cols[m], weights[m]
 * (weights NULL = all 1).  Arrays are copied. */
gga_status gga_graph_from_csr(uint32_t n, uint32_t m, const uint32_t *offsets,
                              const uint32_t *cols, const uint32_t *weights,
                              gga_graph **out);
/* Seeded R-MAT (a, b, c; d = 1-a-b-c) with 2^scale vertices and
 * edge_factor * 2^scale generated edges; symmetrised, self-loops and
 * duplicates removed, vertex ids randomly permuted; weights uniform in
 * [wmin, wmax], equal in both directions. */
gga_status gga_graph_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b,
                              double c, uint64_t seed, uint32_t wmin, uint32_t wmax,
                              gga_graph **out);
/* Seeded width x height 4-neighbour grid, row-major ids; each undirected grid
 * edge deleted with probability del_prob; plus round(longrange_frac * grid
 * edges) random undirected long-range edges; weights uniform in [wmin, wmax]. */
gga_status gga_graph_gen_grid(uint32_t width, uint32_t height, double del_prob,
                              double longrange_frac, uint64_t seed, uint32_t wmin,
                              uint32_t wmax, gga_graph **out);
void gga_graph_free(gga_graph *g);
gga_status gga_graph_get_info(const gga_graph *g, gga_graph_info *info);
/* Borrowed pointers to the unsplit 0-based host CSR (valid until free). */
gga_status gga_graph_csr(const gga_graph *g, const uint32_t **offsets, const uint32_t **cols,
                         const uint32_t **weights);

/* ---- node split (graph.h L1) --------------------------------------------- */

/* Graph::getMaxdeg, graph.h:338-347. */
gga_status gga_max_degree(const gga_graph *g, uint32_t *maxdeg);
/* Graph::getMaxAllowedOutDegree, graph.h:359-385 (degree histogram rule). */
gga_status gga_max_allowed_out_degree(const gga_graph *g, int32_t buckets, uint32_t *mda);
/* Graph::getSizeafterLoadBalance, graph.h:386-414: MDA and the split vertex
 * count for `level` (>0: ceil(maxdeg/level); <0: histogram rule). */
gga_status gga_size_after_split(const gga_graph *g, int32_t level, int32_t buckets,
                                uint32_t *mda, uint32_t *new_nnodes);
/* Graph::NodeSplit, graph.h:415-522, built by device kernels on ctx's GPU.
 * level 0 removes any split.  Returns GGA_ERR_SPLIT_RULE where the reference
 * would divide by zero.  The split graph stays resident on the device. */
gga_status gga_node_split(gga_ctx *ctx, gga_graph *g, int32_t level, int32_t buckets);
/* Copies the split graph out in the reference's own layout (1-based psrc with
 * psrc[n'] = nedges, graph.h:498; edgessrcdst[0] null slot).  Any pointer may
 * be NULL.  Sizes: psrc n'+1, noutgoing/child_count/is_parent/parent_node n',
 * edgessrcdst m+1. */
gga_status gga_graph_split_maps(gga_ctx *ctx, const gga_graph *g, uint32_t *psrc,
                                uint32_t *noutgoing, uint32_t *edgessrcdst,
                                uint32_t *child_count, uint32_t *is_parent,
                                uint32_t *parent_node);
/* myChildIndex / myChildCount, bfs_sssp.cu:256-283: parents that have
 * children (ascending split id) and their child counts.  `count` in/out:
 * capacity in, number of parents out. */
gga_status gga_child_index(gga_ctx *ctx, const gga_graph *g, uint32_t *count,
                           uint32_t *child_index, uint32_t *child_count);

/* ---- device context (graph.h L2) ---------------------------------------- */

gga_status gga_ctx_create(int device, gga_ctx **out);
void gga_ctx_destroy(gga_ctx *ctx);
/* Graph::cudaCopy, graph.h:683-699: uploads g (done lazily by the solvers). */
gga_status gga_graph_upload(gga_ctx *ctx, gga_graph *g);
/* Number of SMs and device name of ctx's GPU. */
gga_status gga_ctx_device_info(gga_ctx *ctx, int *sm_count, char *name, size_t name_len);
/* CUDA-event timing on ctx's stream (the stream every solve launches on):
 * gga_ctx_mark records event `slot` (0..7); gga_ctx_elapsed waits for slot b
 * and returns the milliseconds between slots a and b. */
gga_status gga_ctx_mark(gga_ctx *ctx, int slot);
gga_status gga_ctx_elapsed(gga_ctx *ctx, int a, int b, double *ms);
gga_status gga_ctx_synchronize(gga_ctx *ctx);
/* Page-locks (pin != 0) or unlocks the host CSR so uploads run at full
 * host-to-device bandwidth. */
gga_status gga_graph_pin(gga_graph *g, int pin);
/* Drops the device copy (and split); the next solve uploads again. */
gga_status gga_graph_release_device(gga_graph *g);
/* Uploads g when needed (Graph::cudaCopy, graph.h:683-699) and builds what
 * the frontier engine derives from it once per graph for `algo` under ctx's
 * current parameters: the device symmetry check that bottom-up BFS rounds
 * and pulled SSSP bucket closes rely on, and SSSP's light-first row order
 * for the bucket width in use.  The first solve does the same when this was
 * not called; calling it first takes that one-time work out of the solve. */
gga_status gga_graph_prepare(gga_ctx *ctx, gga_graph *g, gga_algo algo);

/* ---- single-source solve (bfs_sssp.cu:372-468 loop, L3/L4) -------------- */

/* dist_out: host or device buffer of nodes_orig uint32, or NULL to leave the
 * result in the context's device buffer (until its next solve).  stats may
 * be NULL. */
gga_status gga_bfs(gga_ctx *ctx, gga_graph *g, uint32_t src, gga_variant variant,
                   uint32_t *dist_out, gga_stats *stats);
gga_status gga_sssp(gga_ctx *ctx, gga_graph *g, uint32_t src, gga_variant variant,
                    uint32_t *dist_out, gga_stats *stats);
gga_status gga_solve(gga_ctx *ctx, gga_graph *g, gga_algo algo, uint32_t src,
                     gga_variant variant, uint32_t *dist_out, gga_stats *stats);

/* n single-source traversals of g on the frontier engine, one after
 * another; row i of dist_out (n rows of nodes_orig uint32, host or device
 * memory) receives source srcs[i]'s distances, copied on a second stream
 * while the next traversal runs.  Distances and per-source stats are those
 * of n gga_solve calls with GGA_VARIANT_FRONTIER (stats: NULL or n entries;
 * total_ms is the call's wall time / n).  With pageable host memory each
 * copy blocks the host, so use gga_host_alloc memory for the overlap.  No
 * counterpart in the reference, whose executables run one source per
 * process (bfs_sssp.cu:149-330). */
gga_status gga_solve_many(gga_ctx *ctx, gga_graph *g, gga_algo algo, uint32_t n, const uint32_t *srcs,
                          uint32_t *dist_out, gga_stats *stats);
/* Page-locked host memory, e.g. for gga_solve_many's dist_out. */
gga_status gga_host_alloc(size_t bytes, void **out);
void gga_host_free(void *p);

/* Frontier-engine parameters (picked by gga_autotune when not set). */
typedef struct gga_params {
    uint32_t block_threads;  /* CTA size: 256, 512 or 1024 */
    uint32_t unit_iters;     /* edges per work unit = block_threads x this (2..16; 0 = 4096 / block_threads for
                              * BFS, 4 for SSSP) */
    uint32_t sssp_delta;     /* near-far bucket width (0 = plain improved-vertex frontier) */
    uint32_t use_split;      /* 1: the frontier engine expands over the node-split graph when one exists;
                              * 0 (default): over the unsplit CSR, which its edge-balanced units need
                              * no split for (same distances, faster) */
    uint32_t blocks_per_sm;  /* persistent grid = SMs x this (0 = occupancy maximum) */
    /* CDP variants: heavy-vertex threshold as bfs_sssp.cu:224-236 derives it
     * (level > 0: ceil(maxdeg/level); level < 0: histogram rule with buckets) */
    int32_t cdp_level;
    int32_t cdp_buckets;
    /* 0: one CDP2 tail launch per iteration over all heavy vertices;
     * 1: one fire-and-forget <<<1,32>>> child per heavy vertex (the
     *    reference's dynamicP_relax_coal shape); 2: no device launches */
    uint32_t cdp_mode;
    uint32_t cdp_pending_limit; /* cudaLimitDevRuntimePendingLaunchCount to set (0 = leave) */
    uint32_t skip_reached;      /* 1: gga_stats leaves vertices/edges_reached 0 (saves one launch) */
    /* BFS direction: 0 = top-down rounds plus bottom-up rounds (unvisited
     * vertices look for a parent in the frontier) chosen per round by Beamer's
     * rule, on symmetric graphs walked unsplit; 1 = top-down only.  Levels
     * are the same either way. */
    uint32_t bfs_direction;
    uint32_t bfs_alpha; /* go bottom-up when frontier edges x alpha > unexplored edges (0 = 8) */
    uint32_t bfs_beta;  /* go back top-down when frontier vertices x beta < n (0 = 18) */
    /* SSSP edge classes: 0 = delta-stepping light/heavy split when
     * sssp_delta > 0 on the unsplit graph (rows reordered light-first once
     * per graph and delta; near rounds relax light edges, each bucket's
     * vertices relax their heavy edges once when the bucket closes);
     * 1 = every near round relaxes all edges.  Distances are the same. */
    uint32_t sssp_light_heavy;
    /* SSSP bucket close in light/heavy mode.  On graphs whose every edge has
     * its reverse with the same weight a bucket may close by pulling: each
     * unsettled vertex takes the smallest d(u) + w over its heavy edges to
     * settled vertices, instead of the bucket's vertices pushing all their
     * heavy edges.  0 = pull when the bucket's heavy edges outnumber twice
     * the unsettled vertices' heavy edges plus n/2; 1 = always push;
     * 2 = always pull (where allowed).  Distances are the same. */
    uint32_t sssp_pull;
    /* SSSP near-far tail: once a bucket opens with at most n / k far-pile
     * entries and the pile smaller than the largest it has been, the
     * threshold goes to infinity and the remaining vertices run as one
     * label-correcting frontier over whole rows (no more buckets).  0 = k of
     * 2 on graphs averaging 8 or more edges per vertex, never on sparser
     * ones (grids); 1 = never; k > 1 = that k.  Distances are the same. */
    uint32_t sssp_tail;
    /* Expansion strategy of GGA_VARIANT_AUTO (gga_autotune picks it per graph
     * from timed trials; every choice gives the same distances):
     * 0 = edge-balanced CTA-cooperative units over the unsplit CSR;
     * 1 = the same units over the node-split CSR (the split at split_level /
     *     split_buckets, as gga_node_split, graph.h:415-522);
     * 2 = the reference's CDP variant (my_drelax_dynamicP,
     *     cudaKernels.h:438-520) with the heavy-vertex threshold of
     *     split_level / split_buckets. */
    uint32_t expansion;
    int32_t split_level;   /* 0 none, > 0 ceil(maxdeg/level), < 0 histogram rule */
    int32_t split_buckets; /* histogram buckets when split_level < 0 */
    /* SSSP bucket width the batch engine (gga_multi_solve, the server) uses
     * for this graph's queries (0 = Bellman-Ford order); 0xFFFFFFFF = the
     * degree-profile width. */
    uint32_t batch_delta;
} gga_params;
/* p = NULL returns to the per-graph defaults (the graph's autotuned
 * parameters when gga_autotune has run on it, else its degree profile). */
gga_status gga_set_params(gga_ctx *ctx, const gga_params *p);
gga_status gga_get_params(gga_ctx *ctx, gga_params *p);
/* Picks parameters for g from its degree profile and, when trials > 0,
 * short timed trials from two sources: CTA size and SSSP bucket width, BFS
 * direction thresholds (alpha, beta), the expansion strategy (edge units
 * over the unsplit CSR, the node-split CSR at several split levels, or CDP
 * on graphs under 2^21 edges) and the batch engine's bucket width.  The
 * choice is stored on g (used by every solve of g on a context without
 * explicit parameters, and by gga_multi_solve and the server for g's
 * queries) and in ctx.  No counterpart in the reference, whose split level
 * is a command-line argument swept by a shell script (mysc:20-51). */
gga_status gga_autotune(gga_ctx *ctx, gga_graph *g, uint32_t trials, gga_params *chosen);
/* The last gga_autotune's trials on ctx as a JSON object (candidates and
 * their times in ms); at most len bytes with the terminating NUL. */
gga_status gga_autotune_report(gga_ctx *ctx, char *buf, size_t len);

/* ---- instrumentation ------------------------------------------------------
 * Device-counter counterparts of the reference's per-CTA clock64 histogram
 * (my_drelax_metric, cudaKernels.h:1-70, combined per SM in metrics.h:68-84)
 * and of its per-iteration convergence log (convergence.h:100-159). */
typedef struct gga_round_trace {
    uint32_t kind;      /* 0 top-down (SSSP: near) round, 1 bottom-up BFS round, 2 SSSP far pass,
                         * 3 SSSP heavy round (a bucket's heavy edges), 4 SSSP pull scan (lists
                         * the unsettled vertices' heavy edges), 5 SSSP pull round (relaxes them
                         * from the settled side) */
    uint32_t items;     /* vertices expanded (kind 0/1/3/5) or far-pile entries split (kind 2) */
    uint32_t edges;     /* edges owned by the expanded vertices */
    uint32_t far_items; /* SSSP: far-pile size when the round started */
    uint32_t ns;        /* round duration (block 0's clock from this round's start to the next's) */
} gga_round_trace;
/* While enabled, each frontier-engine solve on ctx records one record per
 * round (up to 65536) and each CTA's busy time in kilocycles (clock64 from
 * round start to the grid barrier, summed over rounds). */
gga_status gga_trace_enable(gga_ctx *ctx, int enable);
/* Copies the last traced solve's records: up to `cap` rounds into `rounds`
 * (*nrounds = rounds recorded) and up to `cta_cap` CTA busy times into
 * `cta_kcycles` (*ncta = CTAs of that launch).  Any output may be NULL. */
gga_status gga_trace_get(gga_ctx *ctx, gga_round_trace *rounds, uint32_t cap, uint32_t *nrounds,
                         uint32_t *cta_kcycles, uint32_t cta_cap, uint32_t *ncta);

/* One iteration of a convergence log. */
typedef struct gga_conv_record {
    uint32_t iteration;  /* 1-based relax launch */
    uint32_t pad;
    uint64_t diff_count; /* original vertices whose distance differs from the final one */
    double norm2;        /* sqrt(sum over them of (final - current)^2), the square taken in
                          * 32-bit unsigned arithmetic as the reference's foru does */
} gga_conv_record;
/* Per-iteration convergence of a topology-driven solve, replacing
 * printConv_rtime (convergence.h:100-159, called after every relax launch at
 * bfs_sssp.cu:420-424): after each launch the current distances of the
 * original vertices (the split parents) are compared on the device with
 * final_dist (host, nodes_orig words, e.g. an earlier solve's answer).
 * variant: TOPO_ATOMIC, TOPO_PLAIN, CDP_ATOMIC or CDP_PLAIN (the frontier
 * engine has rounds, not iterations; gga_trace_get covers it).  Up to cap
 * records are written; *nrec receives the number of iterations run.
 * dist_out (host or device, may be NULL) receives the solve's answer. */
gga_status gga_convergence(gga_ctx *ctx, gga_graph *g, gga_algo algo, uint32_t src, gga_variant variant,
                           const uint32_t *final_dist, gga_conv_record *records, uint32_t cap, uint32_t *nrec,
                           uint32_t *dist_out);

/* ---- verification and output (myutils.h, L5) ---------------------------- */

/* verifysolution, myutils.h:1-18: number of edges with wt>0 and
 * dist[u]+wt < dist[v] (weights taken as 1 for BFS), on the split graph when
 * g is split.  dist: host array of nodes_orig entries. */
gga_status gga_verify(const gga_graph *g, gga_algo algo, const uint32_t *dist, uint64_t *nerr);
/* Ary2File, myutils.h:51-62: one "%u\n" line per original vertex. */
gga_status gga_write_dist(const char *path, const gga_graph *g, const uint32_t *dist);
/* E_r and V_r for a distance vector (host array of nodes_orig entries). */
gga_status gga_reached(const gga_graph *g, const uint32_t *dist, uint64_t *vertices_reached,
                       uint64_t *edges_reached);

/* The 17-column row writeResult appends to result.vi (myutils.h:86-113;
 * fields = SResult, graph.h:66-84). */
typedef struct gga_result_row {
    char exename[100];
    char algo[10];
    char graphfile[200];
    uint32_t bucket_size, nnode, nedge, ns_nnode, ns_nedge, extranode, maxdeg, splitlevel,
        max_edges_allowed, iterations, runtime;
    float time, ktime, sktime;
} gga_result_row;
gga_status gga_write_result_row(const char *path, const gga_result_row *row);

/* Allocation-free BFS (no counterpart in the reference, which allocates all
 * of its device memory with cudaMalloc, graph.h:534-553).  For callers that
 * must not allocate GPU memory while they traverse: code running inside a
 * memory pool another framework owns, latency-critical paths where an
 * allocation could synchronise the device, processes whose device memory is
 * reserved up front.  Runs the frontier BFS of gga_bfs with its working
 * memory in a fixed array the library reserves on each GPU it is loaded on
 * (about 6.2 MiB, kept until exit).  Graphs up to 262,144 vertices and
 * 8,388,608 edges; larger ones return GGA_ERR_TOO_LARGE.  Inputs and output
 * are device pointers: d_offsets[n+1] and d_cols[m] a 0-based CSR, d_dist[n]
 * BFS levels (GGA_INFINITY where unreached).  `stream` is a cudaStream_t
 * (NULL = default stream) on the current device.  All calls share the one
 * array: calls that overlap on the GPU race, so serialise them.  The call is
 * synchronous: it returns after the traversal on `stream` has finished, so it
 * must not be made while a stream of the device is being captured into a
 * CUDA graph.  A column id >= n in the caller's CSR returns
 * GGA_ERR_FORMAT (the kernel checks every edge target before using it). */
gga_status gga_bfs_noalloc(const uint32_t *d_offsets, const uint32_t *d_cols, uint32_t n, uint32_t m,
                           uint32_t src, uint32_t *d_dist, void *stream);

/* ---- batched queries ---------------------------------------------------- */

/* Bit-packed multi-source BFS: nsrc <= 64 sources in one traversal (one
 * uint64 mask per vertex; an edge read serves every source whose frontier
 * holds its tail).  Levels equal nsrc single-source gga_bfs runs on the
 * unsplit graph.  dist_out: nsrc x nodes_orig, source-major, host or device.
 * stats: iterations = levels, vertices/edges_reached summed over sources. */
gga_status gga_msbfs(gga_ctx *ctx, gga_graph *g, uint32_t nsrc, const uint32_t *srcs,
                     uint32_t *dist_out, gga_stats *stats);
/* Batched SSSP: nsrc <= 32 sources of one graph in one launch, one warp lane
 * per source (vertex-major distances: an edge read serves every source whose
 * frontier holds its tail).  Distances equal nsrc single-source gga_sssp runs
 * on the unsplit graph.  dist_out: nsrc x nodes_orig, source-major, host or
 * device. */
gga_status gga_sssp_batch(gga_ctx *ctx, gga_graph *g, uint32_t nsrc, const uint32_t *srcs,
                          uint32_t *dist_out, gga_stats *stats);

/* One query of a multi-graph batch. */
typedef struct gga_query {
    gga_graph *graph;
    uint32_t algo; /* gga_algo */
    uint32_t src;
    uint32_t *dist_out; /* host or device, nodes_orig entries */
} gga_query;
/* Runs nq queries over any mix of graphs in one persistent launch: queue
 * entries carry their query, so edge-balanced work units are cut from all
 * queries' frontiers at once and a round costs one grid barrier for the
 * whole batch.  Each result equals the single-source answer (unsplit CSR).
 * stats: iterations = rounds, vertices/edges_reached summed over queries. */
gga_status gga_multi_solve(gga_ctx *ctx, uint32_t nq, const gga_query *queries, gga_stats *stats);

/* ---- serving ------------------------------------------------------------ */

typedef struct gga_server gga_server;
typedef struct gga_server_stats {
    uint64_t submitted, completed, rejected;
    uint32_t max_inflight;
    uint32_t supersteps;
    uint64_t state_bytes_peak; /* peak per-query device state admitted */
} gga_server_stats;

/* Starts a request loop (own thread and stream) over resident graphs:
 * continuous batching on the batch engine in supersteps of a few rounds;
 * finished queries retire and waiting ones join between supersteps.  All
 * device memory (queues, per-query distances and visited/stamp words) is
 * reserved here from mem_cap_bytes; a query whose state can never fit is
 * rejected with GGA_ERR_ADMISSION at submit, others wait for room.  At most
 * max_slots queries are in flight at once. */
gga_status gga_server_create(gga_ctx *ctx, uint32_t ngraphs, gga_graph *const *graphs,
                             uint64_t mem_cap_bytes, uint32_t max_slots, gga_server **out);
/* Queues a query; returns at once with a ticket.  dist_out (host) must stay
 * valid until the ticket completes. */
gga_status gga_server_submit(gga_server *s, uint32_t graph_index, gga_algo algo, uint32_t src,
                             uint32_t *dist_out, uint64_t *ticket);
/* Waits up to timeout_ms (0 = poll) for a ticket; latency_us = completion -
 * submission.  GGA_ERR_NOT_READY if still running.  A ticket is consumed by
 * the wait that returns its result. */
gga_status gga_server_wait(gga_server *s, uint64_t ticket, uint32_t timeout_ms,
                           double *latency_us);
gga_status gga_server_get_stats(gga_server *s, gga_server_stats *st);
/* Stops the loop after the current superstep; queries still queued or in
 * flight are dropped (their buffers are not written after this returns). */
void gga_server_destroy(gga_server *s);

/* ------------------------------------------------------------------------
 * Delaunay mesh refinement (the reference's DMR program, Kepler_DMR/dmr.cu).
 *
 * A mesh is a 2-D triangulation held on the host: points (double x, y),
 * triangles as three point ids in counter-clockwise order, and per triangle
 * the neighbour across each edge (edge i is opposite vertex i;
 * GGA_MESH_NONE on the domain boundary).  gga_mesh_refine inserts points on
 * the GPU until no triangle has an angle below the bound, keeping the mesh
 * Delaunay, and writes the refined mesh back into the same handle.
 * ---------------------------------------------------------------------- */
#define GGA_MESH_NONE 0xFFFFFFFFu
#define GGA_DMR_MIN_ANGLE 25.0 /* MINANGLE, dmr.cu:34 */

typedef struct gga_mesh gga_mesh;

typedef struct gga_mesh_info {
    uint32_t npoints;
    uint32_t ntriangles;
} gga_mesh_info;

typedef struct gga_mesh_check_result {
    uint64_t bad_triangles;      /* smallest angle below the bound */
    uint64_t bad_orientation;    /* zero or negative signed area */
    uint64_t bad_neighbors;      /* links that are not mutual across one shared edge */
    uint64_t non_delaunay_edges; /* the neighbour's far vertex inside the circumcircle */
    uint64_t boundary_edges;     /* edges with no neighbour */
    double area;                 /* sum of signed areas */
} gga_mesh_check_result;

typedef struct gga_refine_stats {
    uint32_t triangles_in, bad_in;   /* myresult.i_ntriangles / i_bad */
    uint32_t triangles_out, bad_out; /* myresult.o_ntriangles / o_bad */
    uint32_t points_out;
    uint32_t rounds;                 /* myresult.iteration */
    uint64_t insertions;             /* circumcentres inserted */
    uint64_t boundary_splits;        /* boundary edges split at their midpoint */
    uint64_t failed_plans;           /* insertions given up (walk, cavity or shape limits) */
    double total_ms;                 /* the whole call: allocation, upload, refinement, download */
    double device_ms;                /* refinement rounds on the device */
    double alloc_ms;                 /* device buffers and their initialisation */
    double upload_ms;                /* mesh to the device */
    double download_ms;              /* refined mesh to the host arrays */
} gga_refine_stats;

/* Reads "<base>.node" and "<base>.ele" (Triangle format, as readNodes /
 * readTriangles in helpers.h:5-63; a .poly file is not needed).  Triangles
 * are reordered counter-clockwise and their neighbours derived.
 * GGA_ERR_FORMAT on a bad count, a bad line, an id out of range, a
 * degenerate triangle or an edge shared by more than two triangles. */
gga_status gga_mesh_load_triangle(const char *base, gga_mesh **out);
gga_status gga_mesh_save_triangle(const gga_mesh *m, const char *base);
/* Builds a mesh from arrays (copied): points x/y[npoints], triangles
 * tri[3 * ntriangles] of point ids; same checks as the loader. */
gga_status gga_mesh_from_arrays(uint32_t npoints, const double *x, const double *y, uint32_t ntriangles,
                                const uint32_t *tri, gga_mesh **out);
/* Seeded Delaunay triangulation of a jittered w x h point grid over the unit
 * square (jitter in cell units, [0, 0.5)). */
gga_status gga_mesh_gen_jittered(uint32_t w, uint32_t h, double jitter, uint64_t seed, gga_mesh **out);
/* Seeded Delaunay triangulation of npoints uniform random points in the unit
 * square plus its four corners (incremental Bowyer-Watson insertion; a point
 * that lands exactly on an edge is left out): about 2 * npoints triangles,
 * the kind of random-point mesh the reference's DMR inputs are. */
gga_status gga_mesh_gen_random(uint32_t npoints, uint64_t seed, gga_mesh **out);
void gga_mesh_free(gga_mesh *m);
gga_status gga_mesh_get_info(const gga_mesh *m, gga_mesh_info *info);
/* Borrowed views of the mesh's arrays, valid until the mesh changes. */
gga_status gga_mesh_arrays(const gga_mesh *m, const double **x, const double **y, const uint32_t **tri,
                           const uint32_t **nbr);
/* Orientation, neighbour symmetry, the local Delaunay property, the count
 * of triangles with an angle below min_angle_deg and the total area. */
gga_status gga_mesh_check(const gga_mesh *m, double min_angle_deg, gga_mesh_check_result *r);
/* Refines m in place on ctx's GPU until no angle is below min_angle_deg
 * (<= 0 means GGA_DMR_MIN_ANGLE).  Each round plans one insertion per bad
 * triangle (at most batch_cap of them, 0 = 1,048,576, lowest ids first),
 * commits the plans whose cavities no higher-priority plan touches, and
 * re-marks the new triangles; the result depends only on the input mesh and
 * the arguments.  max_triangles bounds the refined mesh (0 = 4 x the input +
 * 65,536).  Returns GGA_ERR_TOO_LARGE when a round would pass that bound and
 * GGA_ERR_NO_PROGRESS when every remaining plan fails or 65,536 rounds pass;
 * in both cases m holds the mesh after the last completed round. */
gga_status gga_mesh_refine(gga_ctx *ctx, gga_mesh *m, double min_angle_deg, uint32_t max_triangles,
                           uint32_t batch_cap, gga_refine_stats *st);

/* gga_mesh_refine with the engine's schedule knobs, which change where the
 * work runs, never the result: tail_max is the number of bad triangles at
 * which one block takes over the rounds (0 = 2048; capped at 4096 and at the
 * batch cap; 0xFFFFFFFF keeps every round on the multi-kernel path);
 * prefetch_max is the largest round planned by the prefetching kernel
 * variant (0 = 32,768; 1 plans every larger round with the lean one). */
typedef struct gga_refine_params {
    double min_angle_deg;   /* <= 0: GGA_DMR_MIN_ANGLE */
    uint32_t max_triangles; /* 0: 4 x the input + 65,536 */
    uint32_t batch_cap;     /* 0: 1,048,576 */
    uint32_t tail_max;      /* 0: 2048; 0xFFFFFFFF: never */
    uint32_t prefetch_max;  /* 0: 32,768 */
} gga_refine_params;
gga_status gga_mesh_refine_ex(gga_ctx *ctx, gga_mesh *m, const gga_refine_params *p, gga_refine_stats *st);

#ifdef __cplusplus
}
#endif
#endif /* GGA_H */
