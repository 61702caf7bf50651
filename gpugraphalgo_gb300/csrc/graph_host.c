/*
 * Host graph substrate: .gr I/O, CSR construction, seeded generators, the
 * host-side split rules (getMaxdeg / getMaxAllowedOutDegree /
 * getSizeafterLoadBalance), the verifier and the output writers.
 *
 * Reference items replaced (Programs/CUDA_src/Kepler_BFS_SSSP/):
 *   Graph::readFromGR            graph.h:599-682
 *   Graph::getMaxdeg             graph.h:338-347
 *   Graph::getMaxAllowedOutDegree graph.h:359-385
 *   Graph::getSizeafterLoadBalance graph.h:386-414
 *   verifysolution               myutils.h:1-18
 *   Ary2File                     myutils.h:51-62
 *   writeResult                  myutils.h:86-113
 * The split itself (Graph::NodeSplit) is built on the device
 * (device_graph.cu); nothing here computes distances.
 */
#define _GNU_SOURCE
#include <errno.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

#include "gga_internal.h"

/* ---------------------------------------------------------------- errors */

static _Thread_local char g_errbuf[512];

gga_status gga_fail(gga_status st, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_errbuf, sizeof g_errbuf, fmt, ap);
    va_end(ap);
    return st;
}

void gga_clear_error(void) { g_errbuf[0] = 0; }

const char *gga_last_error(void) { return g_errbuf; }

const char *gga_version(void) { return "gga 0.1.0 (sm_103a)"; }

const char *gga_status_string(gga_status s) {
    switch (s) {
    case GGA_OK: return "ok";
    case GGA_ERR_INVALID_ARG: return "invalid argument";
    case GGA_ERR_IO: return "I/O error";
    case GGA_ERR_FORMAT: return "malformed graph or mesh";
    case GGA_ERR_SPLIT_RULE: return "split rule gives a zero edge limit";
    case GGA_ERR_NO_MEMORY: return "host out of memory";
    case GGA_ERR_CUDA: return "CUDA error";
    case GGA_ERR_NO_DEVICE: return "no CUDA device";
    case GGA_ERR_TIMEOUT: return "device wait timed out";
    case GGA_ERR_ADMISSION: return "admission refused (memory cap)";
    case GGA_ERR_TOO_LARGE: return "graph too large";
    case GGA_ERR_NOT_READY: return "not ready";
    case GGA_ERR_UNSUPPORTED: return "unsupported";
    case GGA_ERR_NO_PROGRESS: return "refinement made no progress";
    }
    return "unknown status";
}

double gga_now_ms(void) {
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return t.tv_sec * 1e3 + t.tv_nsec * 1e-6;
}

void (*gga_dev_graph_release_hook)(gga_graph *g) = NULL;

/* ---------------------------------------------------------------- graph */

gga_status gga_graph_alloc(uint32_t n, uint32_t m, gga_graph **out) {
    if (!out) return gga_fail(GGA_ERR_INVALID_ARG, "out is NULL");
    *out = NULL;
    if (n == 0) return gga_fail(GGA_ERR_INVALID_ARG, "graph needs at least one vertex");
    if (n > GGA_MAX_NODES || m > GGA_MAX_EDGES)
        return gga_fail(GGA_ERR_TOO_LARGE, "n=%u m=%u exceed the uint32 limits", n, m);
    gga_graph *g = (gga_graph *)calloc(1, sizeof *g);
    if (!g) return gga_fail(GGA_ERR_NO_MEMORY, "calloc graph");
    g->n = n;
    g->m = m;
    g->off = (uint32_t *)malloc(((size_t)n + 1) * sizeof(uint32_t));
    g->col = (uint32_t *)malloc(((size_t)m + 1) * sizeof(uint32_t));
    g->wt = (uint32_t *)malloc(((size_t)m + 1) * sizeof(uint32_t));
    if (!g->off || !g->col || !g->wt) {
        free(g->off); free(g->col); free(g->wt); free(g);
        return gga_fail(GGA_ERR_NO_MEMORY, "malloc CSR n=%u m=%u", n, m);
    }
    g->dev_device = -1;
    pthread_mutex_init(&g->lock, NULL);
    *out = g;
    return GGA_OK;
}

void gga_graph_refresh_stats(gga_graph *g) {
    uint32_t md = 0, mw = 0;
    for (uint32_t u = 0; u < g->n; ++u) {
        uint32_t d = g->off[u + 1] - g->off[u];
        if (d > md) md = d;
    }
    uint64_t ws = 0;
    for (uint32_t e = 0; e < g->m; ++e) {
        if (g->wt[e] > mw) mw = g->wt[e];
        ws += g->wt[e];
    }
    g->maxdeg = md;
    g->maxw = mw;
    g->wavg = g->m ? (double)ws / g->m : 1.0;
}

void gga_graph_free(gga_graph *g) {
    if (!g) return;
    if (g->dev && gga_dev_graph_release_hook) gga_dev_graph_release_hook(g);
    free(g->off);
    free(g->col);
    free(g->wt);
    pthread_mutex_destroy(&g->lock);
    free(g);
}

gga_status gga_graph_get_info(const gga_graph *g, gga_graph_info *info) {
    if (!g || !info) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    memset(info, 0, sizeof *info);
    info->nodes_orig = g->n;
    info->nnodes = g->split_level ? g->ns : g->n;
    info->nedges = g->m;
    info->maxdeg = g->maxdeg;
    info->split_level = g->split_level;
    info->split_buckets = g->split_buckets;
    info->mda = g->split_level ? g->mda : 0;
    info->parents_with_children = g->split_level ? g->parents_with_children : 0;
    info->max_weight = g->maxw;
    info->symmetric = g->symmetric;
    info->wsymmetric = g->wsymmetric;
    return GGA_OK;
}

gga_status gga_graph_csr(const gga_graph *g, const uint32_t **offsets, const uint32_t **cols,
                         const uint32_t **weights) {
    if (!g) return gga_fail(GGA_ERR_INVALID_ARG, "NULL graph");
    if (offsets) *offsets = g->off;
    if (cols) *cols = g->col;
    if (weights) *weights = g->wt;
    return GGA_OK;
}

gga_status gga_graph_from_csr(uint32_t n, uint32_t m, const uint32_t *offsets,
                              const uint32_t *cols, const uint32_t *weights,
                              gga_graph **out) {
    if (!offsets || (m && !cols) || !out) return gga_fail(GGA_ERR_INVALID_ARG, "NULL array");
    if (offsets[0] != 0 || offsets[n] != m)
        return gga_fail(GGA_ERR_INVALID_ARG, "offsets must start at 0 and end at m=%u", m);
    for (uint32_t u = 0; u < n; ++u)
        if (offsets[u + 1] < offsets[u])
            return gga_fail(GGA_ERR_INVALID_ARG, "offsets decrease at vertex %u", u);
    for (uint32_t e = 0; e < m; ++e)
        if (cols[e] >= n) return gga_fail(GGA_ERR_INVALID_ARG, "edge %u: dst %u >= n", e, cols[e]);
    gga_graph *g;
    gga_status st = gga_graph_alloc(n, m, &g);
    if (st) return st;
    memcpy(g->off, offsets, ((size_t)n + 1) * sizeof(uint32_t));
    if (m) memcpy(g->col, cols, (size_t)m * sizeof(uint32_t));
    if (weights) {
        if (m) memcpy(g->wt, weights, (size_t)m * sizeof(uint32_t));
    } else {
        for (uint32_t e = 0; e < m; ++e) g->wt[e] = 1;
    }
    gga_graph_refresh_stats(g);
    *out = g;
    return GGA_OK;
}

/* ------------------------------------------------------------- .gr files */

static uint64_t rd64le(const unsigned char *p) {
    uint64_t v = 0;
    for (int i = 7; i >= 0; --i) v = (v << 8) | p[i];
    return v;
}
static uint32_t rd32le(const unsigned char *p) {
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

/* Reads the whole file.  The reference maps it with mmap (graph.h:604-628). */
static gga_status slurp(const char *path, unsigned char **buf, size_t *len) {
    FILE *f = fopen(path, "rb");
    if (!f) return gga_fail(GGA_ERR_IO, "unable to open %s: %s", path, strerror(errno));
    if (fseeko(f, 0, SEEK_END) != 0) { fclose(f); return gga_fail(GGA_ERR_IO, "seek %s", path); }
    off_t sz = ftello(f);
    if (sz < 0) { fclose(f); return gga_fail(GGA_ERR_IO, "tell %s", path); }
    rewind(f);
    unsigned char *b = (unsigned char *)malloc(sz ? (size_t)sz : 1);
    if (!b) { fclose(f); return gga_fail(GGA_ERR_NO_MEMORY, "read buffer %lld", (long long)sz); }
    if (sz && fread(b, 1, (size_t)sz, f) != (size_t)sz) {
        free(b); fclose(f);
        return gga_fail(GGA_ERR_IO, "short read on %s", path);
    }
    fclose(f);
    *buf = b;
    *len = (size_t)sz;
    return GGA_OK;
}

gga_status gga_graph_load_gr(const char *path, gga_graph **out) {
    if (!path || !out) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    *out = NULL;
    unsigned char *buf = NULL;
    size_t len = 0;
    gga_status st = slurp(path, &buf, &len);
    if (st) return st;
    if (len < 32) { free(buf); return gga_fail(GGA_ERR_FORMAT, "%s: header truncated", path); }
    uint64_t version = rd64le(buf), size_edge = rd64le(buf + 8);
    uint64_t n64 = rd64le(buf + 16), m64 = rd64le(buf + 24);
    (void)size_edge; /* ignored, as graph.h:634,644 read u32 edge data regardless */
    if (version != 1) {
        free(buf);
        return gga_fail(GGA_ERR_FORMAT, "%s: version %llu (need 1)", path, (unsigned long long)version);
    }
    if (n64 == 0 || n64 > GGA_MAX_NODES || m64 > GGA_MAX_EDGES) {
        free(buf);
        return gga_fail(n64 == 0 ? GGA_ERR_FORMAT : GGA_ERR_TOO_LARGE,
                        "%s: n=%llu m=%llu outside limits", path, (unsigned long long)n64,
                        (unsigned long long)m64);
    }
    uint64_t need = 32 + 8 * n64 + 4 * m64 + ((m64 & 1) ? 4 : 0) + 4 * m64;
    if (len < need) {
        free(buf);
        return gga_fail(GGA_ERR_FORMAT, "%s: %zu bytes, need %llu", path, len, (unsigned long long)need);
    }
    uint32_t n = (uint32_t)n64, m = (uint32_t)m64;
    gga_graph *g;
    st = gga_graph_alloc(n, m, &g);
    if (st) { free(buf); return st; }
    const unsigned char *idx = buf + 32;
    const unsigned char *outs = idx + 8 * n64;
    const unsigned char *edata = outs + 4 * m64 + ((m64 & 1) ? 4 : 0);
    g->off[0] = 0;
    uint64_t prev = 0;
    for (uint32_t u = 0; u < n; ++u) {
        uint64_t end = rd64le(idx + 8 * (size_t)u);
        if (end < prev || end > m64) {
            free(buf); gga_graph_free(g);
            return gga_fail(GGA_ERR_FORMAT, "%s: outIdx[%u]=%llu not monotone within m", path, u,
                            (unsigned long long)end);
        }
        g->off[u + 1] = (uint32_t)end;
        prev = end;
    }
    if (prev != m64) {
        free(buf); gga_graph_free(g);
        return gga_fail(GGA_ERR_FORMAT, "%s: outIdx ends at %llu, m=%llu", path,
                        (unsigned long long)prev, (unsigned long long)m64);
    }
    for (uint32_t e = 0; e < m; ++e) {
        uint32_t d = rd32le(outs + 4 * (size_t)e);
        if (d >= n) {
            /* the reference only prints "invalid edge" here (graph.h:669-670) */
            free(buf); gga_graph_free(g);
            return gga_fail(GGA_ERR_FORMAT, "%s: invalid edge %u -> dst %u >= n=%u", path, e, d, n);
        }
        g->col[e] = d;
        g->wt[e] = rd32le(edata + 4 * (size_t)e);
    }
    free(buf);
    gga_graph_refresh_stats(g);
    *out = g;
    return GGA_OK;
}

static void wr64le(unsigned char *p, uint64_t v) {
    for (int i = 0; i < 8; ++i) p[i] = (unsigned char)(v >> (8 * i));
}
static void wr32le(unsigned char *p, uint32_t v) {
    for (int i = 0; i < 4; ++i) p[i] = (unsigned char)(v >> (8 * i));
}

gga_status gga_graph_save_gr(const gga_graph *g, const char *path) {
    if (!g || !path) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    FILE *f = fopen(path, "wb");
    if (!f) return gga_fail(GGA_ERR_IO, "unable to create %s: %s", path, strerror(errno));
    unsigned char hdr[32];
    wr64le(hdr, 1);
    wr64le(hdr + 8, 4);
    wr64le(hdr + 16, g->n);
    wr64le(hdr + 24, g->m);
    int ok = fwrite(hdr, 1, 32, f) == 32;
    enum { CH = 1 << 16 };
    unsigned char *tmp = (unsigned char *)malloc(8 * CH);
    if (!tmp) { fclose(f); return gga_fail(GGA_ERR_NO_MEMORY, "write buffer"); }
    for (uint32_t base = 0; ok && base < g->n; base += CH) {
        uint32_t k = g->n - base < CH ? g->n - base : CH;
        for (uint32_t i = 0; i < k; ++i) wr64le(tmp + 8 * i, g->off[base + i + 1]);
        ok = fwrite(tmp, 8, k, f) == k;
    }
    for (int pass = 0; pass < 2 && ok; ++pass) {
        const uint32_t *a = pass ? g->wt : g->col;
        for (uint32_t base = 0; ok && base < g->m; base += CH) {
            uint32_t k = g->m - base < CH ? g->m - base : CH;
            for (uint32_t i = 0; i < k; ++i) wr32le(tmp + 4 * i, a[base + i]);
            ok = fwrite(tmp, 4, k, f) == k;
        }
        if (!pass && (g->m & 1) && ok) {
            memset(tmp, 0, 4);
            ok = fwrite(tmp, 1, 4, f) == 4;
        }
    }
    free(tmp);
    if (fclose(f) != 0) ok = 0;
    return ok ? GGA_OK : gga_fail(GGA_ERR_IO, "write %s failed", path);
}

/* ------------------------------------------------------------ generators */

static inline uint64_t mix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
static inline uint64_t hash3(uint64_t seed, uint64_t a, uint64_t b) {
    return mix64(mix64(seed ^ mix64(a)) + b);
}

static uint32_t pair_weight(uint64_t seed, uint32_t a, uint32_t b, uint32_t wmin, uint32_t wmax) {
    uint64_t span = (uint64_t)wmax - wmin + 1;
    return wmin + (uint32_t)(hash3(seed ^ 0x5EEDF00DCAFEull, a, b) % span);
}

static int host_threads(void) {
    long c = sysconf(_SC_NPROCESSORS_ONLN);
    if (c < 1) c = 1;
    if (c > 32) c = 32;
    return (int)c;
}

typedef void *(*worker_fn)(void *);

/* Runs fn(ctx_t) on nt threads; ctx_t is an array of nt elements of `stride` bytes. */
static void run_threads(int nt, worker_fn fn, void *ctxs, size_t stride) {
    pthread_t th[32];
    for (int t = 0; t < nt; ++t) pthread_create(&th[t], NULL, fn, (char *)ctxs + t * stride);
    for (int t = 0; t < nt; ++t) pthread_join(th[t], NULL);
}

/* Symmetric CSR from undirected pairs (a[i], b[i]); pairs with a == b are
 * dropped, duplicates merged; every adjacency list comes out sorted by
 * neighbour id, so the result does not depend on pair order or thread count.
 * Steps (all threaded): per-thread degree counts -> offsets -> scatter both
 * directions -> per-vertex sort + unique -> compaction -> weights. */
typedef struct {
    int t, nt;
    uint32_t n;
    const uint32_t *a, *b;
    size_t cnt;
    uint32_t *cntv;   /* per-thread counts (n) */
    uint32_t *cur;    /* per-thread cursors (n) */
    uint32_t *tmp;    /* scattered neighbours */
    const uint64_t *toff; /* vertex offsets into tmp */
    uint32_t *udeg;   /* unique degree per vertex */
    const uint32_t *off; /* final offsets */
    uint32_t *col, *wt;
    uint64_t wseed;
    uint32_t wmin, wmax;
    int phase;
} csr_job;

static int cmp_u32(const void *x, const void *y) {
    uint32_t p = *(const uint32_t *)x, q = *(const uint32_t *)y;
    return p < q ? -1 : p > q;
}

static void *csr_worker(void *p) {
    csr_job *j = (csr_job *)p;
    size_t lo = j->cnt * j->t / j->nt, hi = j->cnt * (j->t + 1) / j->nt;
    uint32_t vlo = (uint32_t)((uint64_t)j->n * j->t / j->nt), vhi = (uint32_t)((uint64_t)j->n * (j->t + 1) / j->nt);
    if (j->phase == 0) {
        for (size_t i = lo; i < hi; ++i) {
            uint32_t x = j->a[i], y = j->b[i];
            if (x == y) continue;
            j->cntv[x]++;
            j->cntv[y]++;
        }
    } else if (j->phase == 1) {
        for (size_t i = lo; i < hi; ++i) {
            uint32_t x = j->a[i], y = j->b[i];
            if (x == y) continue;
            j->tmp[j->cur[x]++] = y;
            j->tmp[j->cur[y]++] = x;
        }
    } else if (j->phase == 2) {
        for (uint32_t v = vlo; v < vhi; ++v) {
            uint32_t *l = j->tmp + j->toff[v];
            size_t len = (size_t)(j->toff[v + 1] - j->toff[v]);
            if (len > 1) {
                if (len < 24) {
                    for (size_t q = 1; q < len; ++q) {
                        uint32_t x = l[q];
                        size_t r = q;
                        while (r > 0 && l[r - 1] > x) { l[r] = l[r - 1]; --r; }
                        l[r] = x;
                    }
                } else {
                    qsort(l, len, sizeof(uint32_t), cmp_u32);
                }
            }
            size_t u = 0;
            for (size_t q = 0; q < len; ++q)
                if (u == 0 || l[q] != l[u - 1]) l[u++] = l[q];
            j->udeg[v] = (uint32_t)u;
        }
    } else {
        for (uint32_t v = vlo; v < vhi; ++v) {
            const uint32_t *l = j->tmp + j->toff[v];
            uint32_t o = j->off[v], d = j->off[v + 1] - o;
            for (uint32_t q = 0; q < d; ++q) {
                uint32_t w = l[q];
                j->col[o + q] = w;
                j->wt[o + q] = pair_weight(j->wseed, v < w ? v : w, v < w ? w : v, j->wmin, j->wmax);
            }
        }
    }
    return NULL;
}

static gga_status csr_from_pairs(uint32_t n, const uint32_t *a, const uint32_t *b, size_t cnt, uint64_t wseed,
                                 uint32_t wmin, uint32_t wmax, gga_graph **out) {
    int nt = host_threads();
    if ((uint64_t)n * nt > (1ull << 31)) nt = 4;
    csr_job jobs[32];
    uint32_t *cnts = (uint32_t *)calloc((size_t)n * nt, sizeof(uint32_t));
    uint64_t *toff = (uint64_t *)malloc(((size_t)n + 1) * sizeof(uint64_t));
    uint32_t *udeg = (uint32_t *)malloc((size_t)n * sizeof(uint32_t));
    if (!cnts || !toff || !udeg) {
        free(cnts); free(toff); free(udeg);
        return gga_fail(GGA_ERR_NO_MEMORY, "CSR build buffers (n=%u, %d threads)", n, nt);
    }
    for (int t = 0; t < nt; ++t) {
        memset(&jobs[t], 0, sizeof jobs[t]);
        jobs[t].t = t; jobs[t].nt = nt; jobs[t].n = n; jobs[t].a = a; jobs[t].b = b; jobs[t].cnt = cnt;
        jobs[t].cntv = cnts + (size_t)n * t;
        jobs[t].cur = cnts + (size_t)n * t;
        jobs[t].phase = 0;
    }
    run_threads(nt, csr_worker, jobs, sizeof jobs[0]);
    /* offsets: vertex-major, thread-minor; counts become write cursors */
    uint64_t s = 0;
    for (uint32_t v = 0; v < n; ++v) {
        toff[v] = s;
        for (int t = 0; t < nt; ++t) {
            uint32_t c = cnts[(size_t)n * t + v];
            cnts[(size_t)n * t + v] = (uint32_t)s;
            s += c;
        }
    }
    toff[n] = s;
    if (s > GGA_MAX_EDGES) {
        free(cnts); free(toff); free(udeg);
        return gga_fail(GGA_ERR_TOO_LARGE, "%llu directed edges", (unsigned long long)s);
    }
    uint32_t *tmp = (uint32_t *)malloc((s ? s : 1) * sizeof(uint32_t));
    if (!tmp) {
        free(cnts); free(toff); free(udeg);
        return gga_fail(GGA_ERR_NO_MEMORY, "CSR scatter buffer");
    }
    for (int t = 0; t < nt; ++t) { jobs[t].tmp = tmp; jobs[t].toff = toff; jobs[t].udeg = udeg; jobs[t].phase = 1; }
    run_threads(nt, csr_worker, jobs, sizeof jobs[0]);
    free(cnts);
    for (int t = 0; t < nt; ++t) jobs[t].phase = 2;
    run_threads(nt, csr_worker, jobs, sizeof jobs[0]);
    uint64_t m = 0;
    for (uint32_t v = 0; v < n; ++v) m += udeg[v];
    gga_graph *g;
    gga_status st = gga_graph_alloc(n, (uint32_t)m, &g);
    if (st) { free(tmp); free(toff); free(udeg); return st; }
    uint32_t o = 0;
    for (uint32_t v = 0; v < n; ++v) { g->off[v] = o; o += udeg[v]; }
    g->off[n] = o;
    for (int t = 0; t < nt; ++t) {
        jobs[t].off = g->off; jobs[t].col = g->col; jobs[t].wt = g->wt;
        jobs[t].wseed = wseed; jobs[t].wmin = wmin; jobs[t].wmax = wmax; jobs[t].phase = 3;
    }
    run_threads(nt, csr_worker, jobs, sizeof jobs[0]);
    free(tmp); free(toff); free(udeg);
    g->symmetric = 1;
    g->wsymmetric = 1; /* pair_weight depends on the unordered pair only */
    gga_graph_refresh_stats(g);
    *out = g;
    return GGA_OK;
}

typedef struct {
    uint32_t *sa, *sb;
    const uint32_t *perm;
    uint64_t seed, lo, hi;
    uint32_t scale, ta, tab, tabc;
} rmat_job;

static void *rmat_worker(void *p) {
    rmat_job *j = (rmat_job *)p;
    for (uint64_t i = j->lo; i < j->hi; ++i) {
        uint32_t s = 0, d = 0;
        uint64_t h = 0;
        for (uint32_t l = 0; l < j->scale; ++l) {
            if ((l & 1) == 0) h = hash3(j->seed, i, l >> 1);
            uint32_t r = (l & 1) ? (uint32_t)(h >> 32) : (uint32_t)h;
            uint32_t bit = 1u << (j->scale - 1 - l);
            if (r < j->ta) {
            } else if (r < j->tab) {
                d |= bit;
            } else if (r < j->tabc) {
                s |= bit;
            } else {
                s |= bit;
                d |= bit;
            }
        }
        j->sa[i] = j->perm[s];
        j->sb[i] = j->perm[d];
    }
    return NULL;
}

static uint32_t prob_threshold(double p) {
    double t = p * 4294967296.0;
    if (t <= 0) return 0;
    if (t >= 4294967295.0) return 0xFFFFFFFFu;
    return (uint32_t)t;
}

gga_status gga_graph_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b,
                              double c, uint64_t seed, uint32_t wmin, uint32_t wmax,
                              gga_graph **out) {
    if (!out) return gga_fail(GGA_ERR_INVALID_ARG, "out is NULL");
    if (scale < 1 || scale > 31 || edge_factor < 1)
        return gga_fail(GGA_ERR_INVALID_ARG, "scale %u / edge factor %u out of range", scale, edge_factor);
    if (a < 0 || b < 0 || c < 0 || a + b + c > 1.0 || wmin > wmax)
        return gga_fail(GGA_ERR_INVALID_ARG, "bad R-MAT probabilities or weight range");
    uint32_t n = 1u << scale;
    uint64_t m = (uint64_t)edge_factor << scale;
    if (2 * m > GGA_MAX_EDGES) return gga_fail(GGA_ERR_TOO_LARGE, "R-MAT %u x %u too large", scale, edge_factor);
    uint32_t *perm = (uint32_t *)malloc((size_t)n * sizeof(uint32_t));
    uint32_t *sa = (uint32_t *)malloc((size_t)m * sizeof(uint32_t));
    uint32_t *sb = (uint32_t *)malloc((size_t)m * sizeof(uint32_t));
    if (!perm || !sa || !sb) {
        free(perm); free(sa); free(sb);
        return gga_fail(GGA_ERR_NO_MEMORY, "R-MAT buffers");
    }
    /* Fisher-Yates relabelling from a seeded splitmix stream */
    for (uint32_t v = 0; v < n; ++v) perm[v] = v;
    uint64_t st = seed ^ 0xA5A5A5A55A5A5A5Aull;
    for (uint32_t v = n - 1; v > 0; --v) {
        st += 0x9E3779B97F4A7C15ull;
        uint32_t j = (uint32_t)(mix64(st) % ((uint64_t)v + 1));
        uint32_t t = perm[v]; perm[v] = perm[j]; perm[j] = t;
    }
    int nt = host_threads();
    rmat_job jobs[32];
    uint32_t ta = prob_threshold(a), tab = prob_threshold(a + b), tabc = prob_threshold(a + b + c);
    for (int t = 0; t < nt; ++t) {
        rmat_job j = {sa, sb, perm, seed, m * t / nt, m * (t + 1) / nt, scale, ta, tab, tabc};
        jobs[t] = j;
    }
    run_threads(nt, rmat_worker, jobs, sizeof jobs[0]);
    free(perm);
    gga_status s = csr_from_pairs(n, sa, sb, (size_t)m, seed, wmin, wmax, out);
    free(sa);
    free(sb);
    return s;
}

gga_status gga_graph_gen_grid(uint32_t width, uint32_t height, double del_prob,
                              double longrange_frac, uint64_t seed, uint32_t wmin,
                              uint32_t wmax, gga_graph **out) {
    if (!out) return gga_fail(GGA_ERR_INVALID_ARG, "out is NULL");
    if (width < 1 || height < 1 || del_prob < 0 || del_prob > 1 || longrange_frac < 0 || wmin > wmax)
        return gga_fail(GGA_ERR_INVALID_ARG, "bad grid parameters");
    uint64_t n64 = (uint64_t)width * height;
    if (n64 > GGA_MAX_NODES) return gga_fail(GGA_ERR_TOO_LARGE, "grid %ux%u", width, height);
    uint32_t n = (uint32_t)n64;
    uint64_t nh = (uint64_t)height * (width - 1), nv = (uint64_t)(height - 1) * width;
    uint64_t ngrid = nh + nv;
    uint64_t nlong = (uint64_t)llround(longrange_frac * (double)ngrid);
    if (2 * (ngrid + nlong) > GGA_MAX_EDGES) return gga_fail(GGA_ERR_TOO_LARGE, "grid edges");
    uint32_t *sa = (uint32_t *)malloc((size_t)(ngrid + nlong + 1) * sizeof(uint32_t));
    uint32_t *sb = (uint32_t *)malloc((size_t)(ngrid + nlong + 1) * sizeof(uint32_t));
    if (!sa || !sb) { free(sa); free(sb); return gga_fail(GGA_ERR_NO_MEMORY, "grid pairs"); }
    uint32_t tdel = prob_threshold(del_prob);
    size_t k = 0;
    for (uint64_t id = 0; id < ngrid; ++id) {
        if ((uint32_t)hash3(seed, 1, id) < tdel) continue;
        uint64_t x;
        if (id < nh) {
            uint64_t r = id / (width - 1), c = id % (width - 1);
            x = r * width + c;
            sa[k] = (uint32_t)x;
            sb[k++] = (uint32_t)(x + 1);
        } else {
            x = id - nh; /* vertical edge (r, c) - (r + 1, c) with x = r * width + c */
            sa[k] = (uint32_t)x;
            sb[k++] = (uint32_t)(x + width);
        }
    }
    for (uint64_t i = 0; i < nlong; ++i) {
        sa[k] = (uint32_t)(hash3(seed, 2, i) % n);
        sb[k++] = (uint32_t)(hash3(seed, 3, i) % n);
    }
    gga_status s = csr_from_pairs(n, sa, sb, k, seed, wmin, wmax, out);
    free(sa);
    free(sb);
    return s;
}

/* --------------------------------------------------------- split rules */

gga_status gga_max_degree(const gga_graph *g, uint32_t *maxdeg) {
    if (!g || !maxdeg) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    *maxdeg = g->maxdeg;
    return GGA_OK;
}

/* Degree-histogram rule.  Bucket of a vertex = (int)((deg / (float)(maxdeg+1))
 * * buckets) in single precision, like graph.h:365; the most populated bucket
 * (first on ties) gives MDA = ((maxdeg+1)/buckets) * (bucket+1) in integers
 * (graph.h:375-383).  A bucket index that float rounding pushes to `buckets`
 * is clamped to the last bucket (the reference would write past its array). */
gga_status gga_max_allowed_out_degree(const gga_graph *g, int32_t buckets, uint32_t *mda) {
    if (!g || !mda) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    if (buckets <= 0) return gga_fail(GGA_ERR_INVALID_ARG, "buckets must be positive (got %d)", buckets);
    uint32_t *histo = (uint32_t *)calloc((size_t)buckets, sizeof(uint32_t));
    if (!histo) return gga_fail(GGA_ERR_NO_MEMORY, "histogram");
    int32_t maxdeg1 = (int32_t)g->maxdeg + 1;
    float fmaxdeg1 = (float)maxdeg1, fb = (float)buckets;
    for (uint32_t u = 0; u < g->n; ++u) {
        volatile float q = (float)(g->off[u + 1] - g->off[u]) / fmaxdeg1;
        volatile float p = q * fb;
        int idx = (int)p;
        if (idx >= buckets) idx = buckets - 1;
        histo[idx]++;
    }
    int32_t best = -1, bi = -1;
    for (int32_t i = 0; i < buckets; ++i)
        if ((int32_t)histo[i] > best) { best = (int32_t)histo[i]; bi = i; }
    free(histo);
    *mda = (uint32_t)((maxdeg1 / buckets) * (bi + 1));
    return GGA_OK;
}

gga_status gga_size_after_split(const gga_graph *g, int32_t level, int32_t buckets, uint32_t *mda,
                                uint32_t *new_nnodes) {
    if (!g || !mda || !new_nnodes) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    if (level == 0) return gga_fail(GGA_ERR_INVALID_ARG, "level 0 means no split");
    uint32_t lim;
    if (level > 0) {
        lim = (uint32_t)(((uint64_t)g->maxdeg + (uint32_t)level - 1) / (uint32_t)level);
    } else {
        gga_status st = gga_max_allowed_out_degree(g, buckets, &lim);
        if (st) return st;
    }
    uint64_t cnt = 0;
    for (uint32_t u = 0; u < g->n; ++u) {
        uint32_t d = g->off[u + 1] - g->off[u];
        if (d == 0) { cnt++; continue; }
        if (lim == 0)
            return gga_fail(GGA_ERR_SPLIT_RULE,
                            "edge limit is 0 (maxdeg %u, level %d, buckets %d): the reference divides by zero",
                            g->maxdeg, level, buckets);
        cnt += (d + (uint64_t)lim - 1) / lim;
    }
    if (cnt > GGA_MAX_NODES) return gga_fail(GGA_ERR_TOO_LARGE, "split gives %llu vertices", (unsigned long long)cnt);
    *mda = lim;
    *new_nnodes = (uint32_t)cnt;
    return GGA_OK;
}

/* --------------------------------------------------- verify and output */

/* verifysolution on the split graph visits every edge once with
 * dist[split u] = dist[original u] and targets remapped to parents, so the
 * count equals the one over the unsplit CSR with original-order distances. */
gga_status gga_verify(const gga_graph *g, gga_algo algo, const uint32_t *dist, uint64_t *nerr) {
    if (!g || !dist || !nerr) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    uint64_t e = 0;
    for (uint32_t u = 0; u < g->n; ++u) {
        uint32_t du = dist[u];
        for (uint32_t i = g->off[u]; i < g->off[u + 1]; ++i) {
            uint32_t wt = algo == GGA_SSSP ? g->wt[i] : 1u;
            if (wt > 0 && du + wt < dist[g->col[i]]) ++e;
        }
    }
    *nerr = e;
    return GGA_OK;
}

gga_status gga_reached(const gga_graph *g, const uint32_t *dist, uint64_t *vr, uint64_t *er) {
    if (!g || !dist) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    uint64_t a = 0, b = 0;
    for (uint32_t u = 0; u < g->n; ++u)
        if (dist[u] < GGA_INFINITY) { a++; b += g->off[u + 1] - g->off[u]; }
    if (vr) *vr = a;
    if (er) *er = b;
    return GGA_OK;
}

gga_status gga_write_dist(const char *path, const gga_graph *g, const uint32_t *dist) {
    if (!path || !g || !dist) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    FILE *f = fopen(path, "w");
    if (!f) return gga_fail(GGA_ERR_IO, "unable to create %s: %s", path, strerror(errno));
    int ok = 1;
    for (uint32_t u = 0; u < g->n && ok; ++u) ok = fprintf(f, "%u\n", dist[u]) > 0;
    if (fclose(f) != 0) ok = 0;
    return ok ? GGA_OK : gga_fail(GGA_ERR_IO, "write %s failed", path);
}

gga_status gga_write_result_row(const char *path, const gga_result_row *r) {
    if (!path || !r) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    FILE *f = fopen(path, "a+");
    if (!f) return gga_fail(GGA_ERR_IO, "unable to open %s: %s", path, strerror(errno));
    fprintf(f, "%s,%s,%s,", r->exename, r->algo, r->graphfile);
    fprintf(f, "%u,%u,%u,%u,%u,%u,%u,%u,%u,%u,%u,", r->bucket_size, r->nnode, r->nedge, r->ns_nnode,
            r->ns_nedge, r->extranode, r->maxdeg, r->splitlevel, r->max_edges_allowed, r->iterations,
            r->runtime);
    fprintf(f, "%f,%f,%f\n", r->time, r->ktime, r->sktime);
    return fclose(f) == 0 ? GGA_OK : gga_fail(GGA_ERR_IO, "write %s failed", path);
}
