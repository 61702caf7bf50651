/*
 * ORACLE — test infrastructure, not product code.
 *
 * A plain-C restatement of the reference's host algorithms for the BFS/SSSP
 * path, used only by tests/, __graft_entry__.smoke() and the CPU-baseline leg
 * of bench.py as the checker.  The shipped library never links or calls it.
 * It is pinned against the reference itself: oracle/Makefile's `ref` target compiles the
 * reference's own graph.h/myutils.h into oracle/_ref/ and
 * tests/golden/make_golden.py records that build's outputs, which
 * tests/test_oracle_golden.py compares with this file bit for bit.
 *
 * Layout follows the reference's struct Graph (graph.h:23-64): psrc is
 * 1-based with a null edge slot 0 (graph.h:251-254) and psrc[n] = nedges
 * (graph.h:254 before a split, graph.h:498 after).
 *
 * Each function cites the reference function it restates
 * (paths relative to Programs/CUDA_src/Kepler_BFS_SSSP/).
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define ORACLE_INF 1000000000u /* MYINFINITY, graph.h:96 */

typedef struct oracle_graph {
    uint32_t nnodes, nedges, nodes_b4_ns;
    uint32_t *psrc;        /* nnodes+1 */
    uint32_t *noutgoing;   /* nnodes */
    uint32_t *edgessrcdst; /* nedges+1 */
    uint32_t *edgessrcwt;  /* nedges+1 */
    uint32_t *childCount;  /* nnodes */
    uint32_t *IsParent;    /* nnodes */
    uint32_t *parentNode;  /* nnodes */
    uint32_t mda;          /* MAX_EDGES_ALLOWED of the last split */
    int32_t level;
} oracle_graph;

void oracle_free(oracle_graph *g) {
    if (!g) return;
    free(g->psrc); free(g->noutgoing); free(g->edgessrcdst); free(g->edgessrcwt);
    free(g->childCount); free(g->IsParent); free(g->parentNode);
    free(g);
}

/* Graph::allocOnHost, graph.h:250-264. */
static oracle_graph *alloc_host(uint32_t n, uint32_t m) {
    oracle_graph *g = (oracle_graph *)calloc(1, sizeof *g);
    if (!g) return NULL;
    g->nnodes = n;
    g->nedges = m;
    g->nodes_b4_ns = n;
    g->edgessrcdst = (uint32_t *)calloc((size_t)m + 1, 4);
    g->edgessrcwt = (uint32_t *)calloc((size_t)m + 1, 4);
    g->psrc = (uint32_t *)calloc((size_t)n + 1, 4);
    g->noutgoing = (uint32_t *)calloc(n ? n : 1, 4);
    g->childCount = (uint32_t *)calloc(n ? n : 1, 4);
    g->IsParent = (uint32_t *)calloc(n ? n : 1, 4);
    g->parentNode = (uint32_t *)calloc(n ? n : 1, 4);
    if (!g->edgessrcdst || !g->edgessrcwt || !g->psrc || !g->noutgoing || !g->childCount ||
        !g->IsParent || !g->parentNode) {
        oracle_free(g);
        return NULL;
    }
    g->psrc[n] = m; /* graph.h:254 */
    return g;
}

/* Graph::readFromGR body, graph.h:653-679, from already-decoded arrays:
 * outIdx = end offsets, outs/edgeData = destination and weight per edge. */
static void fill_from_gr(oracle_graph *g, const uint64_t *outIdx, const uint32_t *outs,
                         const uint32_t *edgeData) {
    for (uint32_t ii = 0; ii < g->nnodes; ++ii) {
        g->IsParent[ii] = 1;
        g->childCount[ii] = 0;
        g->parentNode[ii] = ii; /* identity before a split */
        if (ii > 0) {
            g->psrc[ii] = (uint32_t)outIdx[ii - 1] + 1;
            g->noutgoing[ii] = (uint32_t)(outIdx[ii] - outIdx[ii - 1]);
        } else {
            g->psrc[0] = 1;
            g->noutgoing[0] = (uint32_t)outIdx[0];
        }
        for (uint32_t jj = 0; jj < g->noutgoing[ii]; ++jj) {
            uint32_t e = g->psrc[ii] + jj;
            g->edgessrcdst[e] = outs[e - 1];
            g->edgessrcwt[e] = edgeData[e - 1];
        }
    }
}

/* Graph::readFromGR, graph.h:599-682 (little-endian host assumed).
 * Returns NULL on open failure or a malformed file. */
oracle_graph *oracle_load_gr(const char *path) {
    FILE *f = fopen(path, "rb");
    if (!f) return NULL;
    uint64_t h[4];
    if (fread(h, 8, 4, f) != 4 || h[0] != 1) { fclose(f); return NULL; }
    uint64_t n = h[2], m = h[3];
    uint64_t *outIdx = (uint64_t *)malloc((n ? n : 1) * 8);
    uint32_t *outs = (uint32_t *)malloc((m ? m : 1) * 4);
    uint32_t *edata = (uint32_t *)malloc((m ? m : 1) * 4);
    int ok = outIdx && outs && edata && fread(outIdx, 8, n, f) == n && fread(outs, 4, m, f) == m;
    if (ok && (m & 1)) { uint32_t pad; ok = fread(&pad, 4, 1, f) == 1; }
    if (ok) ok = fread(edata, 4, m, f) == m;
    fclose(f);
    oracle_graph *g = ok ? alloc_host((uint32_t)n, (uint32_t)m) : NULL;
    if (g) fill_from_gr(g, outIdx, outs, edata);
    free(outIdx); free(outs); free(edata);
    return g;
}

/* Same as loading a .gr file holding this 0-based CSR. */
oracle_graph *oracle_from_csr(uint32_t n, uint32_t m, const uint32_t *off, const uint32_t *col,
                              const uint32_t *wt) {
    uint64_t *outIdx = (uint64_t *)malloc((n ? n : 1) * 8);
    if (!outIdx) return NULL;
    for (uint32_t i = 0; i < n; ++i) outIdx[i] = off[i + 1];
    oracle_graph *g = alloc_host(n, m);
    if (g) fill_from_gr(g, outIdx, col, wt);
    free(outIdx);
    return g;
}

void oracle_dims(const oracle_graph *g, uint32_t *nnodes, uint32_t *nedges, uint32_t *nodes_b4_ns,
                 uint32_t *mda) {
    if (nnodes) *nnodes = g->nnodes;
    if (nedges) *nedges = g->nedges;
    if (nodes_b4_ns) *nodes_b4_ns = g->nodes_b4_ns;
    if (mda) *mda = g->mda;
}

/* Copies the current arrays out (NULL pointers skipped). */
void oracle_arrays(const oracle_graph *g, uint32_t *psrc, uint32_t *noutgoing, uint32_t *dst,
                   uint32_t *wt, uint32_t *childCount, uint32_t *IsParent, uint32_t *parentNode) {
    size_t n = g->nnodes, m = g->nedges;
    if (psrc) memcpy(psrc, g->psrc, (n + 1) * 4);
    if (noutgoing) memcpy(noutgoing, g->noutgoing, n * 4);
    if (dst) memcpy(dst, g->edgessrcdst, (m + 1) * 4);
    if (wt) memcpy(wt, g->edgessrcwt, (m + 1) * 4);
    if (childCount) memcpy(childCount, g->childCount, n * 4);
    if (IsParent) memcpy(IsParent, g->IsParent, n * 4);
    if (parentNode) memcpy(parentNode, g->parentNode, n * 4);
}

/* Graph::getMaxdeg, graph.h:338-347. */
uint32_t oracle_max_degree(const oracle_graph *g) {
    uint32_t maxdeg = g->noutgoing[0];
    for (uint32_t j = 1; j < g->nnodes; j++)
        if (maxdeg < g->noutgoing[j]) maxdeg = g->noutgoing[j];
    return maxdeg;
}

/* Graph::getMaxAllowedOutDegree, graph.h:359-385.  A bucket index of
 * `maxHisto` (float rounding at degrees above 2^24) is clamped; the reference
 * writes one past its histogram there. */
uint32_t oracle_max_allowed_out_degree(const oracle_graph *g, int maxHisto) {
    uint32_t *histo = (uint32_t *)calloc((size_t)maxHisto, 4);
    int maxdeg = (int)oracle_max_degree(g);
    int maxdeg1 = maxdeg + 1;
    for (uint32_t i = 0; i < g->nnodes; i++) {
        volatile float q = g->noutgoing[i] / (float)maxdeg1;
        volatile float p = q * maxHisto;
        int index = (int)p;
        if (index >= maxHisto) index = maxHisto - 1;
        histo[index]++;
    }
    int max = -1, maxindex = -1;
    for (int i = 0; i < maxHisto; i++) {
        if ((int)histo[i] > max) {
            max = (int)histo[i];
            maxindex = i;
        }
    }
    maxindex++;
    free(histo);
    return (uint32_t)((maxdeg1 / maxHisto) * maxindex);
}

/* Graph::getSizeafterLoadBalance, graph.h:386-414.  Returns 0 on success,
 * 4 where the reference would divide by zero (MDA 0 with a vertex of
 * non-zero degree). */
int oracle_size_after_split(const oracle_graph *g, int level, int maxHisto, uint32_t *mda,
                            uint32_t *count) {
    if (level == 0) return 5; /* level 0 means "no split" (bfs_sssp.cu:170-171) */
    uint32_t maxdeg = oracle_max_degree(g);
    uint32_t lim = (maxdeg + (uint32_t)level - 1) / (uint32_t)level;
    if (level < 0) lim = oracle_max_allowed_out_degree(g, maxHisto);
    uint32_t idx = 0;
    for (uint32_t i = 0; i < g->nnodes; i++) {
        uint32_t nout = g->noutgoing[i];
        if (nout == 0) { idx++; continue; }
        if (lim == 0) return 4;
        idx += (nout + lim - 1) / lim;
    }
    *mda = lim;
    *count = idx;
    return 0;
}

/* Graph::NodeSplit with INT_SPLIT (bfs_sssp.cu:60), graph.h:415-522.
 * Returns 0, or 4 where the reference would divide by zero. */
int oracle_node_split(oracle_graph *g, int level, int maxHisto) {
    uint32_t lim, nn;
    int rc = oracle_size_after_split(g, level, maxHisto, &lim, &nn);
    if (rc) return rc;
    uint32_t *hpsrc = (uint32_t *)calloc((size_t)nn + 1, 4);
    uint32_t *hsrcdist = (uint32_t *)calloc(nn ? nn : 1, 4);
    uint32_t *hnout = (uint32_t *)calloc(nn ? nn : 1, 4);
    uint32_t *isp = (uint32_t *)calloc(nn ? nn : 1, 4);
    uint32_t *cc = (uint32_t *)calloc(nn ? nn : 1, 4);
    uint32_t *presum = (uint32_t *)malloc(((size_t)g->nnodes + 1) * 4);
    uint32_t k = 0;
    presum[0] = 0;
    for (uint32_t i = 0; i < g->nnodes; i++) {
        if (g->noutgoing[i] == 0) {
            presum[i + 1] = presum[i];
            hnout[k] = 0;
            hpsrc[k] = k == 0 ? 1 : hpsrc[k - 1] + hnout[k - 1];
            hsrcdist[k] = i;
            isp[k] = 1;
            k++;
            continue;
        }
        int split = (int)((g->noutgoing[i] + lim - 1) / lim);
        if (split > 1) {
            presum[i + 1] = presum[i] + (uint32_t)split - 1;
            cc[k] = (uint32_t)split - 1;
        } else {
            presum[i + 1] = presum[i];
        }
        isp[k] = 1;
        int local_max_deg = (int)((g->noutgoing[i] + (uint32_t)split - 1) / (uint32_t)split);
        int so_far = 0, count;
        while (split--) {
            if (split == 0) {
                count = (int)g->noutgoing[i] - so_far;
            } else {
                count = local_max_deg;
                so_far += count;
            }
            hnout[k] = (uint32_t)count;
            hpsrc[k] = k == 0 ? 1 : hpsrc[k - 1] + hnout[k - 1];
            hsrcdist[k] = i;
            k++;
        }
    }
    hpsrc[k] = g->nedges; /* graph.h:498 */
    for (uint32_t i = 1; i < g->nedges + 1; i++) g->edgessrcdst[i] += presum[g->edgessrcdst[i]];
    free(presum);
    free(g->psrc); free(g->noutgoing); free(g->IsParent); free(g->childCount); free(g->parentNode);
    g->nodes_b4_ns = g->nnodes;
    g->nnodes = k;
    g->psrc = hpsrc;
    g->noutgoing = hnout;
    g->IsParent = isp;
    g->parentNode = hsrcdist;
    g->childCount = cc;
    g->mda = lim;
    g->level = level;
    return 0;
}

/* myChildIndex / myChildCount construction, bfs_sssp.cu:256-283.  Returns
 * myParentCount; the arrays may be NULL to count only. */
uint32_t oracle_child_index(const oracle_graph *g, uint32_t *idx, uint32_t *cnt) {
    uint32_t p = 0;
    for (uint32_t i = 0; i < g->nnodes; i++) {
        if (g->childCount[i]) {
            if (idx) idx[p] = i;
            if (cnt) cnt[p] = g->childCount[i];
            p++;
        }
    }
    return p;
}

/* Graph::findSerialSSSP / findSerialBFS, graph.h:115-184: in-order
 * Bellman-Ford sweeps, at most nnodes passes, stopping after a pass with no
 * update.  BFS takes every weight as 1.  Writes nnodes distances; returns the
 * number of passes made. */
uint32_t oracle_serial(const oracle_graph *g, int sssp, uint32_t src, uint32_t *localdist) {
    uint32_t n = g->nnodes, passes = 0;
    for (uint32_t i = 0; i < n; i++) localdist[i] = ORACLE_INF;
    localdist[src] = 0;
    for (uint32_t i = 0; i < n; i++) {
        int flag = 1;
        passes++;
        for (uint32_t ver = 0; ver < n; ver++) {
            uint32_t tdist = localdist[ver];
            uint32_t end = g->psrc[ver] + g->noutgoing[ver];
            for (uint32_t ed = g->psrc[ver]; ed < end; ed++) {
                uint32_t wt = sssp ? g->edgessrcwt[ed] : 1u;
                uint32_t v = g->edgessrcdst[ed];
                if (tdist + wt < localdist[v]) {
                    flag = 0;
                    localdist[v] = tdist + wt;
                }
            }
        }
        if (flag) break;
    }
    return passes;
}

/* Host dist initialisation, bfs_sssp.cu:301-318: the set_parent_src-th
 * parent and its children get 0, everything else MYINFINITY. */
void oracle_init_dist(const oracle_graph *g, uint32_t parent_src, uint32_t *hdist) {
    int64_t count = -1;
    for (uint32_t i = 0; i < g->nnodes; i++) {
        if (g->IsParent[i]) count++;
        if (count == (int64_t)parent_src) {
            hdist[i] = 0;
            for (uint32_t k = 1; k <= g->childCount[i]; k++) hdist[i + k] = 0;
            i += g->childCount[i];
        } else {
            hdist[i] = ORACLE_INF;
        }
    }
}

/* verifysolution, myutils.h:1-18: counts edges with wt>0 and
 * dist[u]+wt < dist[v]; `dist` indexed by the current (split) ids. */
uint64_t oracle_verify(const oracle_graph *g, int sssp, const uint32_t *dist) {
    uint64_t nerr = 0;
    for (uint32_t nn = 0; nn < g->nnodes; ++nn) {
        uint32_t start = g->psrc[nn], cnt = g->noutgoing[nn];
        for (uint32_t ii = 0; ii < cnt; ++ii) {
            uint32_t v = g->edgessrcdst[start + ii];
            uint32_t wt = sssp ? g->edgessrcwt[start + ii] : 1u;
            if (wt > 0 && dist[nn] + wt < dist[v]) ++nerr;
        }
    }
    return nerr;
}

/* Ary2File, myutils.h:51-62: "%u\n" for entries whose IsParent is set. */
int oracle_ary2file(const char *fname, const uint32_t *ary, const uint32_t *isparent, uint32_t len) {
    FILE *f = fopen(fname, "w");
    if (!f) return 1;
    for (uint32_t i = 0; i < len; i++)
        if (isparent[i]) fprintf(f, "%u\n", ary[i]);
    return fclose(f) != 0;
}

/* ------------------------------------------------------------------------
 * Exact shortest distances by a second method, for graphs where the
 * reference's O(passes x E) sweeps take minutes (a 4096^2 grid is thousands
 * of BFS levels deep).  Not a restatement of reference code: BFS by a FIFO
 * queue (sssp = 0, every weight 1) and Dijkstra with an indexed binary heap
 * (sssp = 1).  Shortest distances are unique, so on any graph where
 * oracle_serial finishes both give the same array (tests/test_oracle_golden.py
 * checks that on the golden graphs).  Same layout and conventions as
 * oracle_serial: unsplit graph, nnodes distances, ORACLE_INF if unreached.
 * Returns 0, or 1 when memory runs out.
 * ------------------------------------------------------------------------ */
static void heap_sift_up(uint32_t *heap, uint32_t *pos, const uint32_t *key, uint32_t i) {
    const uint32_t v = heap[i];
    while (i > 0) {
        const uint32_t p = (i - 1) / 2;
        if (key[heap[p]] <= key[v]) break;
        heap[i] = heap[p];
        pos[heap[i]] = i;
        i = p;
    }
    heap[i] = v;
    pos[v] = i;
}

static void heap_sift_down(uint32_t *heap, uint32_t *pos, const uint32_t *key, uint32_t size, uint32_t i) {
    const uint32_t v = heap[i];
    for (;;) {
        uint32_t c = 2 * i + 1;
        if (c >= size) break;
        if (c + 1 < size && key[heap[c + 1]] < key[heap[c]]) c++;
        if (key[heap[c]] >= key[v]) break;
        heap[i] = heap[c];
        pos[heap[i]] = i;
        i = c;
    }
    heap[i] = v;
    pos[v] = i;
}

int oracle_shortest(const oracle_graph *g, int sssp, uint32_t src, uint32_t *dist) {
    const uint32_t n = g->nnodes;
    for (uint32_t i = 0; i < n; i++) dist[i] = ORACLE_INF;
    if (src >= n) return 0;
    uint32_t *heap = (uint32_t *)malloc((size_t)(n ? n : 1) * 4);
    uint32_t *pos = (uint32_t *)malloc((size_t)(n ? n : 1) * 4);
    if (!heap || !pos) {
        free(heap);
        free(pos);
        return 1;
    }
    dist[src] = 0;
    if (!sssp) { /* FIFO queue in `heap`; levels grow by one */
        uint32_t head = 0, tail = 0;
        heap[tail++] = src;
        while (head < tail) {
            const uint32_t u = heap[head++];
            const uint32_t end = g->psrc[u] + g->noutgoing[u];
            for (uint32_t ed = g->psrc[u]; ed < end; ed++) {
                const uint32_t v = g->edgessrcdst[ed];
                if (dist[v] == ORACLE_INF) {
                    dist[v] = dist[u] + 1;
                    heap[tail++] = v;
                }
            }
        }
    } else {
        const uint32_t NOPOS = 0xffffffffu;
        for (uint32_t i = 0; i < n; i++) pos[i] = NOPOS;
        uint32_t size = 0;
        heap[size++] = src;
        pos[src] = 0;
        while (size) {
            const uint32_t u = heap[0];
            pos[u] = NOPOS;
            if (--size) {
                heap[0] = heap[size];
                pos[heap[0]] = 0;
                heap_sift_down(heap, pos, dist, size, 0);
            }
            const uint32_t du = dist[u];
            const uint32_t end = g->psrc[u] + g->noutgoing[u];
            for (uint32_t ed = g->psrc[u]; ed < end; ed++) {
                const uint32_t v = g->edgessrcdst[ed];
                const uint32_t nd = du + g->edgessrcwt[ed];
                if (nd < dist[v]) { /* the same test oracle_serial makes */
                    dist[v] = nd;
                    if (pos[v] == NOPOS) {
                        heap[size] = v;
                        pos[v] = size;
                        heap_sift_up(heap, pos, dist, size);
                        size++;
                    } else {
                        heap_sift_up(heap, pos, dist, pos[v]);
                    }
                }
            }
        }
    }
    free(heap);
    free(pos);
    return 0;
}
