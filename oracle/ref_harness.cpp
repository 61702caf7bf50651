/*
 * ORACLE — test infrastructure, not product code.
 *
 * A command-line driver around the reference's OWN host code, compiled from
 * the reference sources where they lie (oracle/Makefile's `ref` target passes the
 * reference directory with -I; nothing of the reference is copied here).  It
 * runs, in the reference's order (bfs_sssp.cu:188-241, 495):
 *   Graph::readFromGR -> getMaxdeg -> findSerialBFS/findSerialSSSP (unsplit,
 *   from `src`) -> NodeSplit(level, buckets) (when level != 0) ->
 *   verifysolution on the split graph -> Ary2File
 * and dumps every array as little-endian uint32 files next to <out>, plus a
 * key=value summary in <out>.meta.  Built twice: with -DSSSP (weights) and
 * without (BFS), as the reference's genexe builds do.
 *
 * usage: ref_{bfs,sssp} <graph.gr> <level> <buckets> <src> <out-prefix>
 */
#include <cuda_runtime.h>

/* The configuration bfs_sssp.cu:59-61 fixes before it includes graph.h:
 * INT_SPLIT selects the equal-slice split of graph.h:461-476. */
#define BFS
#define INT_SPLIT
#define EVERY_IT_CHILD_DIST_UPDATE
#include "graph.h"

#ifdef SSSP
#define BFS_SSSP(index) edgessrcwt[index]
#define ALGO_NAME "SSSP"
#else
#define BFS_SSSP(index) 1
#define ALGO_NAME "BFS"
#endif
#include "myutils.h"

static void dump(const std::string &path, const unsigned *a, size_t n) {
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) { perror(path.c_str()); exit(2); }
    if (n && fwrite(a, sizeof(unsigned), n, f) != n) { perror(path.c_str()); exit(2); }
    fclose(f);
}

int main(int argc, char **argv) {
    if (argc < 6) {
        fprintf(stderr, "usage: %s <graph.gr> <level> <buckets> <src> <out-prefix>\n", argv[0]);
        return 1;
    }
    int level = atoi(argv[2]);
    int buckets = atoi(argv[3]);
    unsigned src = (unsigned)strtoul(argv[4], NULL, 10);
    std::string out = argv[5];

    Graph g;
    if (g.readFromGR(argv[1]) != 0) return 3;
    unsigned maxdeg = g.getMaxdeg();
    unsigned n_orig = g.nnodes;

#ifdef SSSP
    g.findSerialSSSP(src);
    foru *serial = g.sssp;
    foru maxd = g.max_sssp;
#else
    g.findSerialBFS(src);
    foru *serial = g.bfs;
    foru maxd = g.max_bfs;
#endif
    dump(out + ".dist.u32", serial, n_orig);

    if (level != 0) g.NodeSplit(level, buckets);
    unsigned n = g.nnodes;
    if (level == 0) {
        /* readFromGR leaves parentNode unset; before a split it is the identity */
        for (unsigned i = 0; i < n; ++i) g.parentNode[i] = i;
    }
    dump(out + ".psrc.u32", g.psrc, (size_t)n + 1);
    dump(out + ".noutgoing.u32", g.noutgoing, n);
    dump(out + ".edgessrcdst.u32", g.edgessrcdst, (size_t)g.nedges + 1);
    dump(out + ".childCount.u32", g.childCount, n);
    dump(out + ".IsParent.u32", g.IsParent, n);
    dump(out + ".parentNode.u32", g.parentNode, n);

    /* The GPU path's final dist over split ids: a child holds its parent's
     * value (M_my_drelax propagates to children, cudaKernels.h:326-330). */
    foru *hdist = (foru *)malloc(sizeof(foru) * (n ? n : 1));
    for (unsigned i = 0; i < n; ++i) hdist[i] = serial[g.parentNode[i]];
    fflush(stdout);
    verifysolution(g.edgessrcdst, g.edgessrcwt, g.noutgoing, g.psrc, hdist, n, g.nedges, g.srcsrc);
    fflush(stdout);
    std::string ary = out + ".ary.txt";
    unsigned len = n;
    Ary2File((char *)ary.c_str(), hdist, g.IsParent, len);

    FILE *m = fopen((out + ".meta").c_str(), "w");
    fprintf(m, "algo=%s\nnodes_orig=%u\nnnodes=%u\nnedges=%u\nmaxdeg=%u\nmda=%u\nmax_dist=%u\n", ALGO_NAME,
            n_orig, n, g.nedges, maxdeg, level ? myresult.MAX_EDGES_ALLOWED : 0u, maxd);
    fclose(m);
    return 0;
}
