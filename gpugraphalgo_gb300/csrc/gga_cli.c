/*
 * gga_cli — drop-in for the reference's executables.
 *
 * The reference builds one binary per flavour from bfs_sssp.cu (genexe:
 * na_ = atomic relax, n_ = plain relax + child update, da_ / d_ = the same
 * with dynamic-parallelism children, each as bfs or sssp).  This program is
 * one binary whose flavour comes from the name it is run under, so links
 * named like the reference's executables behave like them:
 *
 *   na_bfs, na_sssp  ->  GGA_VARIANT_TOPO_ATOMIC
 *   n_bfs,  n_sssp   ->  GGA_VARIANT_TOPO_PLAIN
 *   da_bfs, da_sssp  ->  GGA_VARIANT_CDP_ATOMIC
 *   d_bfs,  d_sssp   ->  GGA_VARIANT_CDP_PLAIN
 *   anything else    ->  GGA_VARIANT_AUTO (the frontier engine); the
 *                        algorithm is SSSP when the name contains "sssp"
 * (a trailing ".exe" is ignored).  GGA_ALGO=bfs|sssp and
 * GGA_VARIANT=auto|frontier|topo_atomic|topo_plain|cdp_atomic|cdp_plain
 * override the name.
 *
 * Arguments are the reference's (bfs_sssp.cu:149-184):
 *   exe <graph.gr> [level] [buckets | outfile]
 * level 0 or absent: no split; level > 0: split at ceil(maxdeg / level);
 * level -1: the histogram rule with `buckets` (default 10).  A third
 * argument with level != -1 names the file the distances are written to
 * (Ary2File, myutils.h:51-62).  The source is original vertex 0, as in the
 * reference.  The dynamic-parallelism flavours do not split; their
 * heavy-vertex threshold comes from the same level / buckets
 * (bfs_sssp.cu:224-236).  Like the reference, the run appends its 17-column
 * row to result.vi in the working directory (writeResult, myutils.h:86-113).
 *
 * Differences on purpose: errors return a non-zero exit status with a
 * message instead of exit(-1) / SIGFPE (the histogram rule's division by
 * zero reports GGA_ERR_SPLIT_RULE), and the usage check comes before the
 * device is opened (the reference prints its device lines first,
 * bfs_sssp.cu:135-152).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/gga.h"

static const char *base_name(const char *p) {
    const char *s = strrchr(p, '/');
    return s ? s + 1 : p;
}

static int starts_with(const char *s, const char *pre) { return strncmp(s, pre, strlen(pre)) == 0; }

static int fail(const char *what) {
    fprintf(stderr, "%s: %s\n", what, gga_last_error());
    return 2;
}

int main(int argc, char **argv) {
    const char *exe = base_name(argv[0]);
    int sssp = strstr(exe, "sssp") != NULL;
    gga_variant variant = GGA_VARIANT_AUTO;
    if (starts_with(exe, "na_")) variant = GGA_VARIANT_TOPO_ATOMIC;
    else if (starts_with(exe, "n_")) variant = GGA_VARIANT_TOPO_PLAIN;
    else if (starts_with(exe, "da_")) variant = GGA_VARIANT_CDP_ATOMIC;
    else if (starts_with(exe, "d_")) variant = GGA_VARIANT_CDP_PLAIN;
    const char *ea = getenv("GGA_ALGO"), *ev = getenv("GGA_VARIANT");
    if (ea) sssp = strcmp(ea, "sssp") == 0;
    if (ev) {
        static const char *names[] = {"auto", "frontier", "topo_atomic", "topo_plain", "cdp_atomic", "cdp_plain"};
        for (int i = 0; i < 6; ++i)
            if (strcmp(ev, names[i]) == 0) variant = (gga_variant)i;
    }
    const int cdp = variant == GGA_VARIANT_CDP_ATOMIC || variant == GGA_VARIANT_CDP_PLAIN;
    printf("%s\n", sssp ? "SSSP" : "BFS");
    if (argc < 2) {
        printf("Usage: %s <file>\n", argv[0]);
        return 1;
    }

    /* argv handling of bfs_sssp.cu:167-184 */
    int split_level = 1, enable_split = 0, w2f = 0;
    int buckets = 10;
    const char *outfile = NULL;
    if (argc > 2) {
        enable_split = 1;
        split_level = atoi(argv[2]);
        if (split_level == 0) enable_split = 0;
        if (split_level == -1 && argc > 3) buckets = atoi(argv[3]);
    }
    if (split_level != -1 && argc > 3) {
        w2f = 1;
        outfile = argv[3];
    }

    gga_ctx *ctx = NULL;
    gga_graph *g = NULL;
    if (gga_ctx_create(0, &ctx)) return fail("device");
    char dev[256];
    int sms = 0;
    gga_ctx_device_info(ctx, &sms, dev, sizeof dev);
    printf("Device Name:%s\n", dev);
    printf("%s\n%s\n", base_name(argv[1]), argv[1]);
    if (gga_graph_load_gr(argv[1], &g)) return fail(argv[1]);
    gga_graph_info info;
    gga_graph_get_info(g, &info);
    const uint32_t nnode = info.nodes_orig, nedge = info.nedges, maxdeg = info.maxdeg;
    printf("MaxDeg=%u\n", maxdeg);

    uint32_t mda = 0;
    if (cdp) {
        gga_params p;
        gga_get_params(ctx, &p);
        p.cdp_level = split_level;
        p.cdp_buckets = buckets;
        if (gga_set_params(ctx, &p)) return fail("parameters");
        if (split_level < 0) {
            if (gga_max_allowed_out_degree(g, (int32_t)buckets, &mda)) return fail("histogram rule");
            printf("Approx Level=%f\n", mda ? (float)maxdeg / mda : 0.0f);
        } else {
            const uint32_t lv = split_level > 0 ? (uint32_t)split_level : 1u;
            mda = (uint32_t)(((uint64_t)maxdeg + lv - 1) / lv);
        }
    } else if (enable_split) {
        if (gga_node_split(ctx, g, split_level, buckets)) return fail("node split");
        gga_graph_get_info(g, &info);
        mda = info.mda;
        printf("maxOutDegree=%u\n", mda);
        printf("After node split:\nnnodes=%u,nedges=%u (Extranodes=%u)\n", info.nnodes, info.nedges,
               info.nnodes - nnode);
    }

    uint32_t *dist = (uint32_t *)malloc((size_t)(nnode ? nnode : 1) * sizeof(uint32_t));
    if (!dist) return 2;
    gga_stats st;
    if (gga_solve(ctx, g, sssp ? GGA_SSSP : GGA_BFS, 0, variant, dist, &st)) return fail("solve");
    printf("iterations = %u.\n", st.iterations);
    if (w2f) {
        printf("Writing Result To file : %s\n", outfile);
        fflush(stdout);
        if (gga_write_dist(outfile, g, dist)) return fail(outfile);
    }
    uint64_t nerr = 0;
    if (gga_verify(g, sssp ? GGA_SSSP : GGA_BFS, dist, &nerr)) return fail("verify");
    printf("verifying: no of errors = %llu.\n", (unsigned long long)nerr);
    const double time_ms = st.kernel_ms + st.aux_ms;
    printf("%d ms.\n", (int)st.total_ms);
    printf("Time:%.2f ktime=%.2f sktime=%.2f\n", time_ms, st.kernel_ms, st.aux_ms);
    fflush(stdout);

    gga_result_row row;
    memset(&row, 0, sizeof row);
    snprintf(row.exename, sizeof row.exename, "%s", argv[0]);
    snprintf(row.algo, sizeof row.algo, "%s", sssp ? "SSSP" : "BFS");
    snprintf(row.graphfile, sizeof row.graphfile, "%s", base_name(argv[1]));
    gga_graph_get_info(g, &info);
    row.bucket_size = split_level < 0 ? (uint32_t)buckets : 0;
    row.nnode = nnode;
    row.nedge = nedge;
    row.ns_nnode = cdp ? nnode : info.nnodes;
    row.ns_nedge = info.nedges;
    row.extranode = cdp ? 0 : info.nnodes - nnode;
    row.maxdeg = maxdeg;
    row.splitlevel = (uint32_t)split_level;
    row.max_edges_allowed = cdp ? 0 : mda; /* the reference sets it only when it splits (graph.h:397) */
    row.iterations = st.iterations;
    row.runtime = (uint32_t)st.total_ms;
    row.time = (float)time_ms;
    row.ktime = (float)st.kernel_ms;
    row.sktime = (float)st.aux_ms;
    if (gga_write_result_row("result.vi", &row)) return fail("result.vi");

    free(dist);
    gga_graph_free(g);
    gga_ctx_destroy(ctx);
    return nerr ? 3 : 0;
}
