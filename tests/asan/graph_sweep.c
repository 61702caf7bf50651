/* Host graph code (csrc/graph_host.c) and the BFS/SSSP oracle
 * (oracle/gga_oracle.c, oracle/gen_inputs.c) under AddressSanitizer and
 * UndefinedBehaviorSanitizer: seeded R-MAT and grid graphs over a sweep of
 * sizes, a .gr round trip, malformed .gr files, the split-size rules, the
 * oracle's serial traversals, node split, child index, verification and the
 * exact FIFO/Dijkstra checker.  args: tmp-base */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gga_internal.h"

typedef struct oracle_graph oracle_graph;
oracle_graph *oracle_gen_rmat(uint32_t, uint32_t, double, double, double, uint64_t, uint32_t, uint32_t);
oracle_graph *oracle_gen_grid(uint32_t, uint32_t, double, double, uint64_t, uint32_t, uint32_t);
oracle_graph *oracle_load_gr(const char *path);
void oracle_free(oracle_graph *g);
void oracle_dims(const oracle_graph *g, uint32_t *nnodes, uint32_t *nedges, uint32_t *nodes_b4_ns, uint32_t *mda);
uint32_t oracle_max_degree(const oracle_graph *g);
uint32_t oracle_max_allowed_out_degree(const oracle_graph *g, int maxHisto);
int oracle_size_after_split(const oracle_graph *g, int level, int maxHisto, uint32_t *mda, uint32_t *nodes);
int oracle_node_split(oracle_graph *g, int level, int maxHisto);
uint32_t oracle_child_index(const oracle_graph *g, uint32_t *idx, uint32_t *cnt);
uint32_t oracle_serial(const oracle_graph *g, int sssp, uint32_t src, uint32_t *localdist);
void oracle_init_dist(const oracle_graph *g, uint32_t parent_src, uint32_t *hdist);
uint64_t oracle_verify(const oracle_graph *g, int sssp, const uint32_t *dist);
int oracle_shortest(const oracle_graph *g, int sssp, uint32_t src, uint32_t *dist);

static int check_oracle(oracle_graph *o, uint32_t n0) {
    uint32_t nn, ne, nb, mda;
    oracle_dims(o, &nn, &ne, &nb, &mda);
    uint32_t *d = malloc((size_t)(nn + 1) * 4 * 4), *e = malloc((size_t)(nn + 1) * 4 * 4);
    for (int sssp = 0; sssp < 2; ++sssp) {
        oracle_serial(o, sssp, 0, d);
        oracle_shortest(o, sssp, 0, e);
        if (memcmp(d, e, (size_t)n0 * 4)) return 1;
    }
    (void)oracle_max_degree(o);
    for (int b = 2; b <= 15; b += 13) {
        (void)oracle_max_allowed_out_degree(o, b);
        for (int lv = -1; lv <= 8; lv += 3) {
            uint32_t m2, n2;
            (void)oracle_size_after_split(o, lv, b, &m2, &n2);
        }
    }
    free(d);
    free(e);
    return 0;
}

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    long graphs = 0;
    char path[4096];
    snprintf(path, sizeof path, "%s.gr", argv[1]);
    for (uint32_t scale = 4; scale <= 11; ++scale)
        for (uint32_t ef = 2; ef <= 16; ef *= 2) {
            gga_graph *g;
            if (gga_graph_gen_rmat(scale, ef, 0.57, 0.19, 0.19, scale * 7 + ef, 1, 255, &g)) return 3;
            uint32_t md, mda, mda2, ns;
            gga_max_degree(g, &md);
            for (int b = 2; b <= 15; b += 13) {
                gga_max_allowed_out_degree(g, b, &mda);
                for (int lv = -1; lv <= 8; lv += 3) gga_size_after_split(g, lv, b, &mda2, &ns);
            }
            if (gga_graph_save_gr(g, path)) return 4;
            gga_graph *h;
            if (gga_graph_load_gr(path, &h)) return 5;
            if (h->m != g->m || memcmp(h->col, g->col, (size_t)g->m * 4)) return 6;
            gga_graph_free(h);
            oracle_graph *o = oracle_load_gr(path);
            if (!o || check_oracle(o, g->n)) return 7;
            uint32_t nn, ne, nb, mdx;
            for (int lv = 1; lv <= 7; lv += 3) {
                oracle_graph *s = oracle_load_gr(path);
                if (oracle_node_split(s, lv, 10) == 0) {
                    oracle_dims(s, &nn, &ne, &nb, &mdx);
                    uint32_t *idx = malloc((size_t)(nn + 1) * 4), *cnt = malloc((size_t)(nn + 1) * 4),
                             *dist = malloc((size_t)(nn + 1) * 4);
                    (void)oracle_child_index(s, idx, cnt);
                    oracle_init_dist(s, 0, dist);
                    (void)oracle_verify(s, 1, dist);
                    free(idx);
                    free(cnt);
                    free(dist);
                }
                oracle_free(s);
            }
            oracle_free(o);
            gga_graph_free(g);
            ++graphs;
        }
    for (uint32_t w = 2; w < 40; w += 7) {
        oracle_graph *o = oracle_gen_grid(w, w + 3, 0.05, 0.01, w, 1, 1000);
        if (!o || check_oracle(o, w * (w + 3))) return 8;
        oracle_free(o);
        ++graphs;
    }
    /* malformed files: every truncation of a small valid .gr must be refused or read, never overrun */
    gga_graph *g;
    gga_graph_gen_rmat(5, 4, 0.57, 0.19, 0.19, 3, 1, 9, &g);
    gga_graph_save_gr(g, path);
    gga_graph_free(g);
    FILE *f = fopen(path, "rb");
    fseek(f, 0, SEEK_END);
    const long len = ftell(f);
    fseek(f, 0, SEEK_SET);
    unsigned char *buf = malloc(len);
    if (fread(buf, 1, len, f) != (size_t)len) return 9;
    fclose(f);
    char bad[4096];
    snprintf(bad, sizeof bad, "%s.bad.gr", argv[1]);
    for (long cut = 0; cut < len; cut += 3) {
        f = fopen(bad, "wb");
        fwrite(buf, 1, cut, f);
        fclose(f);
        gga_graph *h;
        if (gga_graph_load_gr(bad, &h) == GGA_OK) gga_graph_free(h);
        oracle_graph *o = oracle_load_gr(bad);
        if (o) oracle_free(o);
    }
    free(buf);
    printf("graphs %ld ok\n", graphs);
    return 0;
}
