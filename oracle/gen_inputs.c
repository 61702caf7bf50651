/*
 * ORACLE — test infrastructure, not product code.
 *
 * Input generation for the CPU legs of the benchmark.  The benchmark's
 * workloads are seeded synthetic graphs made by the library's host generator
 * (gga_graph_gen_rmat / gga_graph_gen_grid in
 * gpugraphalgo_gb300/csrc/graph_host.c, plain C with no CUDA).  That file is
 * compiled into liboracle.so as well, so the CPU baseline can build exactly
 * the same graph without loading the GPU library; the graph is then handed
 * over in the reference's own layout (oracle_from_csr, the readFromGR
 * restatement in gga_oracle.c).  Nothing here computes a distance.
 */
#include <stdint.h>

#include "../gpugraphalgo_gb300/csrc/gga_internal.h"

typedef struct oracle_graph oracle_graph;
oracle_graph *oracle_from_csr(uint32_t n, uint32_t m, const uint32_t *off, const uint32_t *col,
                              const uint32_t *wt);

static oracle_graph *to_oracle(gga_status st, gga_graph *g) {
    if (st != GGA_OK) return NULL;
    oracle_graph *o = oracle_from_csr(g->n, g->m, g->off, g->col, g->wt);
    gga_graph_free(g);
    return o;
}

oracle_graph *oracle_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
                              uint32_t wmin, uint32_t wmax) {
    gga_graph *g = NULL;
    gga_status st = gga_graph_gen_rmat(scale, edge_factor, a, b, c, seed, wmin, wmax, &g);
    return to_oracle(st, g);
}

oracle_graph *oracle_gen_grid(uint32_t width, uint32_t height, double del_prob, double longrange_frac,
                              uint64_t seed, uint32_t wmin, uint32_t wmax) {
    gga_graph *g = NULL;
    gga_status st = gga_graph_gen_grid(width, height, del_prob, longrange_frac, seed, wmin, wmax, &g);
    return to_oracle(st, g);
}
