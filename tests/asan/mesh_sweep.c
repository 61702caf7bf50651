/* Host mesh code and the oracle's refinement under AddressSanitizer and
 * UndefinedBehaviorSanitizer: the seeded generators over a sweep of sizes and
 * jitters, a save/load round trip, the checker, and the serial refinement
 * with normal, tiny-batch and capacity-limited runs.  Exits non-zero (the
 * sanitizers abort) on any out-of-bounds access or undefined behaviour.
 * args: tmp-base */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gga_internal.h"

int oracle_mesh_refine(uint32_t *npts, uint32_t *ntri, double *x, double *y, uint32_t *tri, uint32_t *nbr,
                       uint32_t pcap, uint32_t tcap, double cos_bound, uint32_t batch_cap, uint32_t max_rounds,
                       uint64_t *stats);

static int refine(const gga_mesh *m, uint32_t tcap, uint32_t bcap) {
    uint32_t np = m->npts, nt = m->ntri;
    const uint32_t pcap = np + (tcap - nt);
    double *x = calloc(pcap, sizeof(double)), *y = calloc(pcap, sizeof(double));
    uint32_t *t = calloc(3 * (size_t)tcap, 4), *n = calloc(3 * (size_t)tcap, 4);
    memcpy(x, m->x, (size_t)np * 8);
    memcpy(y, m->y, (size_t)np * 8);
    memcpy(t, m->tri, 12 * (size_t)nt);
    memcpy(n, m->nbr, 12 * (size_t)nt);
    uint64_t st[6];
    const int rc = oracle_mesh_refine(&np, &nt, x, y, t, n, pcap, tcap, cos(25.0 * (3.14159265358979323846 / 180.0)),
                                      bcap, 65536, st);
    free(x);
    free(y);
    free(t);
    free(n);
    return rc;
}

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    long meshes = 0;
    for (uint32_t w = 2; w < 50; w += 3)
        for (uint32_t h = 2; h < 30; h += 4)
            for (int j = 0; j < 3; ++j) {
                gga_mesh *q;
                const double jit = j == 0 ? 0.0 : (j == 1 ? 0.3 : 0.49);
                if (gga_mesh_gen_jittered(w, h, jit, w * 31 + h + j, &q)) continue;
                gga_mesh_check_result r;
                gga_mesh_check(q, 25.0, &r);
                if (r.bad_neighbors || r.bad_orientation) return 3;
                gga_mesh_free(q);
                ++meshes;
            }
    for (uint32_t n = 0; n < 2500; n += 61) {
        gga_mesh *q;
        if (gga_mesh_gen_random(n, n + 1, &q)) return 4;
        gga_mesh_free(q);
        ++meshes;
    }
    gga_mesh *m, *l;
    if (gga_mesh_gen_random(2000, 5, &m)) return 5;
    if (gga_mesh_save_triangle(m, argv[1]) || gga_mesh_load_triangle(argv[1], &l)) return 6;
    if (l->ntri != m->ntri || memcmp(l->tri, m->tri, 12 * (size_t)m->ntri)) return 7;
    gga_mesh_free(l);
    if (refine(m, 4 * m->ntri + 65536, 1u << 20) != 0) return 8;
    if (refine(m, 4 * m->ntri + 65536, 3) != 0) return 9;
    if (refine(m, m->ntri + 700, 1u << 20) != 1) return 10; /* capacity stop */
    gga_mesh_free(m);
    printf("meshes %ld ok\n", meshes);
    return 0;
}
