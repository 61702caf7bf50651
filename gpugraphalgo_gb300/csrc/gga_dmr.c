/*
 * gga_dmr — drop-in for the reference's DMR executables (r_dmr.exe,
 * m_dmr.exe, ... built from Kepler_DMR/dmr.cu by genDMR).
 *
 * Arguments are the reference's (dmr.cu:81-84):  exe <basefilename>
 * It reads <basefilename>.node and .ele (readNodes / readTriangles,
 * helpers.h:5-63), refines the mesh on the GPU until no triangle has an
 * angle below 25 degrees (MINANGLE, dmr.cu:34), checks the result (dverify,
 * dmr.cu:371-391, plus the Delaunay and neighbour checks of gga_mesh_check),
 * prints the reference's summary lines and appends its 9-column row to
 * result.vi in the working directory (writeResult, myresult.h:36-52):
 *   exename, input name, triangles in, bad in, triangles out, bad out,
 *   iterations, runtime (ms, wall clock around the refinement), time (ms,
 *   device time of the refinement rounds).
 * GGA_DMR_OUT=<base> also writes the refined mesh as <base>.node / .ele.
 *
 * Differences on purpose: errors return a non-zero exit status with a
 * message, the usage check comes before the device is opened, and the
 * refinement is bit-for-bit reproducible (the reference's result depends on
 * its thread schedule).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/gga.h"

static const char *base_name(const char *p) {
    const char *s = strrchr(p, '/');
    return s ? s + 1 : p;
}

static int fail(const char *what) {
    fprintf(stderr, "%s: %s\n", what, gga_last_error());
    return 2;
}

int main(int argc, char **argv) {
    if (argc != 2) {
        printf("Usage: %s <basefilename>\n", argv[0]);
        return 1;
    }
    printf("reading graphs...\n");
    gga_mesh *m = NULL;
    if (gga_mesh_load_triangle(argv[1], &m)) return fail(argv[1]);
    gga_mesh_info info;
    gga_mesh_get_info(m, &info);
    printf("\t%u nodes\n", info.npoints);
    printf("\t%u triangles.\n", info.ntriangles);

    gga_ctx *ctx = NULL;
    if (gga_ctx_create(0, &ctx)) {
        gga_mesh_free(m);
        return fail("device");
    }
    printf("solving.\n");
    gga_refine_stats st;
    const gga_status rs = gga_mesh_refine(ctx, m, GGA_DMR_MIN_ANGLE, 0, 0, &st);
    if (rs != GGA_OK && rs != GGA_ERR_NO_PROGRESS && rs != GGA_ERR_TOO_LARGE) {
        gga_ctx_destroy(ctx);
        gga_mesh_free(m);
        return fail("refine");
    }
    if (rs != GGA_OK) fprintf(stderr, "refine: %s\n", gga_last_error());
    gga_mesh_check_result chk;
    gga_mesh_check(m, GGA_DMR_MIN_ANGLE, &chk);
    printf("NBAD=%llu,NnonDEl=%u\n", (unsigned long long)chk.bad_triangles, st.triangles_out);
    printf("verifying...\n");
    if (chk.bad_triangles || chk.bad_orientation || chk.bad_neighbors || chk.non_delaunay_edges)
        printf("verification failed: bad triangles exist: %llu (orientation %llu, links %llu, non-Delaunay edges "
               "%llu).\n",
               (unsigned long long)chk.bad_triangles, (unsigned long long)chk.bad_orientation,
               (unsigned long long)chk.bad_neighbors, (unsigned long long)chk.non_delaunay_edges);
    else
        printf("verification succeeded: 0 bad triangles exist.\n");
    printf("iterations = %u.\n", st.rounds);
    printf("%d ms.\n", (int)st.total_ms);

    const char *out = getenv("GGA_DMR_OUT");
    if (out && *out && gga_mesh_save_triangle(m, out)) fprintf(stderr, "write %s: %s\n", out, gga_last_error());
    FILE *fp = fopen("result.vi", "a+t");
    if (fp) {
        fprintf(fp, "%s,%s,%u,%u,%u,%llu,%u,%f,%f,\n", base_name(argv[0]), base_name(argv[1]), st.triangles_in,
                st.bad_in, st.triangles_out, (unsigned long long)chk.bad_triangles, st.rounds, st.total_ms,
                st.device_ms);
        fclose(fp);
    }
    gga_ctx_destroy(ctx);
    gga_mesh_free(m);
    return chk.bad_triangles || chk.non_delaunay_edges ? 1 : 0;
}
