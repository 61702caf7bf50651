/*
 * Host side of the Delaunay mesh refinement path (the reference's DMR
 * programs, Programs/CUDA_src/Kepler_DMR/): mesh storage, input, output and
 * the checker.
 *
 * A mesh is a 2-D triangulation: points (double x, y), triangles of three
 * point ids in counter-clockwise order, and for each triangle the neighbour
 * across each edge (edge i is the one opposite vertex i; GGA_MESH_NONE on the
 * domain boundary).  The reference keeps the same arrays (dmesh.h: nodex,
 * nodey, tnodes, neighbors) and marks boundary segments as two-node elements
 * read from the .poly file; here a boundary edge is simply an edge without a
 * neighbour.
 *
 *   - gga_mesh_load_triangle: the Triangle-format files readNodes /
 *     readTriangles read (helpers.h:5-63): "<base>.node" (count line, then
 *     "index x y ..."), "<base>.ele" (count line, then "index n1 n2 n3"); the
 *     .poly perimeter is not needed (boundary edges are found from the
 *     triangles) and is ignored when present.
 *   - gga_mesh_gen_jittered: a seeded Delaunay triangulation of a jittered
 *     w x h point grid over the unit square (each cell split by its Delaunay
 *     diagonal, then Lawson edge flips until every interior edge is locally
 *     Delaunay, which makes the whole triangulation Delaunay); the synthetic
 *     stand-in for the reference's input meshes, which are not in its
 *     repository.
 *   - gga_mesh_check: orientation, neighbour symmetry, area, the local
 *     Delaunay property of every interior edge and the count of triangles
 *     whose smallest angle is below the bound (the reference's checkbad rule,
 *     MINANGLE 25 in dmr.cu:32).
 */
#define _GNU_SOURCE
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/mman.h>

#include "gga_internal.h"

/* Large mesh arrays are 2 MiB aligned and marked for transparent huge pages
 * where the kernel offers them, so filling a fresh array (a refined mesh
 * copied back from the GPU) takes one page fault per 2 MiB instead of one
 * per base page.  Released with free(). */
static void *mesh_array(size_t bytes) {
    if (bytes == 0) bytes = 1;
    if (bytes < (4u << 20)) return malloc(bytes);
    void *p = NULL;
    if (posix_memalign(&p, 2u << 20, bytes)) return NULL;
#ifdef MADV_HUGEPAGE
    madvise(p, bytes, MADV_HUGEPAGE);
#endif
    return p;
}

static gga_status mesh_alloc(uint32_t npts, uint32_t ntri, gga_mesh **out) {
    gga_mesh *m = (gga_mesh *)calloc(1, sizeof *m);
    if (!m) return gga_fail(GGA_ERR_NO_MEMORY, "mesh");
    m->npts = npts;
    m->ntri = ntri;
    m->x = (double *)mesh_array((size_t)npts * sizeof(double));
    m->y = (double *)mesh_array((size_t)npts * sizeof(double));
    m->tri = (uint32_t *)mesh_array((size_t)ntri * 3 * sizeof(uint32_t));
    m->nbr = (uint32_t *)mesh_array((size_t)ntri * 3 * sizeof(uint32_t));
    if (!m->x || !m->y || !m->tri || !m->nbr) {
        gga_mesh_free(m);
        return gga_fail(GGA_ERR_NO_MEMORY, "mesh arrays (%u points, %u triangles)", npts, ntri);
    }
    *out = m;
    return GGA_OK;
}

gga_status gga_mesh_resize(gga_mesh *m, uint32_t npts, uint32_t ntri) {
    double *x = (double *)mesh_array((size_t)npts * sizeof(double));
    double *y = (double *)mesh_array((size_t)npts * sizeof(double));
    uint32_t *tri = (uint32_t *)mesh_array((size_t)ntri * 3 * sizeof(uint32_t));
    uint32_t *nbr = (uint32_t *)mesh_array((size_t)ntri * 3 * sizeof(uint32_t));
    if (!x || !y || !tri || !nbr) {
        free(x);
        free(y);
        free(tri);
        free(nbr);
        return gga_fail(GGA_ERR_NO_MEMORY, "mesh arrays (%u points, %u triangles)", npts, ntri);
    }
    free(m->x);
    free(m->y);
    free(m->tri);
    free(m->nbr);
    m->x = x;
    m->y = y;
    m->tri = tri;
    m->nbr = nbr;
    m->npts = npts;
    m->ntri = ntri;
    return GGA_OK;
}

void gga_mesh_free(gga_mesh *m) {
    if (!m) return;
    free(m->x);
    free(m->y);
    free(m->tri);
    free(m->nbr);
    free(m);
}

/* ---- geometry (double precision) ---------------------------------------- */

static double orient(const gga_mesh *m, uint32_t a, uint32_t b, uint32_t c) {
    return (m->x[b] - m->x[a]) * (m->y[c] - m->y[a]) - (m->y[b] - m->y[a]) * (m->x[c] - m->x[a]);
}

/* > 0 when d lies inside the circumcircle of the counter-clockwise (a, b, c) */
static double incircle(const gga_mesh *m, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
    const double adx = m->x[a] - m->x[d], ady = m->y[a] - m->y[d];
    const double bdx = m->x[b] - m->x[d], bdy = m->y[b] - m->y[d];
    const double cdx = m->x[c] - m->x[d], cdy = m->y[c] - m->y[d];
    const double ad = adx * adx + ady * ady, bd = bdx * bdx + bdy * bdy, cd = cdx * cdx + cdy * cdy;
    return adx * (bdy * cd - bd * cdy) - ady * (bdx * cd - bd * cdx) + ad * (bdx * cdy - bdy * cdx);
}

/* Square of the largest squared distance from d to a, b or c: the scale of
 * incircle(a, b, c, d), for relative tolerances on cocircular points. */
static double sq_span(const gga_mesh *m, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
    const uint32_t v[3] = {a, b, c};
    double sc = 0;
    for (int k = 0; k < 3; ++k) {
        const double dx = m->x[v[k]] - m->x[d], dy = m->y[v[k]] - m->y[d];
        const double q = dx * dx + dy * dy;
        sc = q > sc ? q : sc;
    }
    return sc * sc;
}

/* Smallest angle of triangle t below the bound: the largest cosine of its
 * three angles against cos(bound). */
static int tri_bad(const gga_mesh *m, uint32_t t, double cos_bound) {
    const uint32_t *v = m->tri + 3 * (size_t)t;
    for (int i = 0; i < 3; ++i) {
        const uint32_t p = v[i], q = v[(i + 1) % 3], r = v[(i + 2) % 3];
        const double ux = m->x[q] - m->x[p], uy = m->y[q] - m->y[p];
        const double wx = m->x[r] - m->x[p], wy = m->y[r] - m->y[p];
        const double cs = (ux * wx + uy * wy) / sqrt((ux * ux + uy * uy) * (wx * wx + wy * wy));
        if (cs > cos_bound) return 1;
    }
    return 0;
}

/* ---- neighbours --------------------------------------------------------- */

typedef struct {
    uint64_t key;  /* (min << 32) | max of the edge's point ids */
    uint32_t code; /* triangle << 2 | edge */
} EdgeRec;

static int cmp_edge(const void *x, const void *y) {
    const EdgeRec *a = (const EdgeRec *)x, *b = (const EdgeRec *)y;
    return a->key < b->key ? -1 : (a->key > b->key ? 1 : (a->code < b->code ? -1 : a->code > b->code));
}

/* nbr from tri: the two triangles that share an edge are neighbours across
 * it; an edge held by one triangle is a boundary edge; an edge held by more
 * than two makes the input invalid. */
gga_status gga_mesh_build_neighbors(gga_mesh *m) {
    const size_t ne = (size_t)m->ntri * 3;
    EdgeRec *e = (EdgeRec *)malloc((ne ? ne : 1) * sizeof(EdgeRec));
    if (!e) return gga_fail(GGA_ERR_NO_MEMORY, "mesh edges");
    for (uint32_t t = 0; t < m->ntri; ++t)
        for (uint32_t i = 0; i < 3; ++i) {
            const uint32_t a = m->tri[3 * t + (i + 1) % 3], b = m->tri[3 * t + (i + 2) % 3];
            EdgeRec *r = e + 3 * (size_t)t + i;
            r->key = ((uint64_t)(a < b ? a : b) << 32) | (a < b ? b : a);
            r->code = (t << 2) | i;
            m->nbr[3 * t + i] = GGA_MESH_NONE;
        }
    qsort(e, ne, sizeof(EdgeRec), cmp_edge);
    gga_status s = GGA_OK;
    for (size_t k = 0; k < ne;) {
        size_t j = k + 1;
        while (j < ne && e[j].key == e[k].key) ++j;
        if (j - k == 2) {
            const uint32_t t0 = e[k].code >> 2, i0 = e[k].code & 3, t1 = e[k + 1].code >> 2, i1 = e[k + 1].code & 3;
            m->nbr[3 * t0 + i0] = t1;
            m->nbr[3 * t1 + i1] = t0;
        } else if (j - k > 2) {
            s = gga_fail(GGA_ERR_FORMAT, "mesh: edge (%u, %u) is shared by %zu triangles", (uint32_t)(e[k].key >> 32),
                         (uint32_t)e[k].key, j - k);
            break;
        }
        k = j;
    }
    free(e);
    return s;
}

/* ---- input -------------------------------------------------------------- */

static void skip_line(FILE *f) {
    int c;
    while ((c = fgetc(f)) != EOF && c != '\n') {}
}

/* Counter-clockwise order (as the refinement's predicates assume), then the
 * neighbours. */
static gga_status mesh_finish(gga_mesh *m) {
    for (uint32_t t = 0; t < m->ntri; ++t) {
        uint32_t *v = m->tri + 3 * (size_t)t;
        if (v[0] >= m->npts || v[1] >= m->npts || v[2] >= m->npts)
            return gga_fail(GGA_ERR_FORMAT, "mesh: triangle %u names a point >= %u", t, m->npts);
        const double o = orient(m, v[0], v[1], v[2]);
        if (!(o != 0.0)) return gga_fail(GGA_ERR_FORMAT, "mesh: triangle %u is degenerate", t);
        if (o < 0) {
            const uint32_t tmp = v[1];
            v[1] = v[2];
            v[2] = tmp;
        }
    }
    return gga_mesh_build_neighbors(m);
}

gga_status gga_mesh_from_arrays(uint32_t npoints, const double *x, const double *y, uint32_t ntriangles,
                                const uint32_t *tri, gga_mesh **out) {
    if (!out || !x || !y || (ntriangles && !tri)) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    *out = NULL;
    if (npoints == 0 || npoints >= GGA_MESH_NONE || ntriangles >= GGA_MESH_NONE / 4)
        return gga_fail(GGA_ERR_INVALID_ARG, "mesh with %u points and %u triangles", npoints, ntriangles);
    gga_mesh *m = NULL;
    gga_status s = mesh_alloc(npoints, ntriangles, &m);
    if (s) return s;
    memcpy(m->x, x, (size_t)npoints * sizeof(double));
    memcpy(m->y, y, (size_t)npoints * sizeof(double));
    if (ntriangles) memcpy(m->tri, tri, (size_t)ntriangles * 3 * sizeof(uint32_t));
    s = mesh_finish(m);
    if (s) {
        gga_mesh_free(m);
        return s;
    }
    *out = m;
    return GGA_OK;
}

gga_status gga_mesh_load_triangle(const char *base, gga_mesh **out) {
    if (!base || !out) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    *out = NULL;
    char path[4096];
    snprintf(path, sizeof path, "%s.node", base);
    FILE *fn = fopen(path, "r");
    if (!fn) return gga_fail(GGA_ERR_IO, "cannot open %s", path);
    unsigned long np = 0, nt = 0;
    if (fscanf(fn, "%lu", &np) != 1 || np == 0 || np >= GGA_MESH_NONE) {
        fclose(fn);
        return gga_fail(GGA_ERR_FORMAT, "%s: bad point count", path);
    }
    skip_line(fn);
    snprintf(path, sizeof path, "%s.ele", base);
    FILE *fe = fopen(path, "r");
    if (!fe) {
        fclose(fn);
        return gga_fail(GGA_ERR_IO, "cannot open %s", path);
    }
    if (fscanf(fe, "%lu", &nt) != 1 || nt >= GGA_MESH_NONE / 4) {
        fclose(fn);
        fclose(fe);
        return gga_fail(GGA_ERR_FORMAT, "%s: bad triangle count", path);
    }
    skip_line(fe);
    gga_mesh *m = NULL;
    gga_status s = mesh_alloc((uint32_t)np, (uint32_t)nt, &m);
    if (s) {
        fclose(fn);
        fclose(fe);
        return s;
    }
    for (unsigned long i = 0; i < np && !s; ++i) {
        unsigned long idx;
        double x, y;
        if (fscanf(fn, "%lu %lf %lf", &idx, &x, &y) != 3 || idx >= np)
            s = gga_fail(GGA_ERR_FORMAT, "%s.node: bad point line %lu", base, i + 1);
        else {
            m->x[idx] = x;
            m->y[idx] = y;
        }
        skip_line(fn);
    }
    for (unsigned long i = 0; i < nt && !s; ++i) {
        unsigned long idx, a, b, c;
        if (fscanf(fe, "%lu %lu %lu %lu", &idx, &a, &b, &c) != 4 || idx >= nt || a >= np || b >= np || c >= np)
            s = gga_fail(GGA_ERR_FORMAT, "%s.ele: bad triangle line %lu", base, i + 1);
        else {
            uint32_t *v = m->tri + 3 * idx;
            v[0] = (uint32_t)a;
            v[1] = (uint32_t)b;
            v[2] = (uint32_t)c;
        }
        skip_line(fe);
    }
    fclose(fn);
    fclose(fe);
    if (!s) s = mesh_finish(m);
    if (s) {
        gga_mesh_free(m);
        return s;
    }
    *out = m;
    return GGA_OK;
}

gga_status gga_mesh_save_triangle(const gga_mesh *m, const char *base) {
    if (!m || !base) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    char path[4096];
    snprintf(path, sizeof path, "%s.node", base);
    FILE *f = fopen(path, "w");
    if (!f) return gga_fail(GGA_ERR_IO, "cannot write %s", path);
    fprintf(f, "%u 2 0 0\n", m->npts);
    for (uint32_t i = 0; i < m->npts; ++i) fprintf(f, "%u %.17g %.17g\n", i, m->x[i], m->y[i]);
    if (fclose(f)) return gga_fail(GGA_ERR_IO, "write %s", path);
    snprintf(path, sizeof path, "%s.ele", base);
    if (!(f = fopen(path, "w"))) return gga_fail(GGA_ERR_IO, "cannot write %s", path);
    fprintf(f, "%u 3 0\n", m->ntri);
    for (uint32_t t = 0; t < m->ntri; ++t)
        fprintf(f, "%u %u %u %u\n", t, m->tri[3 * t], m->tri[3 * t + 1], m->tri[3 * t + 2]);
    if (fclose(f)) return gga_fail(GGA_ERR_IO, "write %s", path);
    return GGA_OK;
}

/* xorshift64* stream for the generator */
static double urand(uint64_t *s) {
    uint64_t x = *s;
    x ^= x >> 12;
    x ^= x << 25;
    x ^= x >> 27;
    *s = x;
    return (double)((x * 0x2545F4914F6CDD1Dull) >> 11) * (1.0 / 9007199254740992.0);
}

/* Lawson flips: while an interior edge has its neighbour's far vertex inside
 * the circumcircle, replace the edge by the other diagonal of the quad.  The
 * stack holds (triangle, edge) codes, each at most once (queued flags), so
 * it never holds more than 3 * ntri entries. */
static gga_status lawson(gga_mesh *m) {
    const size_t ncode = (size_t)m->ntri * 4; /* code = t << 2 | i, i < 3 */
    uint32_t *stack = (uint32_t *)malloc(((size_t)m->ntri * 3 + 1) * sizeof(uint32_t));
    uint8_t *queued = (uint8_t *)calloc(ncode ? ncode : 1, 1);
    if (!stack || !queued) {
        free(stack);
        free(queued);
        return gga_fail(GGA_ERR_NO_MEMORY, "flip stack");
    }
    size_t sp = 0;
    for (uint32_t t = 0; t < m->ntri; ++t)
        for (uint32_t i = 0; i < 3; ++i) {
            stack[sp++] = (t << 2) | i;
            queued[(t << 2) | i] = 1;
        }
#define LAWSON_PUSH(code)                                                                                             \
    do {                                                                                                               \
        const uint32_t c_ = (code);                                                                                    \
        if (!queued[c_]) {                                                                                             \
            queued[c_] = 1;                                                                                            \
            stack[sp++] = c_;                                                                                          \
        }                                                                                                              \
    } while (0)
    uint64_t flips = 0;
    while (sp) {
        const uint32_t code = stack[--sp], t = code >> 2, i = code & 3;
        queued[code] = 0;
        const uint32_t u = m->nbr[3 * t + i];
        if (u == GGA_MESH_NONE) continue;
        uint32_t *tv = m->tri + 3 * (size_t)t, *uv = m->tri + 3 * (size_t)u;
        uint32_t j = 0; /* u's edge back to t */
        while (j < 3 && m->nbr[3 * u + j] != t) ++j;
        if (j == 3) continue;
        const uint32_t a = tv[i], b = tv[(i + 1) % 3], c = tv[(i + 2) % 3], d = uv[j];
        if (incircle(m, a, b, c, d) <= 1e-12 * sq_span(m, a, b, c, d) || orient(m, a, b, d) <= 0 ||
            orient(m, a, d, c) <= 0)
            continue;
        /* t = (a, b, c), u holds (c, b, d): new t = (a, b, d), new u = (a, d, c) */
        const uint32_t nb_ab = m->nbr[3 * t + (i + 2) % 3], nb_ca = m->nbr[3 * t + (i + 1) % 3];
        uint32_t kb = 0, kc = 0; /* in u: positions of b and c */
        while (kb < 3 && uv[kb] != b) ++kb;
        while (kc < 3 && uv[kc] != c) ++kc;
        const uint32_t u_bd = m->nbr[3 * u + kc]; /* edge (b, d) is opposite c in u */
        const uint32_t u_dc = m->nbr[3 * u + kb]; /* edge (d, c) is opposite b in u */
        tv[0] = a; tv[1] = b; tv[2] = d;
        uv[0] = a; uv[1] = d; uv[2] = c;
        m->nbr[3 * t + 0] = u_bd; /* opposite a: (b, d) */
        m->nbr[3 * t + 1] = u;    /* opposite b: (d, a) */
        m->nbr[3 * t + 2] = nb_ab;
        m->nbr[3 * u + 0] = u_dc; /* opposite a: (d, c) */
        m->nbr[3 * u + 1] = nb_ca;
        m->nbr[3 * u + 2] = t;    /* opposite c: (a, d) */
        /* the outer neighbours now face the other triangle on two edges */
        if (u_bd != GGA_MESH_NONE)
            for (int k = 0; k < 3; ++k)
                if (m->nbr[3 * u_bd + k] == u) m->nbr[3 * u_bd + k] = t;
        if (nb_ca != GGA_MESH_NONE)
            for (int k = 0; k < 3; ++k)
                if (m->nbr[3 * nb_ca + k] == t) m->nbr[3 * nb_ca + k] = u;
        LAWSON_PUSH((t << 2) | 0);
        LAWSON_PUSH((t << 2) | 2);
        LAWSON_PUSH((u << 2) | 0);
        LAWSON_PUSH((u << 2) | 1);
        if (++flips > 64ull * m->ntri + 1024) break; /* safety net */
    }
#undef LAWSON_PUSH
    free(stack);
    free(queued);
    return GGA_OK;
}

gga_status gga_mesh_gen_jittered(uint32_t w, uint32_t h, double jitter, uint64_t seed, gga_mesh **out) {
    if (!out) return gga_fail(GGA_ERR_INVALID_ARG, "out is NULL");
    *out = NULL;
    if (w < 2 || h < 2 || jitter < 0 || jitter >= 0.5)
        return gga_fail(GGA_ERR_INVALID_ARG, "jittered mesh: w, h >= 2 and jitter in [0, 0.5) (got %u, %u, %g)", w, h,
                        jitter);
    if ((uint64_t)w * h >= GGA_MESH_NONE / 8 || 2ull * (w - 1) * (h - 1) >= GGA_MESH_NONE / 8)
        return gga_fail(GGA_ERR_TOO_LARGE, "jittered mesh %u x %u", w, h);
    gga_mesh *m = NULL;
    gga_status s = mesh_alloc(w * h, 2 * (w - 1) * (h - 1), &m);
    if (s) return s;
    uint64_t st = seed * 0x9E3779B97F4A7C15ull + 0x2545F4914F6CDD1Dull;
    if (!st) st = 1;
    for (uint32_t j = 0; j < h; ++j)
        for (uint32_t i = 0; i < w; ++i) {
            /* boundary points move only along their side, so the domain stays the unit square */
            double dx = (urand(&st) * 2 - 1) * jitter, dy = (urand(&st) * 2 - 1) * jitter;
            if (i == 0 || i == w - 1) dx = 0;
            if (j == 0 || j == h - 1) dy = 0;
            m->x[j * w + i] = (i + dx) / (w - 1);
            m->y[j * w + i] = (j + dy) / (h - 1);
        }
    uint32_t t = 0;
    for (uint32_t j = 0; j + 1 < h; ++j)
        for (uint32_t i = 0; i + 1 < w; ++i) {
            const uint32_t a = j * w + i, b = a + 1, c = a + w + 1, d = a + w; /* counter-clockwise cell */
            uint32_t *v = m->tri + 3 * (size_t)t;
            /* jitter < 0.5 keeps every cell a simple quad, so one diagonal lies inside it */
            if (orient(m, a, b, c) > 0 && orient(m, a, c, d) > 0) {
                v[0] = a; v[1] = b; v[2] = c; /* diagonal a-c */
                v[3] = a; v[4] = c; v[5] = d;
            } else {
                v[0] = a; v[1] = b; v[2] = d; /* diagonal b-d */
                v[3] = b; v[4] = c; v[5] = d;
            }
            t += 2;
        }
    for (uint32_t k = 0; k < m->ntri && !s; ++k)
        if (orient(m, m->tri[3 * k], m->tri[3 * k + 1], m->tri[3 * k + 2]) <= 0)
            s = gga_fail(GGA_ERR_INVALID_ARG, "jittered mesh: jitter %g folds a cell", jitter);
    if (!s) s = gga_mesh_build_neighbors(m);
    if (!s) s = lawson(m);
    if (s) {
        gga_mesh_free(m);
        return s;
    }
    *out = m;
    return GGA_OK;
}

/* ---- random-point Delaunay mesh ------------------------------------------ */

typedef struct {
    uint32_t *cav, *fa, *fb, *fo, *fm;
    uint32_t ncap, fcap;
} BwBuf;

static int bw_grow(uint32_t **a, uint32_t *cap, uint32_t need) {
    if (need <= *cap) return 1;
    uint32_t nc = *cap ? *cap : 64;
    while (nc < need) nc *= 2;
    uint32_t *p = (uint32_t *)realloc(*a, (size_t)nc * sizeof(uint32_t));
    if (!p) return 0;
    *a = p;
    *cap = nc;
    return 1;
}

/* the four fan arrays share one capacity */
static int bw_fan_room(BwBuf *b, uint32_t need) {
    if (need <= b->fcap) return 1;
    uint32_t c0 = b->fcap, c1 = b->fcap, c2 = b->fcap, c3 = b->fcap;
    if (!bw_grow(&b->fa, &c0, need) || !bw_grow(&b->fb, &c1, need) || !bw_grow(&b->fo, &c2, need) ||
        !bw_grow(&b->fm, &c3, need))
        return 0;
    b->fcap = c0;
    return 1;
}

/* > 0 when (px, py) lies strictly inside the circumcircle of triangle t */
static double incircle_pt(const gga_mesh *m, uint32_t t, double px, double py) {
    const uint32_t *v = m->tri + 3 * (size_t)t;
    const double adx = m->x[v[0]] - px, ady = m->y[v[0]] - py;
    const double bdx = m->x[v[1]] - px, bdy = m->y[v[1]] - py;
    const double cdx = m->x[v[2]] - px, cdy = m->y[v[2]] - py;
    const double ad = adx * adx + ady * ady, bd = bdx * bdx + bdy * bdy, cd = cdx * cdx + cdy * cdy;
    return adx * (bdy * cd - bd * cdy) - ady * (bdx * cd - bd * cdx) + ad * (bdx * cdy - bdy * cdx);
}

static double orient_pt(const gga_mesh *m, uint32_t a, uint32_t b, double px, double py) {
    return (m->x[b] - m->x[a]) * (py - m->y[a]) - (m->y[b] - m->y[a]) * (px - m->x[a]);
}

/* Bowyer-Watson insertion of point id `pid` (coordinates already stored):
 * walk from *hint to the containing triangle, grow the cavity of triangles
 * whose circumcircle holds the point, replace it by a fan.  Returns 1 when
 * inserted, 0 when the point is skipped (on an edge or vertex, or outside),
 * -1 on allocation failure. */
static int bw_insert(gga_mesh *m, uint32_t pid, uint32_t *hint, BwBuf *b) {
    const double px = m->x[pid], py = m->y[pid];
    uint32_t cur = *hint;
    for (uint64_t step = 0;; ++step) {
        uint32_t cross = 3;
        for (uint32_t i = 0; i < 3 && cross == 3; ++i)
            if (orient_pt(m, m->tri[3 * cur + (i + 1) % 3], m->tri[3 * cur + (i + 2) % 3], px, py) < 0) cross = i;
        if (cross == 3) break;
        const uint32_t n = m->nbr[3 * cur + cross];
        if (n == GGA_MESH_NONE || step > 4ull * m->ntri + 64) return 0;
        cur = n;
    }
    for (uint32_t i = 0; i < 3; ++i)
        if (!(orient_pt(m, m->tri[3 * cur + (i + 1) % 3], m->tri[3 * cur + (i + 2) % 3], px, py) > 0)) return 0;
    uint32_t nc = 1, nf = 0;
    if (!bw_grow(&b->cav, &b->ncap, 1)) return -1;
    b->cav[0] = cur;
    for (uint32_t q = 0; q < nc; ++q) {
        const uint32_t c = b->cav[q];
        for (uint32_t i = 0; i < 3; ++i) {
            const uint32_t o = m->nbr[3 * c + i];
            if (o != GGA_MESH_NONE) {
                uint32_t in = 0;
                for (uint32_t k = 0; k < nc && !in; ++k) in = b->cav[k] == o;
                if (in) continue;
                if (incircle_pt(m, o, px, py) > 0) {
                    if (!bw_grow(&b->cav, &b->ncap, nc + 1)) return -1;
                    b->cav[nc++] = o;
                    continue;
                }
            }
            if (!bw_fan_room(b, nf + 1)) return -1;
            b->fa[nf] = m->tri[3 * c + (i + 1) % 3];
            b->fb[nf] = m->tri[3 * c + (i + 2) % 3];
            b->fo[nf] = o;
            b->fm[nf] = c;
            nf++;
        }
    }
    if (nf != nc + 2) return 0; /* not a disk: leave this point out */
    for (uint32_t j = 0; j < nf; ++j)
        if (!(orient_pt(m, b->fa[j], b->fb[j], px, py) > 0)) return 0;
    /* slots: the cavity's, then two new ones */
    const uint32_t base = m->ntri;
    m->ntri += 2;
    for (uint32_t j = 0; j < nf; ++j) {
        const uint32_t s = j < nc ? b->cav[j] : base + (j - nc);
        b->fm[j] = s; /* reuse fm as the fan slot */
    }
    for (uint32_t j = 0; j < nf; ++j) {
        const uint32_t s = b->fm[j];
        uint32_t n0 = GGA_MESH_NONE, n1 = GGA_MESH_NONE;
        for (uint32_t k = 0; k < nf; ++k) {
            if (b->fa[k] == b->fb[j]) n0 = b->fm[k];
            if (b->fb[k] == b->fa[j]) n1 = b->fm[k];
        }
        const uint32_t o = b->fo[j];
        m->tri[3 * s] = b->fa[j];
        m->tri[3 * s + 1] = b->fb[j];
        m->tri[3 * s + 2] = pid;
        m->nbr[3 * s] = n0;
        m->nbr[3 * s + 1] = n1;
        m->nbr[3 * s + 2] = o;
        if (o != GGA_MESH_NONE)
            for (uint32_t e = 0; e < 3; ++e) {
                const uint32_t *ov = m->tri + 3 * (size_t)o;
                if (ov[e] != b->fa[j] && ov[e] != b->fb[j]) m->nbr[3 * o + e] = s;
            }
    }
    *hint = b->fm[0];
    return 1;
}

static int cmp_u64(const void *x, const void *y) {
    const uint64_t a = *(const uint64_t *)x, b = *(const uint64_t *)y;
    return a < b ? -1 : a > b;
}

gga_status gga_mesh_gen_random(uint32_t npoints, uint64_t seed, gga_mesh **out) {
    if (!out) return gga_fail(GGA_ERR_INVALID_ARG, "out is NULL");
    *out = NULL;
    if (npoints >= GGA_MESH_NONE / 8) return gga_fail(GGA_ERR_TOO_LARGE, "random mesh of %u points", npoints);
    const uint32_t N = npoints + 4, T = 2 * N - 6;
    gga_mesh *m = NULL;
    gga_status s = mesh_alloc(N, T, &m);
    if (s) return s;
    uint64_t st = seed * 0x9E3779B97F4A7C15ull + 0x2545F4914F6CDD1Dull;
    if (!st) st = 1;
    /* corners, then the random points in serpentine cell order so that each
     * walk starts next to its target */
    const double cx[4] = {0, 1, 1, 0}, cy[4] = {0, 0, 1, 1};
    for (int i = 0; i < 4; ++i) {
        m->x[i] = cx[i];
        m->y[i] = cy[i];
    }
    uint64_t *key = (uint64_t *)malloc((size_t)(npoints ? npoints : 1) * sizeof(uint64_t));
    double *rx = (double *)malloc((size_t)(npoints ? npoints : 1) * sizeof(double));
    double *ry = (double *)malloc((size_t)(npoints ? npoints : 1) * sizeof(double));
    BwBuf b = {0};
    if (!key || !rx || !ry) s = gga_fail(GGA_ERR_NO_MEMORY, "random mesh points");
    uint32_t G = 1;
    while ((uint64_t)G * G < npoints / 2 + 1) ++G;
    for (uint32_t i = 0; i < npoints && !s; ++i) {
        rx[i] = urand(&st);
        ry[i] = urand(&st);
        uint32_t r = (uint32_t)(ry[i] * G), c = (uint32_t)(rx[i] * G);
        if (r >= G) r = G - 1;
        if (c >= G) c = G - 1;
        if (r & 1) c = G - 1 - c;
        key[i] = ((uint64_t)(r * G + c) << 32) | i;
    }
    if (!s) qsort(key, npoints, sizeof(uint64_t), cmp_u64);
    m->npts = 4;
    m->ntri = 2;
    const uint32_t t0[6] = {0, 1, 2, 0, 2, 3}, n0[6] = {GGA_MESH_NONE, 1, GGA_MESH_NONE, GGA_MESH_NONE, GGA_MESH_NONE, 0};
    memcpy(m->tri, t0, sizeof t0);
    memcpy(m->nbr, n0, sizeof n0);
    uint32_t hint = 0;
    for (uint32_t k = 0; k < npoints && !s; ++k) {
        const uint32_t i = (uint32_t)key[k];
        m->x[m->npts] = rx[i];
        m->y[m->npts] = ry[i];
        const int r = bw_insert(m, m->npts, &hint, &b);
        if (r < 0) s = gga_fail(GGA_ERR_NO_MEMORY, "random mesh cavity");
        else if (r > 0) m->npts++;
    }
    free(key);
    free(rx);
    free(ry);
    free(b.cav);
    free(b.fa);
    free(b.fb);
    free(b.fo);
    free(b.fm);
    if (s) {
        gga_mesh_free(m);
        return s;
    }
    *out = m;
    return GGA_OK;
}

/* ---- queries ------------------------------------------------------------ */

gga_status gga_mesh_get_info(const gga_mesh *m, gga_mesh_info *info) {
    if (!m || !info) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    memset(info, 0, sizeof *info);
    info->npoints = m->npts;
    info->ntriangles = m->ntri;
    return GGA_OK;
}

gga_status gga_mesh_arrays(const gga_mesh *m, const double **x, const double **y, const uint32_t **tri,
                           const uint32_t **nbr) {
    if (!m) return gga_fail(GGA_ERR_INVALID_ARG, "NULL mesh");
    if (x) *x = m->x;
    if (y) *y = m->y;
    if (tri) *tri = m->tri;
    if (nbr) *nbr = m->nbr;
    return GGA_OK;
}

gga_status gga_mesh_check(const gga_mesh *m, double min_angle_deg, gga_mesh_check_result *r) {
    if (!m || !r) return gga_fail(GGA_ERR_INVALID_ARG, "NULL argument");
    memset(r, 0, sizeof *r);
    const double cb = cos(min_angle_deg * 3.14159265358979323846 / 180.0);
    double area = 0;
    for (uint32_t t = 0; t < m->ntri; ++t) {
        const uint32_t *v = m->tri + 3 * (size_t)t;
        const double o = orient(m, v[0], v[1], v[2]);
        area += 0.5 * o;
        if (o <= 0) r->bad_orientation++;
        if (tri_bad(m, t, cb)) r->bad_triangles++;
        for (uint32_t i = 0; i < 3; ++i) {
            const uint32_t u = m->nbr[3 * t + i];
            if (u == GGA_MESH_NONE) {
                r->boundary_edges++;
                continue;
            }
            if (u >= m->ntri) {
                r->bad_neighbors++;
                continue;
            }
            /* u must hold the same edge, with t across it */
            const uint32_t a = v[(i + 1) % 3], b = v[(i + 2) % 3];
            uint32_t j = 0;
            while (j < 3 && m->nbr[3 * u + j] != t) ++j;
            const uint32_t *w = m->tri + 3 * (size_t)u;
            if (j == 3 || !((w[(j + 1) % 3] == b && w[(j + 2) % 3] == a))) {
                r->bad_neighbors++;
                continue;
            }
            /* locally Delaunay: u's far vertex not inside t's circumcircle
             * (relative tolerance for cocircular points) */
            const uint32_t d = w[j];
            if (incircle(m, v[0], v[1], v[2], d) > 1e-9 * sq_span(m, v[0], v[1], v[2], d)) r->non_delaunay_edges++;
        }
    }
    r->area = area;
    return GGA_OK;
}
