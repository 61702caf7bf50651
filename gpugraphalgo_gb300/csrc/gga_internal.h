/*
 * Internal declarations shared by the host C code and the CUDA sources.
 * Not part of the ABI.
 */
#ifndef GGA_INTERNAL_H
#define GGA_INTERNAL_H

#include <pthread.h>
#include <stdint.h>

#include "../../include/gga.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Vertex and edge limits: ids, offsets and counts are uint32 on the device. */
#define GGA_MAX_NODES 0x80000000u
/* edges: 8192 short of 2^32, so that a unit's 32-bit edge positions (a unit
 * start plus up to 4095) cannot wrap */
#define GGA_MAX_EDGES 0xFFFFE000u

/* Host-side graph.  The CSR is 0-based: vertex u owns edges
 * [off[u], off[u+1]).  The reference keeps the same arrays 1-based with a null
 * edge slot 0 (graph.h:251-254); the 1-based view is produced on export. */
struct gga_graph {
    uint32_t n;     /* original vertices */
    uint32_t m;     /* directed edges */
    uint32_t *off;  /* n+1 */
    uint32_t *col;  /* m */
    uint32_t *wt;   /* m */
    uint32_t maxdeg;
    uint32_t maxw;
    double wavg;    /* mean edge weight (1 for an edgeless graph) */
    int symmetric;
    int wsymmetric; /* every edge's reverse has the same weight: 1 yes, -1 no, 0 not known */

    /* node split (graph.h:415-522); arrays live on the device */
    int32_t split_level;
    int32_t split_buckets;
    uint32_t mda;
    uint32_t ns;                    /* split vertex count n' */
    uint32_t parents_with_children; /* myParentCount */

    /* parameters gga_autotune picked for this graph (has_tuned != 0) */
    gga_params tuned;
    int has_tuned;

    /* device residency, owned; see device_graph.cu */
    void *dev;
    int dev_device;
    pthread_mutex_t lock;
};

/* Host-side mesh (gga_mesh_*): points, counter-clockwise triangles and the
 * neighbour across each triangle edge (edge i opposite vertex i). */
struct gga_mesh {
    uint32_t npts;
    uint32_t ntri;
    double *x, *y;  /* npts */
    uint32_t *tri;  /* 3 * ntri */
    uint32_t *nbr;  /* 3 * ntri, GGA_MESH_NONE on the boundary */
};

/* Recomputes nbr from tri (GGA_ERR_FORMAT if an edge has > 2 triangles). */
gga_status gga_mesh_build_neighbors(gga_mesh *m);
/* Replaces the mesh's arrays with fresh ones of the given sizes (contents
 * undefined). */
gga_status gga_mesh_resize(gga_mesh *m, uint32_t npts, uint32_t ntri);

/* Thread-local error message; returns `st` for tail calls. */
gga_status gga_fail(gga_status st, const char *fmt, ...);
void gga_clear_error(void);

/* Allocates an empty graph with n vertices and m edges (arrays uninitialised). */
gga_status gga_graph_alloc(uint32_t n, uint32_t m, gga_graph **out);
/* Recomputes maxdeg / maxw from the CSR. */
void gga_graph_refresh_stats(gga_graph *g);

/* Device-state teardown hook set by device_graph.cu (NULL before first use). */
extern void (*gga_dev_graph_release_hook)(gga_graph *g);

/* Host wall clock in milliseconds. */
double gga_now_ms(void);

#ifdef __cplusplus
}
#endif
#endif
