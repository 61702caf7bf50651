/*
 * ORACLE — test infrastructure, not product code.
 *
 * Serial restatement of Delaunay mesh refinement in the round structure of
 * the reference's DMR (Programs/CUDA_src/Kepler_DMR/): every round, each bad
 * triangle (smallest angle below MINANGLE, dmr.cu:34 and the angle test of
 * helpers.h:150-180) plans a cavity, the plans claim the triangles they
 * would rewrite (the reference's atomic cavity marking, m_refine.h), the
 * plans that hold all their claims are retriangulated, and the new
 * triangles are re-marked; rounds repeat until no bad triangle remains
 * (the iteration loop of dmr.cu:153-346).
 *
 * Insertion rule (Ruppert's refinement, as the reference's refine kernels
 * apply it): the bad triangle's circumcentre is located by a straight walk
 * from the triangle; if the walk leaves the domain, or the circumcentre lies
 * inside the diametral circle of a boundary edge of its cavity, that
 * boundary edge is split at its midpoint instead.  The cavity is every
 * triangle reachable from the containing one whose circumcircle strictly
 * holds the new point; it is replaced by a fan from the point.
 *
 * This file defines the schedule bit for bit so the GPU kernels can be
 * compared with it exactly: the worklist in ascending triangle id (at most
 * batch_cap entries), claims as the maximum of a per-round key that is a
 * bijection of the triangle id, winners allocated point and triangle slots
 * in worklist order, and the same double-precision expressions in the same
 * order (built with -ffp-contract=off, the kernels with --fmad=false, so no
 * multiply-add is fused on either side).
 *
 * Claims.  A plan claims its cavity and its outer ring (the triangles across
 * the cavity's boundary, whose neighbour links it rewrites) in two separate
 * tables.  Two plans conflict when their cavities meet or one's cavity meets
 * the other's ring; two rings may share a triangle, since the plans rewrite
 * different edges of it, and then neither plan's new triangles can hold the
 * other's point (a fan triangle's circumcircle lies inside the union of the
 * circles of the two triangles that shared its outer edge, one in the cavity
 * and one in the ring), so the commits equal some sequential order.  A plan
 * wins a pass when it holds the highest key on every conflicting claim.  A
 * second pass lets the plans that lost, and touch no first-pass winner's
 * cavity or ring, claim again among themselves with higher keys.
 *
 * The reference runs in float (FORD, dmr.cu:36) with a thread schedule that
 * decides which of two conflicting cavities wins, so its own output is not
 * reproducible run to run; parity with it is the mesh's properties (no bad
 * triangle left, Delaunay, conforming, same area), which tests check on
 * both this oracle's and the GPU's result.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define NONE 0xFFFFFFFFu
#define CAV_MAX 64u             /* cavity triangles per plan */
#define FAN_MAX (CAV_MAX + 2u)  /* boundary edges of a cavity */
#define WALK_MAX 65536u         /* steps of the point-location walk */

enum { PLAN_FAIL = 0, PLAN_INSERT = 1, PLAN_SPLIT = 2 };
enum { ST_OK = 0, ST_CAPACITY = 1, ST_STALLED = 2, ST_ROUNDS = 3, ST_NOMEM = 4 };

typedef struct {
    uint32_t npts, ntri;
    double *x, *y;
    uint32_t *tri, *nbr;
} Mesh;

typedef struct {
    uint32_t mode, nc, nf;
    double px, py;
    uint32_t cav[CAV_MAX];
    uint32_t fa[FAN_MAX], fb[FAN_MAX], fo[FAN_MAX], fe[FAN_MAX];
    uint64_t key;
} Plan;

static double orient(const Mesh *m, uint32_t a, uint32_t b, double px, double py) {
    return (m->x[b] - m->x[a]) * (py - m->y[a]) - (m->y[b] - m->y[a]) * (px - m->x[a]);
}

/* > 0: (px, py) strictly inside the circumcircle of counter-clockwise t */
static double incircle(const Mesh *m, uint32_t t, double px, double py) {
    const uint32_t a = m->tri[3 * t], b = m->tri[3 * t + 1], c = m->tri[3 * t + 2];
    const double adx = m->x[a] - px, ady = m->y[a] - py;
    const double bdx = m->x[b] - px, bdy = m->y[b] - py;
    const double cdx = m->x[c] - px, cdy = m->y[c] - py;
    const double ad = adx * adx + ady * ady, bd = bdx * bdx + bdy * bdy, cd = cdx * cdx + cdy * cdy;
    return adx * (bdy * cd - bd * cdy) - ady * (bdx * cd - bd * cdx) + ad * (bdx * cdy - bdy * cdx);
}

/* helpers.h:150-180: an angle whose cosine exceeds cos(MINANGLE) */
static int tri_bad(const Mesh *m, uint32_t t, double cos_bound) {
    for (uint32_t i = 0; i < 3; ++i) {
        const uint32_t p = m->tri[3 * t + i], q = m->tri[3 * t + (i + 1) % 3], r = m->tri[3 * t + (i + 2) % 3];
        const double ux = m->x[q] - m->x[p], uy = m->y[q] - m->y[p];
        const double wx = m->x[r] - m->x[p], wy = m->y[r] - m->y[p];
        const double dot = ux * wx + uy * wy;
        if (dot > cos_bound * sqrt((ux * ux + uy * uy) * (wx * wx + wy * wy))) return 1;
    }
    return 0;
}

static void circumcentre(const Mesh *m, uint32_t t, double *px, double *py) {
    const uint32_t a = m->tri[3 * t], b = m->tri[3 * t + 1], c = m->tri[3 * t + 2];
    const double bx = m->x[b] - m->x[a], by = m->y[b] - m->y[a];
    const double cx = m->x[c] - m->x[a], cy = m->y[c] - m->y[a];
    const double d = 2.0 * (bx * cy - by * cx);
    const double b2 = bx * bx + by * by, c2 = cx * cx + cy * cy;
    *px = m->x[a] + (cy * b2 - by * c2) / d;
    *py = m->y[a] + (bx * c2 - cx * b2) / d;
}

static uint32_t round_prio(uint32_t t, uint32_t round) {
    return (t ^ (round * 0x9E3779B9u)) * 0x85EBCA6Bu; /* a bijection of t */
}

/* pass 0 and 1 keys of a round, above every key of earlier rounds */
static uint64_t claim_key(uint32_t t, uint32_t round, uint32_t pass) {
    return ((uint64_t)(2 * round + pass) << 32) | round_prio(t, round);
}

/* The cavity of (px, py) grown from seed; skip_m/skip_i name the boundary
 * edge being split (left out of the fan).  Returns 0 when a limit is hit. */
static int grow_cavity(const Mesh *m, Plan *p, uint32_t seed, uint32_t skip_m, uint32_t skip_i) {
    p->nc = 1;
    p->nf = 0;
    p->cav[0] = seed;
    for (uint32_t q = 0; q < p->nc; ++q) {
        const uint32_t c = p->cav[q];
        for (uint32_t i = 0; i < 3; ++i) {
            const uint32_t o = m->nbr[3 * c + i];
            if (o != NONE) {
                uint32_t in = 0;
                for (uint32_t k = 0; k < p->nc; ++k) in |= p->cav[k] == o;
                if (in) continue;
                if (incircle(m, o, p->px, p->py) > 0) {
                    if (p->nc == CAV_MAX) return 0;
                    p->cav[p->nc++] = o;
                    continue;
                }
            }
            if (c == skip_m && i == skip_i) continue;
            if (p->nf == FAN_MAX) return 0;
            p->fa[p->nf] = m->tri[3 * c + (i + 1) % 3];
            p->fb[p->nf] = m->tri[3 * c + (i + 2) % 3];
            p->fo[p->nf] = o;
            uint32_t e = 0;
            if (o != NONE)
                while (e < 3 && m->nbr[3 * o + e] != c) ++e;
            p->fe[p->nf] = e;
            p->nf++;
        }
    }
    return 1;
}

/* A fan from the point over the cavity boundary is a valid triangulation
 * only if the boundary is one simple cycle the point sees from inside. */
static int fan_ok(const Mesh *m, const Plan *p) {
    if (p->nf != p->nc + (p->mode == PLAN_SPLIT ? 1u : 2u)) return 0;
    for (uint32_t j = 0; j < p->nf; ++j) {
        if (!(orient(m, p->fa[j], p->fb[j], p->px, p->py) > 0)) return 0;
        for (uint32_t k = 0; k < j; ++k)
            if (p->fa[k] == p->fa[j]) return 0;
    }
    return 1;
}

static void plan_one(const Mesh *m, uint32_t t, uint32_t round, Plan *p) {
    p->mode = PLAN_FAIL;
    p->key = claim_key(t, round, 0);
    circumcentre(m, t, &p->px, &p->py);
    uint32_t cur = t, split_m = NONE, split_i = 0, step = 0;
    for (; step < WALK_MAX; ++step) {
        uint32_t cross = 3;
        for (uint32_t i = 0; i < 3 && cross == 3; ++i)
            if (orient(m, m->tri[3 * cur + (i + 1) % 3], m->tri[3 * cur + (i + 2) % 3], p->px, p->py) < 0) cross = i;
        if (cross == 3) break;
        const uint32_t n = m->nbr[3 * cur + cross];
        if (n == NONE) {
            split_m = cur;
            split_i = cross;
            break;
        }
        cur = n;
    }
    if (step == WALK_MAX) return;
    if (split_m == NONE) {
        if (!grow_cavity(m, p, cur, NONE, 0)) return;
        /* a boundary edge of the cavity whose diametral circle holds the point */
        for (uint32_t j = 0; j < p->nf && split_m == NONE; ++j) {
            if (p->fo[j] != NONE) continue;
            const uint32_t a = p->fa[j], b = p->fb[j];
            if ((p->px - m->x[a]) * (p->px - m->x[b]) + (p->py - m->y[a]) * (p->py - m->y[b]) < 0) {
                /* find the cavity triangle holding edge (a, b) */
                for (uint32_t q = 0; q < p->nc && split_m == NONE; ++q)
                    for (uint32_t i = 0; i < 3; ++i) {
                        const uint32_t c = p->cav[q];
                        if (m->nbr[3 * c + i] == NONE && m->tri[3 * c + (i + 1) % 3] == a &&
                            m->tri[3 * c + (i + 2) % 3] == b) {
                            split_m = c;
                            split_i = i;
                            break;
                        }
                    }
            }
        }
        if (split_m == NONE) {
            p->mode = PLAN_INSERT;
            if (!fan_ok(m, p)) p->mode = PLAN_FAIL;
            return;
        }
    }
    const uint32_t a = m->tri[3 * split_m + (split_i + 1) % 3], b = m->tri[3 * split_m + (split_i + 2) % 3];
    p->px = (m->x[a] + m->x[b]) * 0.5;
    p->py = (m->y[a] + m->y[b]) * 0.5;
    if (!grow_cavity(m, p, split_m, split_m, split_i)) return;
    p->mode = PLAN_SPLIT;
    if (!fan_ok(m, p)) p->mode = PLAN_FAIL;
}

static void claim(const Mesh *m, const Plan *p, uint64_t *owner, uint64_t *ring) {
    (void)m;
    for (uint32_t j = 0; j < p->nc; ++j)
        if (owner[p->cav[j]] < p->key) owner[p->cav[j]] = p->key;
    for (uint32_t j = 0; j < p->nf; ++j)
        if (p->fo[j] != NONE && ring[p->fo[j]] < p->key) ring[p->fo[j]] = p->key;
}

/* no higher key on this plan's cavity (in either table) or on its ring's
 * cavity claims */
static uint8_t holds(const Plan *p, const uint64_t *owner, const uint64_t *ring) {
    uint32_t ok = 1;
    for (uint32_t j = 0; j < p->nc; ++j) ok &= owner[p->cav[j]] == p->key && ring[p->cav[j]] < p->key;
    for (uint32_t j = 0; j < p->nf; ++j) ok &= p->fo[j] == NONE || owner[p->fo[j]] < p->key;
    return (uint8_t)ok;
}

static void commit(Mesh *m, uint8_t *bad, const Plan *p, uint32_t pid, uint32_t tbase, double cos_bound) {
    uint32_t slot[FAN_MAX];
    for (uint32_t j = 0; j < p->nf; ++j) slot[j] = j < p->nc ? p->cav[j] : tbase + (j - p->nc);
    m->x[pid] = p->px;
    m->y[pid] = p->py;
    for (uint32_t j = 0; j < p->nf; ++j) {
        const uint32_t s = slot[j];
        uint32_t n0 = NONE, n1 = NONE;
        for (uint32_t k = 0; k < p->nf; ++k) {
            if (p->fa[k] == p->fb[j]) n0 = slot[k];
            if (p->fb[k] == p->fa[j]) n1 = slot[k];
        }
        m->tri[3 * s] = p->fa[j];
        m->tri[3 * s + 1] = p->fb[j];
        m->tri[3 * s + 2] = pid;
        m->nbr[3 * s] = n0;
        m->nbr[3 * s + 1] = n1;
        m->nbr[3 * s + 2] = p->fo[j];
        if (p->fo[j] != NONE) m->nbr[3 * p->fo[j] + p->fe[j]] = s;
    }
    for (uint32_t j = 0; j < p->nf; ++j) bad[slot[j]] = (uint8_t)tri_bad(m, slot[j], cos_bound);
}

/* stats: [0] rounds, [1] insertions, [2] boundary splits, [3] failed plans,
 *        [4] bad before, [5] bad after.
 * log (optional, 3 words per round up to log_cap rounds): bad triangles at
 * the round's start, plans made, plans committed (dmr.cu:323 prints the
 * same per-iteration counts). */
int oracle_mesh_refine_log(uint32_t *npts, uint32_t *ntri, double *x, double *y, uint32_t *tri, uint32_t *nbr,
                           uint32_t pcap, uint32_t tcap, double cos_bound, uint32_t batch_cap, uint32_t max_rounds,
                           uint64_t *stats, uint32_t *log, uint32_t log_cap) {
    Mesh m = {*npts, *ntri, x, y, tri, nbr};
    memset(stats, 0, 6 * sizeof(uint64_t));
    uint8_t *bad = (uint8_t *)calloc(tcap ? tcap : 1, 1);
    uint64_t *owner = (uint64_t *)calloc(tcap ? tcap : 1, sizeof(uint64_t)); /* cavity claims */
    uint64_t *ring = (uint64_t *)calloc(tcap ? tcap : 1, sizeof(uint64_t));  /* outer-ring claims */
    uint32_t *lock = (uint32_t *)calloc(tcap ? tcap : 1, sizeof(uint32_t));  /* round << 2 | kind of a winner's claim */
    uint8_t *won = (uint8_t *)calloc(batch_cap ? batch_cap : 1, 1);
    uint32_t *work = (uint32_t *)malloc((size_t)(tcap ? tcap : 1) * sizeof(uint32_t));
    Plan *plans = (Plan *)malloc((size_t)(batch_cap ? batch_cap : 1) * sizeof(Plan));
    int st = ST_OK;
    if (!bad || !owner || !ring || !lock || !won || !work || !plans) st = ST_NOMEM;
    uint64_t nb = 0;
    for (uint32_t t = 0; t < m.ntri && !st; ++t) nb += bad[t] = (uint8_t)tri_bad(&m, t, cos_bound);
    stats[4] = nb;
    uint32_t round = 0;
    while (!st) {
        uint32_t nw = 0, nbad = 0;
        for (uint32_t t = 0; t < m.ntri; ++t)
            if (bad[t]) {
                ++nbad;
                if (nw < batch_cap) work[nw++] = t;
            }
        if (nw == 0) break;
        if (round == max_rounds) {
            st = ST_ROUNDS;
            break;
        }
        ++round;
        for (uint32_t k = 0; k < nw; ++k) {
            Plan *p = plans + k;
            plan_one(&m, work[k], round, p);
            if (p->mode != PLAN_FAIL) claim(&m, p, owner, ring);
        }
        /* pass 0; its winners stamp their cavity (kind 1) and ring (kind 2) */
        uint32_t wins = 0, add = 0, fails = 0;
        const uint32_t stamp = round << 2;
        for (uint32_t k = 0; k < nw; ++k) {
            Plan *p = plans + k;
            won[k] = 0;
            if (p->mode == PLAN_FAIL) {
                ++fails;
                continue;
            }
            won[k] = holds(p, owner, ring);
        }
        for (uint32_t k = 0; k < nw; ++k) {
            const Plan *p = plans + k;
            if (!won[k]) continue;
            for (uint32_t j = 0; j < p->nc; ++j) lock[p->cav[j]] = stamp | 1;
            for (uint32_t j = 0; j < p->nf; ++j)
                if (p->fo[j] != NONE) lock[p->fo[j]] = stamp | 2;
        }
        /* pass 1: plans clear of the stamps claim again */
        for (uint32_t k = 0; k < nw; ++k) {
            Plan *p = plans + k;
            if (p->mode == PLAN_FAIL || won[k]) continue;
            uint32_t blocked = 0;
            for (uint32_t j = 0; j < p->nc; ++j) blocked |= (lock[p->cav[j]] >> 2) == round;
            for (uint32_t j = 0; j < p->nf; ++j) blocked |= p->fo[j] != NONE && lock[p->fo[j]] == (stamp | 1);
            if (blocked) {
                won[k] = 2;
                continue;
            }
            p->key = claim_key(work[k], round, 1);
            claim(&m, p, owner, ring);
        }
        for (uint32_t k = 0; k < nw; ++k) {
            Plan *p = plans + k;
            if (p->mode == PLAN_FAIL || won[k] == 1) continue;
            won[k] = won[k] == 0 && holds(p, owner, ring);
        }
        for (uint32_t k = 0; k < nw; ++k) {
            Plan *p = plans + k;
            if (won[k] != 1) {
                if (p->mode != PLAN_FAIL) p->mode = PLAN_FAIL; /* lost this round */
                continue;
            }
            ++wins;
            add += p->nf - p->nc;
        }
        stats[3] += fails;
        if (log && round <= log_cap) {
            log[3 * (round - 1)] = nbad;
            log[3 * (round - 1) + 1] = nw;
            log[3 * (round - 1) + 2] = wins;
        }
        if (wins == 0) {
            st = ST_STALLED;
            break;
        }
        if ((uint64_t)m.npts + wins > pcap || (uint64_t)m.ntri + add > tcap) {
            st = ST_CAPACITY;
            break;
        }
        uint32_t pid = m.npts, tb = m.ntri;
        for (uint32_t k = 0; k < nw; ++k) {
            const Plan *p = plans + k;
            if (p->mode != PLAN_INSERT && p->mode != PLAN_SPLIT) continue;
            commit(&m, bad, p, pid, tb, cos_bound);
            stats[p->mode == PLAN_SPLIT ? 2 : 1]++;
            pid += 1;
            tb += p->nf - p->nc;
        }
        m.npts = pid;
        m.ntri = tb;
    }
    stats[0] = round;
    nb = 0;
    for (uint32_t t = 0; t < m.ntri && st != ST_NOMEM; ++t) nb += bad[t];
    stats[5] = nb;
    *npts = m.npts;
    *ntri = m.ntri;
    free(bad);
    free(owner);
    free(ring);
    free(lock);
    free(won);
    free(work);
    free(plans);
    return st;
}

int oracle_mesh_refine(uint32_t *npts, uint32_t *ntri, double *x, double *y, uint32_t *tri, uint32_t *nbr,
                       uint32_t pcap, uint32_t tcap, double cos_bound, uint32_t batch_cap, uint32_t max_rounds,
                       uint64_t *stats) {
    return oracle_mesh_refine_log(npts, ntri, x, y, tri, nbr, pcap, tcap, cos_bound, batch_cap, max_rounds, stats,
                                  NULL, 0);
}

/* bad-triangle count of a mesh (the initial marking of dmr.cu:128-150) */
uint64_t oracle_mesh_count_bad(uint32_t ntri, const double *x, const double *y, const uint32_t *tri,
                               double cos_bound) {
    Mesh m = {0, ntri, (double *)x, (double *)y, (uint32_t *)tri, NULL};
    uint64_t nb = 0;
    for (uint32_t t = 0; t < ntri; ++t) nb += (uint64_t)tri_bad(&m, t, cos_bound);
    return nb;
}
