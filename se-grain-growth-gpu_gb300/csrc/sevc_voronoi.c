/*
 * Periodic Voronoi microstructures in the reference's input format: the
 * job of the reference's generator voronoi/voronoi.py:12-109 (3x3 tiled
 * scipy Voronoi, vertices merged on a 2^-32 grid, only triple junctions
 * accepted, a new sample drawn otherwise), written in C with OpenMP.
 *
 * Every cell is built on its own: the square around its seed is clipped by
 * the bisector half-planes of the neighbouring seeds, found in a bucket
 * grid of about two seeds per bucket with periodic wrap, in rings until no
 * seed outside can reach the cell (twice the cell's radius).  A Voronoi
 * vertex is the triple of seeds whose bisectors meet there; the cell of the
 * smallest of the three emits it, computed as the circumcentre of the
 * three (relative to that seed), folded into [0, 1) and put on the 2^-32
 * grid as voronoi.py:47-48 does.  A ridge is emitted by the smaller of its
 * two cells.  Anything that is not a clean triple-junction mesh with
 * V = 2N vertices and B = 3N ridges (two cells that disagree about an edge,
 * two vertices on one grid point) makes the sample be drawn again, like
 * voronoi.py:75-84.
 *
 * Random numbers: xoshiro256** (Blackman and Vigna) seeded by splitmix64;
 * the seeds, then the orientations U[0,1), then the stored energies
 * (U[0,1), or triangular(3, 6, 6) by inversion, 3 + 3 sqrt(u)) come from
 * one stream.  The sample is not numpy's for the same seed: meshes agree
 * with voronoi.py's in distribution, not point by point.
 */
#include "sevc_host.h"

#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define VOR_MAXV 96          /* vertices of one cell while it is clipped */
#define VOR_MAXC 512         /* candidate neighbours of one cell */

typedef struct { uint64_t s[4]; } vor_rng;

static uint64_t vor_sm64(uint64_t *x)
{
    uint64_t z = (*x += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
static void vor_seed(vor_rng *r, uint64_t seed)
{
    for (int i = 0; i < 4; i++) r->s[i] = vor_sm64(&seed);
}
static uint64_t vor_rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
static uint64_t vor_next(vor_rng *r)
{
    uint64_t *s = r->s, res = vor_rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
    s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3]; s[2] ^= t; s[3] = vor_rotl(s[3], 45);
    return res;
}
static double vor_unit(vor_rng *r) { return (double)(vor_next(r) >> 11) * 0x1.0p-53; }

typedef struct {
    int n, nb;               /* seeds, buckets per side */
    const double *p;         /* seeds, interleaved */
    int *bstart, *bidx;      /* bucket lists (CSR) */
} vor_grid;

/* one cell: vertices (relative to the seed) and, for edge k from vertex k
 * to vertex k+1, the index (into the cell's candidate list) of the
 * neighbour whose bisector it lies on (-1: the bounding square) */
typedef struct {
    int m;
    double vx[VOR_MAXV], vy[VOR_MAXV];
    int edge[VOR_MAXV];
} vor_cell;

typedef struct { int j; double dx, dy, d2; } vor_cand;

static int cand_cmp(const void *a, const void *b)
{
    const vor_cand *x = (const vor_cand *)a, *y = (const vor_cand *)b;
    if (x->d2 < y->d2) return -1;
    if (x->d2 > y->d2) return 1;
    return x->j - y->j;
}

/* clip the convex polygon by {v : v.d <= |d|^2 / 2} (the half-plane of the
 * seed against the neighbour at displacement d); the new edge gets id j */
static int clip(vor_cell *c, double dx, double dy, int j)
{
    double h = 0.5 * (dx * dx + dy * dy);
    double s[VOR_MAXV];
    int any_out = 0;
    for (int k = 0; k < c->m; k++) {
        s[k] = c->vx[k] * dx + c->vy[k] * dy - h;
        any_out |= s[k] > 0;
    }
    if (!any_out) return 0;
    vor_cell o;
    o.m = 0;
    for (int k = 0; k < c->m; k++) {
        int k1 = (k + 1) % c->m;
        int in0 = s[k] <= 0, in1 = s[k1] <= 0;
        if (in0) {
            if (o.m >= VOR_MAXV) return -1;
            o.vx[o.m] = c->vx[k]; o.vy[o.m] = c->vy[k]; o.edge[o.m] = c->edge[k]; o.m++;
        }
        if (in0 != in1) {                 /* the edge crosses the line */
            double t = s[k] / (s[k] - s[k1]);
            if (o.m >= VOR_MAXV) return -1;
            o.vx[o.m] = c->vx[k] + t * (c->vx[k1] - c->vx[k]);
            o.vy[o.m] = c->vy[k] + t * (c->vy[k1] - c->vy[k]);
            o.edge[o.m] = in0 ? j : c->edge[k];   /* leaving: the clip line follows */
            o.m++;
        }
    }
    *c = o;
    return 0;
}

/* the Voronoi cell of seed i; cand receives its candidate neighbours
 * (edge ids index it).  0 on success. */
static int build_cell(const vor_grid *g, int i, vor_cell *c, vor_cand *cand)
{
    const double xi = g->p[2 * i], yi = g->p[2 * i + 1], hb = 1.0 / g->nb;
    const int bx = (int)(xi * g->nb) < g->nb ? (int)(xi * g->nb) : g->nb - 1;
    const int by = (int)(yi * g->nb) < g->nb ? (int)(yi * g->nb) : g->nb - 1;
    for (int R = 1; R < g->nb; R++) {
        /* candidates of every bucket within Chebyshev distance R */
        int nc = 0;
        for (int dy = -R; dy <= R; dy++)
            for (int dxb = -R; dxb <= R; dxb++) {
                int ux = bx + dxb, uy = by + dy;
                int sx = ux < 0 ? -1 : (ux >= g->nb ? 1 : 0), sy = uy < 0 ? -1 : (uy >= g->nb ? 1 : 0);
                int wx = ux - sx * g->nb, wy = uy - sy * g->nb;
                if (wx < 0 || wx >= g->nb || wy < 0 || wy >= g->nb) return -1;
                int b = wy * g->nb + wx;
                for (int q = g->bstart[b]; q < g->bstart[b + 1]; q++) {
                    int j = g->bidx[q];
                    if (j == i && sx == 0 && sy == 0) continue;
                    if (nc >= VOR_MAXC) return -1;
                    double ddx = g->p[2 * j] + sx - xi, ddy = g->p[2 * j + 1] + sy - yi;
                    cand[nc].j = j; cand[nc].dx = ddx; cand[nc].dy = ddy; cand[nc].d2 = ddx * ddx + ddy * ddy;
                    nc++;
                }
            }
        qsort(cand, (size_t)nc, sizeof(vor_cand), cand_cmp);
        double L = (R + 1) * hb;
        c->m = 4;
        c->vx[0] = -L; c->vy[0] = -L; c->edge[0] = -1;
        c->vx[1] = L; c->vy[1] = -L; c->edge[1] = -1;
        c->vx[2] = L; c->vy[2] = L; c->edge[2] = -1;
        c->vx[3] = -L; c->vy[3] = L; c->edge[3] = -1;
        for (int q = 0; q < nc; q++) {
            double r2 = 0;
            for (int k = 0; k < c->m; k++) {
                double d = c->vx[k] * c->vx[k] + c->vy[k] * c->vy[k];
                r2 = d > r2 ? d : r2;
            }
            if (cand[q].d2 > 4 * r2) break;      /* no seed this far can cut the cell */
            if (clip(c, cand[q].dx, cand[q].dy, q)) return -1;
        }
        double r2 = 0;
        int open = 0;
        for (int k = 0; k < c->m; k++) {
            double d = c->vx[k] * c->vx[k] + c->vy[k] * c->vy[k];
            r2 = d > r2 ? d : r2;
            open |= c->edge[k] < 0;
        }
        /* every seed outside the gathered rings is at least R*hb away */
        if (!open && 4 * r2 <= (R * hb) * (R * hb)) return 0;
    }
    return -1;
}

/* vertex k of a cell lies between edges k-1 and k: its seed triple, sorted */
static void triple_of(const vor_cell *c, const vor_cand *cand, int i, int k, int t[3])
{
    int a = i, b = cand[c->edge[(k + c->m - 1) % c->m]].j, d = cand[c->edge[k]].j, x;
    if (a > b) { x = a; a = b; b = x; }
    if (b > d) { x = b; b = d; d = x; }
    if (a > b) { x = a; a = b; b = x; }
    t[0] = a; t[1] = b; t[2] = d;
}

/* position on the 2^-32 grid of [0, 1), voronoi.py:47-48 (round half to even) */
static double grid32(double x)
{
    double v = nearbyint(x * 4294967296.0);
    v = fmod(v, 4294967296.0);
    if (v < 0) v += 4294967296.0;
    return v / 4294967296.0;
}

static int cmp_u64(const void *a, const void *b)
{
    uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return x < y ? -1 : x > y;
}

/* one attempt on the seeds p; 0 and the mesh on success */
static int vor_attempt(int n, const double *p, double *xy, int32_t *ridges)
{
    vor_grid g;
    g.n = n;
    g.p = p;
    g.nb = (int)floor(sqrt(n / 2.0));
    if (g.nb < 5) g.nb = 5;
    int NB = g.nb * g.nb, rc = -1, bad = 0;
    g.bstart = (int *)calloc((size_t)NB + 1, sizeof(int));
    g.bidx = (int *)malloc(sizeof(int) * (size_t)n);
    int *cnt = (int *)calloc((size_t)n + 1, sizeof(int));      /* corners per cell, then offsets */
    int *tri = NULL, *own = NULL, *voff = NULL, *roff = NULL, *fill = NULL;
    double *pos = NULL;
    uint64_t *key = NULL;
    if (!g.bstart || !g.bidx || !cnt) goto out;
    for (int i = 0; i < n; i++) {
        int bx = (int)(p[2 * i] * g.nb), by = (int)(p[2 * i + 1] * g.nb);
        bx = bx < g.nb ? bx : g.nb - 1;
        by = by < g.nb ? by : g.nb - 1;
        g.bstart[by * g.nb + bx + 1]++;
    }
    for (int b = 0; b < NB; b++) g.bstart[b + 1] += g.bstart[b];
    fill = (int *)malloc(sizeof(int) * (size_t)NB);
    if (!fill) goto out;
    memcpy(fill, g.bstart, sizeof(int) * (size_t)NB);
    for (int i = 0; i < n; i++) {
        int bx = (int)(p[2 * i] * g.nb), by = (int)(p[2 * i + 1] * g.nb);
        bx = bx < g.nb ? bx : g.nb - 1;
        by = by < g.nb ? by : g.nb - 1;
        g.bidx[fill[by * g.nb + bx]++] = i;
    }
    /* pass 1: corner count of every cell */
#pragma omp parallel reduction(| : bad)
    {
        vor_cell *c = (vor_cell *)malloc(sizeof(vor_cell));
        vor_cand *cand = (vor_cand *)malloc(sizeof(vor_cand) * VOR_MAXC);
#pragma omp for schedule(dynamic, 256)
        for (int i = 0; i < n; i++) {
            if (!c || !cand || build_cell(&g, i, c, cand)) { bad = 1; continue; }
            cnt[i + 1] = c->m;
        }
        free(c);
        free(cand);
    }
    if (bad) goto out;
    for (int i = 0; i < n; i++) cnt[i + 1] += cnt[i];
    size_t tot = (size_t)cnt[n];
    if (tot != 6 * (size_t)n) goto out;            /* Euler: the sides sum to 2B = 6N */
    tri = (int *)malloc(sizeof(int) * 3 * tot);
    own = (int *)malloc(sizeof(int) * tot);        /* vertex id of every (cell, corner) */
    voff = (int *)calloc((size_t)n + 1, sizeof(int));
    roff = (int *)calloc((size_t)n + 1, sizeof(int));
    pos = (double *)malloc(sizeof(double) * 2 * tot);
    if (!tri || !own || !voff || !roff || !pos) goto out;
    /* pass 2: triples, positions of the corners a cell emits, ridge counts */
#pragma omp parallel reduction(| : bad)
    {
        vor_cell *c = (vor_cell *)malloc(sizeof(vor_cell));
        vor_cand *cand = (vor_cand *)malloc(sizeof(vor_cand) * VOR_MAXC);
#pragma omp for schedule(dynamic, 256)
        for (int i = 0; i < n; i++) {
            if (!c || !cand || build_cell(&g, i, c, cand) || c->m != cnt[i + 1] - cnt[i]) { bad = 1; continue; }
            int base = cnt[i], owned = 0, rid = 0;
            for (int k = 0; k < c->m; k++) {
                int t[3];
                triple_of(c, cand, i, k, t);
                memcpy(tri + 3 * (size_t)(base + k), t, sizeof t);
                own[base + k] = -1;
                if (t[0] == i) {      /* this cell emits the vertex: circumcentre of the triple */
                    const vor_cand *a = &cand[c->edge[(k + c->m - 1) % c->m]], *b = &cand[c->edge[k]];
                    double D = 2.0 * (a->dx * b->dy - a->dy * b->dx);
                    double cx = (b->dy * a->d2 - a->dy * b->d2) / D, cy = (a->dx * b->d2 - b->dx * a->d2) / D;
                    pos[2 * (size_t)(base + k)] = grid32(p[2 * i] + cx);
                    pos[2 * (size_t)(base + k) + 1] = grid32(p[2 * i + 1] + cy);
                    own[base + k] = -2;
                    owned++;
                }
                if (i < cand[c->edge[k]].j) rid++;
            }
            voff[i + 1] = owned;
            roff[i + 1] = rid;
        }
        free(c);
        free(cand);
    }
    if (bad) goto out;
    for (int i = 0; i < n; i++) { voff[i + 1] += voff[i]; roff[i + 1] += roff[i]; }
    if (voff[n] != 2 * n || roff[n] != 3 * n) goto out;
    /* vertex ids: emitted corners in cell order; every other corner looks
     * its triple up among the corners of the cell that emitted it */
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) {
        int id = voff[i];
        for (int q = cnt[i]; q < cnt[i + 1]; q++)
            if (own[q] == -2) {
                xy[2 * (size_t)id] = pos[2 * (size_t)q];
                xy[2 * (size_t)id + 1] = pos[2 * (size_t)q + 1];
                own[q] = id++;
            }
    }
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int i = 0; i < n; i++)
        for (int q = cnt[i]; q < cnt[i + 1]; q++) {
            if (own[q] >= 0) continue;
            const int *t = tri + 3 * (size_t)q;
            int o = t[0], found = -1;
            for (int r = cnt[o]; r < cnt[o + 1]; r++) {
                const int *u = tri + 3 * (size_t)r;
                if (u[0] == t[0] && u[1] == t[1] && u[2] == t[2]) { found = r; break; }
            }
            if (found < 0 || own[found] < 0) { bad = 1; continue; }
            own[q] = own[found];
        }
    if (bad) goto out;
    /* ridges, emitted by the smaller cell of the two */
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int i = 0; i < n; i++) {
        int r = roff[i], m = cnt[i + 1] - cnt[i];
        for (int k = 0; k < m; k++) {
            int q0 = cnt[i] + k, q1 = cnt[i] + (k + 1) % m;
            /* the edge from corner k to k+1 is shared with the seed that is in
             * both corners' triples besides i */
            const int *a = tri + 3 * (size_t)q0, *b = tri + 3 * (size_t)q1;
            int other = -1, shared = 0;
            for (int x = 0; x < 3; x++)
                for (int y = 0; y < 3; y++)
                    if (a[x] == b[y] && a[x] != i) { other = a[x]; shared++; }
            if (shared != 1) { bad = 1; break; }
            if (i < other) {
                ridges[2 * (size_t)r] = own[q0];
                ridges[2 * (size_t)r + 1] = own[q1];
                r++;
            }
        }
    }
    if (bad) goto out;
    /* two vertices on one grid point (voronoi.py:95-98): draw again */
    key = (uint64_t *)malloc(sizeof(uint64_t) * 2 * (size_t)n);
    if (!key) goto out;
    for (int v = 0; v < 2 * n; v++)
        key[v] = ((uint64_t)(xy[2 * (size_t)v] * 4294967296.0) << 32) | (uint64_t)(xy[2 * (size_t)v + 1] * 4294967296.0);
    qsort(key, 2 * (size_t)n, sizeof(uint64_t), cmp_u64);
    for (int v = 1; v < 2 * n; v++) bad |= key[v] == key[v - 1];
    if (bad) goto out;
    rc = 0;
out:
    free(g.bstart); free(g.bidx); free(cnt); free(tri); free(own); free(voff); free(roff); free(fill); free(pos);
    free(key);
    return rc;
}

sevc_status sevc_voronoi_generate(int n, uint64_t seed, int se_dist, double *xy, int32_t *ridges, double *oris,
                                  double *se)
{
    if (n < 64 || !xy || !ridges) {
        sevc_set_error("sevc_voronoi_generate: need n >= 64 and output arrays");
        return SEVC_ERR_ARG;
    }
    double *p = (double *)malloc(sizeof(double) * 2 * (size_t)n);
    if (!p) return SEVC_ERR_CAPACITY;
    vor_rng r;
    vor_seed(&r, seed);
    for (int attempt = 0; attempt < 20; attempt++) {            /* voronoi.py:14-84 */
        for (int i = 0; i < 2 * n; i++) p[i] = vor_unit(&r);
        if (vor_attempt(n, p, xy, ridges) == 0) {
            free(p);
            for (int g = 0; g < n; g++) {
                double o = vor_unit(&r);
                if (oris) oris[g] = o;
            }
            for (int g = 0; g < n; g++) {
                double u = vor_unit(&r);
                if (se) se[g] = se_dist == 1 ? 3.0 + 3.0 * sqrt(u) : u;   /* triangular(3, 6, 6) or U[0,1) */
            }
            return SEVC_OK;
        }
    }
    free(p);
    sevc_set_error("sevc_voronoi_generate: no triple-junction mesh in 20 samples");
    return SEVC_ERR_TOPOLOGY;
}

/* the four files of voronoi.py:141-164 (same formats) */
sevc_status sevc_voronoi_write(int n, const double *xy, const int32_t *ridges, const double *oris, const double *se,
                               const char *fv, const char *fr, const char *fo, const char *fse)
{
    FILE *f;
    char a[64], b[64];
    if (!(f = fopen(fv, "w"))) { sevc_set_error("cannot write %s", fv); return SEVC_ERR_IO; }
    for (int v = 0; v < 2 * n; v++) {
        sevc_format_fixed16(xy[2 * (size_t)v], a);
        sevc_format_fixed16(xy[2 * (size_t)v + 1], b);
        fprintf(f, "%s %s\n", a, b);
    }
    fclose(f);
    if (!(f = fopen(fr, "w"))) { sevc_set_error("cannot write %s", fr); return SEVC_ERR_IO; }
    for (int r = 0; r < 3 * n; r++) fprintf(f, "%d %d\n", ridges[2 * (size_t)r], ridges[2 * (size_t)r + 1]);
    fclose(f);
    const double *col[2] = { oris, se };
    const char *path[2] = { fo, fse };
    for (int k = 0; k < 2; k++) {
        if (!(f = fopen(path[k], "w"))) { sevc_set_error("cannot write %s", path[k]); return SEVC_ERR_IO; }
        for (int g = 0; g < n; g++) {
            sevc_format_fixed16(col[k][g], a);
            fprintf(f, "%s\n", a);
        }
        fclose(f);
    }
    return SEVC_OK;
}
