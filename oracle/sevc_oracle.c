/*
 * ORACLE — TEST INFRASTRUCTURE ONLY (see sevc_oracle.h).
 *
 * CPU restatement of the reference time step.  Build with
 * -ffp-contract=off so that every a*b+c rounds twice, like the reference
 * compiled without FMA contraction.
 */
#include "sevc_oracle.h"
#include "synth_rng.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

static const double GRAD_EPS = 1e-8; /* src/calculus.h:7 */
#define MAXV ORC_MAX_VRT_PER_GRN

#define OMP_FOR _Pragma("omp parallel for schedule(static) if(st->nthreads_omp > 1) num_threads(st->nthreads_omp)")

typedef struct { double x, y; } v2;

static inline void set_err(orc_state *st, int code) { if (st->status == ORC_OK) st->status = code; }

/* ------------------------------------------------------------------ */
/* periodic geometry, src/geometry.h:133-331                           */
/* ------------------------------------------------------------------ */
static inline double dom_mod(double a, double D)          /* :133 */
{
    if (a < 0) return a + D;
    else if (a >= D) return a - D;
    return a;
}
static inline double wrap_dist(double dest, double orig, double D) /* :147 */
{
    double delta = dest - orig;
    if (delta > +(D / 2.0)) return (delta - D);
    if (delta < -(D / 2.0)) return (D + delta);
    return delta;
}
static inline v2 delta_to(v2 dest, v2 orig, double D)     /* :162 */
{
    v2 r; r.x = wrap_dist(dest.x, orig.x, D); r.y = wrap_dist(dest.y, orig.y, D); return r;
}
static inline double mag(v2 a)                             /* :217 */
{
    double p = fmax(fabs(a.x), fabs(a.y));
    if (p == 0) return 0;
    double q = fmin(fabs(a.x), fabs(a.y));
    return p * sqrt(1.0 + (q / p) * (q / p));
}
static inline v2 unitary(v2 v)                             /* :274 */
{
    v2 r;
    double m = mag(v);
    if (m == 0) { r.x = 0; r.y = 0; }
    else { double angle = atan2(v.y, v.x); r.x = cos(angle); r.y = sin(angle); }
    return r;
}
static inline v2 adjust(v2 v, double D)                    /* :296 */
{
    v2 r; r.x = dom_mod(v.x, D); r.y = dom_mod(v.y, D); return r;
}
static inline v2 vmean(v2 a, v2 b, double D)               /* :311 */
{
    v2 c = a;
    v2 d = delta_to(b, a, D);
    c.x += d.x / 2;
    c.y += d.y / 2;
    return adjust(c, D);
}
static inline double arclen(v2 ini, v2 end, double D)      /* :328 */
{
    return mag(delta_to(ini, end, D));
}
/* src/geometry.h:908-931 */
static void adjust_origin(double *xs, double *ys, int n, double D)
{
    if (n > 0) {
        v2 prev; prev.x = xs[0]; prev.y = ys[0];
        xs[0] = 0; ys[0] = 0;
        for (int i = 1; i < n; i++) {
            v2 cur; cur.x = xs[i]; cur.y = ys[i];
            v2 d = delta_to(cur, prev, D);
            prev.x = xs[i]; prev.y = ys[i];
            v2 ap; ap.x = xs[i - 1]; ap.y = ys[i - 1];
            cur.x = ap.x + d.x; cur.y = ap.y + d.y;
            xs[i] = cur.x; ys[i] = cur.y;
        }
    }
}
/* src/geometry.h:757-765 */
static double compute_area(double *X, double *Y, int n, double D)
{
    double area = 0;
    adjust_origin(X, Y, n, D);
    for (int k = 0; k < n; k++)
        area += X[k] * Y[(k + 1) % n] - Y[k] * X[(k + 1) % n];
    area *= 0.5;
    return area;
}
/* src/geometry.h:779-787 */
static double compute_dadt(double *X, double *Y, double *VX, double *VY, int n, double D)
{
    double d = 0;
    adjust_origin(X, Y, n, D);
    for (int k = 0; k < n; k++) {
        d += (VX[k] * Y[(k + 1) % n] + X[k] * VY[(k + 1) % n]);
        d -= (VY[k] * X[(k + 1) % n] + Y[k] * VX[(k + 1) % n]);
    }
    return d;
}
/* src/geometry.h:548-550 */
static inline double gb_energy_func(double d_alpha, double eps)
{
    return (1 + 0.5 * eps * (1 - pow(cos(4 * d_alpha), 3)));
}

static inline v2 vpos(const orc_state *st, int v) { v2 p; p.x = st->px[v]; p.y = st->py[v]; return p; }
static inline int other_end(const orc_state *st, int b, int v) { return st->bini[b] == v ? st->bend[b] : st->bini[b]; }

/* src/geometry.h:837-848; returns how many grains were found */
static int grains_intersect(const orc_state *st, int a, int b, int *out)
{
    int k = 0;
    out[0] = -1; out[1] = -1;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            if (st->vg[3 * a + i] == st->vg[3 * b + j]) {
                out[k++] = st->vg[3 * a + i];
                if (k == 2) return k;
            }
    return k;
}
/* src/geometry.h:863-875 */
static void grains_union(const orc_state *st, int a, int b, int *out)
{
    for (int i = 0; i < 3; i++) out[i] = st->vg[3 * a + i];
    out[3] = -1;
    for (int i = 0; i < 3; i++) {
        int g = st->vg[3 * b + i];
        if (g != out[0] && g != out[1] && g != out[2]) { out[3] = g; break; }
    }
}
/* src/geometry.h:886-898 */
static void grains_symdiff(const orc_state *st, int a, int b, int *out)
{
    int gic[2], gun[4];
    grains_intersect(st, a, b, gic);
    grains_union(st, a, b, gun);
    int k = 0;
    out[0] = -1; out[1] = -1;
    for (int i = 0; i < 4; i++)
        if (gun[i] != gic[0] && gun[i] != gic[1]) {
            out[k++] = gun[i];
            if (k == 2) return;
        }
}

/* ------------------------------------------------------------------ */
/* entity helpers, src/geometry.h:346-706                              */
/* ------------------------------------------------------------------ */
static void reset_mod_list(orc_state *st, int v)           /* :369 */
{
    for (int i = 0; i < 4; i++) {
        orc_mod *m = &st->vmod[4 * v + i];
        m->vrt = -1; m->prev = -1; m->grn = -1; m->fix = ORC_NONE;
    }
}
static void init_vertex(orc_state *st, int v, v2 pos)      /* :346 */
{
    st->px[v] = pos.x; st->py[v] = pos.y;
    st->vx[v] = 0.0; st->vy[v] = 0.0;
    st->venergy[v] = 0.0;
    st->ven[v] = 1;
    st->vnucleate[v] = 0;
    for (int i = 0; i < 3; i++) { st->vg[3 * v + i] = -1; st->vb[3 * v + i] = -1; }
    st->voted[v] = -1;
    reset_mod_list(st, v);
}
static void vertex_add_boundary(orc_state *st, int v, int b) /* :385 */
{
    for (int i = 0; i < 3; i++)
        if (st->vb[3 * v + i] == -1) { st->vb[3 * v + i] = b; return; }
}
static void vertex_add_grain(orc_state *st, int v, int g)  /* :406 */
{
    for (int i = 0; i < 3; i++)
        if (st->vg[3 * v + i] == -1) { st->vg[3 * v + i] = g; return; }
}
static void vertex_invert_boundary_order(orc_state *st, int v) /* :424 */
{
    int b = st->vb[3 * v + 1];
    st->vb[3 * v + 1] = st->vb[3 * v + 0];
    st->vb[3 * v + 0] = b;
}
static void vertex_set_boundaries_clockwise(orc_state *st, int v) /* :437 */
{
    double D = st->opt.domain_bound;
    double angle[3];
    for (int i = 0; i < 3; i++) {
        int b = st->vb[3 * v + i];
        v2 d;
        if (st->bini[b] == v) d = delta_to(vpos(st, st->bend[b]), vpos(st, v), D);
        else d = delta_to(vpos(st, st->bini[b]), vpos(st, v), D);
        angle[i] = atan2(d.y, d.x);
    }
    for (int i = 0; i < 2; i++)
        for (int p = 1; p < 3 - i; p++)
            if (angle[p - 1] < angle[p]) {
                double a = angle[p - 1]; angle[p - 1] = angle[p]; angle[p] = a;
                int b = st->vb[3 * v + p - 1]; st->vb[3 * v + p - 1] = st->vb[3 * v + p]; st->vb[3 * v + p] = b;
            }
}
/* src/geometry.h:472-479 */
static double vertex_compute_energy(const orc_state *st, int v)
{
    double e = 0.0;
    for (int i = 0; i < 3; i++) {
        int b = st->vb[3 * v + i], g = st->vg[3 * v + i];
        e += (st->blen[b] * st->benergy[b] * 0.5);
        e += (st->gse[g] * st->garea[g] / st->gvlen[g]);
    }
    return e;
}
/* src/geometry.h:491-504 */
static void init_boundary(orc_state *st, int b, int ini, int end)
{
    st->bini[b] = ini; vertex_add_boundary(st, ini, b);
    st->bend[b] = end; vertex_add_boundary(st, end, b);
    st->blen[b] = 0;
    st->btext[b] = ORC_MAX_T_EXT;
    st->ben[b] = 1;
    st->bcand[b] = 0;
    st->bvotes[b] = 0;
    st->bconf[b] = -1;
}
/* src/geometry.h:513-517 */
static inline int boundary_is_candidate(const orc_state *st, int b, double dt)
{
    return (st->btext[b] >= 0 && st->btext[b] <= dt);
}
/* src/geometry.h:559-564 */
static double boundary_compute_energy(orc_state *st, int b, double eps)
{
    int gic[2];
    if (grains_intersect(st, st->bini[b], st->bend[b], gic) < 2 || gic[0] < 0 || gic[1] < 0) {
        set_err(st, ORC_ERR_TOPOLOGY);
        return st->benergy[b];
    }
    double d_alpha = st->gori[gic[0]] - st->gori[gic[1]];
    return gb_energy_func(d_alpha, eps);
}
static void init_grain(orc_state *st, int g)               /* :578 */
{
    for (int i = 0; i < MAXV; i++) st->glist[MAXV * g + i] = -1;
    st->gvlen[g] = 0; st->garea[g] = 0; st->gse[g] = 0; st->gori[g] = 0;
    st->gen[g] = 1; st->gcand[g] = 0; st->gfix[g] = 0; st->gtype[g] = ORC_COMMON;
}
static void nucleate_grain(orc_state *st, int g)           /* :596 */
{
    for (int i = 0; i < MAXV; i++) st->glist[MAXV * g + i] = -1;
    st->gvlen[g] = 0; st->garea[g] = 0; st->gse[g] = 0; st->gori[g] = 0;
    st->gen[g] = 1; st->gcand[g] = 0; st->gfix[g] = 0; st->gtype[g] = ORC_NUCLEATED;
}
static void grain_add_vertex(orc_state *st, int g, int v)  /* :614 */
{
    if (st->gvlen[g] >= MAXV) { set_err(st, ORC_ERR_CAPACITY); return; }
    st->glist[MAXV * g + st->gvlen[g]] = v;
    st->gvlen[g]++;
}
static void grain_add_vertex_after(orc_state *st, int g, int v, int prev) /* :629 */
{
    int vlen = st->gvlen[g], pos = -1;
    int *L = &st->glist[MAXV * g];
    for (int i = 0; i < vlen; i++)
        if (L[i] == prev) { pos = i + 1; break; }
    if (pos < 0 || vlen >= MAXV) { set_err(st, pos < 0 ? ORC_ERR_TOPOLOGY : ORC_ERR_CAPACITY); return; }
    for (int i = vlen; i > pos; i--) L[i] = L[i - 1];
    L[pos] = v;
    st->gvlen[g]++;
}
static void grain_remove_vertex(orc_state *st, int g, int v) /* :653 */
{
    int *L = &st->glist[MAXV * g];
    for (int i = 0; i < st->gvlen[g]; i++)
        if (L[i] == v) {
            for (int j = i; j < st->gvlen[g] - 1; j++) L[j] = L[j + 1];
            st->gvlen[g]--;
            L[st->gvlen[g]] = -1;
            return;
        }
}
static void grain_replace_vertex(orc_state *st, int g, int oldv, int newv) /* :686 */
{
    int *L = &st->glist[MAXV * g];
    for (int i = 0; i < st->gvlen[g]; i++)
        if (L[i] == oldv) { L[i] = newv; return; }
}
static int grain_contains_vertex(const orc_state *st, int g, int v) /* :703 */
{
    const int *L = &st->glist[MAXV * g];
    for (int i = 0; i < st->gvlen[g]; i++)
        if (L[i] == v) return i;
    return -1;
}
static int grain_contains_consecutive(const orc_state *st, int g, int A, int B) /* :724 */
{
    const int *L = &st->glist[MAXV * g];
    int n = st->gvlen[g];
    for (int i = 0; i < n; i++) {
        if (L[i] == A && L[(i + 1) % n] == B) return 1;
        if (L[i] == B && L[(i + 1) % n] == A) return 2;
    }
    return -1;
}
static double grain_compute_area(const orc_state *st, int g) /* :797 */
{
    double X[MAXV], Y[MAXV];
    int n = st->gvlen[g];
    for (int i = 0; i < n; i++) { int v = st->glist[MAXV * g + i]; X[i] = st->px[v]; Y[i] = st->py[v]; }
    return compute_area(X, Y, n, st->opt.domain_bound);
}

/* ------------------------------------------------------------------ */
/* options, src/options.h:55-206                                       */
/* ------------------------------------------------------------------ */
void orc_default_options(orc_options *o)
{
    memset(o, 0, sizeof(*o));
    o->tmax = -1; o->nmax = -1;                  /* :71-72 */
    o->GB_eps = 0.02; o->GB_scaling = 1.0;       /* :73-74 */
    o->SE_eps = 1.0; o->SE_min = 999; o->SE_max = 999;
    o->MC_k = 1.0; o->nucleation_scaling = 0.9;
    o->domain_bound = 1.0; o->do_nucleation = 1;
    o->nucleation_gap = 1; o->debug_lvl = 0;
    o->output_folder[0] = '\0';
    o->leave_percent = -1;
    o->n_blocks = 32; o->n_threads = 256;
    o->min_grains = 5000;
}

static void fix_string(char *s) { size_t n = strlen(s); if (n > 0) s[n - 1] = '\0'; } /* :55 */

void orc_finish_options(orc_options *o)
{
    o->nucleation_gap = (int)(o->dtau / o->dt);  /* :172 */
    if (o->tmax > 0 && o->nmax == -1) {
    } else if (o->tmax == -1 && o->nmax > 0) {
    } else { o->tmax = 1.0; o->nmax = -1; }      /* :173-181 */
}

int orc_parse_ini(const char *path, orc_options *o)
{
    orc_default_options(o);
    FILE *f = fopen(path, "r");
    if (!f) return ORC_ERR_IO;
    char buf[1000], var[1000];
    while (fgets(buf, sizeof buf, f)) {
        if (buf[0] == '#' || buf[0] == '[') continue;
        char *p = strchr(buf, '=');
        if (!p) continue;
        size_t k = (size_t)(p - buf);
        memcpy(var, buf, k); var[k] = '\0';
        const char *val = p + 1;
        if (!strcmp(var, "dt")) o->dt = atof(val);
        else if (!strcmp(var, "dtau")) o->dtau = atof(val);
        else if (!strcmp(var, "tmax")) o->tmax = atof(val);
        else if (!strcmp(var, "nmax")) o->nmax = atoi(val);
        else if (!strcmp(var, "snap_gap")) o->snap_gap = atoi(val);
        else if (!strcmp(var, "leave_percent")) o->leave_percent = atof(val);
        else if (!strcmp(var, "n_grains")) o->n_grains = atoi(val);
        else if (!strcmp(var, "vertex_fname")) { snprintf(o->vertex_fname, 256, "%s", val); fix_string(o->vertex_fname); }
        else if (!strcmp(var, "boundary_fname")) { snprintf(o->boundary_fname, 256, "%s", val); fix_string(o->boundary_fname); }
        else if (!strcmp(var, "orientation_fname")) { snprintf(o->orientation_fname, 256, "%s", val); fix_string(o->orientation_fname); }
        else if (!strcmp(var, "SE_fname")) { snprintf(o->SE_fname, 256, "%s", val); fix_string(o->SE_fname); }
        else if (!strcmp(var, "n_blocks")) o->n_blocks = atoi(val);
        else if (!strcmp(var, "n_threads")) o->n_threads = atoi(val);
        else if (!strcmp(var, "debug_lvl")) o->debug_lvl = atoi(val);
        else if (!strcmp(var, "folder")) { snprintf(o->output_folder, 256, "%s", val); fix_string(o->output_folder); }
        else if (!strcmp(var, "GB_eps")) o->GB_eps = atof(val);
        else if (!strcmp(var, "GB_scaling")) o->GB_scaling = atof(val);
        else if (!strcmp(var, "SE_eps")) o->SE_eps = atof(val);
        else if (!strcmp(var, "SE_min")) o->SE_min = atof(val);
        else if (!strcmp(var, "SE_max")) o->SE_max = atof(val);
        else if (!strcmp(var, "MC_k")) o->MC_k = atof(val);
        else if (!strcmp(var, "nucleation_scaling")) o->nucleation_scaling = atof(val);
        else if (!strcmp(var, "domain_bound")) o->domain_bound = atof(val);
        else if (!strcmp(var, "do_nucleation")) o->do_nucleation = !strcmp(val, "true\n");
    }
    fclose(f);
    orc_finish_options(o);
    return ORC_OK;
}

/* ------------------------------------------------------------------ */
/* allocation                                                          */
/* ------------------------------------------------------------------ */
static void *xcalloc(size_t n, size_t s) { void *p = calloc(n ? n : 1, s); if (!p) abort(); return p; }

static orc_state *alloc_state(const orc_options *opt, int nv, int nb, int ng)
{
    orc_state *st = (orc_state *)xcalloc(1, sizeof(orc_state));
    st->opt = *opt;
    st->nv = nv; st->nb = nb; st->ng = ng;
#define A(f, n) st->f = xcalloc((size_t)(n), sizeof(*st->f))
    A(px, nv); A(py, nv); A(vx, nv); A(vy, nv); A(venergy, nv);
    A(vel_bnd_x, nv); A(vel_grn_x, nv); A(vel_bnd_y, nv); A(vel_grn_y, nv);
    A(nucl_r, nv); A(nucl_ori, nv); A(DeltaE, nv); A(nfactor, nv);
    A(ven, nv); A(vnucleate, nv); A(vb, 3 * (size_t)nv); A(vg, 3 * (size_t)nv);
    A(vmod, 4 * (size_t)nv); A(voted, nv);
    A(bini, nb); A(bend, nb); A(benergy, nb); A(blen, nb); A(btext, nb);
    A(ben, nb); A(bcand, nb); A(bvotes, nb); A(bconf, nb);
    A(glist, (size_t)MAXV * ng); A(gvlen, ng); A(garea, ng); A(gdadt, ng); A(gori, ng); A(gse, ng);
    A(gen, ng); A(gcand, ng); A(gfix, ng); A(gtype, ng);
    A(cand_buf, nb);
#undef A
    st->rng_nstreams = opt->n_blocks * opt->n_threads;
    st->rng_pos = (int64_t *)xcalloc((size_t)st->rng_nstreams, sizeof(int64_t));
    st->rng_kind = 0; st->rng_seed = 0;
    st->vrt_id_candidate = 0;
    st->polling_cap = 100000;
    st->nthreads_omp = 1;
    return st;
}

void orc_free(orc_state *st)
{
    if (!st) return;
    void *ptrs[] = { st->px, st->py, st->vx, st->vy, st->venergy, st->vel_bnd_x, st->vel_grn_x,
        st->vel_bnd_y, st->vel_grn_y, st->nucl_r, st->nucl_ori, st->DeltaE, st->nfactor, st->ven,
        st->vnucleate, st->vb, st->vg, st->vmod, st->voted, st->bini, st->bend, st->benergy,
        st->blen, st->btext, st->ben, st->bcand, st->bvotes, st->bconf, st->glist, st->gvlen,
        st->garea, st->gdadt, st->gori, st->gse, st->gen, st->gcand, st->gfix, st->gtype,
        st->cand_buf, st->rng_pos };
    for (size_t i = 0; i < sizeof ptrs / sizeof ptrs[0]; i++) free(ptrs[i]);
    free(st);
}

void orc_rng_synthetic(orc_state *st, uint64_t seed)
{
    st->rng_kind = 0; st->rng_seed = seed;
    memset(st->rng_pos, 0, sizeof(int64_t) * (size_t)st->rng_nstreams);
}
void orc_rng_table(orc_state *st, int nstreams, int ndraws, const double *table)
{
    st->rng_kind = 1; st->rng_table = table; st->rng_ndraws = ndraws;
    if (nstreams < st->rng_nstreams) set_err(st, ORC_ERR_RNG);
    memset(st->rng_pos, 0, sizeof(int64_t) * (size_t)st->rng_nstreams);
}
/* curand_uniform_double(&state[tid]) stand-in */
static double rng_u(orc_state *st, int tid)
{
    int64_t k = st->rng_pos[tid]++;
    if (st->rng_kind == 1) {
        if (k >= st->rng_ndraws) { set_err(st, ORC_ERR_RNG); return 0.5; }
        return st->rng_table[(size_t)tid * (size_t)st->rng_ndraws + (size_t)k];
    }
    return sevc_synth_uniform(st->rng_seed, (uint64_t)tid, (uint64_t)k);
}

/* ------------------------------------------------------------------ */
/* loader, src/io.h:66-264                                             */
/* ------------------------------------------------------------------ */
static int load_core(const orc_options *opt, int nv, const double *xy, int nb, const int *ridges,
                     int n_ori, const double *oris, int n_se, const double *se, orc_state **out)
{
    *out = NULL;
    if (nv <= 0 || nb <= 0 || opt->n_grains <= 0) return ORC_ERR_PARSE;
    if (n_ori > opt->n_grains || n_se > opt->n_grains) return ORC_ERR_CAPACITY;
    orc_state *st = alloc_state(opt, nv, nb, opt->n_grains);
    double D = opt->domain_bound;
    for (int i = 0; i < nv; i++) {                       /* :84-93 */
        v2 p; p.x = xy[2 * i] * D; p.y = xy[2 * i + 1] * D;
        init_vertex(st, i, p);
    }
    for (int i = 0; i < nb; i++) {                       /* :124-126 */
        int a = ridges[2 * i], b = ridges[2 * i + 1];
        if (a < 0 || a >= nv || b < 0 || b >= nv) { orc_free(st); return ORC_ERR_PARSE; }
        init_boundary(st, i, a, b);
    }
    for (int j = 0; j < nv; j++)                          /* :132-134 */
        for (int i = 0; i < 3; i++)
            if (st->vb[3 * j + i] < 0) { orc_free(st); return ORC_ERR_TOPOLOGY; }
    for (int j = 0; j < nv; j++) vertex_set_boundaries_clockwise(st, j);

    int lengrains = 0;                                   /* :137-180 */
    uint8_t *cons = (uint8_t *)xcalloc(3 * (size_t)nv, 1);
    int *tmp = (int *)xcalloc(MAXV, sizeof(int));
    for (int j = 0; j < nv; j++) {
        if (!st->ven[j]) continue;
        for (int g = 0; g < 3; g++) {
            if (cons[3 * j + g]) continue;
            int vlen = 0, cur = j, side = g;
            do {
                if (cons[3 * cur + side] || !st->ven[cur] || vlen >= MAXV) {
                    free(cons); free(tmp); orc_free(st); return ORC_ERR_TOPOLOGY;
                }
                cons[3 * cur + side] = 1;
                tmp[vlen++] = cur;
                int b = st->vb[3 * cur + side];
                cur = (st->bini[b] == cur) ? st->bend[b] : st->bini[b];
                int i = 0;
                while (i < 3 && st->vb[3 * cur + i] != b) i++;
                if (i == 3) { free(cons); free(tmp); orc_free(st); return ORC_ERR_TOPOLOGY; }
                side = (i + 1) % 3;
            } while (cur != j);
            if (lengrains >= opt->n_grains) { free(cons); free(tmp); orc_free(st); return ORC_ERR_TOPOLOGY; }
            init_grain(st, lengrains);
            for (int k = 0; k < vlen; k++) st->glist[MAXV * lengrains + k] = tmp[k];
            st->gvlen[lengrains] = vlen;
            lengrains++;
        }
    }
    free(cons); free(tmp);
    if (lengrains != opt->n_grains) { orc_free(st); return ORC_ERR_TOPOLOGY; } /* :182-186 */
    for (int j = 0; j < nv; j++) {                       /* :189-192 */
        vertex_set_boundaries_clockwise(st, j);
        vertex_invert_boundary_order(st, j);
    }
    for (int i = 0; i < st->ng; i++)                      /* :196-200 */
        for (int k = 0; k < st->gvlen[i]; k++)
            vertex_add_grain(st, st->glist[MAXV * i + k], i);
    for (int i = 0; i < n_ori; i++) st->gori[i] = oris[i];           /* :214 */
    for (int j = 0; j < st->ng; j++) st->gori[j] = st->gori[j] * 2 * M_PI; /* :216-218, :536 */
    for (int i = 0; i < n_se; i++) st->gse[i] = se[i];                /* :223 */
    if (opt->SE_min == 999 && opt->SE_max == 999) {                    /* :228-248 */
        for (int j = 0; j < st->ng; j++) st->gse[j] *= opt->SE_eps;
    } else if (opt->SE_min == opt->SE_max) {
        for (int j = 0; j < st->ng; j++) st->gse[j] = opt->SE_max * opt->SE_eps;
    } else {
        double fm = (opt->SE_max - opt->SE_min), fb = opt->SE_min;
        for (int j = 0; j < st->ng; j++) st->gse[j] = fm * st->gse[j] + fb;
    }
    st->curr_n_grains = st->ng;                           /* main.cu:72 */
    *out = st;
    return ORC_OK;
}

int orc_load_arrays(const orc_options *opt, int nv, const double *xy, int nb, const int *ridges,
                    int ng, const double *oris, const double *se, orc_state **out)
{
    return load_core(opt, nv, xy, nb, ridges, ng, oris, ng, se, out);
}

/* A state of nv vertices, nb boundaries and ng grains with every entity
 * in its initial (init_vertex / init_boundary / init_grain) condition and
 * no connectivity, for the caller to fill field by field (orc_field) with
 * a mesh taken in the middle of a run; curr_n_grains = ng. */
orc_state *orc_alloc_blank(const orc_options *opt, int nv, int nb, int ng)
{
    orc_state *st = alloc_state(opt, nv, nb, ng);
    v2 z = { 0.0, 0.0 };
    for (int i = 0; i < nv; i++) init_vertex(st, i, z);
    for (int b = 0; b < nb; b++) {
        st->bini[b] = st->bend[b] = -1;
        st->btext[b] = ORC_MAX_T_EXT;
        st->ben[b] = 1;
        st->bconf[b] = -1;
    }
    for (int g = 0; g < ng; g++) init_grain(st, g);
    st->curr_n_grains = ng;
    return st;
}

static int read_doubles(const char *path, int per_line, double **out, int *n)
{
    FILE *f = fopen(path, "r");
    if (!f) return ORC_ERR_IO;
    size_t cap = 1024, len = 0;
    double *a = (double *)malloc(cap * sizeof(double));
    double x, y;
    for (;;) {
        int r = per_line == 2 ? fscanf(f, "%lf %lf\n", &x, &y) : fscanf(f, "%lf\n", &x);
        if (r == EOF) break;
        if (r != per_line) { free(a); fclose(f); return ORC_ERR_PARSE; }
        if (len + 2 > cap) { cap *= 2; a = (double *)realloc(a, cap * sizeof(double)); }
        a[len++] = x;
        if (per_line == 2) a[len++] = y;
    }
    fclose(f);
    *out = a; *n = (int)(len / (size_t)per_line);
    return ORC_OK;
}
static int read_ridges(const char *path, int **out, int *n)
{
    FILE *f = fopen(path, "r");
    if (!f) return ORC_ERR_IO;
    size_t cap = 1024, len = 0;
    int *a = (int *)malloc(cap * sizeof(int));
    int x, y;
    for (;;) {
        int r = fscanf(f, "%d %d\n", &x, &y);
        if (r == EOF) break;
        if (r != 2) { free(a); fclose(f); return ORC_ERR_PARSE; }
        if (len + 2 > cap) { cap *= 2; a = (int *)realloc(a, cap * sizeof(int)); }
        a[len++] = x; a[len++] = y;
    }
    fclose(f);
    *out = a; *n = (int)(len / 2);
    return ORC_OK;
}

int orc_load_files(const orc_options *opt, orc_state **out)
{
    double *xy = NULL, *oris = NULL, *se = NULL; int *ridges = NULL;
    int nv = 0, nb = 0, no = 0, ns = 0, rc;
    *out = NULL;
    if ((rc = read_doubles(opt->vertex_fname, 2, &xy, &nv))) goto done;
    if ((rc = read_ridges(opt->boundary_fname, &ridges, &nb))) goto done;
    if ((rc = read_doubles(opt->orientation_fname, 1, &oris, &no))) goto done;
    if ((rc = read_doubles(opt->SE_fname, 1, &se, &ns))) goto done;
    rc = load_core(opt, nv, xy, nb, ridges, no, oris, ns, se, out);
done:
    free(xy); free(ridges); free(oris); free(se);
    return rc;
}

/* ------------------------------------------------------------------ */
/* geometry kernels, src/calculus.h                                    */
/* ------------------------------------------------------------------ */
void orc_compute_boundary_arclengths(orc_state *st)       /* calculus.h:83 */
{
    double D = st->opt.domain_bound;
    OMP_FOR
    for (int b = 0; b < st->nb; b++)
        if (st->ben[b]) st->blen[b] = arclen(vpos(st, st->bini[b]), vpos(st, st->bend[b]), D);
}
void orc_compute_boundary_energies(orc_state *st)         /* calculus.h:104 */
{
    double eps = st->opt.GB_eps, s = st->opt.GB_scaling;
    OMP_FOR
    for (int b = 0; b < st->nb; b++)
        if (st->ben[b]) st->benergy[b] = boundary_compute_energy(st, b, eps) * s;
}
void orc_compute_vertex_energies(orc_state *st)           /* calculus.h:123 */
{
    OMP_FOR
    for (int v = 0; v < st->nv; v++)
        if (st->ven[v]) st->venergy[v] = vertex_compute_energy(st, v);
}
void orc_compute_grain_areas(orc_state *st)               /* calculus.h:224 */
{
    OMP_FOR
    for (int g = 0; g < st->ng; g++)
        if (st->gen[g]) st->garea[g] = grain_compute_area(st, g);
}
void orc_compute_grain_dadts(orc_state *st)               /* calculus.h:243, geometry.h:813 */
{
    double D = st->opt.domain_bound;
    OMP_FOR
    for (int g = 0; g < st->ng; g++) {
        if (!st->gen[g]) continue;
        double X[MAXV], Y[MAXV], VX[MAXV], VY[MAXV];
        int n = st->gvlen[g];
        for (int i = 0; i < n; i++) {
            int v = st->glist[MAXV * g + i];
            X[i] = st->px[v]; VX[i] = st->vx[v]; Y[i] = st->py[v]; VY[i] = st->vy[v];
        }
        st->gdadt[g] = compute_dadt(X, Y, VX, VY, n, D);
    }
}

/* src/calculus.h:19-73 */
static double energy_diff(orc_state *st, int comp, int v)
{
    double D = st->opt.domain_bound;
    v2 np = vpos(st, v);
    if (comp == 0) np.x += GRAD_EPS; else np.y += GRAD_EPS;
    np = adjust(np, D);
    double L[3] = { 0, 0, 0 };
    for (int j = 0; j < 3; j++) {
        int b = st->vb[3 * v + j];
        if (st->bini[b] == v) L[j] = arclen(np, vpos(st, st->bend[b]), D);
        else L[j] = arclen(np, vpos(st, st->bini[b]), D);
    }
    double Ar[3] = { 0, 0, 0 };
    for (int j = 0; j < 3; j++) {
        double X[MAXV], Y[MAXV];
        int g = st->vg[3 * v + j];
        int n = st->gvlen[g];
        for (int k = 0; k < n; k++) {
            int u = st->glist[MAXV * g + k];
            X[k] = st->px[u]; Y[k] = st->py[u];
            if (u == v) { X[k] = np.x; Y[k] = np.y; }
        }
        Ar[j] = compute_area(X, Y, n, D);
    }
    double bt = 0.0, gt = 0.0;
    for (int j = 0; j < 3; j++) {
        int b = st->vb[3 * v + j], g = st->vg[3 * v + j];
        bt += (st->benergy[b] * (L[j] - st->blen[b]));
        gt += (st->gse[g] * (fabs(Ar[j]) - fabs(st->garea[g])));
    }
    if (comp == 0) { st->vel_bnd_x[v] = -bt / GRAD_EPS; st->vel_grn_x[v] = -gt / GRAD_EPS; }
    else { st->vel_bnd_y[v] = -bt / GRAD_EPS; st->vel_grn_y[v] = -gt / GRAD_EPS; }
    return bt + gt;
}
void orc_compute_vertex_velocities(orc_state *st)         /* calculus.h:143 */
{
    OMP_FOR
    for (int v = 0; v < st->nv; v++)
        if (st->ven[v]) {
            st->vx[v] = -energy_diff(st, 0, v) / GRAD_EPS;
            st->vy[v] = -energy_diff(st, 1, v) / GRAD_EPS;
        }
}
static void update_vertices_positions(orc_state *st)      /* calculus.h:391 */
{
    double dt = st->opt.dt, D = st->opt.domain_bound;
    OMP_FOR
    for (int v = 0; v < st->nv; v++)
        if (st->ven[v]) {
            st->px[v] += st->vx[v] * dt;
            st->py[v] += st->vy[v] * dt;
            st->px[v] = dom_mod(st->px[v], D);
            st->py[v] = dom_mod(st->py[v], D);
        }
}
int orc_current_n_grains(const orc_state *st)             /* calculus.h:264-313 */
{
    int c = 0;
    for (int g = 0; g < st->ng; g++) c += st->gen[g] ? 1 : 0;
    return c;
}
/* block tree reduction of src/calculus.h:338-345 for n_threads values */
static double block_tree_sum(double *t, int nthr)
{
    for (int i = nthr / 2; i != 0; i /= 2)
        for (int c = 0; c < i; c++) t[c] += t[c + i];
    return t[0];
}
double orc_nucleated_fraction_area(const orc_state *st)   /* calculus.h:322-378 */
{
    int nblk = st->opt.n_blocks, nthr = st->opt.n_threads, grid = nblk * nthr;
    double *t = (double *)malloc(sizeof(double) * (size_t)nthr);
    double total = 0.0;
    for (int b = 0; b < nblk; b++) {
        for (int c = 0; c < nthr; c++) {
            double a = 0.0;
            for (int g = b * nthr + c; g < st->ng; g += grid)
                if (st->gen[g] && st->gtype[g] == ORC_NUCLEATED) a += st->garea[g];
            t[c] = a;
        }
        total += block_tree_sum(t, nthr);
    }
    free(t);
    double D = st->opt.domain_bound;
    return 100 * total / (D * D);
}

/* ------------------------------------------------------------------ */
/* topological transitions, src/topological.h                          */
/* ------------------------------------------------------------------ */
void orc_compute_t_ext(orc_state *st)                     /* topological.h:303 */
{
    double D = st->opt.domain_bound;
    OMP_FOR
    for (int b = 0; b < st->nb; b++) {
        if (!st->ben[b]) continue;
        st->bcand[b] = 0;
        int ini = st->bini[b], end = st->bend[b];
        double xp[2] = { st->px[ini], st->px[end] }, yp[2] = { st->py[ini], st->py[end] };
        adjust_origin(xp, yp, 2, D);
        v2 diff; diff.x = xp[1] - xp[0]; diff.y = yp[1] - yp[0];
        double norm = mag(diff);
        v2 T = unitary(diff);
        v2 P; P.x = st->vx[end] - st->vx[ini]; P.y = st->vy[end] - st->vy[ini];
        double aux = T.x * P.x + T.y * P.y;
        st->btext[b] = (aux == 0) ? 100 : -norm / aux;
    }
}
static void label_boundaries(orc_state *st)               /* topological.h:343 */
{
    double dt = st->opt.dt;
    OMP_FOR
    for (int b = 0; b < st->nb; b++) {
        st->bcand[b] = (uint8_t)boundary_is_candidate(st, b, dt);
        st->bconf[b] = -1;
    }
}
/* topological.h:486-537: AND over each thread's stride set, OR within a
 * block (bool += in the tree), AND over blocks */
static int compare_candidates(const orc_state *st)
{
    int nblk = st->opt.n_blocks, nthr = st->opt.n_threads, grid = nblk * nthr;
    double *t = (double *)malloc(sizeof(double) * (size_t)nthr);
    int all = 1;
    for (int blk = 0; blk < nblk; blk++) {
        for (int c = 0; c < nthr; c++) {
            int tmp = 1;
            for (int b = blk * nthr + c; b < st->nb; b += grid)
                if (st->ben[b]) tmp = tmp && (st->bcand[b] == st->cand_buf[b]);
            t[c] = tmp;
        }
        for (int i = nthr / 2; i != 0; i /= 2)
            for (int c = 0; c < i; c++) t[c] = (t[c] != 0 || t[c + i] != 0) ? 1 : 0;
        all = all && (t[0] != 0);
    }
    free(t);
    return all;
}
static int polling_system(orc_state *st)                  /* topological.h:549-578 */
{
    int conv = 0, it = 0;
    while (!conv) {
        if (it >= st->polling_cap) { set_err(st, ORC_ERR_NONCONVERGED); return -1; }
        it++;
        for (int b = 0; b < st->nb; b++) if (st->ben[b]) st->bvotes[b] = 0;   /* :426 */
        for (int v = 0; v < st->nv; v++) if (st->ven[v]) st->voted[v] = -1;   /* :388 */
        for (int v = 0; v < st->nv; v++) {                                    /* :362 */
            if (!st->ven[v]) continue;
            double mt = 99999999;
            int am = 0;
            for (int i = 0; i < 3; i++) {
                int b = st->vb[3 * v + i];
                if (st->btext[b] <= mt && st->bcand[b]) { mt = st->btext[b]; am = i; }
            }
            st->voted[v] = st->vb[3 * v + am];
        }
        for (int b = 0; b < st->nb; b++)                                      /* :406 */
            if (st->ben[b] && st->bcand[b]) {
                if (st->voted[st->bini[b]] == b) st->bvotes[b]++;
                if (st->voted[st->bend[b]] == b) st->bvotes[b]++;
            }
        for (int b = 0; b < st->nb; b++)                                      /* :441 */
            if (st->ben[b] && st->bcand[b] && st->bvotes[b] == 2)
                for (int i = 0; i < 3; i++) {
                    int bi = st->vb[3 * st->bini[b] + i], be = st->vb[3 * st->bend[b] + i];
                    if (b != bi) st->bcand[bi] = 0;
                    if (b != be) st->bcand[be] = 0;
                }
        conv = compare_candidates(st);
        for (int b = 0; b < st->nb; b++) st->cand_buf[b] = st->ben[b] ? st->bcand[b] : 0; /* :466 */
    }
    st->polling_iters = it;
    return it;
}
static void check_conflictive_boundaries(orc_state *st)  /* topological.h:83 */
{
    for (int b = 0; b < st->nb; b++) {
        if (!(st->ben[b] && !st->bcand[b])) continue;
        int bi = -1, be = -1;
        for (int i = 0; i < 3; i++) {
            int x = st->vb[3 * st->bini[b] + i];
            if (x != b && st->bcand[x]) { bi = x; break; }
        }
        for (int i = 0; i < 3; i++) {
            int x = st->vb[3 * st->bend[b] + i];
            if (x != b && st->bcand[x]) { be = x; break; }
        }
        if (bi >= 0 && be >= 0) {
            if (st->btext[bi] == st->btext[be]) st->bconf[b] = bi < be ? bi : be;
            else st->bconf[b] = st->btext[bi] < st->btext[be] ? bi : be;
            st->ev_conflicts++;
        }
    }
}
static void unlabel_conflictive_boundaries(orc_state *st) /* topological.h:129 */
{
    for (int b = 0; b < st->nb; b++) {
        if (!(st->ben[b] && st->bcand[b])) continue;
        for (int i = 0; i < 3; i++) {
            int x = st->vb[3 * st->bini[b] + i];
            if (b != x && st->bconf[x] != -1 && st->bconf[x] != b) { st->bcand[b] = 0; break; }
        }
        for (int i = 0; i < 3; i++) {
            int x = st->vb[3 * st->bend[b] + i];
            if (b != x && st->bconf[x] != -1 && st->bconf[x] != b) { st->bcand[b] = 0; break; }
        }
    }
}
static int gic_ok(orc_state *st, int b, int *gic)
{
    if (grains_intersect(st, st->bini[b], st->bend[b], gic) < 2 || gic[0] < 0 || gic[1] < 0) {
        set_err(st, ORC_ERR_TOPOLOGY);
        return 0;
    }
    return 1;
}
static int two_three_sided_grains(orc_state *st)          /* topological.h:22-73 */
{
    int c = 0;
    for (int b = 0; b < st->nb; b++) {
        if (!st->ben[b]) continue;
        int gic[2];
        if (!gic_ok(st, b, gic)) continue;
        if (st->gvlen[gic[0]] == 3 && st->gvlen[gic[1]] == 3) c++;
    }
    return c;
}
/* topological.h:840-955 */
static void remove_two_grains(orc_state *st, int bnd, const int *gnic)
{
    int A = st->bini[bnd], B = st->bend[bnd];
    int i, j, AC = -1, BD = -1;
    for (i = 0; i < 3; i++) if (st->vb[3 * A + i] == bnd) { i = (i + 1) % 3; AC = st->vb[3 * A + i]; break; }
    for (j = 0; j < 3; j++) if (st->vb[3 * B + j] == bnd) { j = (j + 1) % 3; BD = st->vb[3 * B + j]; break; }
    if (AC < 0 || BD < 0) { set_err(st, ORC_ERR_TOPOLOGY); return; }
    int C = (st->bini[AC] == A) ? st->bend[AC] : st->bini[AC];
    int D = (st->bini[BD] == B) ? st->bend[BD] : st->bini[BD];
    int k, l, CE = -1, DF = -1;
    for (k = 0; k < 3; k++) if (st->vb[3 * C + k] == AC) { k = (k + 2) % 3; CE = st->vb[3 * C + k]; break; }
    for (l = 0; l < 3; l++) if (st->vb[3 * D + l] == BD) { l = (l + 2) % 3; DF = st->vb[3 * D + l]; break; }
    if (CE < 0 || DF < 0) { set_err(st, ORC_ERR_TOPOLOGY); return; }
    int F = (st->bini[DF] == D) ? st->bend[DF] : st->bini[DF];
    if (st->bini[CE] == C) st->bini[CE] = F; else st->bend[CE] = F;
    for (int p = 0; p < 3; p++) if (st->vb[3 * F + p] == DF) { st->vb[3 * F + p] = CE; break; }
    int G3, G4;
    if (gnic[0] < 0 || gnic[1] < 0) { set_err(st, ORC_ERR_TOPOLOGY); return; }
    if (grain_contains_vertex(st, gnic[0], A) >= 0) { G3 = gnic[0]; G4 = gnic[1]; }
    else { G3 = gnic[1]; G4 = gnic[0]; }
    orc_mod *ma = &st->vmod[4 * A], *mb = &st->vmod[4 * B];
    ma[0].fix = ORC_REMOVE; ma[0].grn = G3; ma[0].vrt = A; st->gfix[G3] = 1;
    ma[1].fix = ORC_REMOVE; ma[1].grn = G3; ma[1].vrt = C;
    ma[2].fix = ORC_REMOVE; ma[2].grn = G3; ma[2].vrt = D;
    mb[0].fix = ORC_REMOVE; mb[0].grn = G4; mb[0].vrt = B; st->gfix[G4] = 1;
    mb[1].fix = ORC_REMOVE; mb[1].grn = G4; mb[1].vrt = C;
    mb[2].fix = ORC_REMOVE; mb[2].grn = G4; mb[2].vrt = D;
    for (int q = 0; q < 3; q++) { st->ben[st->vb[3 * A + q]] = 0; st->ben[st->vb[3 * B + q]] = 0; }
    st->ben[DF] = 0; st->ben[bnd] = 0;
    st->ven[A] = 0; st->ven[D] = 0; st->ven[C] = 0; st->ven[B] = 0;
}
static void remove_two_grains_configurations(orc_state *st) /* topological.h:965 */
{
    for (int b = 0; b < st->nb; b++) {
        if (!st->ben[b]) continue;
        int gic[2], gnic[2];
        if (!gic_ok(st, b, gic)) continue;
        grains_symdiff(st, st->bini[b], st->bend[b], gnic);
        if (st->gvlen[gic[0]] == 3 && st->gvlen[gic[1]] == 3) {
            remove_two_grains(st, b, gnic);
            st->gen[gic[0]] = 0;
            st->gen[gic[1]] = 0;
            st->ev_two_three++;
        }
    }
}
/* topological.h:1035-1227 */
static void fix_grain_lists(orc_state *st)
{
    for (int g = 0; g < st->ng; g++) {                   /* ADD :1035 */
        if (!(st->gen[g] && st->gfix[g])) continue;
        for (int i = 0; i < st->gvlen[g]; i++) {
            int v = st->glist[MAXV * g + i];
            for (int j = 0; j < 4; j++) {
                orc_mod m = st->vmod[4 * v + j];
                if (m.fix == ORC_ADD && m.grn == g) grain_add_vertex_after(st, g, m.vrt, m.prev);
            }
        }
    }
    orc_mod *buff = (orc_mod *)malloc(sizeof(orc_mod) * MAXV * 4);
    for (int g = 0; g < st->ng; g++) {                   /* REMOVE :1081 */
        if (!(st->gen[g] && st->gfix[g])) continue;
        for (int i = 0; i < MAXV * 4; i++) buff[i].fix = ORC_NONE;
        int vlen = st->gvlen[g];
        for (int i = 0; i < vlen; i++) {
            int v = st->glist[MAXV * g + i];
            for (int j = 0; j < 4; j++) buff[i * 4 + j] = st->vmod[4 * v + j];
        }
        for (int i = 0; i < MAXV * 4; i++)
            if (buff[i].fix == ORC_REMOVE && buff[i].grn == g) grain_remove_vertex(st, g, buff[i].vrt);
    }
    free(buff);
    for (int g = 0; g < st->ng; g++) {                   /* REPLACE :1119 */
        if (!(st->gen[g] && st->gfix[g])) continue;
        for (int i = 0; i < st->gvlen[g]; i++) {
            int v = st->glist[MAXV * g + i];
            for (int j = 0; j < 4; j++) {
                orc_mod m = st->vmod[4 * v + j];
                if (m.fix == ORC_REPLACE && m.grn == g) grain_replace_vertex(st, g, m.prev, m.vrt);
            }
        }
    }
    for (int g = 0; g < st->ng; g++) {                   /* clear :1150 */
        if (!st->gen[g]) continue;
        st->gfix[g] = 0;
        for (int i = 0; i < st->gvlen[g]; i++) reset_mod_list(st, st->glist[MAXV * g + i]);
    }
}
static void label_3sided_grains(orc_state *st)            /* topological.h:634 */
{
    double dt = st->opt.dt;
    for (int g = 0; g < st->ng; g++) {
        if (!(st->gen[g] && st->gvlen[g] == 3)) continue;
        int ans = 0;
        for (int i = 0; i < 3; i++) {
            int v = st->glist[MAXV * g + i];
            for (int k = 0; k < 3; k++) {
                int b = st->vb[3 * v + k];
                int ip = grain_contains_vertex(st, g, st->bini[b]);
                int ep = grain_contains_vertex(st, g, st->bend[b]);
                if (ip >= 0 && ep >= 0 && st->bcand[b] && st->ben[b]) { st->gcand[g] = 1; break; }
                if (ip >= 0 && ep >= 0 && boundary_is_candidate(st, b, dt) && st->ben[b]) ans++;
            }
        }
        ans /= 2;
        if (ans == 3) st->gcand[g] = 1;
    }
}
/* topological.h:687-822 */
static void remove_grain(orc_state *st, int grn)
{
    double Dm = st->opt.domain_bound;
    int A = st->glist[MAXV * grn + 0], B = st->glist[MAXV * grn + 1], C = st->glist[MAXV * grn + 2];
    double xp[3] = { st->px[A], st->px[B], st->px[C] };
    double yp[3] = { st->py[A], st->py[B], st->py[C] };
    double nAB = arclen(vpos(st, A), vpos(st, B), Dm);
    double nBC = arclen(vpos(st, B), vpos(st, C), Dm);
    double nCA = arclen(vpos(st, C), vpos(st, A), Dm);
    double denom = nAB + nBC + nCA;
    adjust_origin(xp, yp, 3, Dm);
    st->px[A] += (nBC * xp[0] + nCA * xp[1] + nAB * xp[2]) / denom;
    st->py[A] += (nBC * yp[0] + nCA * yp[1] + nAB * yp[2]) / denom;
    st->px[A] = dom_mod(st->px[A], Dm);
    st->py[A] = dom_mod(st->py[A], Dm);
    int gbc[2], gab[2], gac[2], G1, G2, G3;
    grains_intersect(st, B, C, gbc); G3 = (gbc[0] == grn) ? gbc[1] : gbc[0];
    grains_intersect(st, A, B, gab); G2 = (gab[0] == grn) ? gab[1] : gab[0];
    grains_intersect(st, A, C, gac); G1 = (gac[0] == grn) ? gac[1] : gac[0];
    if (G1 < 0 || G2 < 0 || G3 < 0) { set_err(st, ORC_ERR_TOPOLOGY); return; }
    st->vx[A] = 0.0; st->vy[A] = 0.0;
    for (int i = 0; i < 3; i++) {
        int x = st->vb[3 * C + i];
        if ((st->bini[x] == B && st->bend[x] == C) || (st->bend[x] == B && st->bini[x] == C)) { st->ben[x] = 0; break; }
    }
    int BE = -1, CF = -1;
    for (int i = 0; i < 3; i++) {
        int x = st->vb[3 * B + i];
        if (!(st->bini[x] == A || st->bend[x] == A) && !(st->bini[x] == C || st->bend[x] == C)) { BE = x; break; }
    }
    for (int i = 0; i < 3; i++) {
        int x = st->vb[3 * C + i];
        if (!(st->bini[x] == A || st->bend[x] == A) && !(st->bini[x] == B || st->bend[x] == B)) { CF = x; break; }
    }
    if (BE < 0 || CF < 0) { set_err(st, ORC_ERR_TOPOLOGY); return; }
    if (st->bini[BE] == B) st->bini[BE] = A; else st->bend[BE] = A;
    if (st->bini[CF] == C) st->bini[CF] = A; else st->bend[CF] = A;
    for (int i = 0; i < 3; i++) {
        int x = st->vb[3 * A + i];
        if (st->bini[x] == B || st->bend[x] == B) { st->ben[x] = 0; st->vb[3 * A + i] = BE; break; }
    }
    for (int i = 0; i < 3; i++) {
        int x = st->vb[3 * A + i];
        if (st->bini[x] == C || st->bend[x] == C) { st->ben[x] = 0; st->vb[3 * A + i] = CF; break; }
    }
    st->ven[B] = 0; st->ven[C] = 0; st->gen[grn] = 0;
    orc_mod *mb = &st->vmod[4 * B], *mc = &st->vmod[4 * C];
    mb[0].grn = G2; mb[0].fix = ORC_REMOVE; mb[0].vrt = B; st->gfix[G2] = 1;
    mc[0].grn = G1; mc[0].fix = ORC_REMOVE; mc[0].vrt = C; st->gfix[G1] = 1;
    mb[1].grn = G3; mb[1].fix = ORC_REMOVE; mb[1].vrt = B; st->gfix[G3] = 1;
    mc[1].fix = ORC_REPLACE; mc[1].vrt = A; mc[1].prev = C; mc[1].grn = G3;
    for (int i = 0; i < 3; i++) if (st->vg[3 * A + i] == grn) st->vg[3 * A + i] = G3;
}
static void remove_grains(orc_state *st)                  /* topological.h:994 */
{
    for (int g = 0; g < st->ng; g++)
        if (st->gen[g] && st->gcand[g]) { remove_grain(st, g); st->ev_removals++; }
}
static void unlabel_boundaries_st2(orc_state *st)         /* topological.h:588 */
{
    for (int b = 0; b < st->nb; b++) {
        if (!(st->ben[b] && st->bcand[b])) continue;
        int gic[2];
        if (!gic_ok(st, b, gic)) continue;
        if (st->gvlen[gic[0]] == 3 || st->gvlen[gic[1]] == 3) st->bcand[b] = 0;
    }
}
/* topological.h:174-291 */
static void flip(orc_state *st, int bnd)
{
    double eps = st->opt.GB_eps, Dm = st->opt.domain_bound;
    int A = st->bini[bnd], B = st->bend[bnd];
    int gic[2], gnic[2];
    if (!gic_ok(st, bnd, gic)) return;
    grains_symdiff(st, A, B, gnic);
    int i, j, AC = -1, BE = -1;
    for (i = 0; i < 3; i++) if (st->vb[3 * A + i] == bnd) { i = (i + 1) % 3; AC = st->vb[3 * A + i]; break; }
    for (j = 0; j < 3; j++) if (st->vb[3 * B + j] == bnd) { j = (j + 1) % 3; BE = st->vb[3 * B + j]; break; }
    if (AC < 0 || BE < 0 || gnic[0] < 0 || gnic[1] < 0) { set_err(st, ORC_ERR_TOPOLOGY); return; }
    st->vb[3 * A + i] = BE;
    st->vb[3 * B + j] = AC;
    if (st->bini[AC] == A) st->bini[AC] = B; else st->bend[AC] = B;
    if (st->bini[BE] == B) st->bini[BE] = A; else st->bend[BE] = A;
    int g1, g2, g3, g4;
    for (g2 = 0; g2 < 2; g2++)
        if (grain_contains_consecutive(st, gic[g2], A, B) == 1) {
            orc_mod *m = &st->vmod[4 * A + 0];
            m->fix = ORC_REMOVE; m->vrt = A; m->grn = gic[g2]; st->gfix[gic[g2]] = 1; break;
        }
    for (g4 = 0; g4 < 2; g4++)
        if (grain_contains_consecutive(st, gic[g4], B, A) == 1) {
            orc_mod *m = &st->vmod[4 * B + 0];
            m->fix = ORC_REMOVE; m->vrt = B; m->grn = gic[g4]; st->gfix[gic[g4]] = 1; break;
        }
    for (g3 = 0; g3 < 2; g3++)
        if (grain_contains_vertex(st, gnic[g3], A) >= 0) {
            orc_mod *m = &st->vmod[4 * A + 1];
            m->fix = ORC_ADD; m->vrt = B; m->prev = A; m->grn = gnic[g3]; st->gfix[gnic[g3]] = 1; break;
        }
    for (g1 = 0; g1 < 2; g1++)
        if (grain_contains_vertex(st, gnic[g1], B) >= 0) {
            orc_mod *m = &st->vmod[4 * B + 1];
            m->fix = ORC_ADD; m->vrt = A; m->prev = B; m->grn = gnic[g1]; st->gfix[gnic[g1]] = 1; break;
        }
    if (g1 == 2 || g2 == 2 || g3 == 2 || g4 == 2) { set_err(st, ORC_ERR_TOPOLOGY); return; }
    for (int k = 0; k < 3; k++) {
        if (st->vg[3 * A + k] == gic[g2]) st->vg[3 * A + k] = gnic[g1];
        if (st->vg[3 * B + k] == gic[g4]) st->vg[3 * B + k] = gnic[g3];
    }
    v2 c = vmean(vpos(st, A), vpos(st, B), Dm);
    st->px[A] = c.x; st->py[A] = c.y;
    st->px[B] = c.x; st->py[B] = c.y;
    vertex_invert_boundary_order(st, A);
    vertex_invert_boundary_order(st, B);
    st->benergy[bnd] = boundary_compute_energy(st, bnd, eps);
    st->vx[A] = 0; st->vy[A] = 0; st->vx[B] = 0; st->vy[B] = 0;
}
static void apply_flippings(orc_state *st)                /* topological.h:1016 */
{
    for (int b = 0; b < st->nb; b++)
        if (st->ben[b] && st->bcand[b]) { flip(st, b); st->ev_flips++; }
}

/* ------------------------------------------------------------------ */
/* nucleation, src/nucleation2.cu                                      */
/* ------------------------------------------------------------------ */
typedef struct { v2 Apos, Bpos, Cpos; int D, E, F, AD, AE, AF, g1, g2, g3; double DeltaE; } nucl_geo;

/* nucleation2.cu:116-212 */
static int generate_grain_for_nucleation(orc_state *st, int A, double energy_eps, double energy_scaling,
                                         nucl_geo *o, int do_scale)
{
    double Dm = st->opt.domain_bound;
    double E0 = 0.0, E1 = 0.0;
    o->AD = st->vb[3 * A + 0]; o->AE = st->vb[3 * A + 1]; o->AF = st->vb[3 * A + 2];
    o->D = other_end(st, o->AD, A); o->E = other_end(st, o->AE, A); o->F = other_end(st, o->AF, A);
    int gAD[2], gAE[2], gAF[2];
    grains_intersect(st, A, o->D, gAD);
    grains_intersect(st, A, o->E, gAE);
    grains_intersect(st, A, o->F, gAF);
    if (gAD[0] == gAE[0] || gAD[0] == gAE[1]) { o->g2 = gAD[0]; o->g1 = gAD[1]; }
    else if (gAD[1] == gAE[0] || gAD[1] == gAE[1]) { o->g2 = gAD[1]; o->g1 = gAD[0]; }
    else return -1;
    if (gAE[0] == o->g2) o->g3 = gAE[1];
    else if (gAE[1] == o->g2) o->g3 = gAE[0];
    else return -1;
    if (o->g1 < 0 || o->g2 < 0 || o->g3 < 0) return -1;
    v2 pa = vpos(st, A);
    v2 tmp = delta_to(vpos(st, o->D), pa, Dm);
    double w = st->nucl_r[A] / mag(tmp);
    if (do_scale) w *= 0.99;
    o->Apos.x = w * tmp.x + pa.x; o->Apos.y = w * tmp.y + pa.y; o->Apos = adjust(o->Apos, Dm);
    tmp = delta_to(vpos(st, o->E), pa, Dm);
    w = st->nucl_r[A] / mag(tmp);
    if (do_scale) w *= 0.99;
    o->Bpos.x = w * tmp.x + pa.x; o->Bpos.y = w * tmp.y + pa.y; o->Bpos = adjust(o->Bpos, Dm);
    tmp = delta_to(vpos(st, o->F), pa, Dm);
    w = st->nucl_r[A] / mag(tmp);
    if (do_scale) w *= 0.99;
    o->Cpos.x = w * tmp.x + pa.x; o->Cpos.y = w * tmp.y + pa.y; o->Cpos = adjust(o->Cpos, Dm);
    double LAB = arclen(o->Apos, o->Bpos, Dm);
    double LBC = arclen(o->Bpos, o->Cpos, Dm);
    double LCA = arclen(o->Cpos, o->Apos, Dm);
    double xx[3], yy[3];
    xx[0] = pa.x; xx[1] = o->Cpos.x; xx[2] = o->Apos.x;
    yy[0] = pa.y; yy[1] = o->Cpos.y; yy[2] = o->Apos.y;
    double A1 = compute_area(xx, yy, 3, Dm);
    xx[0] = pa.x; xx[1] = o->Apos.x; xx[2] = o->Bpos.x;
    yy[0] = pa.y; yy[1] = o->Apos.y; yy[2] = o->Bpos.y;
    double A2 = compute_area(xx, yy, 3, Dm);
    xx[0] = pa.x; xx[1] = o->Bpos.x; xx[2] = o->Cpos.x;
    yy[0] = pa.y; yy[1] = o->Bpos.y; yy[2] = o->Cpos.y;
    double A3 = compute_area(xx, yy, 3, Dm);
    for (int i = 0; i < 3; i++) {
        if (do_scale) E0 += 0.99 * st->nucl_r[A] * st->benergy[st->vb[3 * A + i]];
        else E0 += st->nucl_r[A] * st->benergy[st->vb[3 * A + i]];
    }
    E0 += A1 * st->gse[o->g1] + A2 * st->gse[o->g2] + A3 * st->gse[o->g3];
    E1 = gb_energy_func(st->nucl_ori[A] - st->gori[o->g1], energy_eps) * energy_scaling * LCA;
    E1 += gb_energy_func(st->nucl_ori[A] - st->gori[o->g2], energy_eps) * energy_scaling * LAB;
    E1 += gb_energy_func(st->nucl_ori[A] - st->gori[o->g3], energy_eps) * energy_scaling * LBC;
    o->DeltaE = E1 - E0;
    return 0;
}
/* nucleation2.cu:239-282 */
static void compute_nucleation_factor(orc_state *st)
{
    int grid = st->opt.n_blocks * st->opt.n_threads;
    double eps = st->opt.GB_eps, s = st->opt.GB_scaling;
    for (int tid = 0; tid < grid; tid++)
        for (int v = tid; v < st->nv; v += grid) {
            if (!st->ven[v]) continue;
            st->DeltaE[v] = 0;
            st->nfactor[v] = 0;
            double ALs[3], mn;
            for (int i = 0; i < 3; i++) ALs[i] = st->blen[st->vb[3 * v + i]];
            mn = ALs[0];
            for (int i = 0; i < 3; i++) if (mn > ALs[i]) mn = ALs[i];
            st->nucl_r[v] = 0.8 * mn * rng_u(st, tid) + 0.1;
            st->nucl_ori[v] = 2 * M_PI * rng_u(st, tid);
            nucl_geo g0, g1;
            if (generate_grain_for_nucleation(st, v, eps, s, &g0, 0) ||
                generate_grain_for_nucleation(st, v, eps, s, &g1, 1)) {
                set_err(st, ORC_ERR_TOPOLOGY);
                continue;
            }
            st->DeltaE[v] = g0.DeltaE;
            st->nfactor[v] = g0.DeltaE - g1.DeltaE;
        }
}
/* nucleation2.cu:292-363 */
static void get_vertex_id_per_block(orc_state *st)
{
    int nblk = st->opt.n_blocks, nthr = st->opt.n_threads, grid = nblk * nthr;
    int *alive = (int *)malloc(sizeof(int) * (size_t)nthr);
    int *pick = (int *)malloc(sizeof(int) * (size_t)nthr);
    for (int blk = 0; blk < nblk; blk++) {
        for (int c = 0; c < nthr; c++) {
            int tid = blk * nthr + c, n_alive = 0, rid = -1;
            for (int v = tid; v < st->nv; v += grid) if (st->ven[v]) n_alive++;
            alive[c] = n_alive;
            if (n_alive > 0) {
                int n_steps = (int)(rng_u(st, tid) * (n_alive - 1));
                int k = 0;
                for (int v = tid; v < st->nv; v += grid)
                    if (st->ven[v]) { if (k == n_steps) { rid = v; break; } k++; }
                pick[c] = rid;
            } else pick[c] = -1;
        }
        int tot = 0;
        for (int i = 0; i < nthr; i++) tot += alive[i];
        if (tot > 0) {
            double p = rng_u(st, blk * nthr);
            double pc = 0.0;
            for (int i = 0; i < nthr; i++) {
                if (pick[i] != -1 && pc <= p && p < (pc + (alive[i] / (double)tot))) {
                    pick[0] = pick[i]; alive[0] = alive[i]; break;
                }
                pc += alive[i] / (double)tot;
            }
            st->vertex_buffer[blk] = pick[0];
            st->vertex_buffer[32 + blk] = tot;
        } else {
            st->vertex_buffer[blk] = -1;
            st->vertex_buffer[32 + blk] = 0;
        }
    }
    free(alive); free(pick);
}
/* nucleation2.cu:375-443 */
static int get_vertex_id2(orc_state *st)
{
    int tot = 0;
    for (int i = 0; i < 32; i++) tot += st->vertex_buffer[32 + i];
    double p = rng_u(st, 0);
    double pc = 0.0, pn = 0.0;
    for (int i = 0; i < 32; i++) {
        pn = ((double)st->vertex_buffer[32 + i]) / tot;
        if (st->vertex_buffer[i] != -1 && pc < p && p <= (pc + pn)) { st->vrt_id_candidate = st->vertex_buffer[i]; break; }
        pc += pn;
    }
    int v = st->vrt_id_candidate;
    if (v < 0 || v >= st->nv) { set_err(st, ORC_ERR_TOPOLOGY); return -1; }
    st->vnucleate[v] = 0;
    if (st->DeltaE[v] < 0) st->vnucleate[v] = 1;
    else if (st->nfactor[v] < 0) {
        double q = rng_u(st, 0);
        double thr = exp(-st->opt.MC_k * st->DeltaE[v]);
        if (q < thr) st->vnucleate[v] = 1;
        else st->vrt_id_candidate = -1;
    } else st->vrt_id_candidate = -1;
    return 0;
}
/* nucleation2.cu:33-72 */
static void get_nucleation_ids(orc_state *st)
{
    st->vrt_ids[0] = st->vrt_ids[1] = -1;
    st->bnd_ids[0] = st->bnd_ids[1] = st->bnd_ids[2] = -1;
    st->grn_id = -1;
    for (int i = 0; i < st->ng; i++) if (!st->gen[i]) { st->grn_id = i; break; }
    int f = 0;
    for (int i = 0; i < st->nb; i++) if (!st->ben[i]) { st->bnd_ids[f++] = i; if (f == 3) break; }
    f = 0;
    for (int i = 0; i < st->nv; i++) if (!st->ven[i]) { st->vrt_ids[f++] = i; if (f == 2) break; }
}
/* nucleation2.cu:474-676 */
static void nucleate(orc_state *st)
{
    int dv = st->vrt_ids[0] != st->vrt_ids[1];
    int db = (st->bnd_ids[0] != st->bnd_ids[1] && st->bnd_ids[1] != st->bnd_ids[2] && st->bnd_ids[2] != st->bnd_ids[0]);
    int dg = st->grn_id != -1;
    if (st->vrt_id_candidate == -1) return;
    if (!db || !dv || !dg) return;
    int A = st->vrt_id_candidate;
    if (!st->vnucleate[A]) return;
    if (st->vrt_ids[0] < 0 || st->vrt_ids[1] < 0 || st->bnd_ids[2] < 0) { set_err(st, ORC_ERR_CAPACITY); return; }
    int B = st->vrt_ids[0], C = st->vrt_ids[1];
    int AB = st->bnd_ids[0], BC = st->bnd_ids[1], CA = st->bnd_ids[2];
    int g = st->grn_id;
    nucl_geo o;
    /* the reference passes (energy_scaling, energy_eps) swapped here; it
     * only changes the DeltaE that this call discards */
    if (generate_grain_for_nucleation(st, A, st->opt.GB_scaling, st->opt.GB_eps, &o, 1)) {
        set_err(st, ORC_ERR_TOPOLOGY); return;
    }
    init_vertex(st, B, o.Bpos);
    init_vertex(st, C, o.Cpos);
    st->px[A] = o.Apos.x; st->py[A] = o.Apos.y;
    for (int i = 0; i < 3; i++) st->vb[3 * A + i] = -1;
    init_boundary(st, AB, A, B);
    init_boundary(st, BC, B, C);
    init_boundary(st, CA, C, A);
    vertex_add_boundary(st, A, o.AD);
    nucleate_grain(st, g);
    st->gori[g] = st->nucl_ori[A];
    grain_add_vertex(st, g, A);
    grain_add_vertex(st, g, B);
    grain_add_vertex(st, g, C);
    for (int i = 0; i < 3; i++) if (st->vg[3 * A + i] == o.g3) { st->vg[3 * A + i] = g; break; }
    vertex_add_grain(st, B, g); vertex_add_grain(st, B, o.g2); vertex_add_grain(st, B, o.g3);
    vertex_add_grain(st, C, g); vertex_add_grain(st, C, o.g3); vertex_add_grain(st, C, o.g1);
    grain_add_vertex_after(st, o.g1, C, A);
    if (st->bini[o.AE] == A) grain_add_vertex_after(st, o.g2, B, st->bend[o.AE]);
    else if (st->bend[o.AE] == A) grain_add_vertex_after(st, o.g2, B, st->bini[o.AE]);
    grain_add_vertex_after(st, o.g3, C, A);
    grain_add_vertex_after(st, o.g3, B, C);
    grain_remove_vertex(st, o.g3, A);
    vertex_invert_boundary_order(st, B);
    vertex_invert_boundary_order(st, C);
    if (st->bini[o.AE] == A) st->bini[o.AE] = B;
    else if (st->bend[o.AE] == A) st->bend[o.AE] = B;
    st->vb[3 * B + 2] = o.AE;
    if (st->bini[o.AF] == A) st->bini[o.AF] = C; else st->bend[o.AF] = C;
    st->vb[3 * C + 2] = o.AF;
    st->ev_nucleations++;
}

/* ------------------------------------------------------------------ */
/* main loop, src/main.cu:120-394                                      */
/* ------------------------------------------------------------------ */
int orc_should_continue(const orc_state *st)
{
    const orc_options *o = &st->opt;
    int mg = o->min_grains;
    return ((st->t <= o->tmax && o->tmax > 0) || (st->n <= o->nmax && o->nmax > 0)) &&
           (st->curr_n_grains >= mg && mg > 0);
}
int orc_should_export(const orc_state *st)
{
    int mg = st->opt.min_grains;
    return (st->opt.snap_gap > 0 && st->n % st->opt.snap_gap == 0) || (st->curr_n_grains <= mg && mg > 0);
}

int orc_step(orc_state *st)
{
    orc_options *o = &st->opt;
    st->ev_flips = st->ev_removals = st->ev_two_three = st->ev_nucleations = st->ev_conflicts = 0;
    st->n_two_three_iters = 0;
    orc_compute_boundary_arclengths(st);                  /* :124 */
    orc_compute_grain_areas(st);                          /* :127 */
    orc_compute_boundary_energies(st);                    /* :130 */
    orc_compute_vertex_energies(st);                      /* :133 */
    if (st->curr_n_grains <= 5 * o->n_grains / 6) st->allow_nucleation = 1; /* :137 */
    if (o->do_nucleation && o->nucleation_gap > 0 && (st->n % o->nucleation_gap) == 0 && st->allow_nucleation) {
        compute_nucleation_factor(st);                    /* :144 */
        get_vertex_id_per_block(st);                      /* :147 */
        if (get_vertex_id2(st) == 0) {                    /* :149 */
            get_nucleation_ids(st);                       /* :161 */
            nucleate(st);                                 /* :164 */
        }
        orc_compute_boundary_arclengths(st);              /* :171-181 */
        orc_compute_grain_areas(st);
        orc_compute_boundary_energies(st);
        orc_compute_vertex_energies(st);
    }
    /* compute_dihedral_angles (:200) has no observable output: skipped */
    orc_compute_vertex_velocities(st);                    /* :203 */
    orc_compute_grain_dadts(st);                          /* :206 */
    orc_compute_t_ext(st);                                /* :212 */
    label_boundaries(st);                                 /* :216 */
    polling_system(st);                                   /* :219 */
    check_conflictive_boundaries(st);                     /* :222 */
    unlabel_conflictive_boundaries(st);                   /* :224 */
    for (int it = 0; it < 20; it++) {                     /* :227-250 */
        int c = two_three_sided_grains(st);
        st->last_two_three[it] = c;
        st->n_two_three_iters = it + 1;
        if (c == 0) break;
        remove_two_grains_configurations(st);
        fix_grain_lists(st);
    }
    for (int g = 0; g < st->ng; g++) if (st->gen[g]) st->gcand[g] = 0; /* :252 */
    label_3sided_grains(st);                              /* :255 */
    remove_grains(st);                                    /* :259 */
    fix_grain_lists(st);                                  /* :262 */
    orc_compute_grain_areas(st);                          /* :266 */
    unlabel_boundaries_st2(st);                           /* :282 */
    apply_flippings(st);                                  /* :289 */
    fix_grain_lists(st);                                  /* :294 */
    update_vertices_positions(st);                        /* :314 */
    st->curr_n_grains = orc_current_n_grains(st);         /* :317 */
    st->nucleated_area = orc_nucleated_fraction_area(st); /* :321 */
    return st->status;
}

/* src/main.cu:388-393; returns 1 to keep looping */
int orc_finish_step(orc_state *st)
{
    st->n++;
    st->t = st->n * st->opt.dt;
    int mg = st->opt.min_grains;
    if (st->curr_n_grains <= mg && mg > 0) return 0;
    return orc_should_continue(st);
}

/* ------------------------------------------------------------------ */
/* snapshot, src/io.h:280-377                                          */
/* ------------------------------------------------------------------ */
int orc_export(const orc_state *st, const char *path, double time)
{
    const orc_options *o = &st->opt;
    FILE *f = fopen(path, "w");
    if (!f) return ORC_ERR_IO;
    int cv = 0, cb = 0, cg = 0;
    for (int i = 0; i < st->nv; i++) cv += st->ven[i] ? 1 : 0;
    for (int i = 0; i < st->nb; i++) cb += st->ben[i] ? 1 : 0;
    for (int i = 0; i < st->ng; i++) cg += st->gen[i] ? 1 : 0;
    fprintf(f, "TIME %.16f\n", time);
    fprintf(f, "DELTA T %.16f\n", o->dt);
    fprintf(f, "DELTA TAU %.16f\n", o->dtau);
    fprintf(f, "MAX TIME %.16f\n", o->tmax);
    fprintf(f, "NUCLEATION %d\n", o->do_nucleation ? 1 : 0);
    fprintf(f, "DOMAIN BOUND %.16f\n", o->domain_bound);
    fprintf(f, "GB EPSILON %.16f\n", o->GB_eps);
    fprintf(f, "GB SCALING %.16f\n", o->GB_scaling);
    fprintf(f, "SE EPSILON %.16f\n", o->SE_eps);
    fprintf(f, "SE MIN %.16f\n", o->SE_min);
    fprintf(f, "SE MAX %.16f\n", o->SE_max);
    fprintf(f, "NUCLEATION SCALING %.16f\n", o->nucleation_scaling);
    fprintf(f, "MAX VERTICES PER GRN %d\n", MAXV);
    fprintf(f, "VERTICES %d\n", st->nv);
    fprintf(f, "BOUNDARIES %d\n", st->nb);
    fprintf(f, "GRAINS %d\n", st->ng);
    fprintf(f, "CURR VERTICES %d\n", cv);
    fprintf(f, "CURR BOUNDARIES %d\n", cb);
    fprintf(f, "CURR GRAINS %d\n", cg);
    fprintf(f, "#VERTEX ENABLED ENERGY X Y VX VY VXbnd VXgrn VYbnd VYgrn VG1 G2 G3 N1 N2 N3\n");
    for (int i = 0; i < st->nv; i++) {
        fprintf(f, "%d %d %.16f %.16f %.16f %.16f %.16f %.16f %.16f %.16f %.16f %d %d %d ",
                i, st->ven[i] ? 1 : 0, st->venergy[i], st->px[i], st->py[i], st->vx[i], st->vy[i],
                st->vel_bnd_x[i], st->vel_grn_x[i], st->vel_bnd_y[i], st->vel_grn_y[i],
                st->vg[3 * i], st->vg[3 * i + 1], st->vg[3 * i + 2]);
        for (int j = 0; j < 3; j++) {
            int b = st->vb[3 * i + j];
            int nbr = b < 0 ? -1 : (st->bini[b] == i ? st->bend[b] : st->bini[b]);
            fprintf(f, j == 2 ? "%d\n" : "%d ", nbr);
        }
    }
    fprintf(f, "#BOUNDARY ENABLED INI END ENERGY ARCLEN EXTTIME CANDIDATE\n");
    for (int i = 0; i < st->nb; i++)
        fprintf(f, "%d %d %d %d %.16f %.16f %.16f %d\n", i, st->ben[i] ? 1 : 0, st->bini[i], st->bend[i],
                st->benergy[i], st->blen[i], st->btext[i], st->bcand[i] ? 1 : 0);
    fprintf(f, "#GRAIN ID ENABLED NUCLEATED ORIENT SE AREA dAdt VLEN VERTICES\n");
    for (int i = 0; i < st->ng; i++) {
        fprintf(f, "%d %d %d %.16f %.16f %.16f %.16f %d ", i, st->gen[i] ? 1 : 0, (int)st->gtype[i],
                st->gori[i], st->gse[i], st->garea[i], st->gdadt[i], st->gvlen[i]);
        for (int j = 0; j < MAXV; j++) {
            if (j < st->gvlen[i]) fprintf(f, "%d ", st->glist[MAXV * i + j]);
            else if (j == MAXV - 1) fprintf(f, "%d", -1);
            else fprintf(f, "%d ", -1);
        }
        fprintf(f, "\n");
    }
    fclose(f);
    return ORC_OK;
}

/* ------------------------------------------------------------------ */
/* invariant checker, src/utils.h:85-336 (counts is_valid=false hits)  */
/* ------------------------------------------------------------------ */
int orc_check_data(const orc_state *st)
{
    int bad = 0;
    for (int b = 0; b < st->nb; b++) {
        if (!st->ben[b]) continue;
        int ini = st->bini[b], end = st->bend[b];
        if (ini == end) bad++;
        if (!st->ven[ini] || !st->ven[end]) bad++;
        if (st->vb[3 * ini] != b && st->vb[3 * ini + 1] != b && st->vb[3 * ini + 2] != b) bad++;
        if (st->vb[3 * end] != b && st->vb[3 * end + 1] != b && st->vb[3 * end + 2] != b) bad++;
        if (!st->ben[st->vb[3 * end]] || !st->ben[st->vb[3 * end + 1]] || !st->ben[st->vb[3 * end + 2]]) bad++;
        if (!st->ben[st->vb[3 * ini]] || !st->ben[st->vb[3 * ini + 1]] || !st->ben[st->vb[3 * ini + 2]]) bad++;
        int gic[2];
        if (grains_intersect((orc_state *)st, ini, end, gic) < 2 || gic[0] == gic[1]) bad++;
    }
    for (int v = 0; v < st->nv; v++) {
        if (!st->ven[v]) continue;
        const int *B = &st->vb[3 * v], *G = &st->vg[3 * v];
        if (B[0] == B[1] || B[1] == B[2] || B[2] == B[0]) bad++;
        if (G[0] == G[1] || G[1] == G[2] || G[2] == G[0]) bad++;
        for (int j = 0; j < 3; j++) if (!st->ben[B[j]]) bad++;
        for (int j = 0; j < 3; j++) if (G[j] < 0 || !st->gen[G[j]]) bad++;
        for (int j = 0; j < 3; j++) if (st->bini[B[j]] == st->bend[B[j]]) bad++;
        int arr[3];
        for (int j = 0; j < 3; j++) arr[j] = st->bini[B[j]] == v ? st->bend[B[j]] : st->bini[B[j]];
        if (arr[0] == arr[1] || arr[1] == arr[2] || arr[2] == arr[0]) bad++;
        for (int j = 0; j < 3; j++) if (st->bini[B[j]] != v && st->bend[B[j]] != v) bad++;
        for (int j = 0; j < 3; j++) {
            if (G[j] < 0) { bad++; continue; }
            if (grain_contains_vertex(st, G[j], v) < 0) bad++;
        }
    }
    for (int g = 0; g < st->ng; g++) {
        if (!st->gen[g]) continue;
        const int *L = &st->glist[MAXV * g];
        for (int j = 0; j < st->gvlen[g]; j++) if (!st->ven[L[j]]) bad++;
        for (int j = 0; j < st->gvlen[g]; j++) {
            int v = L[j];
            if (st->vg[3 * v] != g && st->vg[3 * v + 1] != g && st->vg[3 * v + 2] != g) { bad++; break; }
        }
        int cnt = 0;
        for (int j = 0; j < MAXV; j++) cnt += L[j] != -1;
        if (cnt != st->gvlen[g]) bad++;
    }
    return bad;
}

/* ------------------------------------------------------------------ */
/* bindings helpers                                                    */
/* ------------------------------------------------------------------ */
void *orc_field(orc_state *st, const char *name, int64_t *count, int *kind)
{
    struct { const char *n; void *p; int64_t c; int k; } t[] = {
        { "px", st->px, st->nv, 0 }, { "py", st->py, st->nv, 0 }, { "vx", st->vx, st->nv, 0 },
        { "vy", st->vy, st->nv, 0 }, { "venergy", st->venergy, st->nv, 0 },
        { "vel_bnd_x", st->vel_bnd_x, st->nv, 0 }, { "vel_grn_x", st->vel_grn_x, st->nv, 0 },
        { "vel_bnd_y", st->vel_bnd_y, st->nv, 0 }, { "vel_grn_y", st->vel_grn_y, st->nv, 0 },
        { "nucl_r", st->nucl_r, st->nv, 0 }, { "nucl_ori", st->nucl_ori, st->nv, 0 },
        { "DeltaE", st->DeltaE, st->nv, 0 }, { "nfactor", st->nfactor, st->nv, 0 },
        { "ven", st->ven, st->nv, 2 }, { "vnucleate", st->vnucleate, st->nv, 2 },
        { "vb", st->vb, 3 * (int64_t)st->nv, 1 }, { "vg", st->vg, 3 * (int64_t)st->nv, 1 },
        { "vmod", st->vmod, 4 * (int64_t)st->nv, 4 }, { "voted", st->voted, st->nv, 1 },
        { "bini", st->bini, st->nb, 1 }, { "bend", st->bend, st->nb, 1 },
        { "benergy", st->benergy, st->nb, 0 }, { "blen", st->blen, st->nb, 0 },
        { "btext", st->btext, st->nb, 0 }, { "ben", st->ben, st->nb, 2 }, { "bcand", st->bcand, st->nb, 2 },
        { "bvotes", st->bvotes, st->nb, 1 }, { "bconf", st->bconf, st->nb, 1 },
        { "glist", st->glist, (int64_t)MAXV * st->ng, 1 }, { "gvlen", st->gvlen, st->ng, 1 },
        { "garea", st->garea, st->ng, 0 }, { "gdadt", st->gdadt, st->ng, 0 }, { "gori", st->gori, st->ng, 0 },
        { "gse", st->gse, st->ng, 0 }, { "gen", st->gen, st->ng, 2 }, { "gcand", st->gcand, st->ng, 2 },
        { "gfix", st->gfix, st->ng, 2 }, { "gtype", st->gtype, st->ng, 2 },
        { "cand_buf", st->cand_buf, st->nb, 2 }, { "rng_pos", st->rng_pos, st->rng_nstreams, 3 },
    };
    for (size_t i = 0; i < sizeof t / sizeof t[0]; i++)
        if (!strcmp(t[i].n, name)) { *count = t[i].c; *kind = t[i].k; return t[i].p; }
    return NULL;
}

orc_state *orc_clone(const orc_state *src)
{
    orc_state *st = alloc_state(&src->opt, src->nv, src->nb, src->ng);
    int64_t *pos = st->rng_pos;
    void *keep[64]; int nk = 0;
    (void)keep; (void)nk;
    /* copy scalars then arrays */
    orc_state tmp = *st;
    *st = *src;
    /* restore our own array pointers */
#define P(f) st->f = tmp.f
    P(px); P(py); P(vx); P(vy); P(venergy); P(vel_bnd_x); P(vel_grn_x); P(vel_bnd_y); P(vel_grn_y);
    P(nucl_r); P(nucl_ori); P(DeltaE); P(nfactor); P(ven); P(vnucleate); P(vb); P(vg); P(vmod); P(voted);
    P(bini); P(bend); P(benergy); P(blen); P(btext); P(ben); P(bcand); P(bvotes); P(bconf);
    P(glist); P(gvlen); P(garea); P(gdadt); P(gori); P(gse); P(gen); P(gcand); P(gfix); P(gtype); P(cand_buf);
#undef P
    st->rng_pos = pos;
    memcpy(st->rng_pos, src->rng_pos, sizeof(int64_t) * (size_t)src->rng_nstreams);
    const char *names[] = { "px","py","vx","vy","venergy","vel_bnd_x","vel_grn_x","vel_bnd_y","vel_grn_y",
        "nucl_r","nucl_ori","DeltaE","nfactor","ven","vnucleate","vb","vg","vmod","voted","bini","bend",
        "benergy","blen","btext","ben","bcand","bvotes","bconf","glist","gvlen","garea","gdadt","gori","gse",
        "gen","gcand","gfix","gtype","cand_buf" };
    static const size_t ksz[] = { 8, 4, 1, 8, 16 };
    for (size_t i = 0; i < sizeof names / sizeof names[0]; i++) {
        int64_t c1, c2; int k1, k2;
        void *d = orc_field(st, names[i], &c1, &k1);
        void *s = orc_field((orc_state *)src, names[i], &c2, &k2);
        memcpy(d, s, (size_t)c1 * ksz[k1]);
    }
    return st;
}

/* Digests of the state in the definition of sevc_state_digest (the
 * engine's include/sevc.h): per field, the sum mod 2^64 over its elements
 * i of splitmix64_finaliser((f << 56) + i * 0x9E3779B97F4A7C15 + bits_i),
 * bits_i = the double's bit pattern, the int32 as unsigned 32-bit, or the
 * byte.  Lets the tests compare a run with the engine's every step. */
static uint64_t dg_mix(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
void orc_state_digest(orc_state *st, uint64_t *out)
{
    static const char *names[20] = { "px", "py", "vx", "vy", "ven", "vb", "vg", "bini", "bend", "benergy", "blen",
                                     "ben", "bcand", "glist", "gvlen", "garea", "gori", "gse", "gen", "gtype" };
    for (int f = 0; f < 20; f++) {
        int64_t n;
        int kind;
        void *p = orc_field(st, names[f], &n, &kind);
        uint64_t salt = (uint64_t)f << 56, acc = 0;
        int nt = st->nthreads_omp > 1 && n > 65536 ? st->nthreads_omp : 1;
#pragma omp parallel for reduction(+ : acc) schedule(static) num_threads(nt)
        for (int64_t i = 0; i < n; i++) {
            uint64_t b;
            if (kind == 0) memcpy(&b, (const double *)p + i, 8);
            else if (kind == 1) b = (uint32_t)((const int32_t *)p)[i];
            else b = ((const uint8_t *)p)[i];
            acc += dg_mix(salt + (uint64_t)i * 0x9E3779B97F4A7C15ULL + b);
        }
        out[f] = acc;
    }
}
