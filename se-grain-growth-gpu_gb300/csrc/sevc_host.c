/*
 * Host side of the engine, in C: .ini options (src/options.h:69-206),
 * initial mesh construction (src/io.h:66-264), snapshot text
 * (src/io.h:280-377) and the invariant checker (src/utils.h:85-336).
 *
 * These run on the CPU in the reference too; they are restated here so the
 * engine accepts the same files and writes byte-identical snapshots.
 * Compiled without FMA contraction so the boundary ordering angles
 * (atan2 of wrapped deltas) match the reference's host build.
 */
#include "sevc_host.h"

#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

static __thread char g_err[512];

void sevc_set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}

const char *sevc_last_error(void) { return g_err; }

/* ---------------------------------------------------------------- */
/* options                                                           */
/* ---------------------------------------------------------------- */
sevc_status sevc_default_options(sevc_options *o)
{
    if (!o) return SEVC_ERR_ARG;
    memset(o, 0, sizeof(*o));
    o->tmax = -1;                 /* src/options.h:71-85 */
    o->nmax = -1;
    o->GB_eps = 0.02;
    o->GB_scaling = 1.0;
    o->SE_eps = 1.0;
    o->SE_min = 999;
    o->SE_max = 999;
    o->MC_k = 1.0;
    o->nucleation_scaling = 0.9;
    o->domain_bound = 1.0;
    o->do_nucleation = 1;
    o->nucleation_gap = 1;
    o->debug_lvl = 0;
    o->leave_percent = -1;
    o->n_blocks = 32;
    o->n_threads = 256;
    o->min_grains = 5000;         /* src/main.cu:49 */
    return SEVC_OK;
}

static void chop_last(char *s)    /* fix_string, src/options.h:55 */
{
    size_t n = strlen(s);
    if (n) s[n - 1] = '\0';
}

static void copy_name(char *dst, const char *val)
{
    snprintf(dst, 256, "%s", val);
    chop_last(dst);
}

sevc_status sevc_load_ini(const char *path, sevc_options *o)
{
    sevc_default_options(o);
    FILE *f = fopen(path, "r");
    if (!f) { sevc_set_error("cannot open %s", path); return SEVC_ERR_IO; }
    char line[1000], key[1000];
    while (fgets(line, sizeof line, f)) {
        if (line[0] == '#' || line[0] == '[') continue;
        char *eq = strchr(line, '=');
        if (!eq) continue;
        size_t k = (size_t)(eq - line);
        memcpy(key, line, k);
        key[k] = '\0';
        const char *v = eq + 1;
        /* keys compare without trimming, like src/options.h:103-106 */
        if (!strcmp(key, "dt")) o->dt = atof(v);
        else if (!strcmp(key, "dtau")) o->dtau = atof(v);
        else if (!strcmp(key, "tmax")) o->tmax = atof(v);
        else if (!strcmp(key, "nmax")) o->nmax = atoi(v);
        else if (!strcmp(key, "snap_gap")) o->snap_gap = atoi(v);
        else if (!strcmp(key, "leave_percent")) o->leave_percent = atof(v);
        else if (!strcmp(key, "n_grains")) o->n_grains = atoi(v);
        else if (!strcmp(key, "vertex_fname")) copy_name(o->vertex_fname, v);
        else if (!strcmp(key, "boundary_fname")) copy_name(o->boundary_fname, v);
        else if (!strcmp(key, "orientation_fname")) copy_name(o->orientation_fname, v);
        else if (!strcmp(key, "SE_fname")) copy_name(o->SE_fname, v);
        else if (!strcmp(key, "n_blocks")) o->n_blocks = atoi(v);
        else if (!strcmp(key, "n_threads")) o->n_threads = atoi(v);
        else if (!strcmp(key, "debug_lvl")) o->debug_lvl = atoi(v);
        else if (!strcmp(key, "folder")) copy_name(o->output_folder, v);
        else if (!strcmp(key, "GB_eps")) o->GB_eps = atof(v);
        else if (!strcmp(key, "GB_scaling")) o->GB_scaling = atof(v);
        else if (!strcmp(key, "SE_eps")) o->SE_eps = atof(v);
        else if (!strcmp(key, "SE_min")) o->SE_min = atof(v);
        else if (!strcmp(key, "SE_max")) o->SE_max = atof(v);
        else if (!strcmp(key, "MC_k")) o->MC_k = atof(v);
        else if (!strcmp(key, "nucleation_scaling")) o->nucleation_scaling = atof(v);
        else if (!strcmp(key, "domain_bound")) o->domain_bound = atof(v);
        else if (!strcmp(key, "do_nucleation")) o->do_nucleation = strcmp(v, "true\n") == 0;
    }
    fclose(f);
    o->nucleation_gap = (int)(o->dtau / o->dt);  /* src/options.h:172 */
    if (o->tmax > 0 && o->nmax == -1) {
    } else if (o->tmax == -1 && o->nmax > 0) {
    } else {
        o->tmax = 1.0;
        o->nmax = -1;
    }
    return SEVC_OK;
}

/* ---------------------------------------------------------------- */
/* host mesh storage                                                 */
/* ---------------------------------------------------------------- */
int sevc_hmesh_alloc(sevc_hmesh *hm, int nv, int nb, int ng)
{
    memset(hm, 0, sizeof(*hm));
    size_t V = (size_t)nv, B = (size_t)nb, G = (size_t)ng;
    size_t bytes = 9 * V * 8 + V + 6 * V * 4 + 2 * B * 4 + 3 * B * 8 + 2 * B +
                   (SEVC_MAX_VRT_PER_GRN + 1) * G * 4 + 4 * G * 8 + 2 * G + 64 * 8;
    char *p = (char *)calloc(1, bytes);
    if (!p) return SEVC_ERR_CAPACITY;
    hm->block = p;
    sevc_mesh_host *m = &hm->m;
    m->nv = nv; m->nb = nb; m->ng = ng;
#define TAKE(f, n, t) do { m->f = (t *)p; p += (n) * sizeof(t); } while (0)
    TAKE(px, V, double); TAKE(py, V, double); TAKE(vx, V, double); TAKE(vy, V, double);
    TAKE(venergy, V, double); TAKE(vel_bnd_x, V, double); TAKE(vel_grn_x, V, double);
    TAKE(vel_bnd_y, V, double); TAKE(vel_grn_y, V, double);
    TAKE(benergy, B, double); TAKE(blen, B, double); TAKE(btext, B, double);
    TAKE(garea, G, double); TAKE(gdadt, G, double); TAKE(gori, G, double); TAKE(gse, G, double);
    TAKE(vb, 3 * V, int32_t); TAKE(vg, 3 * V, int32_t);
    TAKE(bini, B, int32_t); TAKE(bend, B, int32_t);
    TAKE(glist, SEVC_MAX_VRT_PER_GRN * G, int32_t); TAKE(gvlen, G, int32_t);
    TAKE(ven, V, uint8_t); TAKE(ben, B, uint8_t); TAKE(bcand, B, uint8_t);
    TAKE(gen, G, uint8_t); TAKE(gtype, G, uint8_t);
#undef TAKE
    return SEVC_OK;
}

void sevc_hmesh_free(sevc_hmesh *hm)
{
    free(hm->block);
    memset(hm, 0, sizeof(*hm));
}

/* ---------------------------------------------------------------- */
/* mesh construction, src/io.h:66-264                                */
/* ---------------------------------------------------------------- */
static double wrapd(double dest, double orig, double D) /* src/geometry.h:147 */
{
    double d = dest - orig;
    if (d > +(D / 2.0)) return (d - D);
    if (d < -(D / 2.0)) return (D + d);
    return d;
}

/* vertex_set_boundaries_clockwise, src/geometry.h:437-460: order the three
 * boundaries by decreasing atan2 angle of the edge vector (three
 * compare-swaps, stable on ties). */
static void order_boundaries(sevc_mesh_host *m, int v, double D)
{
    int *s = &m->vb[3 * v];
    double a[3];
    for (int i = 0; i < 3; i++) {
        int b = s[i];
        int o = (m->bini[b] == v) ? m->bend[b] : m->bini[b];
        a[i] = atan2(wrapd(m->py[o], m->py[v], D), wrapd(m->px[o], m->px[v], D));
    }
    static const int pairs[3][2] = { { 0, 1 }, { 1, 2 }, { 0, 1 } };
    for (int k = 0; k < 3; k++) {
        int i = pairs[k][0], j = pairs[k][1];
        if (a[i] < a[j]) {
            double t = a[i]; a[i] = a[j]; a[j] = t;
            int tb = s[i]; s[i] = s[j]; s[j] = tb;
        }
    }
}

int sevc_host_build(const sevc_options *opt, int nv, const double *xy, int nb, const int *ridges,
                    int n_ori, const double *oris, int n_se, const double *se, sevc_hmesh *out)
{
    int ng = opt->n_grains;
    if (nv <= 0 || nb <= 0 || ng <= 0) { sevc_set_error("empty mesh"); return SEVC_ERR_PARSE; }
    if (n_ori > ng || n_se > ng) { sevc_set_error("more orientations/SE values than grains"); return SEVC_ERR_PARSE; }
    if (sevc_hmesh_alloc(out, nv, nb, ng)) { sevc_set_error("out of host memory"); return SEVC_ERR_CAPACITY; }
    sevc_mesh_host *m = &out->m;
    double D = opt->domain_bound;
    for (int i = 0; i < nv; i++) {              /* init_vertex, src/geometry.h:346 */
        m->px[i] = xy[2 * i] * D;
        m->py[i] = xy[2 * i + 1] * D;
        m->ven[i] = 1;
        m->vb[3 * i] = m->vb[3 * i + 1] = m->vb[3 * i + 2] = -1;
        m->vg[3 * i] = m->vg[3 * i + 1] = m->vg[3 * i + 2] = -1;
    }
    for (int b = 0; b < nb; b++) {              /* init_boundary, src/geometry.h:491 */
        int a = ridges[2 * b], c = ridges[2 * b + 1];
        if (a < 0 || a >= nv || c < 0 || c >= nv) { sevc_set_error("ridge %d out of range", b); goto bad; }
        m->bini[b] = a;
        m->bend[b] = c;
        int ends[2] = { a, c };
        for (int e = 0; e < 2; e++) {
            int *s = &m->vb[3 * ends[e]];
            if (s[0] < 0) s[0] = b; else if (s[1] < 0) s[1] = b; else if (s[2] < 0) s[2] = b;
        }
        m->btext[b] = SEVC_MAX_T_EXT;
        m->ben[b] = 1;
    }
    for (int v = 0; v < nv; v++)
        if (m->vb[3 * v] < 0 || m->vb[3 * v + 1] < 0 || m->vb[3 * v + 2] < 0) {
            sevc_set_error("vertex %d has fewer than three boundaries", v);
            goto bad;
        }
#pragma omp parallel for schedule(static)
    for (int v = 0; v < nv; v++) order_boundaries(m, v, D);

    {   /* face traversal, src/io.h:137-186.  The reference walks a face from
         * the first of its (vertex, side) half-edges met in index order and
         * numbers faces in that order; that half-edge is the smallest index
         * on the face's cycle of successors.  So: every successor in
         * parallel, every half-edge's cycle minimum by pointer doubling
         * (7 rounds cover 128 >= the 100 vertices a grain may have), faces
         * numbered by ascending minimum, and each face walked from its
         * minimum, in parallel. */
        size_t H = 3 * (size_t)nv;
        int *next = (int *)malloc(H * sizeof(int)), *fid = (int *)malloc(H * sizeof(int));
        int *j0 = (int *)malloc(H * sizeof(int)), *j1 = (int *)malloc(H * sizeof(int));
        int *c0 = (int *)malloc(H * sizeof(int)), *c1 = (int *)malloc(H * sizeof(int));
        int bad_next = 0, bad_walk = 0;
        if (!next || !fid || !j0 || !j1 || !c0 || !c1) {
            free(next); free(fid); free(j0); free(j1); free(c0); free(c1);
            sevc_set_error("out of host memory");
            goto bad;
        }
#pragma omp parallel for schedule(static) reduction(| : bad_next)
        for (long long h = 0; h < (long long)H; h++) {
            int cur = (int)(h / 3), b = m->vb[h];
            int nx = (m->bini[b] == cur) ? m->bend[b] : m->bini[b];
            int i = 0;
            while (i < 3 && m->vb[3 * nx + i] != b) i++;
            next[h] = i == 3 ? -1 : 3 * nx + (i + 1) % 3;
            bad_next |= i == 3;
            j0[h] = i == 3 ? (int)h : next[h];
            c0[h] = (int)h;
            fid[h] = -1;
        }
        for (int r = 0; r < 7; r++) {
#pragma omp parallel for schedule(static)
            for (long long h = 0; h < (long long)H; h++) {
                int s = j0[h], a = c0[s];
                c1[h] = a < c0[h] ? a : c0[h];
                j1[h] = j0[s];
            }
            int *t = j0; j0 = j1; j1 = t;
            t = c0; c0 = c1; c1 = t;
        }
        int ngr = 0;                                 /* faces in the reference's order */
        for (size_t h = 0; h < H; h++)
            if (c0[h] == (int)h) j1[h] = ngr++;
        if (!bad_next && ngr == ng) {
#pragma omp parallel for schedule(dynamic, 1024) reduction(| : bad_walk)
            for (long long h0 = 0; h0 < (long long)H; h0++) {
                if (c0[h0] != (int)h0) continue;
                int g = j1[h0], n = 0, h = (int)h0, start = (int)(h0 / 3);
                int *L = &m->glist[(size_t)SEVC_MAX_VRT_PER_GRN * g];
                do {
                    if (n >= SEVC_MAX_VRT_PER_GRN || fid[h] >= 0) { bad_walk = 1; break; }
                    fid[h] = g;
                    L[n++] = h / 3;
                    h = next[h];
                } while (h / 3 != start);
                for (int k = n; k < SEVC_MAX_VRT_PER_GRN; k++) L[k] = -1;
                m->gvlen[g] = n;
                m->gen[g] = 1;
            }
            for (size_t h = 0; h < H && !bad_walk; h++) bad_walk |= fid[h] < 0;
        }
        if (!bad_next && !bad_walk && ngr == ng) {
#pragma omp parallel for schedule(static)
            for (int v = 0; v < nv; v++) {          /* src/io.h:196-200: slots in ascending grain order */
                int a = fid[3 * v], b = fid[3 * v + 1], c = fid[3 * v + 2], t;
                if (a > b) { t = a; a = b; b = t; }
                if (b > c) { t = b; b = c; c = t; }
                if (a > b) { t = a; a = b; b = t; }
                m->vg[3 * v] = a; m->vg[3 * v + 1] = b; m->vg[3 * v + 2] = c;
            }
        }
        free(next); free(fid); free(j0); free(j1); free(c0); free(c1);
        if (bad_next || bad_walk) { sevc_set_error("inconsistent ridges: the faces do not close"); goto bad; }
        if (ngr != ng) {
            sevc_set_error("face traversal found %d grains, expected %d", ngr, ng);
            goto bad;
        }
    }
    /* src/io.h:189-192 sorts each vertex's boundaries again, then swaps the
     * first two.  Nothing moved since the first sort and the three
     * compare-swaps leave a sorted triple unchanged, so only the swap
     * remains. */
    for (int v = 0; v < nv; v++) {
        int t = m->vb[3 * v + 1]; m->vb[3 * v + 1] = m->vb[3 * v]; m->vb[3 * v] = t;
    }
    for (int g = 0; g < ng; g++) m->gori[g] = (g < n_ori ? oris[g] : 0.0) * 2 * M_PI; /* :214-218 */
    for (int g = 0; g < ng; g++) m->gse[g] = g < n_se ? se[g] : 0.0;                   /* :223 */
    if (opt->SE_min == 999 && opt->SE_max == 999) {                                    /* :228-248 */
        for (int g = 0; g < ng; g++) m->gse[g] *= opt->SE_eps;
    } else if (opt->SE_min == opt->SE_max) {
        for (int g = 0; g < ng; g++) m->gse[g] = opt->SE_max * opt->SE_eps;
    } else {
        double slope = (opt->SE_max - opt->SE_min), shift = opt->SE_min;
        for (int g = 0; g < ng; g++) m->gse[g] = slope * m->gse[g] + shift;
    }
    return SEVC_OK;
bad:
    sevc_hmesh_free(out);
    return SEVC_ERR_PARSE;
}

static int slurp_numbers(const char *path, int per_line, int as_int, void **out, int *count)
{
    FILE *f = fopen(path, "r");
    if (!f) { sevc_set_error("cannot open %s", path); return SEVC_ERR_IO; }
    size_t cap = 4096, n = 0, w = as_int ? sizeof(int) : sizeof(double);
    char *buf = (char *)malloc(cap * w);
    for (;;) {
        int r;
        if (as_int) {
            int a, b;
            r = fscanf(f, "%d %d\n", &a, &b);
            if (r == EOF) break;
            if (r != 2) goto parse_err;
            if (n + 2 > cap) { cap *= 2; buf = (char *)realloc(buf, cap * w); }
            ((int *)buf)[n++] = a;
            ((int *)buf)[n++] = b;
        } else if (per_line == 2) {
            double a, b;
            r = fscanf(f, "%lf %lf\n", &a, &b);
            if (r == EOF) break;
            if (r != 2) goto parse_err;
            if (n + 2 > cap) { cap *= 2; buf = (char *)realloc(buf, cap * w); }
            ((double *)buf)[n++] = a;
            ((double *)buf)[n++] = b;
        } else {
            double a;
            r = fscanf(f, "%lf\n", &a);
            if (r == EOF) break;
            if (r != 1) goto parse_err;
            if (n + 1 > cap) { cap *= 2; buf = (char *)realloc(buf, cap * w); }
            ((double *)buf)[n++] = a;
        }
    }
    fclose(f);
    *out = buf;
    *count = (int)(n / (size_t)per_line);
    return SEVC_OK;
parse_err:
    fclose(f);
    free(buf);
    sevc_set_error("malformed line in %s", path);
    return SEVC_ERR_PARSE;
}

int sevc_host_load_files(const sevc_options *opt, sevc_hmesh *out)
{
    void *xy = NULL, *rd = NULL, *ori = NULL, *se = NULL;
    int nv, nb, no, ns, rc;
    if ((rc = slurp_numbers(opt->vertex_fname, 2, 0, &xy, &nv))) goto done;
    if ((rc = slurp_numbers(opt->boundary_fname, 2, 1, &rd, &nb))) goto done;
    if ((rc = slurp_numbers(opt->orientation_fname, 1, 0, &ori, &no))) goto done;
    if ((rc = slurp_numbers(opt->SE_fname, 1, 0, &se, &ns))) goto done;
    rc = sevc_host_build(opt, nv, (double *)xy, nb, (int *)rd, no, (double *)ori, ns, (double *)se, out);
done:
    free(xy); free(rd); free(ori); free(se);
    return rc;
}

sevc_status sevc_load_mesh_host(const sevc_options *opt, sevc_mesh_host *out, int *nv, int *nb, int *ng)
{
    if (!opt) return SEVC_ERR_ARG;
    sevc_hmesh hm;
    int rc = sevc_host_load_files(opt, &hm);
    if (rc) return (sevc_status)rc;
    if (nv) *nv = hm.m.nv;
    if (nb) *nb = hm.m.nb;
    if (ng) *ng = hm.m.ng;
    if (out) {
        if (out->nv != hm.m.nv || out->nb != hm.m.nb || out->ng != hm.m.ng) {
            sevc_hmesh_free(&hm);
            sevc_set_error("output sizes do not match the mesh");
            return SEVC_ERR_ARG;
        }
        size_t V = (size_t)hm.m.nv, B = (size_t)hm.m.nb, G = (size_t)hm.m.ng;
#define CP(f, n) memcpy(out->f, hm.m.f, (n) * sizeof(*hm.m.f))
        CP(px, V); CP(py, V); CP(vx, V); CP(vy, V); CP(venergy, V); CP(vel_bnd_x, V); CP(vel_grn_x, V);
        CP(vel_bnd_y, V); CP(vel_grn_y, V); CP(ven, V); CP(vb, 3 * V); CP(vg, 3 * V); CP(bini, B); CP(bend, B);
        CP(benergy, B); CP(blen, B); CP(btext, B); CP(ben, B); CP(bcand, B); CP(glist, SEVC_MAX_VRT_PER_GRN * G);
        CP(gvlen, G); CP(garea, G); CP(gdadt, G); CP(gori, G); CP(gse, G); CP(gen, G); CP(gtype, G);
#undef CP
    }
    sevc_hmesh_free(&hm);
    return SEVC_OK;
}

/* ---------------------------------------------------------------- */
/* exact "%.16f" and "%d" into a buffer                               */
/* ---------------------------------------------------------------- */
/* A finite double is m * 2^e with m < 2^53.  Its value times 10^16 is
 * m * 10^16 * 2^e, and m * 10^16 < 2^107 fits an unsigned 128-bit integer,
 * so the correctly rounded N = round(x * 10^16) (ties to even, as printf
 * rounds in the default rounding mode) is an integer shift with an exact
 * remainder; the text is N / 10^16, '.', and the 16 digits of N mod 10^16.
 * Values of 2^73 or more, NaN and infinities go to snprintf. */
typedef unsigned __int128 u128;

static char *put_u128(char *p, u128 v)
{
    char tmp[48];
    int n = 0;
    do {
        tmp[n++] = (char)('0' + (int)(v % 10));
        v /= 10;
    } while (v);
    while (n) *p++ = tmp[--n];
    return p;
}

static char *put_f16(char *p, double x)
{
    if (!isfinite(x) || fabs(x) >= 9.4e21) return p + sprintf(p, "%.16f", x);
    if (signbit(x)) { *p++ = '-'; x = -x; }
    u128 N = 0;
    if (x != 0) {
        int k;
        double f = frexp(x, &k);                     /* x = f * 2^k, f in [0.5, 1) */
        uint64_t mant = (uint64_t)ldexp(f, 53);      /* exact: 53 significant bits */
        int e = k - 53;
        u128 P = (u128)mant * (u128)10000000000000000ULL;
        if (e >= 0) {
            N = P << e;                              /* e <= 20 here: no overflow */
        } else {
            int s = -e;
            if (s >= 108) {
                N = 0;                               /* P < 2^107 <= half: rounds to 0 */
            } else {
                u128 q = P >> s, r = P - (q << s), half = (u128)1 << (s - 1);
                if (r > half || (r == half && (q & 1))) q++;
                N = q;
            }
        }
    }
    const u128 TEN16 = (u128)10000000000000000ULL;
    p = put_u128(p, N / TEN16);
    uint64_t frac = (uint64_t)(N % TEN16);
    *p++ = '.';
    for (int i = 15; i >= 0; i--) {
        p[i] = (char)('0' + (int)(frac % 10));
        frac /= 10;
    }
    return p + 16;
}

static char *put_int(char *p, int v)
{
    unsigned int u = (unsigned int)v;
    if (v < 0) { *p++ = '-'; u = 0u - u; }
    char tmp[12];
    int n = 0;
    do {
        tmp[n++] = (char)('0' + u % 10);
        u /= 10;
    } while (u);
    while (n) *p++ = tmp[--n];
    return p;
}

int sevc_format_fixed16(double x, char *out)
{
    char *e = put_f16(out, x);
    *e = 0;
    return (int)(e - out);
}

/* ---------------------------------------------------------------- */
/* snapshot text, src/io.h:280-377                                   */
/* ---------------------------------------------------------------- */
/* lines are formatted with the exact formatter above into per-thread
 * blocks and written in large writes */

/* One line of each section.  A binary64 in %.16f takes at most 327
 * characters (309 integer digits, sign, point, 16 decimals), an int 11. */
#define F16_MAX 330
#define VLINE_MAX (9 * (F16_MAX + 1) + 8 * 12 + 2)
#define BLINE_MAX (3 * (F16_MAX + 1) + 5 * 12 + 2)
#define GLINE_MAX (4 * (F16_MAX + 1) + (4 + SEVC_MAX_VRT_PER_GRN) * 12 + 2)
static char *line_vertex(const sevc_mesh_host *m, int i, char *p)
{
    const int *s = &m->vb[3 * i];
    int nbr[3];
    for (int j = 0; j < 3; j++)
        nbr[j] = s[j] < 0 ? -1 : (m->bini[s[j]] == i ? m->bend[s[j]] : m->bini[s[j]]);
    p = put_int(p, i); *p++ = ' ';
    p = put_int(p, m->ven[i] ? 1 : 0);
    const double vals[9] = { m->venergy[i], m->px[i], m->py[i], m->vx[i], m->vy[i], m->vel_bnd_x[i],
                             m->vel_grn_x[i], m->vel_bnd_y[i], m->vel_grn_y[i] };
    for (int k = 0; k < 9; k++) { *p++ = ' '; p = put_f16(p, vals[k]); }
    const int ints[6] = { m->vg[3 * i], m->vg[3 * i + 1], m->vg[3 * i + 2], nbr[0], nbr[1], nbr[2] };
    for (int k = 0; k < 6; k++) { *p++ = ' '; p = put_int(p, ints[k]); }
    *p++ = '\n';
    return p;
}
static char *line_boundary(const sevc_mesh_host *m, int i, char *p)
{
    p = put_int(p, i); *p++ = ' ';
    p = put_int(p, m->ben[i] ? 1 : 0); *p++ = ' ';
    p = put_int(p, m->bini[i]); *p++ = ' ';
    p = put_int(p, m->bend[i]); *p++ = ' ';
    p = put_f16(p, m->benergy[i]); *p++ = ' ';
    p = put_f16(p, m->blen[i]); *p++ = ' ';
    p = put_f16(p, m->btext[i]); *p++ = ' ';
    p = put_int(p, m->bcand[i] ? 1 : 0);
    *p++ = '\n';
    return p;
}
static char *line_grain(const sevc_mesh_host *m, int i, char *p)
{
    int n = m->gvlen[i];
    p = put_int(p, i); *p++ = ' ';
    p = put_int(p, m->gen[i] ? 1 : 0); *p++ = ' ';
    p = put_int(p, (int)m->gtype[i]); *p++ = ' ';
    p = put_f16(p, m->gori[i]); *p++ = ' ';
    p = put_f16(p, m->gse[i]); *p++ = ' ';
    p = put_f16(p, m->garea[i]); *p++ = ' ';
    p = put_f16(p, m->gdadt[i]); *p++ = ' ';
    p = put_int(p, n); *p++ = ' ';
    const int *L = &m->glist[(size_t)SEVC_MAX_VRT_PER_GRN * i];
    for (int j = 0; j < SEVC_MAX_VRT_PER_GRN; j++) {
        if (j < n) { p = put_int(p, L[j]); *p++ = ' '; }
        else if (j == SEVC_MAX_VRT_PER_GRN - 1) { *p++ = '-'; *p++ = '1'; }
        else { *p++ = '-'; *p++ = '1'; *p++ = ' '; }
    }
    *p++ = '\n';
    return p;
}

/* A section's lines, formatted in chunks of SEC_LINES by the OpenMP
 * threads, a round of chunks at a time, and written in order: the file is
 * byte for byte the serial one. */
#define SEC_LINES 512
static int write_section(FILE *f, const sevc_mesh_host *m, int n, char *(*line)(const sevc_mesh_host *, int, char *),
                         size_t maxline)
{
    int nchunks = (n + SEC_LINES - 1) / SEC_LINES;
    if (nchunks == 0) return 0;
    int per_round = 64;
    size_t chunk_bytes = (size_t)SEC_LINES * maxline;
    char *pool = (char *)malloc((size_t)per_round * chunk_bytes);
    size_t lens[64];
    if (!pool) return -1;
    int err = 0;
    for (int c0 = 0; c0 < nchunks && !err; c0 += per_round) {
        int cn = nchunks - c0 < per_round ? nchunks - c0 : per_round;
#pragma omp parallel for schedule(dynamic, 1)
        for (int c = 0; c < cn; c++) {
            int lo = (c0 + c) * SEC_LINES, hi = lo + SEC_LINES < n ? lo + SEC_LINES : n;
            char *b = pool + (size_t)c * chunk_bytes, *p = b;
            for (int i = lo; i < hi; i++) p = line(m, i, p);
            lens[c] = (size_t)(p - b);
        }
        for (int c = 0; c < cn && !err; c++)
            if (fwrite(pool + (size_t)c * chunk_bytes, 1, lens[c], f) != lens[c]) err = 1;
    }
    free(pool);
    return err;
}

int sevc_host_export(const sevc_mesh_host *m, const sevc_options *o, const char *path, double time)
{
    FILE *f = fopen(path, "w");
    if (!f) { sevc_set_error("cannot write %s", path); return SEVC_ERR_IO; }
    int cv = 0, cb = 0, cg = 0;
    for (int i = 0; i < m->nv; i++) cv += m->ven[i] != 0;
    for (int i = 0; i < m->nb; i++) cb += m->ben[i] != 0;
    for (int i = 0; i < m->ng; i++) cg += m->gen[i] != 0;
    fprintf(f, "TIME %.16f\nDELTA T %.16f\nDELTA TAU %.16f\nMAX TIME %.16f\nNUCLEATION %d\n", time, o->dt, o->dtau,
            o->tmax, o->do_nucleation ? 1 : 0);
    fprintf(f, "DOMAIN BOUND %.16f\nGB EPSILON %.16f\nGB SCALING %.16f\nSE EPSILON %.16f\nSE MIN %.16f\n",
            o->domain_bound, o->GB_eps, o->GB_scaling, o->SE_eps, o->SE_min);
    fprintf(f, "SE MAX %.16f\nNUCLEATION SCALING %.16f\nMAX VERTICES PER GRN %d\n", o->SE_max,
            o->nucleation_scaling, SEVC_MAX_VRT_PER_GRN);
    fprintf(f, "VERTICES %d\nBOUNDARIES %d\nGRAINS %d\nCURR VERTICES %d\nCURR BOUNDARIES %d\nCURR GRAINS %d\n",
            m->nv, m->nb, m->ng, cv, cb, cg);
    int err = fputs("#VERTEX ENABLED ENERGY X Y VX VY VXbnd VXgrn VYbnd VYgrn VG1 G2 G3 N1 N2 N3\n", f) < 0;
    if (!err) err = write_section(f, m, m->nv, line_vertex, VLINE_MAX) != 0;
    if (!err) err = fputs("#BOUNDARY ENABLED INI END ENERGY ARCLEN EXTTIME CANDIDATE\n", f) < 0;
    if (!err) err = write_section(f, m, m->nb, line_boundary, BLINE_MAX) != 0;
    if (!err) err = fputs("#GRAIN ID ENABLED NUCLEATED ORIENT SE AREA dAdt VLEN VERTICES\n", f) < 0;
    if (!err) err = write_section(f, m, m->ng, line_grain, GLINE_MAX) != 0;
    if (fclose(f) || err) { sevc_set_error("write error on %s", path); return SEVC_ERR_IO; }
    return SEVC_OK;
}

sevc_status sevc_write_snapshot(const sevc_mesh_host *mesh, const sevc_options *opt, const char *path, double time)
{
    if (!mesh || !opt || !path) return SEVC_ERR_ARG;
    return (sevc_status)sevc_host_export(mesh, opt, path, time);
}

/* ---------------------------------------------------------------- */
/* invariants, src/utils.h:85-336 (the is_valid = false checks)      */
/* ---------------------------------------------------------------- */
static int two_common(const sevc_mesh_host *m, int a, int b, int *g0, int *g1)
{
    int k = 0, out[2] = { -1, -1 };
    for (int i = 0; i < 3 && k < 2; i++)
        for (int j = 0; j < 3 && k < 2; j++)
            if (m->vg[3 * a + i] == m->vg[3 * b + j]) out[k++] = m->vg[3 * a + i];
    *g0 = out[0];
    *g1 = out[1];
    return k;
}

static int in_list(const sevc_mesh_host *m, int g, int v)
{
    const int *L = &m->glist[(size_t)SEVC_MAX_VRT_PER_GRN * g];
    int n = m->gvlen[g];
    if (n > SEVC_MAX_VRT_PER_GRN) n = SEVC_MAX_VRT_PER_GRN;
    for (int i = 0; i < n; i++)
        if (L[i] == v) return 1;
    return 0;
}

/* An index outside its array counts as one violation and is not followed
 * (the reference would read out of bounds there); the device checker
 * (sevc_check.cu) counts the same way. */
static int inr(int x, int n) { return x >= 0 && x < n; }

int sevc_host_check(const sevc_mesh_host *m)
{
    int bad = 0;
    for (int b = 0; b < m->nb; b++) {
        if (!m->ben[b]) continue;
        int a = m->bini[b], c = m->bend[b];
        if (!inr(a, m->nv) || !inr(c, m->nv)) { bad++; continue; }
        const int *sa = &m->vb[3 * a], *sc = &m->vb[3 * c];
        bad += a == c;
        bad += !m->ven[a] || !m->ven[c];
        bad += sa[0] != b && sa[1] != b && sa[2] != b;
        bad += sc[0] != b && sc[1] != b && sc[2] != b;
        int ok_c = 1, ok_a = 1;
        for (int j = 0; j < 3; j++) {
            ok_c &= inr(sc[j], m->nb) && m->ben[sc[j]];
            ok_a &= inr(sa[j], m->nb) && m->ben[sa[j]];
        }
        bad += !ok_c;
        bad += !ok_a;
        int g0, g1;
        bad += two_common(m, a, c, &g0, &g1) < 2 || g0 == g1;
    }
    for (int v = 0; v < m->nv; v++) {
        if (!m->ven[v]) continue;
        const int *s = &m->vb[3 * v], *g = &m->vg[3 * v];
        bad += s[0] == s[1] || s[1] == s[2] || s[2] == s[0];
        bad += g[0] == g[1] || g[1] == g[2] || g[2] == g[0];
        int nb[3] = { -1, -2, -3 };
        for (int j = 0; j < 3; j++) {
            int gok = inr(g[j], m->ng);
            bad += !gok || !m->gen[g[j]];
            bad += !gok || !in_list(m, g[j], v);
            if (!inr(s[j], m->nb)) { bad++; continue; }
            bad += !m->ben[s[j]];
            bad += m->bini[s[j]] == m->bend[s[j]];
            nb[j] = m->bini[s[j]] == v ? m->bend[s[j]] : m->bini[s[j]];
            bad += m->bini[s[j]] != v && m->bend[s[j]] != v;
        }
        bad += nb[0] == nb[1] || nb[1] == nb[2] || nb[2] == nb[0];
    }
    for (int gi = 0; gi < m->ng; gi++) {
        if (!m->gen[gi]) continue;
        const int *L = &m->glist[(size_t)SEVC_MAX_VRT_PER_GRN * gi];
        int n = m->gvlen[gi];
        if (n < 0 || n > SEVC_MAX_VRT_PER_GRN) { bad++; continue; }
        int listed = 1;
        for (int j = 0; j < n; j++) {
            if (!inr(L[j], m->nv)) { bad++; listed = 0; continue; }
            bad += !m->ven[L[j]];
        }
        for (int j = 0; j < n && listed; j++) {
            const int *g = &m->vg[3 * L[j]];
            if (g[0] != gi && g[1] != gi && g[2] != gi) { bad++; break; }
        }
        int cnt = 0;
        for (int j = 0; j < SEVC_MAX_VRT_PER_GRN; j++) cnt += L[j] != -1;
        bad += cnt != n;
    }
    return bad;
}
