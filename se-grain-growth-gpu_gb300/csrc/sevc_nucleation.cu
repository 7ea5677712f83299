/*
 * Monte-Carlo nucleation (src/nucleation2.cu of the reference) with an
 * exact replay of its random stream.
 *
 * The reference keeps 8192 cuRAND XORWOW states seeded with
 * curand_init(32, tid, 0) (:12-16) and lets thread tid of its 32x256 grid
 * consume, per attempt: 2 uniforms for every enabled vertex of its stride
 * set (compute_nucleation_factor :262-263), 1 uniform if that set has an
 * enabled vertex and, for thread 0 of each block, 1 more
 * (get_vertex_id_per_block :315, :342), then state 0 draws 1 or 2 in
 * get_vertex_id2 (:392, :421).
 *
 * Here the same states are kept and advanced by the same calls, but the
 * triangle construction (two per vertex in the reference) is done only for
 * the one vertex the selection picks: the vertex choice depends only on
 * the enabled flags and the draws, never on the per-vertex energies.  The
 * chosen vertex's two uniforms are regenerated from a copy of its stream
 * taken before the attempt.
 */
#include "sevc_internal.h"
#include "sevc_host.h"

#include <cmath>
#include <mutex>
#include <vector>

namespace {

constexpr int NBLK = 32, NTHR = 256, GRID = NBLK * NTHR;
constexpr int NUCL_BUF = 3 * NBLK;   /* per instance: each block's pick, alive count, pick's rank */

__global__ void k_rng_init(curandState *st, int n)
{
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid < n) curand_init(32, tid, 0, &st[tid]);
}

__global__ void k_rng_draw(curandState *st, int n, int ndraws, double *out)
{
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= n) return;
    curandState s = st[tid];
    for (int k = 0; k < ndraws; k++) out[(size_t)tid * ndraws + k] = curand_uniform_double(&s);
    st[tid] = s;
}

/* compute_nucleation_factor's draws + get_vertex_id_per_block
 * (src/nucleation2.cu:239-363), on the reference's 32x256 grid; blockIdx.y
 * is the instance, whose own 8192 streams walk its own vertex indices */
__global__ void __launch_bounds__(NTHR) k_nucl_blocks(DevMesh m, curandState *rng, curandState *saved, int *buf,
                                                     const int *nucl_on)
{
    __shared__ int alive[NTHR], pick[NTHR], nst[NTHR], stot;
    __shared__ double share[NTHR];
    int inst = blockIdx.y;
    if (!nucl_on[inst]) return;
    int vo = m.voff[inst], nvi = m.voff[inst + 1] - vo;
    rng += (size_t)inst * GRID;
    saved += (size_t)inst * GRID;
    buf += NUCL_BUF * inst;
    if (threadIdx.x == 0) stot = 0;
    int tid = blockIdx.x * NTHR + threadIdx.x;
    curandState s = rng[tid];
    saved[tid] = s;
    int n_alive = 0;
    for (int v = tid; v < nvi; v += GRID) n_alive += m.ven[vo + v] ? 1 : 0;
    for (int k = 0; k < 2 * n_alive; k++) (void)curand_uniform_double(&s);
    alive[threadIdx.x] = n_alive;
    int rid = -1, rid_k = -1;   /* the pick and its rank among the stream's enabled vertices */
    if (n_alive > 0) {
        int n_steps = (int)(curand_uniform_double(&s) * (n_alive - 1));
        int k = 0;
        for (int v = tid; v < nvi; v += GRID)
            if (m.ven[vo + v]) {
                if (k == n_steps) { rid = vo + v; rid_k = k; break; }
                k++;
            }
    }
    pick[threadIdx.x] = rid;
    nst[threadIdx.x] = rid_k;
    __syncthreads();
    atomicAdd(&stot, n_alive);                   /* integers: the same sum in any order */
    __syncthreads();
    const int tot = stot;
    /* each thread's share alive[i] / tot, the quotient the selection below
     * compares against (computed once per thread instead of one after
     * another by thread 0) */
    share[threadIdx.x] = tot > 0 ? alive[threadIdx.x] / (double)tot : 0.0;
    __syncthreads();
    if (threadIdx.x == 0) {
        if (tot > 0) {
            double p = curand_uniform_double(&s);
            double pc = 0.0;
            int kk = nst[0];
            for (int i = 0; i < NTHR; i++) {
                if (pick[i] != -1 && pc <= p && p < (pc + share[i])) {
                    pick[0] = pick[i];
                    kk = nst[i];
                    break;
                }
                pc += share[i];
            }
            buf[blockIdx.x] = pick[0];
            buf[NBLK + blockIdx.x] = tot;
            buf[2 * NBLK + blockIdx.x] = kk;
        } else {
            buf[blockIdx.x] = -1;
            buf[NBLK + blockIdx.x] = 0;
            buf[2 * NBLK + blockIdx.x] = -1;
        }
    }
    rng[tid] = s;
}

struct NuclGeo {
    double2 Apos, Bpos, Cpos;
    int D, E, F, AD, AE, AF, g1, g2, g3;
    double DeltaE;
};

/* 3-point compute_area (src/geometry.h:757) */
__device__ double area3(double2 a, double2 b, double2 c, double D)
{
    double x1 = 0 + wrapd(b.x, a.x, D), y1 = 0 + wrapd(b.y, a.y, D);
    double x2 = x1 + wrapd(c.x, b.x, D), y2 = y1 + wrapd(c.y, b.y, D);
    double x0 = 0, y0 = 0;
    double area = 0;
    area += x0 * y1 - y0 * x1;
    area += x1 * y2 - y1 * x2;
    area += x2 * y0 - y2 * x0;
    area *= 0.5;
    return area;
}

/* generate_grain_for_nucleation, src/nucleation2.cu:116-212 */
__device__ int gen_triangle(const DevMesh &m, int A, double nucl_r, double nucl_ori, double eps, double scaling,
                            bool do_scale, const double *gam3, NuclGeo &o)
{
    double D = m.D;
    int4 sa = m.vb[A];
    o.AD = sa.x; o.AE = sa.y; o.AF = sa.z;
    o.D = other_end(m.bv[o.AD], A);
    o.E = other_end(m.bv[o.AE], A);
    o.F = other_end(m.bv[o.AF], A);
    int gAD[2], gAE[2], gAF[2];
    int4 ga = m.vg[A];
    gintersect(ga, m.vg[o.D], gAD);
    gintersect(ga, m.vg[o.E], gAE);
    gintersect(ga, m.vg[o.F], gAF);
    if (gAD[0] == gAE[0] || gAD[0] == gAE[1]) { o.g2 = gAD[0]; o.g1 = gAD[1]; }
    else if (gAD[1] == gAE[0] || gAD[1] == gAE[1]) { o.g2 = gAD[1]; o.g1 = gAD[0]; }
    else return -1;
    if (gAE[0] == o.g2) o.g3 = gAE[1];
    else if (gAE[1] == o.g2) o.g3 = gAE[0];
    else return -1;
    if (o.g1 < 0 || o.g2 < 0 || o.g3 < 0) return -1;
    double2 pa = m.pos[A];
    int far[3] = { o.D, o.E, o.F };
    double2 out[3];
    for (int k = 0; k < 3; k++) {
        double2 q = m.pos[far[k]];
        double tx = wrapd(q.x, pa.x, D), ty = wrapd(q.y, pa.y, D);
        double w = nucl_r / vmag(tx, ty);
        if (do_scale) w *= 0.99;
        double2 r = make_double2(w * tx + pa.x, w * ty + pa.y);
        r.x = dmod(r.x, D);
        r.y = dmod(r.y, D);
        out[k] = r;
    }
    o.Apos = out[0]; o.Bpos = out[1]; o.Cpos = out[2];
    double LAB = arclen(o.Apos, o.Bpos, D), LBC = arclen(o.Bpos, o.Cpos, D), LCA = arclen(o.Cpos, o.Apos, D);
    double A1 = area3(pa, o.Cpos, o.Apos, D);
    double A2 = area3(pa, o.Apos, o.Bpos, D);
    double A3 = area3(pa, o.Bpos, o.Cpos, D);
    double E0 = 0.0, E1 = 0.0;
    for (int i = 0; i < 3; i++) {
        double gam = gam3[i];   /* the energy of A's i-th boundary this step */
        if (do_scale) E0 += 0.99 * nucl_r * gam;
        else E0 += nucl_r * gam;
    }
    E0 += A1 * m.gse[o.g1] + A2 * m.gse[o.g2] + A3 * m.gse[o.g3];
    E1 = gb_energy(nucl_ori - m.gori[o.g1], eps) * scaling * LCA;
    E1 += gb_energy(nucl_ori - m.gori[o.g2], eps) * scaling * LAB;
    E1 += gb_energy(nucl_ori - m.gori[o.g3], eps) * scaling * LBC;
    o.DeltaE = E1 - E0;
    return 0;
}

__device__ void add_bnd_slot(const DevMesh &m, int v, int b)   /* vertex_add_boundary :385 */
{
    int4 s = m.vb[v];
    if (s.x < 0) s.x = b; else if (s.y < 0) s.y = b; else if (s.z < 0) s.z = b;
    m.vb[v] = s;
}
__device__ void add_grn_slot(const DevMesh &m, int v, int g)   /* vertex_add_grain :406 */
{
    int4 s = m.vg[v];
    if (s.x < 0) s.x = g; else if (s.y < 0) s.y = g; else if (s.z < 0) s.z = g;
    m.vg[v] = s;
}
__device__ bool list_add_after(const DevMesh &m, int g, int v, int prev) /* grain_add_vertex :629 */
{
    int *L = m.glist + (size_t)SEVC_MAXV * g;
    int n = m.gvlen[g], pos = -1;
    for (int i = 0; i < n; i++)
        if (L[i] == prev) { pos = i + 1; break; }
    if (pos < 0 || n >= SEVC_MAXV) return false;
    for (int i = n; i > pos; i--) L[i] = L[i - 1];
    L[pos] = v;
    m.gvlen[g] = n + 1;
    return true;
}
__device__ void list_remove(const DevMesh &m, int g, int v)   /* grain_remove_vertex :653 */
{
    int *L = m.glist + (size_t)SEVC_MAXV * g;
    int n = m.gvlen[g];
    for (int i = 0; i < n; i++)
        if (L[i] == v) {
            for (int j = i; j < n - 1; j++) L[j] = L[j + 1];
            m.gvlen[g] = n - 1;
            L[n - 1] = -1;
            return;
        }
}
__device__ void init_vertex_dev(const DevMesh &m, int v, double2 p) /* init_vertex :346 */
{
    m.pos[v] = p;
    m.vel[v] = make_double2(0.0, 0.0);
    m.venergy[v] = 0.0;
    m.ven[v] = 1;
    m.vg[v] = make_int4(-1, -1, -1, -1);
    m.vb[v] = make_int4(-1, -1, -1, -1);
    m.voted[v] = -1;
    for (int j = 0; j < 4; j++) m.vmod[4 * (size_t)v + j] = make_int4(-1, -1, -1, FIX_NONE);
}
__device__ void init_boundary_dev(const DevMesh &m, int b, int ini, int end) /* init_boundary :491 */
{
    m.bv[b] = make_int2(ini, end);
    add_bnd_slot(m, ini, b);
    add_bnd_slot(m, end, b);
    m.blen[b] = 0;
    m.btext[b] = SEVC_MAX_T_EXT_D;
    m.ben[b] = 1;
    m.bcand[b] = 0;
    m.bvotes[b] = 0;
    m.bconf[b] = -1;
}

/* get_vertex_id2 (:375-443), the chosen vertex's factor
 * (compute_nucleation_factor for that vertex), get_nucleation_ids (:33-72)
 * and nucleate (:474-676); one thread per instance */
__global__ void k_nucl_finish(DevMesh m, curandState *rng, const curandState *saved, const int *buf, int *ctr,
                              const int *nucl_on, double eps, double scaling, double MC_k)
{
    int inst = blockIdx.x * blockDim.x + threadIdx.x;
    if (inst >= m.ninst || !nucl_on[inst]) return;
    int vo = m.voff[inst], v_end = m.voff[inst + 1];
    int bo = m.boff[inst], b_end = m.boff[inst + 1];
    int go = m.goff[inst], g_end = m.goff[inst + 1];
    rng += (size_t)inst * GRID;
    saved += (size_t)inst * GRID;
    buf += NUCL_BUF * inst;
    ctr += (size_t)inst * CTR_COUNT;
    int *nlist = m.nlist + go, *nnlist = m.nnlist + inst;
    int tot = 0;
    for (int i = 0; i < NBLK; i++) tot += buf[NBLK + i];
    curandState s0 = rng[0];
    double p = curand_uniform_double(&s0);
    double pc = 0.0, pn = 0.0;
    int cand = ctr[CTR_CANDIDATE], kpick = -1;
    for (int i = 0; i < NBLK; i++) {
        pn = ((double)buf[NBLK + i]) / tot;
        if (buf[i] != -1 && pc < p && p <= (pc + pn)) { cand = buf[i]; kpick = buf[2 * NBLK + i]; break; }
        pc += pn;
    }
    int v = cand;
    if (v < vo || v >= v_end || !m.ven[v]) {
        /* the reference would read a stale or out-of-range vertex here */
        raise_err(m, ERRB_RNG);
        ctr[CTR_CANDIDATE] = -1;
        rng[0] = s0;
        return;
    }
    /* the two draws compute_nucleation_factor made for v: v is the k-th
     * enabled vertex of stream ((v - vo) mod 8192); k_nucl_blocks recorded
     * that rank with its pick (a candidate kept from an earlier attempt is
     * counted here) */
    int t = (v - vo) % GRID, k = kpick;
    if (k < 0) {
        k = 0;
        for (int u = vo + t; u < v; u += GRID) k += m.ven[u] ? 1 : 0;
    }
    curandState s = saved[t];
    for (int j = 0; j < 2 * k; j++) (void)curand_uniform_double(&s);
    double u1 = curand_uniform_double(&s);
    double u2 = curand_uniform_double(&s);
    /* the arclengths and energies of v's boundaries this step
     * (compute_boundaries_lengths / _energies, src/main.cu:124-130, run on
     * every boundary before the attempt in the reference; only v's three
     * are read, so they are computed here, with the same arithmetic as
     * the step's boundary pass that follows) */
    int4 sb = m.vb[v];
    double AL[3], gam3[3];
    for (int i = 0; i < 3; i++) {
        int b = slot3(sb, i);
        int2 e = m.bv[b];
        AL[i] = arclen(m.pos[e.x], m.pos[e.y], m.D);
        if (!boundary_gamma(m, b, eps, scaling, gam3[i])) {
            raise_err(m, ERRB_TOPOLOGY);
            ctr[CTR_CANDIDATE] = -1;
            rng[0] = s0;
            return;
        }
    }
    double mn = AL[0];
    int imin = 0;
    for (int i = 0; i < 3; i++) if (mn > AL[i]) { mn = AL[i]; imin = i; }   /* min(), src/geometry.h:116 */
    double nucl_r = 0.8 * mn * u1 + 0.1;
    double nucl_ori = 2 * M_PI * u2;
    NuclGeo o0, o1;
    if (gen_triangle(m, v, nucl_r, nucl_ori, eps, scaling, false, gam3, o0) ||
        gen_triangle(m, v, nucl_r, nucl_ori, eps, scaling, true, gam3, o1)) {
        raise_err(m, ERRB_TOPOLOGY);
        ctr[CTR_CANDIDATE] = -1;
        rng[0] = s0;
        return;
    }
    double DeltaE = o0.DeltaE, factor = o0.DeltaE - o1.DeltaE;
    bool nucl = false;
    if (DeltaE < 0) nucl = true;
    else if (factor < 0) {
        double q = curand_uniform_double(&s0);
        double thr = exp(-MC_k * DeltaE);
        if (q < thr) nucl = true; else cand = -1;
    } else cand = -1;
    ctr[CTR_CANDIDATE] = cand;
    rng[0] = s0;
    if (cand < 0 || !nucl) return;

    /* get_nucleation_ids: lowest free slots */
    int gfree = -1, bfree[3] = { -1, -1, -1 }, vfree[2] = { -1, -1 };
    for (int i = go; i < g_end; i++) if (!m.gen[i]) { gfree = i; break; }
    for (int i = bo, f = 0; i < b_end && f < 3; i++) if (!m.ben[i]) bfree[f++] = i;
    for (int i = vo, f = 0; i < v_end && f < 2; i++) if (!m.ven[i]) vfree[f++] = i;
    bool diff_vrt = vfree[0] != vfree[1];
    bool diff_bnd = bfree[0] != bfree[1] && bfree[1] != bfree[2] && bfree[2] != bfree[0];
    if (!diff_bnd || !diff_vrt || gfree == -1) return;      /* :496-499 */
    if (vfree[1] < 0 || bfree[2] < 0) { raise_err(m, ERRB_CAPACITY); return; }

    int A = v, B = vfree[0], C = vfree[1];
    int AB = bfree[0], BC = bfree[1], CA = bfree[2], g = gfree;
    /* the reference passes (scaling, eps) swapped here; only the unused
     * energy changes */
    NuclGeo o;
    if (gen_triangle(m, A, nucl_r, nucl_ori, scaling, eps, true, gam3, o)) { raise_err(m, ERRB_TOPOLOGY); return; }
    {   /* the triangle's position map, for an adjoint replay */
        EventRec r0, r1;
        r0.type = EV_NUCL; r0.a = A; r0.b = B; r0.c = C;
        r0.pa = m.pos[A]; r0.pb = m.pos[o.D]; r0.pc = m.pos[o.E];
        r1.type = EV_NUCL_AUX; r1.a = o.D; r1.b = o.E; r1.c = o.F;
        r1.pa = m.pos[o.F]; r1.pb = make_double2(0.8 * u1, nucl_r); r1.pc = make_double2(imin, 0.0);
        log_event_pair(m, r0, r1);
    }
    init_vertex_dev(m, B, o.Bpos);
    init_vertex_dev(m, C, o.Cpos);
    m.pos[A] = o.Apos;
    m.vb[A] = make_int4(-1, -1, -1, -1);
    init_boundary_dev(m, AB, A, B);
    init_boundary_dev(m, BC, B, C);
    init_boundary_dev(m, CA, C, A);
    add_bnd_slot(m, A, o.AD);
    if (m.gtype[g] != GT_NUCLEATED) {                      /* keep nlist ascending */
        int k = (*nnlist)++;
        while (k > 0 && nlist[k - 1] > g) { nlist[k] = nlist[k - 1]; k--; }
        nlist[k] = g;
    }
    int *L = m.glist + (size_t)SEVC_MAXV * g;              /* nucleate_grain :596 */
    for (int i = 0; i < SEVC_MAXV; i++) L[i] = -1;
    m.gvlen[g] = 0; m.garea[g] = 0; m.gse[g] = 0; m.gori[g] = 0;
    m.gen[g] = 1; m.gcand[g] = 0; m.gfix[g] = 0; m.gtype[g] = GT_NUCLEATED;
    m.gori[g] = nucl_ori;
    L[0] = A; L[1] = B; L[2] = C;
    m.gvlen[g] = 3;
    int4 ga = m.vg[A];
    if (ga.x == o.g3) ga.x = g; else if (ga.y == o.g3) ga.y = g; else if (ga.z == o.g3) ga.z = g;
    m.vg[A] = ga;
    add_grn_slot(m, B, g); add_grn_slot(m, B, o.g2); add_grn_slot(m, B, o.g3);
    add_grn_slot(m, C, g); add_grn_slot(m, C, o.g3); add_grn_slot(m, C, o.g1);
    bool ok = list_add_after(m, o.g1, C, A);
    int2 ae = m.bv[o.AE];
    if (ae.x == A) ok &= list_add_after(m, o.g2, B, ae.y);
    else if (ae.y == A) ok &= list_add_after(m, o.g2, B, ae.x);
    ok &= list_add_after(m, o.g3, C, A);
    ok &= list_add_after(m, o.g3, B, C);
    list_remove(m, o.g3, A);
    if (!ok) raise_err(m, ERRB_TOPOLOGY);
    int4 t4;
    t4 = m.vb[B]; { int x = t4.y; t4.y = t4.x; t4.x = x; } m.vb[B] = t4;  /* vertex_invert_boundary_order */
    t4 = m.vb[C]; { int x = t4.y; t4.y = t4.x; t4.x = x; } m.vb[C] = t4;
    ae = m.bv[o.AE];
    if (ae.x == A) ae.x = B; else if (ae.y == A) ae.y = B;
    m.bv[o.AE] = ae;
    t4 = m.vb[B]; t4.z = o.AE; m.vb[B] = t4;
    int2 af = m.bv[o.AF];
    if (af.x == A) af.x = C; else af.y = C;
    m.bv[o.AF] = af;
    t4 = m.vb[C]; t4.z = o.AF; m.vb[C] = t4;
    m.evt[EVT_COUNT * inst + EVT_NUCLEATIONS]++;
}

} // namespace

void launch_rng_init(curandState *st, int n, cudaStream_t s)
{
    COUNT_LAUNCHES(1), k_rng_init<<<(n + 255) / 256, 256, 0, s>>>(st, n);
}

void launch_nucleation(const DevMesh &m, const DevScratch &x, const StepParams &p, cudaStream_t s)
{
    COUNT_LAUNCHES(1), k_nucl_blocks<<<dim3(NBLK, p.ninst), NTHR, 0, s>>>(m, x.rng, x.rng_saved, x.nucl_buf, x.nucl_on);
    COUNT_LAUNCHES(1), k_nucl_finish<<<(p.ninst + 31) / 32, 32, 0, s>>>(m, x.rng, x.rng_saved, x.nucl_buf, x.counters,
                                                                      x.nucl_on, p.eps, p.scaling, p.MC_k);
}

int rng_record(int nstreams, int ndraws, double *host_out)
{
    curandState *st = nullptr;
    double *d = nullptr;
    size_t bytes = (size_t)nstreams * ndraws * sizeof(double);
    if (cudaMalloc(&st, sizeof(curandState) * nstreams) != cudaSuccess) return 1;
    if (cudaMalloc(&d, bytes) != cudaSuccess) { cudaFree(st); return 1; }
    COUNT_LAUNCHES(1), k_rng_init<<<(nstreams + 255) / 256, 256>>>(st, nstreams);
    COUNT_LAUNCHES(1), k_rng_draw<<<(nstreams + 255) / 256, 256>>>(st, nstreams, ndraws, d);
    cudaError_t e = cudaMemcpy(host_out, d, bytes, cudaMemcpyDeviceToHost);
    cudaFree(st);
    cudaFree(d);
    return e == cudaSuccess ? 0 : 1;
}

/* ------------------------------------------------------------------ */
/* Allocation-free recording of the random stream                      */
/* ------------------------------------------------------------------ */
/* Scratch of sevc_rng_record_noalloc: one cuRAND XORWOW state per stream,
 * 8192 x 48 bytes = 384 KiB, held by every GPU that loads the library
 * until the process exits.  8192 is the reference's whole 32 x 256 grid,
 * so every stream it uses fits. */
#define SEVC_NOALLOC_MAX_STREAMS 8192
static __device__ __align__(256) curandState g_noalloc_rng[SEVC_NOALLOC_MAX_STREAMS];

namespace {
std::mutex g_noalloc_mu;
constexpr int NOALLOC_MAX_DEVICES = 64;
curandState *g_noalloc_ptr[NOALLOC_MAX_DEVICES];   /* device address per device, set once */
} // namespace

extern "C" sevc_status sevc_rng_record_noalloc(int nstreams, int ndraws, double *d_out, void *stream)
{
    if (nstreams <= 0 || ndraws <= 0 || !d_out) {
        sevc_set_error("sevc_rng_record_noalloc: need nstreams > 0, ndraws > 0 and an output buffer");
        return SEVC_ERR_ARG;
    }
    if (nstreams > SEVC_NOALLOC_MAX_STREAMS) {
        sevc_set_error("sevc_rng_record_noalloc: nstreams %d exceeds the fixed scratch of %d streams", nstreams,
                       SEVC_NOALLOC_MAX_STREAMS);
        return SEVC_ERR_ARG;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) { sevc_set_error("no CUDA device"); return SEVC_ERR_CUDA; }
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) { sevc_set_error("device index %d out of range", dev); return SEVC_ERR_ARG; }
    curandState *scratch;
    {
        /* the array's host-side name is not a device address: resolve it
         * once per device, with that device current */
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!g_noalloc_ptr[dev]) {
            curandState *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress((void **)&p, g_noalloc_rng);
            if (e != cudaSuccess || !p) {
                sevc_set_error("cudaGetSymbolAddress: %s", cudaGetErrorString(e));
                return SEVC_ERR_CUDA;
            }
            g_noalloc_ptr[dev] = p;
        }
        scratch = g_noalloc_ptr[dev];
    }
    cudaStream_t s = (cudaStream_t)stream;
    /* every state is re-seeded by curand_init, so nothing left by an
     * earlier call survives into the draws */
    COUNT_LAUNCHES(1), k_rng_init<<<(nstreams + 255) / 256, 256, 0, s>>>(scratch, nstreams);
    COUNT_LAUNCHES(1), k_rng_draw<<<(nstreams + 255) / 256, 256, 0, s>>>(scratch, nstreams, ndraws, d_out);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { sevc_set_error("sevc_rng_record_noalloc: %s", cudaGetErrorString(e)); return SEVC_ERR_CUDA; }
    return SEVC_OK;
}
