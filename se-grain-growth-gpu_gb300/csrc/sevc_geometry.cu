/*
 * Geometry and kinetics kernels of one time step (src/calculus.h and
 * src/topological.h:303-353 of the reference), one thread per entity.
 *
 * The finite-difference velocity (src/calculus.h:19-73,143-154) is split
 * in two passes so that no thread re-reads another grain's polygon:
 *   grain pass   for every grain: its area, and for every list slot p the
 *                areas with that vertex moved by +eps in x and in y; the
 *                stored-energy terms SE*(|A'|-|A|) are scattered to the
 *                vertex's grain slot;
 *   vertex pass  for every vertex: the three perturbed arclengths, the
 *                boundary terms, the velocity, and the vertex energy.
 * Both passes repeat the reference's arithmetic in the same order, so the
 * results are the ones energy_diff computes.
 */
#include "sevc_internal.h"

#include <cmath>

namespace {

constexpr int TPB = 256;
inline int nblk(int n) { return (n + TPB - 1) / TPB; }

/* src/calculus.h:83-114 */
__global__ void k_boundary_geometry(DevMesh m, double eps, double scaling)
{
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= m.nb || !m.ben[b]) return;
    int2 e = m.bv[b];
    double2 a = m.pos[e.x], c = m.pos[e.y];
    m.blen[b] = arclen(a, c, m.D);
    double gamma;
    if (!boundary_gamma(m, b, eps, scaling, gamma)) { raise_err(m, ERRB_TOPOLOGY); return; }
    m.benergy[b] = gamma;
}

/* Store the stored-energy finite-difference terms of list vertex v
 * (SE * (|A'| - |A|), src/calculus.h:60) in v's slot for grain g. */
__device__ __forceinline__ void put_contrib(const DevMesh &m, int g, int v, double se, double absA, double Ax,
                                           double Ay)
{
    int4 sg = m.vg[v];
    int j = sg.x == g ? 0 : (sg.y == g ? 1 : (sg.z == g ? 2 : -1));
    if (j >= 0) m.contrib[3 * v + j] = make_double2(se * (dabs(Ax) - absA), se * (dabs(Ay) - absA));
}

/* Grain pass for a grain of N sides (compile-time), polygon in registers.
 *
 * compute_area of the polygon with vertex p moved (src/geometry.h:757,
 * :908) differs from the unmoved one only from vertex p on: the unwrapped
 * coordinates of vertices 0..p-1 and the partial shoelace sum of terms
 * 0..p-2 are the same operations on the same values, so they are taken
 * from the unmoved pass; the moved component's unwrapped chain and the
 * terms from p-1 on are recomputed in the reference's order.  The other
 * component is unchanged (its dom_mod is the identity; if it is not, the
 * slot falls back to a full recomputation). */
/* Area of the polygon with vertex p moved along component C (0 = x,
 * 1 = y).  R/A0/DD are the moved component's raw positions, unwrapped
 * coordinates and wrapped deltas, Ro/B0 the other component's. */
__device__ __noinline__ double area_stream_slow(const int *__restrict__ L, int n, const double2 *__restrict__ pos,
                                                int ps, double2 pp, double D)
{
    return area_stream(L, n, pos, ps, pp, D);
}

/* shoelace term k of the moved component C: P = its unwrapped
 * coordinates k and k+1, B = the other component's */
template <int C>
__device__ __forceinline__ double moved_term(double pk, double bk, double pk1, double bk1)
{
    return C == 0 ? pk * bk1 - bk * pk1 : bk * pk1 - pk * bk1;
}

/* Moving vertex p (0 < p < N-1) changes the unwrapped chain at p, then
 * at p+1 by the wrapped deltas into and out of the moved point.  When the
 * moved chain arrives at p+1 on the unmoved value (bit for bit: the two
 * deltas cancel exactly, which they do unless a wrap or a tiny coordinate
 * makes a difference inexact), every later coordinate is the same
 * operation on the same values as in the unmoved pass, so terms p+1.. are
 * the unmoved terms T[k] and only the running sum is redone.  Otherwise
 * the polygon is recomputed from memory. */
template <int N, int C>
__device__ __forceinline__ double moved_area_mid(const DevMesh &m, const int *__restrict__ L, int p, double moved,
                                                 double other, const double (&R)[N], const double (&A0)[N],
                                                 const double (&B0)[N], const double (&S)[N], const double (&T)[N])
{
    const double D = m.D;
    double pp = p == 1 ? zero_plus(wrapd(moved, R[0], D)) : A0[p - 1] + wrapd(moved, R[p - 1], D);
    double pn = pp + wrapd(R[p + 1], moved, D);
    if (dbits(pn) != dbits(A0[p + 1])) {
        double2 q = C == 0 ? make_double2(moved, other) : make_double2(other, moved);
        return area_stream_slow(L, N, m.pos, p, q, D);
    }
    /* terms p-1 and p (the products that involve only unmoved
     * coordinates are the unmoved pass's; the compiler shares them) */
    double a = 0;
    if (p >= 2) {
        double t = moved_term<C>(A0[p - 1], B0[p - 1], pp, B0[p]);
        a = p == 2 ? zero_plus(t) : S[p - 2] + t;
    }
    double t = moved_term<C>(pp, B0[p], A0[p + 1], B0[p + 1]);
    a = p == 1 ? zero_plus(t) : a + t;
#pragma unroll
    for (int k = 2; k < N - 1; k++)
        if (k > p) a = a + T[k];
    a = C == 0 ? add_closing_term(a, A0[N - 1], B0[N - 1]) : add_closing_term(a, B0[N - 1], A0[N - 1]);
    return dscale_down<1>(a);
}

template <int N, int C>
__device__ __forceinline__ double moved_area(const DevMesh &m, const int *__restrict__ L, int p, const double (&R)[N],
                                             const double (&Ro)[N], const double (&A0)[N], const double (&B0)[N],
                                             const double (&DD)[N], const double (&S)[N], const double (&T)[N])
{
    const double D = m.D;
    double moved = dmod(R[p] + SEVC_GRAD_EPS_D, D);
    double other = dmod(Ro[p], D);
    if (dbits(other) != dbits(Ro[p])) {
        double2 pp = C == 0 ? make_double2(moved, other) : make_double2(other, moved);
        return area_stream(L, N, m.pos, p, pp, D);
    }
    if (p > 0 && p < N - 1) return moved_area_mid<N, C>(m, L, p, moved, other, R, A0, B0, S, T);
    double Pm[N];
    Pm[0] = 0;
#pragma unroll
    for (int k = 1; k < N; k++) {
        if (k < p) Pm[k] = A0[k];
        else if (k == 1) Pm[k] = zero_plus(k == p ? wrapd(moved, R[0], D) : wrapd(R[1], moved, D));   /* +0 + w */
        else if (k == p) Pm[k] = A0[k - 1] + wrapd(moved, R[k - 1], D);
        else if (k == p + 1) Pm[k] = Pm[k - 1] + wrapd(R[k], moved, D);
        else Pm[k] = Pm[k - 1] + DD[k];
    }
    double a = (p >= 2) ? S[p - 2] : 0.0;  /* S[0] = +0: term 0 never changes the sum */
#pragma unroll
    for (int k = 1; k < N - 1; k++) {
        if (k < p - 1) continue;
        double term = C == 0 ? Pm[k] * B0[k + 1] - B0[k] * Pm[k + 1] : B0[k] * Pm[k + 1] - Pm[k] * B0[k + 1];
        a = (k == 1 && p <= 2) ? zero_plus(term) : a + term;   /* the sum is still +0 */
    }
    a = C == 0 ? add_closing_term(a, Pm[N - 1], B0[N - 1]) : add_closing_term(a, B0[N - 1], Pm[N - 1]);
    return dscale_down<1>(a);
}

template <int N>
__device__ __forceinline__ void grain_fd_fixed(const DevMesh &m, int g, const int *__restrict__ L)
{
    const double D = m.D;
    int V[N];
    double RX[N], RY[N], AX[N], AY[N], DX[N], DY[N], S[N], T[N];
#pragma unroll
    for (int k = 0; k < N; k++) {
        V[k] = L[k];
        double2 q = m.pos[V[k]];
        RX[k] = q.x;
        RY[k] = q.y;
    }
    AX[0] = 0; AY[0] = 0; DX[0] = 0; DY[0] = 0;
#pragma unroll
    for (int k = 1; k < N; k++) {
        DX[k] = wrapd(RX[k], RX[k - 1], D);
        DY[k] = wrapd(RY[k], RY[k - 1], D);
        AX[k] = k == 1 ? zero_plus(DX[k]) : AX[k - 1] + DX[k];   /* AX[0] = +0 */
        AY[k] = k == 1 ? zero_plus(DY[k]) : AY[k - 1] + DY[k];
    }
    double acc = 0;                    /* terms 0 and N-1 involve the origin */
    S[0] = 0;
    T[0] = 0;
#pragma unroll
    for (int k = 1; k < N - 1; k++) {
        double term = AX[k] * AY[k + 1] - AY[k] * AX[k + 1];
        T[k] = term;
        acc = k == 1 ? zero_plus(term) : acc + term;
        S[k] = acc;
    }
    T[N - 1] = 0;
    acc = add_closing_term(acc, AX[N - 1], AY[N - 1]);
    S[N - 1] = acc;
    double A = dscale_down<1>(acc);
    m.garea[g] = A;
    double se = m.gse[g];
    m.gq[g] = div_small<N>(se * A);
    double absA = dabs(A);
#pragma unroll
    for (int p = 0; p < N; p++) {
        double ax = moved_area<N, 0>(m, L, p, RX, RY, AX, AY, DX, S, T);
        double ay = moved_area<N, 1>(m, L, p, RY, RX, AY, AX, DY, S, T);
        put_contrib(m, g, V[p], se, absA, ax, ay);
    }
}

/* Grain pass, any side count: each polygon streamed from memory. */
__device__ __noinline__ void grain_fd_generic(const DevMesh &m, int g, const int *__restrict__ L, int n)
{
    double2 none = make_double2(0, 0);
    double A = area_stream(L, n, m.pos, -1, none, m.D);
    m.garea[g] = A;
    double se = m.gse[g];
    m.gq[g] = se * A / n;
    double absA = dabs(A);
    for (int p = 0; p < n; p++) {
        int v = L[p];
        double2 q = m.pos[v];
        double2 px = make_double2(dmod(q.x + SEVC_GRAD_EPS_D, m.D), dmod(q.y, m.D));
        double2 py = make_double2(dmod(q.x, m.D), dmod(q.y + SEVC_GRAD_EPS_D, m.D));
        double Ax = area_stream(L, n, m.pos, p, px, m.D);
        double Ay = area_stream(L, n, m.pos, p, py, m.D);
        put_contrib(m, g, v, se, absA, Ax, Ay);
    }
}

/* grain pass over the grains of fewer than `wide` sides (11 by default), ordered by
 * side count (warps see one N), most sides first so that the longest
 * blocks start in the first wave.  The pass is FP64 bound and waits on
 * FP64 results: OCC resident blocks of 128 per SM (4: 128 registers, 5:
 * 96, 6: 80, 8: 64) trades registers (and spills) for warps to hide that
 * latency; the launch-shape autotuner picks it (6 on the 1M-grain mesh).
 * Capping registers at 128 measured 9% faster than the compiler's
 * 218-register choice. */
template <int OCC>
__global__ void __launch_bounds__(128, OCC) k_grain_fd_sorted(DevMesh m, const int *perm, const int *vbucket, int wide)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int total = vbucket[VB_START(wide)];
    if (i >= total) return;
    int g = perm[total - 1 - i];
    const int *L = m.glist + (size_t)SEVC_MAXV * g;
    int n = m.gvlen[g];
    switch (n) {
    case 3: grain_fd_fixed<3>(m, g, L); break;
    case 4: grain_fd_fixed<4>(m, g, L); break;
    case 5: grain_fd_fixed<5>(m, g, L); break;
    case 6: grain_fd_fixed<6>(m, g, L); break;
    case 7: grain_fd_fixed<7>(m, g, L); break;
    case 8: grain_fd_fixed<8>(m, g, L); break;
    case 9: grain_fd_fixed<9>(m, g, L); break;
    case 10: grain_fd_fixed<10>(m, g, L); break;
    default: grain_fd_generic(m, g, L, n); break;
    }
}

/* area_stream over a polygon staged in shared memory (raw positions P[k]
 * of vertex k), same operations in the same order. */
__device__ __forceinline__ double area_shared(const double2 *P, int n, int ps, double2 pp, double D)
{
    double area = 0;
    if (n > 0) {
        double2 r0 = (ps == 0) ? pp : P[0];
        double ax = 0, ay = 0, rx = r0.x, ry = r0.y;
        for (int k = 1; k < n; k++) {
            double2 r = (k == ps) ? pp : P[k];
            double nx = ax + wrapd(r.x, rx, D);
            double ny = ay + wrapd(r.y, ry, D);
            if (k > 1) area += ax * ny - ay * nx;
            ax = nx; ay = ny; rx = r.x; ry = r.y;
        }
        area = add_closing_term(area, ax, ay);
    }
    return dscale_down<1>(area);
}

/* grain pass over the grains of `wide` or more sides (the tail of the
 * side-count order): one warp per grain, polygon staged in shared memory.
 * The 2n+1 areas of a grain (vertex p moved along x: task 2p, along y:
 * task 2p+1, unmoved: task 2n) are spread over the lanes, so a grain of
 * up to 15 sides costs one polygon walk per lane.  A thread per grain
 * would walk 2n+1 polygons of n dependent loads each and hold up the
 * whole pass. */
constexpr int WIDE_WARPS = 4;
__global__ void __launch_bounds__(32 * WIDE_WARPS) k_grain_fd_wide(DevMesh m, const int *perm, const int *vbucket,
                                                                  const int *total, int wide)
{
    __shared__ double2 poly[WIDE_WARPS][SEVC_MAXV];
    __shared__ double area[WIDE_WARPS][2 * SEVC_MAXV + 1];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    double2 *P = poly[w];
    double *R = area[w];
    int first = vbucket[VB_START(wide)], end = *total;
    int nwarps = gridDim.x * WIDE_WARPS;
    const double D = m.D;
    for (int i = first + blockIdx.x * WIDE_WARPS + w; i < end; i += nwarps) {
        int g = perm[i];
        const int *L = m.glist + (size_t)SEVC_MAXV * g;
        int n = m.gvlen[g];
        __syncwarp();
        for (int k = lane; k < n; k += 32) P[k] = m.pos[L[k]];
        __syncwarp();
        for (int t = lane; t <= 2 * n; t += 32) {
            int p = t >> 1;
            double2 pp = make_double2(0, 0);
            if (t < 2 * n) {
                double2 q = P[p];
                pp = (t & 1) ? make_double2(dmod(q.x, D), dmod(q.y + SEVC_GRAD_EPS_D, D))
                             : make_double2(dmod(q.x + SEVC_GRAD_EPS_D, D), dmod(q.y, D));
            } else {
                p = -1;
            }
            R[t] = area_shared(P, n, p, pp, D);
        }
        __syncwarp();
        double A = R[2 * n];
        double se = m.gse[g];
        if (lane == 0) {
            m.garea[g] = A;
            m.gq[g] = se * A / n;
        }
        double absA = dabs(A);
        for (int p = lane; p < n; p += 32) put_contrib(m, g, L[p], se, absA, R[2 * p], R[2 * p + 1]);
    }
}

/* counting sort of the enabled grains by side count (16 buckets, the last
 * one for 15 or more sides) */
constexpr int NBUCKET = 16;
/* Side-count histogram of the enabled grains into cnt[0..15]; the last
 * block to finish turns it into cursor[16..31] (bucket starts, advanced by
 * the scatter), start[32..47] and count[48..63] (kept for later passes
 * over one bucket) and leaves cnt[0..15] zero for the next step. */
__global__ void k_vlen_hist(DevMesh m, int *cnt, int *cursor, int *total)
{
    __shared__ int h[NBUCKET];
    if (threadIdx.x < NBUCKET) h[threadIdx.x] = 0;
    __syncthreads();
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g < m.ng && m.gen[g]) atomicAdd(&h[min(m.gvlen[g], NBUCKET - 1)], 1);
    __syncthreads();
    if (threadIdx.x < NBUCKET && h[threadIdx.x]) atomicAdd(&cnt[threadIdx.x], h[threadIdx.x]);
    bool last = last_block(m.lastblk + 1);
    if (last && threadIdx.x == 0) {
        __threadfence();
        int acc = 0;
        for (int b = 0; b < NBUCKET; b++) {
            int c = __ldcg(cnt + b);
            cursor[b] = acc;
            cnt[2 * NBUCKET + b] = acc;
            cnt[3 * NBUCKET + b] = c;
            acc += c;
            cnt[b] = 0;
        }
        *total = acc;
    }
}

/* The step computes every output-only value (extinction times of all
 * boundaries, dA/dt of all grains) when it can export or is asked to
 * (flags[1], set by the host), or when it could end at the stop threshold
 * (a final export): every removal takes a 3-sided grain, and a pass of the
 * 2x3 loop can make at most two per pair; the bound is generous, as the
 * threshold is crossed once per run.  Else only what the step can observe
 * is computed.  flags[0] = the decision, taken on the device so that no
 * host round trip separates the step's first half from its second. */
__global__ void k_full_flag(const int *n_two_three, const int *vbucket, int *flags, unsigned *stamp)
{
    int mg = flags[2], curr = flags[3], n3 = vbucket[3 * NBUCKET + 3];
    long long reach = (long long)curr - n3 - 40LL * *n_two_three - 64;
    flags[0] = flags[1] || (mg > 0 && reach <= mg);
    *stamp += 1;   /* a new step: every value saved by the last step's events is stale */
}
__global__ void k_vlen_scatter(DevMesh m, int *cursor, int *perm)
{
    __shared__ int h[NBUCKET], base[NBUCKET];
    if (threadIdx.x < NBUCKET) h[threadIdx.x] = 0;
    __syncthreads();
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    int b = -1, r = 0;
    if (g < m.ng && m.gen[g]) { b = min(m.gvlen[g], NBUCKET - 1); r = atomicAdd(&h[b], 1); }
    __syncthreads();
    if (threadIdx.x < NBUCKET) base[threadIdx.x] = h[threadIdx.x] ? atomicAdd(&cursor[threadIdx.x], h[threadIdx.x]) : 0;
    __syncthreads();
    if (b >= 0) perm[base[b] + r] = g;
}


/* vertex pass: src/calculus.h:19-73 (boundary part) and :143-154;
 * vertex_compute_energy src/geometry.h:472-479.
 *
 * UNIT_GAMMA: every boundary energy is exactly 1 this step (isotropic
 * boundaries, GB_scaling = 1: the geometry pass wrote 1 * 1 into every
 * enabled boundary), so the products gamma * x are x and are skipped.
 * Sums that the reference starts from 0.0 take their first term through
 * zero_plus, which keeps the first addition off the FP64 pipe. */
template <bool UNIT_GAMMA>
__global__ void k_vertex_fd(DevMesh m, double mu)
{
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= m.nv || !m.ven[v]) return;
    double2 p = m.pos[v];
    int4 sb = m.vb[v], sg = m.vg[v];
    double2 q[3];
    double gam[3], len[3];
    for (int j = 0; j < 3; j++) {
        int b = slot3(sb, j);
        q[j] = m.pos[other_end(m.bv[b], v)];
        gam[j] = m.benergy[b];
        len[j] = m.blen[b];
    }
    double2 cg[3];
    for (int j = 0; j < 3; j++) cg[j] = m.contrib[3 * v + j];
    DevMesh::FdTerms t;
    double vel[2];
#pragma unroll
    for (int c = 0; c < 2; c++) {
        double2 np = p;
        if (c == 0) np.x += SEVC_GRAD_EPS_D; else np.y += SEVC_GRAD_EPS_D;
        np.x = dmod(np.x, m.D);
        np.y = dmod(np.y, m.D);
        double bt = 0.0, gt = 0.0;
#pragma unroll
        for (int j = 0; j < 3; j++) {
            double Lj = arclen(np, q[j], m.D);
            double term = UNIT_GAMMA ? (Lj - len[j]) : (gam[j] * (Lj - len[j]));
            double gj = c == 0 ? cg[j].x : cg[j].y;
            if (j == 0) { bt = zero_plus(term); gt = zero_plus(gj); }
            else { bt += term; gt += gj; }
        }
        if (c == 0) { t.bx = bt; t.gx = gt; } else { t.by = bt; t.gy = gt; }
        vel[c] = div_grad_eps(-(bt + gt));
        if (mu != 1.0) vel[c] = mu * vel[c];   /* mobility; 1 * v is v exactly */
    }
    m.terms[v] = t;
    m.vel[v] = make_double2(vel[0], vel[1]);
    m.vspd[v] = speed_bound(vel[0], vel[1]);
    double e = 0.0;
#pragma unroll
    for (int j = 0; j < 3; j++) {
        int g = slot3(sg, j);
        double ej = dscale_down<1>(UNIT_GAMMA ? len[j] : (len[j] * gam[j]));
        e = j == 0 ? zero_plus(ej) : e + ej;
        e += g >= 0 ? m.gq[g] : 0.0;
    }
    m.venergy[v] = e;
}

/* compute_grain_dAdts, src/calculus.h:243 with compute_dAdt
 * src/geometry.h:779-787 streamed over the list */
__device__ void dadt_of(const DevMesh &m, int g);

/* every enabled grain when flags[0], else the 3-sided ones (bucket 3 of
 * the side-count order) */
__global__ void k_grain_dadt(DevMesh m, const int *perm, const int *vbucket, const int *flags)
{
    int stride = gridDim.x * blockDim.x;
    if (flags[0]) {
        for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.ng; g += stride)
            if (m.gen[g]) dadt_of(m, g);
    } else {
        int n3 = vbucket[3 * NBUCKET + 3], start = vbucket[2 * NBUCKET + 3];
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += stride) dadt_of(m, perm[start + i]);
    }
}

__device__ void dadt_of(const DevMesh &m, int g)
{
    m.gdadt[g] = dadt_from(m, g, m.pos, m.vel);
    m.gexact[g] = 1;
}

/* compute_t_ext (src/topological.h:303-334) then label_boundaries
 * (:343-353), which runs on every slot including disabled ones */
/*
 * When flags[0] is 0 a boundary that provably is not a candidate skips
 * the transcendental evaluation and gets a t_ext outside [0, dt], so the
 * labels (this kernel's and label_3sided's) see what they would see; the
 * value itself is not observed: exports happen only on steps that compute
 * every value, and a boundary an event disables gets its exact value then
 * (finalize_boundary).  The proof that a boundary is not a candidate is the
 * binary32 certificate text_outside_dt.
 */
__device__ __forceinline__ void text_label_one(const DevMesh &m, int b, uint8_t en, double2 pi, double2 pe,
                                               double2 vi, double2 ve, double dt, float Df, float hDf, float inv_dt,
                                               int full)
{
    long long tb;
    if (en) {
        if (!full && text_outside_dt(pi, pe, vi, ve, Df, hDf, inv_dt)) {
            /* not a candidate: its t_ext is outside [0, dt]; the value
             * itself is only observed if an event disables the boundary,
             * which then computes it (finalize_boundary) */
            m.btext[b] = SEVC_MAX_T_EXT_D;
            m.bexact[b] = 0;
            m.bcand[b] = 0;
            m.bconf[b] = -1;
            return;
        }
        double text = text_exact_call(pi, pe, vi, ve, m.D);
        m.btext[b] = text;
        m.bexact[b] = 1;
        tb = dbits(text);
    } else {
        tb = dbits(m.btext[b]);
    }
    /* text >= 0 && text <= dt on the bit pattern (dt > 0): +-0, or a
     * non-negative pattern not above dt's; NaN fails as in the comparison.
     * Written in PTX so that it stays two integer comparisons (as C the
     * compiler may turn it back into FP64 ones). */
    unsigned cand;
    asm("{\n\t.reg .pred p, q, z;\n\t"
        "setp.ge.s64 p, %1, 0;\n\t"
        "setp.le.s64 q, %1, %2;\n\t"
        "setp.eq.s64 z, %1, 0x8000000000000000;\n\t"
        "and.pred p, p, q;\n\t"
        "or.pred p, p, z;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(cand) : "l"(tb), "l"(dbits(dt)));
    m.bcand[b] = (uint8_t)cand;
    m.bconf[b] = -1;
}
/* Two boundaries per thread (b and b + blockDim.x of the block's pair of
 * tiles), every load of both issued before either is labelled: the pass
 * waits on rounds of gathers, and twice the loads in flight per thread
 * hide more of that latency than the registers they cost.
 *
 * Speed bound.  A candidate has 0 <= t_ext = -|d| / (u.(ve - vi)) <= dt
 * (u = d/|d| through atan2/cos/sin, |u| <= 1 + 1e-15), so
 * |d| <= dt (|vi|_1 + |ve|_1) (1 + 1e-14).  The vertex pass leaves an upper
 * bound of each |v|_1 in binary32 (speed_bound); a boundary whose
 * arclength this step (blen, the same |d| up to 1e-15) cut down to binary32
 * exceeds dt_up (s_i + s_e), dt_up >= dt (1 + 1e-6), rounded up, is no
 * candidate, and is labelled as the certificate labels one (without
 * reading its ends' positions and velocities).  The others take the
 * certificate and, if undecided, the exact value. */
__global__ void k_text_label(DevMesh m, double dt, float Df, float hDf, float inv_dt, float dt_up, const int *flags)
{
    griddep_wait();
    int b0 = 2 * blockIdx.x * blockDim.x + threadIdx.x;
    int full = flags[0];
    uint8_t en[2];
    int2 e[2];
#pragma unroll
    for (int k = 0; k < 2; k++) {
        int b = b0 + k * blockDim.x;
        bool in = b < m.nb;
        en[k] = in ? m.ben[b] : 0;
        e[k] = in ? m.bv[b] : make_int2(0, 0);   /* loaded beside the flag: one round trip less */
    }
    bool far[2] = { false, false };
    if (!full) {
        float bl[2] = { 0.f, 0.f }, si[2] = { 0.f, 0.f }, se[2] = { 0.f, 0.f };
#pragma unroll
        for (int k = 0; k < 2; k++)
            if (en[k]) { bl[k] = f32_cut(m.blen[b0 + k * blockDim.x]); si[k] = m.vspd[e[k].x]; se[k] = m.vspd[e[k].y]; }
#pragma unroll
        for (int k = 0; k < 2; k++) far[k] = en[k] && bl[k] > __fmul_ru(__fadd_ru(si[k], se[k]), dt_up);
    }
    double2 z = make_double2(0, 0), pi[2] = { z, z }, pe[2] = { z, z }, vi[2] = { z, z }, ve[2] = { z, z };
#pragma unroll
    for (int k = 0; k < 2; k++)
        if (en[k] && !far[k]) { pi[k] = m.pos[e[k].x]; pe[k] = m.pos[e[k].y]; vi[k] = m.vel[e[k].x]; ve[k] = m.vel[e[k].y]; }
#pragma unroll
    for (int k = 0; k < 2; k++) {
        int b = b0 + k * blockDim.x;
        if (b >= m.nb) continue;
        if (far[k]) {
            m.btext[b] = SEVC_MAX_T_EXT_D;       /* as text_label_one's certified skip */
            m.bexact[b] = 0;
            m.bcand[b] = 0;
            m.bconf[b] = -1;
        } else {
            text_label_one(m, b, en[k], pi[k], pe[k], vi[k], ve[k], dt, Df, hDf, inv_dt, full);
        }
    }
}


/* the step's summary in one buffer, for one readback: counters, events,
 * error bits, polling iterations, 2x3 pass counts (all per instance) and
 * the output decision */
/* The step's summary in one buffer; each per-step record it packs (event
 * counts, error bits, polling iterations and convergence, 2x3 pass counts)
 * is zeroed once read, and so are the exactness marks of the grains' dA/dt
 * and the polling iteration total, so the next step starts from zeros
 * without resets of its own (the reset each step would otherwise begin
 * with: src/main.cu's per-step clears of these values). */
__global__ void k_pack_summary(DevMesh m, DevScratch x, int ninst, int *out)
{
    griddep_wait();
    size_t nc = (size_t)ninst * CTR_COUNT, ne = (size_t)ninst * EVT_COUNT, np = ninst,
           ns = (size_t)ninst * TWO_THREE_PASSES;
    size_t total = nc + ne + 4 + np + ns + 1;
    const size_t stride = (size_t)gridDim.x * blockDim.x, t0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (size_t i = t0; i < total; i += stride) {
        size_t k = i;
        int v;
        if (k < nc) v = x.counters[k];
        else if ((k -= nc) < ne) { v = m.evt[k]; m.evt[k] = 0; }
        else if ((k -= ne) < 4) { v = m.err[k]; m.err[k] = 0; }
        else if ((k -= 4) < np) { v = x.piters[k]; x.piters[k] = 0; m.pdone[k] = 0; }
        else if ((k -= np) < ns) { v = x.segcnt[k]; x.segcnt[k] = 0; }
        else { v = x.flags[0]; *x.ptot = 0; }
        out[i] = v;
    }
    const size_t nw = (size_t)m.ng / 16;                   /* gexact as 16-byte words (256-byte aligned array) */
    for (size_t i = t0; i < nw; i += stride) reinterpret_cast<uint4 *>(m.gexact)[i] = make_uint4(0, 0, 0, 0);
    for (size_t i = 16 * nw + t0; i < (size_t)m.ng; i += stride) m.gexact[i] = 0;
}
__global__ void k_reset_ngrains(int *counters, int ninst)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ninst) counters[(size_t)i * CTR_COUNT + CTR_NGRAINS] = 0;
}

/* update_vertices_positions, src/calculus.h:391-404 */
__global__ void k_update(DevMesh m, double dt)
{
    griddep_wait();
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= m.nv || !m.ven[v]) return;
    double2 p = m.pos[v], w = m.vel[v];
    p.x += w.x * dt;
    p.y += w.y * dt;
    p.x = dmod(p.x, m.D);
    p.y = dmod(p.y, m.D);
    m.pos[v] = p;
}

/* current_n_grains (src/calculus.h:264-313): an integer count per
 * instance (blockIdx.y), added into counters[inst * CTR_COUNT + CTR_NGRAINS] */
__global__ void k_count_grains(DevMesh m, int *counters)
{
    int inst = blockIdx.y;
    int lo = m.goff[inst], hi = m.goff[inst + 1];
    int c = 0;
    for (int g = lo + blockIdx.x * blockDim.x + threadIdx.x; g < hi; g += gridDim.x * blockDim.x) c += m.gen[g] ? 1 : 0;
    __shared__ int part[32];
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += part[w];
        if (t) atomicAdd(counters + (size_t)inst * CTR_COUNT + CTR_NGRAINS, t);
    }
}

/* nucl_area_per_block (src/calculus.h:322-348): launched on the
 * reference's grid (blockIdx.y = instance) so that the floating-point sum
 * order is the same: per-thread strided partial sums over the instance's
 * grain indices, then the shared-memory tree. */
__global__ void k_nucl_area_blocks(DevMesh m, double *block_out)
{
    __shared__ double t[256];
    int inst = blockIdx.y;
    int go = m.goff[inst];
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    int stride = gridDim.x * blockDim.x;
    double a = 0.0;
    /* the thread's stride set in ascending order, restricted to the slots
     * that can be NUCLEATED (the instance's nlist part is ascending) */
    int nn = m.nnlist[inst];
    const int *nl = m.nlist + go;
    for (int i = 0; i < nn; i++) {
        int g = nl[i];
        if ((g - go) % stride == tid && m.gen[g] && m.gtype[g] == GT_NUCLEATED) a += m.garea[g];
    }
    t[threadIdx.x] = a;
    __syncthreads();
    for (int i = blockDim.x / 2; i != 0; i /= 2) {
        if ((int)threadIdx.x < i) t[threadIdx.x] += t[threadIdx.x + i];
        __syncthreads();
    }
    if (threadIdx.x == 0) block_out[(size_t)inst * gridDim.x + blockIdx.x] = t[0];
}

/* host loop of nucleated_fraction_area, src/calculus.h:373-377, one
 * thread per instance */
__global__ void k_nucl_area_final(const double *block_out, int nblocks, int ninst, double D, int *counters)
{
    int inst = blockIdx.x * blockDim.x + threadIdx.x;
    if (inst >= ninst) return;
    double s = 0.0;
    for (int i = 0; i < nblocks; i++) s += block_out[(size_t)inst * nblocks + i];
    *reinterpret_cast<double *>(counters + (size_t)inst * CTR_COUNT + CTR_NUCL_AREA_SLOT) = 100 * s / (D * D);
}

} // namespace

void launch_boundary_geometry(const DevMesh &m, double eps, double scaling, const LaunchShape &sh, cudaStream_t s)
{
    int t = sh.tpb_boundary;
    COUNT_LAUNCHES(1), k_boundary_geometry<<<(m.nb + t - 1) / t, t, 0, s>>>(m, eps, scaling);
}
void launch_grain_sort(const DevMesh &m, const DevScratch &x, cudaStream_t s)
{
    COUNT_LAUNCHES(1), k_vlen_hist<<<nblk(m.ng), TPB, 0, s>>>(m, x.vbucket, x.vbucket + NBUCKET, x.n_perm);
    COUNT_LAUNCHES(1), k_vlen_scatter<<<nblk(m.ng), TPB, 0, s>>>(m, x.vbucket + NBUCKET, x.perm);
}
void launch_grain_fd_wide(const DevMesh &m, const DevScratch &x, const LaunchShape &sh, cudaStream_t s)
{
    /* one warp per grain, grid-stride: enough warps that each takes only a
     * few of the widest grains (their areas are chains of dependent FP64
     * operations, so warps in flight hide the latency) */
    COUNT_LAUNCHES(1), k_grain_fd_wide<<<8 * 152, 32 * WIDE_WARPS, 0, s>>>(m, x.perm, x.vbucket, x.n_perm, sh.wide_sides);
}
void launch_grain_fd_sorted(const DevMesh &m, const DevScratch &x, const LaunchShape &sh, cudaStream_t s)
{
    int g = (m.ng + 127) / 128;
    if (sh.grain_occ >= 8) COUNT_LAUNCHES(1), k_grain_fd_sorted<8><<<g, 128, 0, s>>>(m, x.perm, x.vbucket, sh.wide_sides);
    else if (sh.grain_occ >= 6) COUNT_LAUNCHES(1), k_grain_fd_sorted<6><<<g, 128, 0, s>>>(m, x.perm, x.vbucket, sh.wide_sides);
    else if (sh.grain_occ == 5) COUNT_LAUNCHES(1), k_grain_fd_sorted<5><<<g, 128, 0, s>>>(m, x.perm, x.vbucket, sh.wide_sides);
    else COUNT_LAUNCHES(1), k_grain_fd_sorted<4><<<g, 128, 0, s>>>(m, x.perm, x.vbucket, sh.wide_sides);
}

void launch_vertex_fd(const DevMesh &m, double mu, bool unit_gamma, const LaunchShape &sh, cudaStream_t s)
{
    int t = sh.tpb_vertex;
    if (unit_gamma) COUNT_LAUNCHES(1), k_vertex_fd<true><<<(m.nv + t - 1) / t, t, 0, s>>>(m, mu);
    else COUNT_LAUNCHES(1), k_vertex_fd<false><<<(m.nv + t - 1) / t, t, 0, s>>>(m, mu);
}
void launch_full_flag(const DevMesh &m, const DevScratch &x, cudaStream_t s)
{
    COUNT_LAUNCHES(1), k_full_flag<<<1, 1, 0, s>>>(x.n_b, x.vbucket, x.flags, m.stamp);
}
void launch_grain_dadt(const DevMesh &m, const DevScratch &x, cudaStream_t s)
{
    int g = nblk(m.ng);   /* grid-stride: every grain, or only the 3-sided ones, decided on the device */
    COUNT_LAUNCHES(1), k_grain_dadt<<<g < 8 * 152 ? g : 8 * 152, TPB, 0, s>>>(m, x.perm, x.vbucket, x.flags);
}
void launch_text_label(const DevMesh &m, const DevScratch &x, double dt, const LaunchShape &sh, cudaStream_t s)
{
    int t = sh.tpb_boundary;
    /* binary32 copies for the certificate (text_outside_dt): rounded to
     * nearest, within 2^-24 of the binary64 values */
    float Df = (float)m.D, hDf = (float)(m.D / 2.0), inv_dt = (float)(1.0 / dt);
    /* dt (1 + 1e-6) rounded up to binary32, for the speed bound */
    float dt_up = std::nextafter((float)(dt * (1.0 + 1e-6)), INFINITY);
    if ((double)dt_up < dt * (1.0 + 1e-6)) dt_up = std::nextafter(dt_up, INFINITY);
    if (m.nb > 0)
        launch_dep(k_text_label, (m.nb + 2 * t - 1) / (2 * t), t, s, m, dt, Df, hDf, inv_dt, dt_up, x.flags);
}
void launch_update_positions(const DevMesh &m, double dt, cudaStream_t s) { launch_dep(k_update, nblk(m.nv), TPB, s, m, dt); }

void launch_pack_summary(const DevMesh &m, const DevScratch &x, int ninst, int *out, cudaStream_t s)
{
    size_t total = (size_t)ninst * (CTR_COUNT + EVT_COUNT + 1 + TWO_THREE_PASSES) + 5;
    int g = (int)((total + TPB - 1) / TPB);
    launch_dep(k_pack_summary, g < 152 ? g : 152, TPB, s, m, x, ninst, out);
}

void launch_counts(const DevMesh &m, const DevScratch &x, const StepParams &p, cudaStream_t s)
{
    COUNT_LAUNCHES(1), k_reset_ngrains<<<(p.ninst + 127) / 128, 128, 0, s>>>(x.counters, p.ninst);
    int gx = nblk(p.max_inst_ng);
    if (gx > 4096) gx = 4096;
    if (gx < 1) gx = 1;
    COUNT_LAUNCHES(1), k_count_grains<<<dim3(gx, p.ninst), TPB, 0, s>>>(m, x.counters);
    COUNT_LAUNCHES(1), k_nucl_area_blocks<<<dim3(p.n_blocks, p.ninst), p.n_threads, 0, s>>>(m, x.block_area);
    COUNT_LAUNCHES(1), k_nucl_area_final<<<(p.ninst + 127) / 128, 128, 0, s>>>(x.block_area, p.n_blocks, p.ninst, m.D,
                                                                              x.counters);
}
