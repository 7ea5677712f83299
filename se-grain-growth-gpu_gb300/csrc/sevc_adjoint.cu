/*
 * Adjoint of the time step over the positions, and the grain-area
 * histogram used as a differentiable statistic.  No counterpart in the
 * reference.
 *
 * Forward map of one step (fixed event sequence):
 *   v_i^c = mu * ( -[ sum_j gamma_j (L_j(x + eps e_i^c) - L_j(x))
 *                     + sum_g SE_g (|A_g(x + eps e_i^c)| - |A_g(x)|) ] / eps )
 *                                          (src/calculus.h:19-73, eps = 1e-8)
 *   events: a T1 flip sets both ends to their midpoint, a 3-sided removal
 *           moves the survivor to the length-weighted point of the three
 *           vertices (src/topological.h:174-291, :687-822); both zero the
 *           velocities of the vertices they move; disabled vertices stop
 *   x_{n+1} = x' + dt * v'                 (src/calculus.h:391-404)
 * with gamma_j = s * f_j (s = GB_scaling, f_j = 1 for GB_eps = 0).
 * A step with a nucleation first maps the positions by the inserted
 * triangle (src/nucleation2.cu:116-212 with the factor 0.99): with
 * A's boundaries ending at D, E, F, d_X = X - A (wrapped), u_X = d_X/|d_X|
 * and r = k * |d_X*| + 0.1 (X* the end of the shortest boundary, k = 0.8
 * times the replayed draw), the new A, B, C are A + 0.99 r u_D, u_E, u_F;
 * the rest of the step acts on that mesh.  The nucleated grain's stored
 * energy is 0, not a parameter.
 *
 * The adjoint below is the exact derivative of that map in real
 * arithmetic.  Two identities keep it cheap: the shoelace area is linear in
 * each coordinate of one vertex, so (|A(x + eps e)| - |A(x)|) / eps =
 * sign(A) dA/dx (away from a sign change), whose derivatives are constants
 * on the two list neighbours; and the arclength term's derivative is
 * (n' - n) / eps with n, n' the unit vectors of the unmoved and moved edge.
 * Every accumulation is a gather in a fixed order, so results do not depend
 * on scheduling.
 */
#include "sevc_internal.h"

namespace {

constexpr int TPB = 256;
inline int nblk(int n) { return (n + TPB - 1) / TPB; }

/* quadratic B-spline (partition of unity over unit-spaced bins) and its derivative */
__device__ __forceinline__ double bspline2(double s)
{
    double a = fabs(s);
    if (a <= 0.5) return 0.75 - s * s;
    if (a <= 1.5) { double t = 1.5 - a; return 0.5 * t * t; }
    return 0.0;
}
__device__ __forceinline__ double bspline2_d(double s)
{
    double a = fabs(s);
    if (a <= 0.5) return -2.0 * s;
    if (a <= 1.5) return s > 0 ? -(1.5 - a) : (1.5 - a);
    return 0.0;
}

/* signed area of grain g (src/geometry.h:757 order) */
__device__ __forceinline__ double grain_area(const DevMesh &m, int g)
{
    double2 none = make_double2(0, 0);
    return area_stream(m.glist + (size_t)SEVC_MAXV * g, m.gvlen[g], m.pos, -1, none, m.D);
}

/* position of vertex v in grain g's list, its list neighbours */
__device__ __forceinline__ int list_pos(const DevMesh &m, int g, int v, int *prev, int *next)
{
    const int *L = m.glist + (size_t)SEVC_MAXV * g;
    int n = m.gvlen[g];
    for (int p = 0; p < n; p++)
        if (L[p] == v) {
            *prev = L[p == 0 ? n - 1 : p - 1];
            *next = L[p == n - 1 ? 0 : p + 1];
            return p;
        }
    return -1;
}

/* ---------------- histogram of normalised grain areas ---------------- */
/* a_g = |A_g| sc with sc = N / (total domain area): N enabled grains tile
 * the domain, so 1/sc is their mean area;
 * h_k = (1/N) sum_g B2(a_g / w - k - 1/2), w = amax / nbins */
__global__ void k_hist_blocks(DevMesh m, int nbins, double amax, double sc, double *blockbins)
{
    __shared__ double red[TPB];
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    double a = -1.0;
    if (g < m.ng && m.gen[g]) a = fabs(grain_area(m, g)) * sc;
    double w = amax / nbins;
    for (int k = 0; k < nbins; k++) {
        red[threadIdx.x] = a >= 0 ? bspline2(a / w - k - 0.5) : 0.0;
        __syncthreads();
        for (int s = TPB / 2; s > 0; s >>= 1) {
            if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
            __syncthreads();
        }
        if (threadIdx.x == 0) blockbins[(size_t)blockIdx.x * nbins + k] = red[0];
        __syncthreads();
    }
}
__global__ void k_hist_final(const double *blockbins, int nblocks, int nbins, double nnorm, double *hist)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nbins) return;
    double s = 0.0;
    for (int b = 0; b < nblocks; b++) s += blockbins[(size_t)b * nbins + k];
    hist[k] = s / nnorm;
}

/* dL/dA_g of the histogram (signed area) given dL/dh */
__global__ void k_hist_grad_area(DevMesh m, int nbins, double amax, double sc, double nnorm, const double *dldh,
                                 double *dlda)
{
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= m.ng) return;
    if (!m.gen[g]) { dlda[g] = 0.0; return; }
    double A = grain_area(m, g);
    double a = fabs(A) * sc, w = amax / nbins;
    double d = 0.0;
    for (int k = 0; k < nbins; k++) d += dldh[k] * bspline2_d(a / w - k - 0.5);
    d *= sc / (w * nnorm);
    dlda[g] = A < 0 ? -d : d;
}

/* lambda_k = sum over k's grains of dL/dA_g dA_g/dx_k, with
 * dA/dx_k = (y_next - y_prev) / 2, dA/dy_k = (x_prev - x_next) / 2 */
__global__ void k_area_grad_to_vertices(DevMesh m, const double *dlda, double2 *lam)
{
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= m.nv) return;
    double2 out = make_double2(0, 0);
    if (m.ven[v]) {
        double2 p = m.pos[v];
        int4 sg = m.vg[v];
        for (int j = 0; j < 3; j++) {
            int g = slot3(sg, j);
            if (g < 0 || !m.gen[g]) continue;
            int pv, nx;
            if (list_pos(m, g, v, &pv, &nx) < 0) continue;
            double2 a = m.pos[pv], b = m.pos[nx];
            /* unwrapped neighbour coordinates relative to v */
            double xp = wrapd(a.x, p.x, m.D), yp = wrapd(a.y, p.y, m.D);
            double xn = wrapd(b.x, p.x, m.D), yn = wrapd(b.y, p.y, m.D);
            out.x += dlda[g] * 0.5 * (yn - yp);
            out.y += dlda[g] * 0.5 * (xp - xn);
        }
    }
    lam[v] = out;
}

/* ---------------- adjoint of one step ---------------- */
/* vertices moved by an event this step (their velocity was zeroed) */
__global__ void k_adj_mark_events(uint8_t *mark, const EventRec *log, const int *nlog)
{
    int n = *nlog;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        EventRec r = log[i];
        if (r.type != EV_FLIP && r.type != EV_REMOVE) continue;
        mark[r.a] = 1;
        mark[r.b] = 1;
        if (r.type == EV_REMOVE) mark[r.c] = 1;
    }
}

/* translation x_{n+1} = x' + dt v': lambda_x' = lambda (vertices alive
 * after the step), lambda_v = dt lambda (alive, not moved by an event);
 * d/dmu of the step: dt * lambda . v' / mu */
__global__ void k_adj_translate(int nv, double dt, double mu, const double2 *lam, const uint8_t *ven1,
                                const double2 *vel1, const uint8_t *mark, double2 *lx, double2 *lv, double *gmu)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    double2 l = ven1[i] ? lam[i] : make_double2(0, 0);
    lx[i] = l;
    lv[i] = (ven1[i] && !mark[i]) ? make_double2(dt * l.x, dt * l.y) : make_double2(0, 0);
    double2 w = vel1[i];
    gmu[i] += dt * (l.x * w.x + l.y * w.y) / mu;
}

/* one logged flip or 3-sided removal, backward */
__device__ void adj_event_one(double D, const EventRec &r, double2 *lx)
{
    if (r.type == EV_FLIP) {                          /* both ends -> midpoint */
        double2 a = lx[r.a], b = lx[r.b];
        double2 s = make_double2(0.5 * (a.x + b.x), 0.5 * (a.y + b.y));
        lx[r.a] = s;
        lx[r.b] = s;
        return;
    }
    if (r.type != EV_REMOVE) return;                  /* nucleations: k_adj_nucleation */
    /* A' = A + F(u, w), u = B - A, w = C - A,
     * F = (|w| u + |u| w) / (|u| + |w - u| + |w|) */
    double2 lp = lx[r.a];
    double ux = wrapd(r.pb.x, r.pa.x, D), uy = wrapd(r.pb.y, r.pa.y, D);
    double wx = ux + wrapd(r.pc.x, r.pb.x, D), wy = uy + wrapd(r.pc.y, r.pb.y, D);
    double nu = sqrt(ux * ux + uy * uy), nw = sqrt(wx * wx + wy * wy);
    double rx = wx - ux, ry = wy - uy, nr = sqrt(rx * rx + ry * ry);
    double S = nu + nr + nw;
    double Nx = nw * ux + nu * wx, Ny = nw * uy + nu * wy;
    double lN = lp.x * Nx + lp.y * Ny, lw = lp.x * wx + lp.y * wy, lu = lp.x * ux + lp.y * uy;
    double hux = ux / nu, huy = uy / nu, hwx = wx / nw, hwy = wy / nw, hrx = rx / nr, hry = ry / nr;
    if (nu == 0) { hux = 0; huy = 0; }                /* coincident vertices: zero subgradient */
    if (nw == 0) { hwx = 0; hwy = 0; }
    if (nr == 0) { hrx = 0; hry = 0; }
    if (!(S > 0)) return;                             /* degenerate triangle: the map is not moved */
    double S2 = S * S;
    /* J_u^T lambda' and J_w^T lambda' */
    double jux = (nw * lp.x + lw * hux) / S - lN * (hux - hrx) / S2;
    double juy = (nw * lp.y + lw * huy) / S - lN * (huy - hry) / S2;
    double jwx = (lu * hwx + nu * lp.x) / S - lN * (hrx + hwx) / S2;
    double jwy = (lu * hwy + nu * lp.y) / S - lN * (hry + hwy) / S2;
    lx[r.a] = make_double2(lp.x - jux - jwx, lp.y - juy - jwy);
    double2 b = lx[r.b], c = lx[r.c];
    lx[r.b] = make_double2(b.x + jux, b.y + juy);
    lx[r.c] = make_double2(c.x + jwx, c.y + jwy);
}

/* Walk the step's log from its end in chunks of ADJ_TPB records, one block
 * per instance: the threads test a chunk at once (record kind and the
 * instance of its first vertex) and thread 0 takes the hits in descending
 * log order.  Events of different instances touch disjoint vertices, so
 * the instances run side by side; within an instance the events keep the
 * reverse of the order they were applied in (the log order: the parallel
 * events, which share no vertex, then the deferred ones). */
constexpr int ADJ_TPB = 256;
template <class Want, class Take>
__device__ void walk_log_reverse(const EventRec *log, int n, Want want, Take take)
{
    __shared__ unsigned hit[ADJ_TPB / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int top = n; top > 0; top -= ADJ_TPB) {
        int e = top - 1 - (int)threadIdx.x;
        bool f = e >= 0 && want(e);
        unsigned w = __ballot_sync(0xffffffffu, f);
        if (lane == 0) hit[warp] = w;
        __syncthreads();
        if (threadIdx.x == 0)
            for (int k = 0; k < ADJ_TPB / 32; k++)
                for (unsigned h = hit[k]; h; h &= h - 1) take(top - 1 - (32 * k + __ffs(h) - 1));
        __syncthreads();
    }
}
__device__ __forceinline__ bool in_instance(const int *voff, int ninst, int inst, int v)
{
    return ninst <= 1 || (v >= voff[inst] && v < voff[inst + 1]);
}

/* the step's flips and 3-sided removals in reverse order, per instance */
__global__ void __launch_bounds__(ADJ_TPB) k_adj_events(double D, const EventRec *log, const int *nlog, double2 *lx,
                                                        const int *voff, int ninst)
{
    const int inst = blockIdx.x;
    walk_log_reverse(
        log, *nlog,
        [&](int e) {
            EventRec r = log[e];
            return (r.type == EV_FLIP || r.type == EV_REMOVE) && in_instance(voff, ninst, inst, r.a);
        },
        [&](int e) { adj_event_one(D, log[e], lx); });
}

/* boundary weight f_j = gamma_j / s (k_boundary_geometry's definition) */
__device__ __forceinline__ double gb_weight(const DevMesh &m, int b, double eps)
{
    if (eps == 0.0) return 1.0;
    int2 e = m.bv[b];
    int gic[2];
    if (gintersect(m.vg[e.x], m.vg[e.y], gic) < 2) return 0.0;
    return gb_energy(m.gori[gic[0]] - m.gori[gic[1]], eps);
}

/* the nucleations of the step, last first: lambda of the positions
 * before it from lambda after it (one block per instance, as
 * k_adj_events).  For each new position Y = A + c u_X (c = 0.99 r):
 *   dY/dX = c (I - u u^T) / |d_X|,  dY/dA = I - dY/dX + u (dc/dA)^T,
 *   dc/dX* = 0.99 k u_X* = -dc/dA;
 * the new vertices B and C had no position before. */
__device__ void adj_nucleation_one(double D, const EventRec &r, const EventRec &x, double2 *lam)
{
    int Y[3] = { r.a, r.b, r.c }, X[3] = { x.a, x.b, x.c };
    double2 pa = r.pa, px[3] = { r.pb, r.pc, x.pa };
    double k = x.pb.x, c = 0.99 * x.pb.y;
    int is = (int)x.pc.x;
    double2 ly[3] = { lam[Y[0]], lam[Y[1]], lam[Y[2]] };
    double usx = wrapd(px[is].x, pa.x, D), usy = wrapd(px[is].y, pa.y, D);
    double ns = sqrt(usx * usx + usy * usy);
    usx = ns > 0 ? usx / ns : 0.0;
    usy = ns > 0 ? usy / ns : 0.0;
    double2 la = make_double2(0, 0);
    double2 lstar = make_double2(0, 0);
    for (int i = 0; i < 3; i++) {
        double dx = wrapd(px[i].x, pa.x, D), dy = wrapd(px[i].y, pa.y, D), n = sqrt(dx * dx + dy * dy);
        if (!(n > 0)) continue;
        double ux = dx / n, uy = dy / n, l_u = ux * ly[i].x + uy * ly[i].y;
        double gx = c / n * (ly[i].x - ux * l_u), gy = c / n * (ly[i].y - uy * l_u);
        double t = 0.99 * k * l_u;
        la.x += ly[i].x - gx - t * usx;
        la.y += ly[i].y - gy - t * usy;
        lam[X[i]].x += gx;
        lam[X[i]].y += gy;
        lstar.x += t * usx;
        lstar.y += t * usy;
    }
    lam[X[is]].x += lstar.x;
    lam[X[is]].y += lstar.y;
    lam[Y[0]] = la;
    lam[Y[1]] = make_double2(0, 0);
    lam[Y[2]] = make_double2(0, 0);
}
__global__ void __launch_bounds__(ADJ_TPB) k_adj_nucleation(double D, const EventRec *log, const int *nlog,
                                                            double2 *lam, const int *voff, int ninst)
{
    const int inst = blockIdx.x, n = *nlog;
    walk_log_reverse(
        log, n,
        [&](int e) {
            if (e + 1 >= n) return false;
            EventRec r = log[e];
            return r.type == EV_NUCL && log[e + 1].type == EV_NUCL_AUX && in_instance(voff, ninst, inst, r.a);
        },
        [&](int e) { adj_nucleation_one(D, log[e], log[e + 1], lam); });
}

/* per grain: sign of the area at the step's start, and
 * dL/dSE_g += sum_p lambda_v(p) . (-mu sign(A) dA/dx_p) (not for a
 * nucleated grain, whose stored energy is 0, not a parameter) */
__global__ void k_adj_grains(DevMesh m, double mu, const double2 *lv, double *sgn, double *gse)
{
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= m.ng) return;
    if (!m.gen[g]) { sgn[g] = 0.0; return; }
    const int *L = m.glist + (size_t)SEVC_MAXV * g;
    int n = m.gvlen[g];
    double A = grain_area(m, g);
    double s = A > 0 ? 1.0 : (A < 0 ? -1.0 : 0.0);
    sgn[g] = s;
    double acc = 0.0;
    for (int p = 0; p < n; p++) {
        int v = L[p], pv = L[p == 0 ? n - 1 : p - 1], nx = L[p == n - 1 ? 0 : p + 1];
        double2 q = m.pos[v], a = m.pos[pv], b = m.pos[nx];
        double xp = wrapd(a.x, q.x, m.D), yp = wrapd(a.y, q.y, m.D);
        double xn = wrapd(b.x, q.x, m.D), yn = wrapd(b.y, q.y, m.D);
        double2 l = lv[v];
        acc += l.x * (0.5 * (yn - yp)) + l.y * (0.5 * (xp - xn));
    }
    if (m.gtype[g] != GT_NUCLEATED) gse[g] += -mu * s * acc;
}

/* For the edge vector d (length L) and its end moved by eps along axis c,
 * d' = d + eps e_c, L' = |d'|: *g = (d'/L' - d/L) / eps, the gradient with
 * respect to the moved end of (L' - L) / eps, and *s = (L' - L) / eps, both
 * in forms without cancellation:
 *   (L' - L) / eps = (2 d_c + eps) / (L + L')
 *   (d'/L' - d/L) / eps = e_c / L' - d (2 d_c + eps) / (L L' (L + L'))
 * (the same values as the difference quotients, which lose about eight
 * digits to cancellation).  L = 0, an edge whose ends coincide after a
 * flip, takes the zero subgradient for d/L. */
/*
 * The adjoint is checked against an FP64 reference and difference quotients
 * to a tolerance (it is not a bit-exact restatement), so its square roots
 * and reciprocals use a binary32 seed on the mantissa (the exponent split
 * off on the integer pipe) and one FP64 Newton step: ~2^-45 relative,
 * 3 and 2 FP64 instructions instead of ~8 each.  x > 0 and normal; other x
 * take the native operation.
 */
static __device__ __noinline__ double rsqrt_slow(double x) { return 1.0 / sqrt(x); }
static __device__ __noinline__ double rcp_slow(double x) { return 1.0 / x; }
__device__ __forceinline__ double rsqrt_newton(double x)
{
    long long b = dbits(x);
    int eb = (int)(b >> 52);
    if (eb < 2 || eb > 2045) return rsqrt_slow(x);
    int k = (eb - 1023) >> 1;                             /* x = m' 4^k, m' in [1, 4) */
    double mp = __longlong_as_double(b - (long long)(2 * k) * (1LL << 52));
    float y0 = rsqrt_seed(f32_cut(mp));
    double y = __longlong_as_double(dbits(f2d_bits(y0)) - (long long)k * (1LL << 52));
    double h = dscale_down<1>(x);
    double r = __fma_rn(-h * y, y, 0.5);                  /* 1/2 - x y^2 / 2 */
    return __fma_rn(y, r, y);
}
__device__ __forceinline__ double rcp_newton(double x)
{
    long long b = dbits(x);
    int eb = (int)(b >> 52);
    if (eb < 2 || eb > 2045) return rcp_slow(x);
    long long sh = (long long)(eb - 1023) * (1LL << 52);  /* x = m 2^e, m in [1, 2) */
    float y0 = rcp_seed(f32_cut(__longlong_as_double(b - sh)));
    double y = __longlong_as_double(dbits(f2d_bits(y0)) - sh);
    double e = __fma_rn(-x, y, 1.0);
    return __fma_rn(y, e, y);
}

/* The same quantities for the edge d (squared length L2, length L, 1/L,
 * 0 when L = 0) with the end moved by eps along axis c, written with one
 * reciprocal square root and one reciprocal:
 *   num = 2 d_c + eps, L'^2 = L2 + eps num, s = num / (L + L'),
 *   g = e_c / L' - d s / (L L'). */
__device__ __forceinline__ void edge_fd_grad(double dx, double dy, double L2, double L, double invL, double E, int c,
                                             double2 *g, double *s)
{
    double dc = c == 0 ? dx : dy, dother = c == 0 ? dy : dx;
    double num = __fma_rn(2.0, dc, E);
    double inv1 = rsqrt_newton(__fma_rn(E, num, L2));     /* 1 / L' */
    double L1 = __fma_rn(E, num, L2) * inv1;
    double sv = num * rcp_newton(L + L1);
    double t = sv * inv1 * invL;
    double gc = __fma_rn(-dc, t, inv1), go = -dother * t;
    *s = sv;
    *g = c == 0 ? make_double2(gc, go) : make_double2(go, gc);
}

/* per vertex k (gather): lambda_n[k] = lambda_x[k] + (J_v^T lambda_v)[k];
 * d/ds of k's own velocity into ggam[k] */
__global__ void k_adj_vertices(DevMesh m, double mu, double eps, double s_gb, const double2 *lx, const double2 *lv,
                               const double *sgn, double2 *lam_out, double *ggam)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m.nv) return;
    if (!m.ven[k]) { lam_out[k] = make_double2(0, 0); return; }
    const double E = SEVC_GRAD_EPS_D;
    double2 out = lx[k];
    double2 p = m.pos[k];
    double2 lk = lv[k];
    int4 sb = m.vb[k];
    double dgam = 0.0;
    for (int j = 0; j < 3; j++) {
        int b = slot3(sb, j);
        if (b < 0) continue;
        int q = other_end(m.bv[b], k);
        double f = gb_weight(m, b, eps), gam = s_gb * f;
        double2 pq = m.pos[q];
        double dx = wrapd(p.x, pq.x, m.D), dy = wrapd(p.y, pq.y, m.D);
        double L2 = dx * dx + dy * dy;
        double invL = L2 > 0 ? rsqrt_newton(L2) : 0.0, L = L2 * invL;
        /* k moved along x / y (d -> d + eps e_c) and q moved (-d -> -d + eps e_c) */
        double2 gkx, gky, gqx, gqy;
        double skx, sky;
        edge_fd_grad(dx, dy, L2, L, invL, E, 0, &gkx, &skx);
        edge_fd_grad(dx, dy, L2, L, invL, E, 1, &gky, &sky);
        double sqx, sqy;
        edge_fd_grad(-dx, -dy, L2, L, invL, E, 0, &gqx, &sqx);
        edge_fd_grad(-dx, -dy, L2, L, invL, E, 1, &gqy, &sqy);
        double cg = -mu * gam;
        out.x += cg * (lk.x * gkx.x + lk.y * gky.x);
        out.y += cg * (lk.x * gkx.y + lk.y * gky.y);
        dgam += -mu * f * (lk.x * skx + lk.y * sky);
        /* q's velocity: d/dx_k of -(gam/eps) (L(x_q + eps e_c) - L(x)) is
         * minus the gradient with respect to the moved end */
        double2 lq = lv[q];
        double cq = mu * gam;
        out.x += cq * (lq.x * gqx.x + lq.y * gqy.x);
        out.y += cq * (lq.x * gqx.y + lq.y * gqy.y);
    }
    int4 sg = m.vg[k];
    for (int j = 0; j < 3; j++) {
        int g = slot3(sg, j);
        if (g < 0 || !m.gen[g]) continue;
        int pv, nx;
        if (list_pos(m, g, k, &pv, &nx) < 0) continue;
        double se = m.gtype[g] == GT_NUCLEATED ? 0.0 : m.gse[g];
        double c = 0.5 * mu * se * sgn[g];
        double2 a = lv[pv], b = lv[nx];
        out.x += c * (a.y - b.y);
        out.y += c * (b.x - a.x);
    }
    lam_out[k] = out;
    ggam[k] += dgam;
}

/* grain statistics over grains [lo, hi): count, sum |A|, sum A^2, sum of
 * side counts, 3-sided count, min |A|, max |A| (one block, fixed order) */
__global__ void __launch_bounds__(512) k_grain_stats(DevMesh m, int lo, int hi, double *out)
{
    __shared__ double red[7][512];
    double c = 0, s1 = 0, s2 = 0, sv = 0, n3 = 0, mn = 1e300, mx = 0;
    for (int g = lo + threadIdx.x; g < hi; g += blockDim.x) {
        if (!m.gen[g]) continue;
        double a = fabs(grain_area(m, g));
        c += 1;
        s1 += a;
        s2 += a * a;
        sv += m.gvlen[g];
        n3 += m.gvlen[g] == 3;
        mn = fmin(mn, a);
        mx = fmax(mx, a);
    }
    double v[7] = { c, s1, s2, sv, n3, mn, mx };
    for (int k = 0; k < 7; k++) red[k][threadIdx.x] = v[k];
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s)
            for (int k = 0; k < 7; k++) {
                double a = red[k][threadIdx.x], b = red[k][threadIdx.x + s];
                red[k][threadIdx.x] = k == 5 ? fmin(a, b) : (k == 6 ? fmax(a, b) : a + b);
            }
        __syncthreads();
    }
    if (threadIdx.x < 7) out[threadIdx.x] = red[threadIdx.x][0];
}

__global__ void k_sum_ordered(const double *a, int n, double *out)
{
    __shared__ double red[TPB];
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += TPB) s += a[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int k = TPB / 2; k > 0; k >>= 1) {
        if ((int)threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

} // namespace

void launch_histogram(const DevMesh &m, int nbins, double amax, double sc, double nnorm, double *blockbins,
                      double *hist, cudaStream_t s)
{
    int nb = nblk(m.ng);
    COUNT_LAUNCHES(1), k_hist_blocks<<<nb, TPB, 0, s>>>(m, nbins, amax, sc, blockbins);
    COUNT_LAUNCHES(1), k_hist_final<<<(nbins + 63) / 64, 64, 0, s>>>(blockbins, nb, nbins, nnorm, hist);
}
int histogram_blocks(const DevMesh &m) { return nblk(m.ng); }

void launch_hist_seed(const DevMesh &m, int nbins, double amax, double sc, double nnorm, const double *dldh,
                      double *dlda, double2 *lam, cudaStream_t s)
{
    COUNT_LAUNCHES(1), k_hist_grad_area<<<nblk(m.ng), TPB, 0, s>>>(m, nbins, amax, sc, nnorm, dldh, dlda);
    COUNT_LAUNCHES(1), k_area_grad_to_vertices<<<nblk(m.nv), TPB, 0, s>>>(m, dlda, lam);
}

void launch_adjoint_step(const DevMesh &rec, const AdjointBuffers &a, double dt, double mu, double eps, double s_gb,
                         const EventRec *log, const int *nlog, const uint8_t *ven1, const double2 *vel1,
                         cudaStream_t s)
{
    cudaMemsetAsync(a.mark, 0, rec.nv, s);
    COUNT_LAUNCHES(1), k_adj_mark_events<<<4, TPB, 0, s>>>(a.mark, log, nlog);
    COUNT_LAUNCHES(1), k_adj_translate<<<nblk(rec.nv), TPB, 0, s>>>(rec.nv, dt, mu, a.lam, ven1, vel1, a.mark, a.lx,
                                                                    a.lv, a.gmu);
    COUNT_LAUNCHES(1), k_adj_events<<<rec.ninst, ADJ_TPB, 0, s>>>(rec.D, log, nlog, a.lx, rec.voff, rec.ninst);
    COUNT_LAUNCHES(1), k_adj_grains<<<nblk(rec.ng), TPB, 0, s>>>(rec, mu, a.lv, a.sgn, a.gse);
    COUNT_LAUNCHES(1), k_adj_vertices<<<nblk(rec.nv), TPB, 0, s>>>(rec, mu, eps, s_gb, a.lx, a.lv, a.sgn, a.lam,
                                                                   a.ggam);
    COUNT_LAUNCHES(1), k_adj_nucleation<<<rec.ninst, ADJ_TPB, 0, s>>>(rec.D, log, nlog, a.lam, rec.voff, rec.ninst);
}

void launch_grain_stats(const DevMesh &m, int lo, int hi, double *out, cudaStream_t s)
{
    COUNT_LAUNCHES(1), k_grain_stats<<<1, 512, 0, s>>>(m, lo, hi, out);
}

void launch_sum_ordered(const double *a, int n, double *out, cudaStream_t s)
{
    COUNT_LAUNCHES(1), k_sum_ordered<<<1, TPB, 0, s>>>(a, n, out);
}
