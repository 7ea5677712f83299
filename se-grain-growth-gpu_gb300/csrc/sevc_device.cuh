/*
 * Device-side mesh layout and exact periodic geometry.
 *
 * Layout (structure of arrays, entity = int32 index, -1 = NULL):
 *   vertex   pos/vel double2, terms double4 (finite-difference energy
 *            terms, kept raw), energy double, enabled u8, boundaries int4
 *            (x,y,z used), grains int4, mods int4[4] (grn, vrt, prev, fix)
 *   boundary ends int2 (ini, end), energy/arclength/t_ext double,
 *            enabled/candidate/candidate-buffer u8, votes/conflict int
 *   grain    list int32[100] row-major, vlen int32, area/dAdt/orientation/
 *            stored-energy double, enabled/candidate/fix/type u8
 * Field meanings follow src/geometry.h:39-86 of the reference.
 *
 * Arithmetic: every helper restates the reference's expression tree
 * operation by operation.  The library is compiled with -fmad=false, so no
 * multiply-add is fused and results equal the reference semantics computed
 * in IEEE binary64 without contraction.
 */
#ifndef SEVC_DEVICE_CUH
#define SEVC_DEVICE_CUH

#include <climits>
#include <cstdint>
#include <cuda_runtime.h>

#define SEVC_MAXV 100
#define SEVC_GRAD_EPS_D 1e-8          /* src/calculus.h:7 */
#define SEVC_MAX_T_EXT_D 100000.0     /* src/geometry.h:11 */

enum { FIX_ADD = 0, FIX_REMOVE = 1, FIX_REPLACE = 2, FIX_NONE = 3 }; /* src/geometry.h:17 */
enum { GT_COMMON = 0, GT_NUCLEATED = 1 };                            /* src/geometry.h:19 */

/* error bits raised by kernels (read back once per step) */
enum {
    ERRB_CAPACITY = 1,
    ERRB_TOPOLOGY = 2,
    ERRB_RNG = 4,
    ERRB_WORKLIST = 8,
    ERRB_NONCONVERGED = 16
};

struct DevMesh {
    int nv, nb, ng;
    double D;            /* domain bound */
    /* vertices */
    double2 *pos, *vel;
    struct alignas(16) FdTerms { double bx, gx, by, gy; } *terms; /* energy terms of src/calculus.h:59-69 */
    double2 *contrib;    /* 3 per vertex: stored-energy FD term per grain slot */
    float *vspd;         /* upper bound of |vx| + |vy| from the step's vertex pass */
    double *venergy;
    uint8_t *ven;
    int4 *vb, *vg;
    int4 *vmod;          /* 4 per vertex */
    int *voted;
    uint8_t *vmodmark;
    /* boundaries */
    int2 *bv;
    double *benergy, *blen, *btext;
    uint8_t *ben, *bcand, *bcandbuf;
    int *bvotes, *bconf;
    /* grains */
    int *glist, *gvlen;
    double *garea, *gdadt, *gori, *gse, *gq;
    uint8_t *gen, *gcand, *gfix, *gtype;
    /* worklists of the grain-list fix-up (src/topological.h:1209); the
     * capacities are the array sizes unless sevc_set_limits lowers them */
    int *fixlist, *nfix;
    int *modlist, *nmod;
    int fixcap, modcap;
    int *err;            /* ERRB_* bits */
    int *evt;            /* event counters, EVT_COUNT per instance */
    /* Instances.  A batched handle holds several independent meshes one
     * after another in every array (indices are global, no edge crosses an
     * instance); instance i owns vertices [voff[i], voff[i+1]) and likewise
     * boundaries and grains.  A plain handle is one instance. */
    int ninst;
    int *voff, *boff, *goff;
    int *binst, *ginst;  /* instance of every boundary / grain */
    int *pdone;          /* per instance: polling has converged this step */
    /* position-moving events of the step in application order, recorded
     * only while an adjoint tape replays a segment (elog->buf == nullptr
     * else); the control block lives in device memory so that captured
     * launches stay valid whether or not events are recorded */
    struct EventLog *elog;
    /* slots that ever held a nucleated grain, ascending; instance i's
     * entries start at nlist[goff[i]], nnlist[i] of them */
    int *nlist, *nnlist;
    /* Output-only values (extinction time, dA/dt) are computed exactly for
     * every entity only on steps that can export; on other steps the values
     * of entities an event disables are computed at that moment from the
     * positions, velocities and boundary ends the step started its events
     * with.  Events save those before they first overwrite them in a step
     * (save_vertex, save_ends): pos0 / vel0 / bv0 hold the saved values
     * and vstamp / bstamp the step stamp (*stamp, advanced once per step)
     * under which they were saved; an entry with an older stamp is stale
     * and the live value is still the step's starting one.  bexact /
     * gexact say which values are already exact this step. */
    double2 *pos0, *vel0;
    int2 *bv0;
    unsigned *vstamp, *bstamp, *stamp;
    uint8_t *bexact, *gexact;
    uint8_t *bmark;      /* boundaries marked by a sparse pass, compacted next */
    int *lastblk;        /* arrival counters of last_block, zero between launches */
};

/* per-instance event counters of a step; EVT_CONFLICTS counts the
 * boundaries check_conflictive_boundaries marks (src/topological.h:116
 * prints one line for each) */
enum { EVT_TWO_THREE = 0, EVT_REMOVALS = 1, EVT_FLIPS = 2, EVT_NUCLEATIONS = 3, EVT_CONFLICTS = 4, EVT_COUNT = 5 };

/* one position-moving event: a T1 flip (vertices a, b move to their
 * midpoint) or a 3-sided grain removal (a moves to the length-weighted
 * point of a, b, c; b and c are disabled), with the positions it read.
 * A nucleation takes two records in a row: EV_NUCL {a = A, b = B, c = C
 * (the new vertices), pa, pb, pc = A, D, E before it} and EV_NUCL_AUX
 * {a, b, c = D, E, F (the far ends of A's boundaries), pa = F,
 * pb = (k, r) with r = k * min length + 0.1 the triangle's radius,
 * pc.x = the slot (0..2) of the shortest boundary}. */
enum { EV_FLIP = 1, EV_REMOVE = 2, EV_NUCL = 3, EV_NUCL_AUX = 4 };
struct EventRec {
    int type, a, b, c;
    double2 pa, pb, pc;
};

struct EventLog {
    EventRec *buf;   /* nullptr: not recording */
    int *n;
    int cap;
};

__device__ __forceinline__ void log_event(const DevMesh &m, int type, int a, int b, int c, double2 pa, double2 pb,
                                          double2 pc)
{
    EventLog L = *m.elog;
    if (!L.buf) return;
    int i = atomicAdd(L.n, 1);
    if (i >= L.cap) { atomicOr(m.err, ERRB_WORKLIST); return; }
    EventRec r;
    r.type = type; r.a = a; r.b = b; r.c = c; r.pa = pa; r.pb = pb; r.pc = pc;
    L.buf[i] = r;
}
/* two records in consecutive slots (an event that takes two) */
__device__ __forceinline__ void log_event_pair(const DevMesh &m, const EventRec &r0, const EventRec &r1)
{
    EventLog L = *m.elog;
    if (!L.buf) return;
    int i = atomicAdd(L.n, 2);
    if (i + 1 >= L.cap) { atomicOr(m.err, ERRB_WORKLIST); return; }
    L.buf[i] = r0;
    L.buf[i + 1] = r1;
}

/* first statement of a kernel launched with launch_dep: wait until the
 * previous kernel of the stream has completed and its writes are visible
 * (a no-op for a kernel launched without the attribute) */
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

/* True in the last block of the grid to get here: every other block has
 * finished (its reads of work-list counts included), so that block may
 * reset state the whole grid read.  All threads of every block must call
 * it; *ctr is zero on entry and left zero. */
__device__ __forceinline__ bool last_block(int *ctr)
{
    __shared__ int last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(ctr, 1) == (int)(gridDim.x * gridDim.y) - 1;
        if (last) *ctr = 0;
    }
    __syncthreads();
    return last != 0;
}

/* ---- periodic geometry, src/geometry.h:133-331 ----
 * Comparisons, absolute values and min/max work on the IEEE-754 bit
 * patterns with integer instructions: for finite doubles the signed
 * 64-bit order of the patterns of non-negative values is their numeric
 * order, so every branch takes the same side as the floating-point
 * comparison of the reference while the (scarce) FP64 pipe only executes
 * the arithmetic.  Inputs are never NaN.
 *
 * Two compiler behaviours are kept away from the FP64 pipe (counted with
 * ncu: each cost one FP64 instruction per call):
 *  - a short branch whose body is FP64 arithmetic gets if-converted, the
 *    arithmetic then runs for every thread; rare bodies are therefore
 *    calls (the *_slow functions), which cannot be speculated;
 *  - an absolute value taken from the bit pattern (sign masked or shifted
 *    out) and compared is recognised as an FP comparison of fabs and
 *    emitted on the FP64 pipe; magnitudes are therefore compared through
 *    mag2, whose shift is opaque inline PTX, or, for a negative b, through
 *    b itself (b = magnitude - 2^63). */
#define SEVC_ABSMASK 0x7FFFFFFFFFFFFFFFLL
__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ double dabs(double x) { return __longlong_as_double(dbits(x) & SEVC_ABSMASK); }
/* the magnitude's bit pattern shifted left by one: ordered like |x| */
__device__ __forceinline__ unsigned long long mag2(double x)
{
    unsigned long long r;
    asm("shl.b64 %0, %1, 1;" : "=l"(r) : "l"(dbits(x)));
    return r;
}

static __device__ __noinline__ double dadd_slow(double a, double b) { return a + b; }
static __device__ __noinline__ double dsub_slow(double a, double b) { return a - b; }
static __device__ __noinline__ double dmul_slow(double x, double s) { return x * s; }
static __device__ __noinline__ double ddiv_slow(double x, double y) { return x / y; }

__device__ __forceinline__ double dmod(double a, double D)        /* dom_mod :133 */
{
    long long b = dbits(a);
    if (b < 0 && b != (long long)0x8000000000000000ULL) return dadd_slow(a, D);   /* a < 0 (not -0) */
    else if (b >= dbits(D)) return dsub_slow(a, D);                               /* a >= D (D > 0) */
    return a;
}
/* Exact scalings and divisions kept off the FP64 pipe (on GB300 one FP64
 * operation costs as much issue time as dozens of integer ones). */

/* +0.0 + x, exactly, on the integer pipe: x, except that -0 becomes +0
 * (for the first term of a sum the reference starts from 0.0) */
__device__ __forceinline__ double zero_plus(double x)
{
    long long b = dbits(x);
    return __longlong_as_double(b == LLONG_MIN ? 0LL : b);
}

/* x * 2^-K (K = 1..3), exactly: an exponent decrement on the integer pipe
 * when x and the result are normal, else the multiplication */
template <int K> __device__ __forceinline__ double dscale_down(double x)
{
    long long b = dbits(x);
    unsigned ex = (unsigned)(b >> 52) & 0x7ffu;
    if (ex > (unsigned)K && ex < 0x7ffu) return __longlong_as_double(b - ((long long)K << 52));
    return dmul_slow(x, K == 1 ? 0.5 : (K == 2 ? 0.25 : 0.125));
}

/* x / N for a small integer N, correctly rounded, with one multiplication
 * and one fma (Brisebarre, Muller and Raina, "Accelerating correctly
 * rounded floating-point division when the divisor is known in advance",
 * IEEE Trans. Computers 53(8), 2004): zh = RN(1/N), zl = RN(1/N - zh).
 * The fma's exact argument x zh + RN(x zl) is within 2^-105.8 of x/N
 * (relative, worst N = 7), while x/N, a 53-bit integer over N <= 10
 * scaled by a power of two, is never within 2^-59 (relative) of a
 * rounding midpoint: the fma returns RN(x/N).  Valid while x zl is normal
 * and x/N finite, 2^-900 <= |x| < 2^900; other x divide.  N = 4 and 8 are
 * exact scalings. */
template <int N> struct InvSplit;
template <> struct InvSplit<3> { static constexpr double hi = 0x1.5555555555555p-2, lo = 0x1.5555555555555p-56; };
template <> struct InvSplit<5> { static constexpr double hi = 0x1.999999999999ap-3, lo = -0x1.999999999999ap-57; };
template <> struct InvSplit<6> { static constexpr double hi = 0x1.5555555555555p-3, lo = 0x1.5555555555555p-57; };
template <> struct InvSplit<7> { static constexpr double hi = 0x1.2492492492492p-3, lo = 0x1.2492492492492p-57; };
template <> struct InvSplit<9> { static constexpr double hi = 0x1.c71c71c71c71cp-4, lo = 0x1.c71c71c71c71cp-58; };
template <> struct InvSplit<10> { static constexpr double hi = 0x1.999999999999ap-4, lo = -0x1.999999999999ap-58; };
template <int N> __device__ __forceinline__ double div_small(double x)
{
    if constexpr (N == 4) {
        return dscale_down<2>(x);
    } else if constexpr (N == 8) {
        return dscale_down<3>(x);
    } else {
        unsigned long long b = mag2(x);
        if (b >= (0x07B0000000000000ULL << 1) && b < (0x7830000000000000ULL << 1))
            return __fma_rn(x, InvSplit<N>::hi, __dmul_rn(x, InvSplit<N>::lo));
        return ddiv_slow(x, (double)N);
    }
}

__device__ __forceinline__ double wrapd(double dest, double orig, double D) /* wrap_dist :147 */
{
    double d = dest - orig;
    /* D/2 by an exponent decrement (D is a positive normal domain bound) */
    long long b = dbits(d), h = dbits(D) - (1LL << 52);
    if (b > h) return dsub_slow(d, D);                            /* d > +D/2 */
    if (b < 0 && b > h + LLONG_MIN) return dadd_slow(D, d);       /* d < -D/2 */
    return d;
}
/* ---- correctly rounded division and square root for vector2_mag ----
 * On GB300 a binary64 division or square root costs ~10-12 FP64
 * instructions (ncu: 16 for the pair), and the FP64 pipe is the scarce
 * one (1/64 of the binary32 rate).  These versions use none: a binary32
 * seed from the special-function unit is refined on the FP32 pipe to a
 * float-float approximation of the result (~45 bits), its 53-bit
 * significand K is formed on the integer pipe, and the result is then
 * corrected and CERTIFIED in integer arithmetic.  With the operands'
 * significands as integers, the exact quotient or root X lies in one
 * binade [2^52, 2^53) of the integer scale, and K = RN(X) exactly when
 * the remainder (N - K Mp for a quotient N / Mp, M - K^2 for a root of M)
 * lies inside the half-unit band (neither a quotient of two 53-bit
 * significands nor a square root is ever a rounding midpoint).  The
 * remainder is formed as a 128-bit integer (64-bit multiply low and
 * high), so the test is exact; one correction step (remainder times the
 * binary32 reciprocal, rounded to an integer) and a final +-1 bring K to
 * the nearest integer.  A candidate that does not pass (special operands,
 * or a seed too far off) is discarded and the native operation runs, so
 * the returned value is always the correctly rounded one; the error
 * analysis of the seed only bounds how often that happens.  The method is
 * the exact-remainder test of Markstein (P. Markstein, "IA-64 and
 * elementary functions", 2000, ch. 8; J.-M. Muller et al., Handbook of
 * Floating-Point Arithmetic, 2nd ed., 2018, sec. 4.7 and 5.5) carried out
 * on integer significands. */

/* binary32 -> binary64 by bit manipulation (exact for normal x; zero and
 * subnormal x give 0, an error the certification absorbs) */
__device__ __forceinline__ double f2d_bits(float x)
{
    unsigned u = __float_as_uint(x);
    unsigned e = (u >> 23) & 0xffu;
    unsigned long long r = ((unsigned long long)(u & 0x80000000u) << 32) |
                           ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)(u & 0x7fffffu) << 29);
    return e == 0u ? 0.0 : __longlong_as_double((long long)r);
}
/* a binary64 in [1, 2) (bit pattern b) as hi + lo binary32, hi holding
 * the leading 24 bits */
__device__ __forceinline__ void split_unit(long long b, float &hi, float &lo)
{
    hi = __uint_as_float(0x3F800000u | (unsigned)((b >> 29) & 0x7fffffLL));
    lo = __uint2float_rn((unsigned)(b & 0x1fffffffLL)) * 0x1p-52f;
}
/* the same for a positive binary64 of biased exponent 949..1150 */
__device__ __forceinline__ void split_pos(long long b, float &hi, float &lo)
{
    unsigned eb = (unsigned)(b >> 52);
    hi = __uint_as_float(((eb - 896u) << 23) | (unsigned)((b >> 29) & 0x7fffffLL));
    lo = __uint2float_rn((unsigned)(b & 0x1fffffffLL)) * __uint_as_float((eb - 948u) << 23);
}
/* hi + lo as a binary64, on the integer pipe, for binary32 hi > 0 (normal)
 * and |lo| < 2^-8 hi: the 53-bit significand of hi plus lo's significand
 * shifted into its units, renormalised by one bit if needed.  Bits of lo
 * below hi's 53-bit window are cut: the result is within 2^-52 (relative)
 * of hi + lo. */
__device__ __forceinline__ double ff_to_double(float hi, float lo)
{
    unsigned uh = __float_as_uint(hi), ul = __float_as_uint(lo);
    int eh = (int)(uh >> 23), el = (int)((ul >> 23) & 0xffu);
    long long M = (long long)((uh & 0x7fffffu) | 0x800000u) << 29;
    long long ml = (long long)((ul & 0x7fffffu) | 0x800000u);
    int s = el - eh + 29;
    long long add = (el == 0 || s <= -24) ? 0LL : (s >= 0 ? (ml << s) : (ml >> -s));
    M += (int)ul < 0 ? -add : add;
    int e = eh + 896;
    if (M >= (1LL << 53)) { M >>= 1; e++; }
    else if (M < (1LL << 52)) { M <<= 1; e--; }
    return __longlong_as_double(((long long)e << 52) | (M & 0x000FFFFFFFFFFFFFLL));
}
__device__ __forceinline__ float rcp_seed(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float rsqrt_seed(float x)
{
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

constexpr unsigned long long SEVC_MANT = 0x000FFFFFFFFFFFFFULL, SEVC_HIDDEN = 1ULL << 52;

/* r = x - y z for the 128-bit x = (xhi, xlo) and 64-bit y, z, all
 * unsigned, wrapping; true when the difference fits in a signed 64-bit
 * integer (then r is its exact value) */
__device__ __forceinline__ bool rem128(unsigned long long xhi, unsigned long long xlo, unsigned long long y,
                                       unsigned long long z, long long &r)
{
    unsigned long long plo = y * z, phi = __umul64hi(y, z);
    unsigned long long lo = xlo - plo, hi = xhi - phi - (xlo < plo ? 1ULL : 0ULL);
    r = (long long)lo;
    return hi == (unsigned long long)(r >> 63);
}
/* the significand of the binary64 pattern b as an integer aligned to the
 * binade of biased exponent E (2^52 <= result < 2^53 when b's exponent is
 * E); false when b is more than one binade away */
__device__ __forceinline__ bool sig_at(long long b, int E, unsigned long long &K)
{
    int e = (int)(b >> 52);
    unsigned long long M = ((unsigned long long)b & SEVC_MANT) | SEVC_HIDDEN;
    if (e == E) K = M;
    else if (e == E + 1) K = M << 1;
    else if (e == E - 1) K = M >> 1;
    else return false;
    return true;
}
/* binary32 estimate of x / 2^32 for a signed 64-bit x, on the FP32 side */
__device__ __forceinline__ float hi32f(long long x) { return __int2float_rn((int)(x >> 32)); }

/* r = RN(q / p) for 0 <= q <= p; false when not certified */
__device__ __forceinline__ bool div_fast(double q, double p, double &r)
{
    long long pb = dbits(p), qb = dbits(q);
    if (qb == 0) { r = 0.0; return true; }                /* q = +0 */
    int ep = (int)(pb >> 52), eq = (int)(qb >> 52);
    if (eq < 1 || eq > ep || ep > 2046 || ep - eq > 60) return false;
    /* P = p scaled into [1, 2), Q = q by the same power of two (Q / P =
     * q / p, Q >= 2^-60) */
    double P = __longlong_as_double((pb & 0x000FFFFFFFFFFFFFLL) | (1023LL << 52));
    double Q = __longlong_as_double(qb - (long long)(ep - 1023) * (1LL << 52));
    float ph, pl, qh, ql;
    split_unit(dbits(P), ph, pl);
    split_pos(dbits(Q), qh, ql);
    float y0 = rcp_seed(ph);                              /* 1/P to ~2^-23 */
    float e = fmaf(-ph, y0, 1.0f);
    e = fmaf(-pl, y0, e);                                 /* 1 - P y0 to ~2^-46 */
    float yl = y0 * e;                                    /* 1/P ~ y0 + yl to ~2^-45 */
    float ah = qh * y0;                                   /* Q (y0 + yl) as ah + al */
    float al = fmaf(qh, y0, -ah);
    al = fmaf(qh, yl, al);
    al = fmaf(ql, y0, al);
    /* integer scale: X = N / Mp in [2^52, 2^53), the result's biased
     * exponent E */
    unsigned long long Mp = ((unsigned long long)pb & SEVC_MANT) | SEVC_HIDDEN;
    unsigned long long Mq = ((unsigned long long)qb & SEVC_MANT) | SEVC_HIDDEN;
    int up = Mq >= Mp ? 0 : 1;
    int E = eq - ep + 1023 - up, sh = 52 + up;
    unsigned long long Nhi = Mq >> (64 - sh), Nlo = Mq << sh;
    unsigned long long K;
    if (!sig_at(dbits(ff_to_double(ah, al)), E, K)) return false;
    long long R;                                          /* N - K Mp */
    if (!rem128(Nhi, Nlo, K, Mp, R)) return false;
    /* K += R / Mp (1/Mp = y0 2^-52) rounded, then the nearest integer */
    int d = __float2int_rn(hi32f(R) * y0 * 0x1p-20f);
    K += (unsigned long long)(long long)d;
    unsigned long long Ru = (unsigned long long)R - (unsigned long long)(long long)d * Mp;
    long long half = (long long)((Mp - 1) >> 1);          /* |R| < Mp/2 <=> |R| <= half */
    if ((long long)Ru > half) K += 1;
    else if ((long long)Ru < -half) K -= 1;
    if (!rem128(Nhi, Nlo, K, Mp, R) || R > half || R < -half) return false;
    if (K < SEVC_HIDDEN || K > (SEVC_HIDDEN << 1)) return false;
    /* K = 2^53 carries into the exponent */
    r = __longlong_as_double(((long long)E << 52) + (long long)(K - SEVC_HIDDEN));
    return true;
}

/* r = RN(sqrt(t)) for t in [1, 2); false when not certified */
__device__ __forceinline__ bool sqrt_fast(double t, double &r)
{
    long long tb = dbits(t);
    if ((tb >> 52) != 1023) return false;
    float th, tl;
    split_unit(tb, th, tl);
    float y0 = rsqrt_seed(th);                            /* 1/sqrt(t) to ~2^-23 */
    float ah = y0 * y0, al = fmaf(y0, y0, -ah);           /* y0^2 = ah + al exactly */
    float e = fmaf(-th, ah, 1.0f);
    e = fmaf(-th, al, e);
    e = fmaf(-tl, ah, e);                                 /* 1 - t y0^2 to ~2^-46 */
    float yl = 0.5f * (y0 * e);                           /* Newton: 1/sqrt(t) ~ y0 + yl */
    float sh = th * y0;                                   /* t (y0 + yl) as sh + sl */
    float sl = fmaf(th, y0, -sh);
    sl = fmaf(th, yl, sl);
    sl = fmaf(tl, y0, sl);
    /* integer scale: X = sqrt(M) for M = Mt 2^52, X in [2^52, 2^52.5),
     * result exponent 1023; RN(X) = S iff -S < M - S^2 <= S */
    unsigned long long Mt = ((unsigned long long)tb & SEVC_MANT) | SEVC_HIDDEN;
    unsigned long long Mhi = Mt >> 12, Mlo = Mt << 52;
    long long b0 = dbits(ff_to_double(sh, sl));
    unsigned long long S;
    if ((b0 >> 52) == 1022) S = SEVC_HIDDEN;              /* just below 1 */
    else if (!sig_at(b0, 1023, S)) return false;
    long long F;                                          /* M - S^2 */
    if (!rem128(Mhi, Mlo, S, S, F)) return false;
    /* S += F / (2 S) (1/(2S) = y0 2^-53) rounded, then the nearest integer */
    int d = __float2int_rn(hi32f(F) * y0 * 0x1p-21f);
    unsigned long long dd = (unsigned long long)(long long)d;
    unsigned long long Fu = (unsigned long long)F - 2 * S * dd - dd * dd;
    S += dd;
    if ((long long)Fu > (long long)S) S += 1;
    else if ((long long)Fu <= -(long long)S) S -= 1;
    if (!rem128(Mhi, Mlo, S, S, F) || F > (long long)S || F <= -(long long)S) return false;
    if (S < SEVC_HIDDEN || S >= (SEVC_HIDDEN << 1)) return false;
    r = __longlong_as_double((1023LL << 52) + (long long)(S - SEVC_HIDDEN));
    return true;
}

/* vector2_mag (src/geometry.h:217): p sqrt(1 + (q/p)^2) with p = max(|x|,
 * |y|), q = min, every operation correctly rounded as in the reference */
__device__ __forceinline__ double vmag_native(double x, double y)
{
    long long ax = dbits(x) & SEVC_ABSMASK, ay = dbits(y) & SEVC_ABSMASK;
    long long pb = ax > ay ? ax : ay, qb = ax > ay ? ay : ax;    /* fmax / fmin of |x|, |y| */
    if (pb == 0) return 0;
    double p = __longlong_as_double(pb), q = __longlong_as_double(qb);
    double r = q / p;
    return p * sqrt(1.0 + r * r);
}
static __device__ __noinline__ double sqrt_slow(double t) { return sqrt(t); }
/* |x|'s bit pattern, masked in opaque inline PTX (see mag2) */
__device__ __forceinline__ long long absbits(double x)
{
    long long r;
    asm("and.b64 %0, %1, 0x7FFFFFFFFFFFFFFF;" : "=l"(r) : "l"(dbits(x)));
    return r;
}
__device__ __forceinline__ double vmag(double x, double y)      /* vector2_mag :217 */
{
    long long ax = absbits(x), ay = absbits(y);
    long long pb = ax > ay ? ax : ay, qb = ax > ay ? ay : ax;    /* fmax / fmin of |x|, |y| */
    if (pb == 0) return 0;
    double p = __longlong_as_double(pb), q = __longlong_as_double(qb);
    double r, s;
    if (!div_fast(q, p, r)) r = ddiv_slow(q, p);
    double t = 1.0 + r * r;
    if (!sqrt_fast(t, s)) s = sqrt_slow(t);
    return p * s;
}
/* x / SEVC_GRAD_EPS_D, correctly rounded, with one multiplication and one
 * fma instead of a division: the divisor y is known in advance
 * (Brisebarre, Muller and Raina, "Accelerating correctly rounded
 * floating-point division when the divisor is known in advance", IEEE
 * Trans. Computers 53(8), 2004).  With zh = RN(1/y) (exactly 1e8) and
 * zl = RN(1/y - zh), the fma's exact argument x zh + RN(x zl) is within
 * 2^-107.4 of x/y (relative), while the quotient of two 53-bit
 * significands is never within 2^-107 (relative) of a rounding midpoint,
 * so the fma returns RN(x/y).  That holds while x zl stays normal and
 * x/y finite: 2^-990 <= |x| < 2^990; other x (zero, tiny, huge,
 * non-finite) take the division. */
#define SEVC_INV_EPS_HI 0x1.7d784p+26
#define SEVC_INV_EPS_LO (-0x1.1f8eb76e8p-29)
__device__ __forceinline__ double div_grad_eps(double x)
{
    unsigned long long b = mag2(x);
    if (b >= (0x0210000000000000ULL << 1) && b < (0x7DD0000000000000ULL << 1))
        return __fma_rn(x, SEVC_INV_EPS_HI, __dmul_rn(x, SEVC_INV_EPS_LO));
    return ddiv_slow(x, SEVC_GRAD_EPS_D);
}

/* compute_arclength(a, b) = |delta_to(a, b)|, :328 */
__device__ __forceinline__ double arclen(double2 a, double2 b, double D)
{
    return vmag(wrapd(a.x, b.x, D), wrapd(a.y, b.y, D));
}
/* boundary_energy_func, :548 */
__device__ __forceinline__ double gb_energy(double d_alpha, double eps)
{
    return (1 + 0.5 * eps * (1 - pow(cos(4 * d_alpha), 3)));
}

/* Shoelace terms that involve the origin point (0, 0), decided on the
 * integer pipe with IEEE signed-zero rules:
 *  - the first term +0*y1 - (+0)*x1 is +-0, and +0 + (+-0) is +0, so a
 *    sum that starts at +0 is still +0 after it;
 *  - the closing term x*(+0) - y*(+0) is -0 exactly when x has its sign
 *    bit set and y has not (else +0); acc + (+-0) equals acc except that
 *    -0 + +0 is +0. */
__device__ __forceinline__ double add_closing_term(double acc, double x, double y)
{
    if (dbits(acc) == (long long)0x8000000000000000ULL) {
        bool neg = dbits(x) < 0 && dbits(y) >= 0;
        return neg ? acc : 0.0;
    }
    return acc;
}

/* compute_area (src/geometry.h:757-765, with adjust_origin_for_points
 * :908-931) streamed over a grain list: point 0 becomes the origin,
 * later points accumulate wrapped deltas, shoelace terms add in list
 * order.  Slot `ps` (if >= 0) is replaced by position `pp`. */
__device__ __forceinline__ double area_stream(const int *__restrict__ L, int n, const double2 *__restrict__ pos,
                                              int ps, double2 pp, double D)
{
    double area = 0;
    if (n > 0) {
        double2 r0 = (ps == 0) ? pp : pos[L[0]];
        double ax = 0, ay = 0, rx = r0.x, ry = r0.y;
        for (int k = 1; k < n; k++) {
            double2 r = (k == ps) ? pp : pos[L[k]];
            double nx = ax + wrapd(r.x, rx, D);
            double ny = ay + wrapd(r.y, ry, D);
            if (k > 1) area += ax * ny - ay * nx;   /* term k-1; term 0 leaves +0 */
            ax = nx; ay = ny; rx = r.x; ry = r.y;
        }
        area = add_closing_term(area, ax, ay);
    }
    return dscale_down<1>(area);
}

/* grains_intersect, src/geometry.h:837-848; returns count found */
__device__ __forceinline__ int gintersect(int4 a, int4 b, int *out)
{
    int k = 0;
    out[0] = -1; out[1] = -1;
    int A[3] = { a.x, a.y, a.z }, B[3] = { b.x, b.y, b.z };
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            if (A[i] == B[j]) {
                out[k++] = A[i];
                if (k == 2) return k;
            }
    return k;
}
/* compute_boundaries_energies for boundary b (src/calculus.h:100-114):
 * the energy of the misorientation between its two grains, times
 * GB_scaling; isotropic boundaries take 1 * scaling without the
 * transcendental (1 + 0.5 * 0 * (1 - cos^3) is exactly 1 for every finite
 * cosine).  False (energy unset) when the ends share fewer than two
 * grains. */
__device__ __forceinline__ bool boundary_gamma(const DevMesh &m, int b, double eps, double scaling, double &gamma)
{
    if (eps == 0.0) { gamma = 1.0 * scaling; return true; }
    int2 e = m.bv[b];
    int gic[2];
    if (gintersect(m.vg[e.x], m.vg[e.y], gic) < 2) return false;
    gamma = gb_energy(m.gori[gic[0]] - m.gori[gic[1]], eps) * scaling;
    return true;
}
/* grains_union + grains_symdiff, src/geometry.h:863-898 */
__device__ __forceinline__ void gsymdiff(int4 a, int4 b, int *out)
{
    int gic[2], gun[4];
    gintersect(a, b, gic);
    gun[0] = a.x; gun[1] = a.y; gun[2] = a.z; gun[3] = -1;
    int B[3] = { b.x, b.y, b.z };
    for (int i = 0; i < 3; i++)
        if (B[i] != gun[0] && B[i] != gun[1] && B[i] != gun[2]) { gun[3] = B[i]; break; }
    int k = 0;
    out[0] = -1; out[1] = -1;
    for (int i = 0; i < 4; i++)
        if (gun[i] != gic[0] && gun[i] != gic[1]) {
            out[k++] = gun[i];
            if (k == 2) return;
        }
}

__device__ __forceinline__ int slot3(int4 s, int i) { return i == 0 ? s.x : (i == 1 ? s.y : s.z); }
__device__ __forceinline__ void set_slot3(int4 &s, int i, int v)
{
    if (i == 0) s.x = v; else if (i == 1) s.y = v; else s.z = v;
}
__device__ __forceinline__ int other_end(int2 e, int v) { return e.x == v ? e.y : e.x; }

__device__ __forceinline__ void raise_err(const DevMesh &m, int bits) { atomicOr(m.err, bits); }

/* compute_t_ext for one boundary (src/topological.h:303-334): ends at
 * pi, pe with velocities vi, ve */
__device__ __forceinline__ double text_exact(double2 pi, double2 pe, double2 vi, double2 ve, double D)
{
    double dx = 0.0 + wrapd(pe.x, pi.x, D);   /* adjust_origin_for_points on 2 points */
    double dy = 0.0 + wrapd(pe.y, pi.y, D);
    dx = dx - 0.0;
    dy = dy - 0.0;
    double norm = vmag(dx, dy);
    double tx = 0, ty = 0;
    if (norm != 0) {                          /* vector2_unitary, src/geometry.h:274 */
        double ang = atan2(dy, dx);
        tx = cos(ang);
        ty = sin(ang);
    }
    double aux = tx * (ve.x - vi.x) + ty * (ve.y - vi.y);
    return (aux == 0) ? 100 : -norm / aux;
}
/* text_exact as a call, for kernels where it is the rare branch (keeps its
 * FP64 work from being speculated into the common path) */
static __device__ __noinline__ double text_exact_call(double2 pi, double2 pe, double2 vi, double2 ve, double D)
{
    return text_exact(pi, pe, vi, ve, D);
}

/* binary64 -> binary32 by cutting the significand, on the integer pipe:
 * for 2^-126 <= |x| < 2^128 the result has x's sign and
 * (1 - 2^-23)|x| < |r| <= |x|; smaller |x| give +-0 (error < 2^-126);
 * larger or non-finite x give NaN, which fails every comparison. */
__device__ __forceinline__ float f32_cut(double x)
{
    unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    unsigned e = (hi >> 20) & 0x7ffu;
    unsigned mag = ((e - 896u) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
    mag = e <= 896u ? 0u : mag;
    mag = e >= 1151u ? 0x7fc00000u : mag;
    return __uint_as_float((hi & 0x80000000u) | mag);
}

/* Upper bound of |vx| + |vy| in binary32, on the integer and FP32 pipes:
 * f32_cut(x) is within a factor (1 - 2^-23) of x for normal binary32
 * magnitudes, so scaling it up by 1 + 2^-21 (rounded up) and adding the
 * largest magnitude it maps to 0 covers |x|; non-finite and huge x give
 * NaN or infinity, which no comparison passes. */
__device__ __forceinline__ float speed_bound(double vx, double vy)
{
    float ax = fabsf(f32_cut(vx)), ay = fabsf(f32_cut(vy));
    const float up = 1.0f + 0x1p-21f;
    return __fadd_ru(__fadd_ru(__fmul_ru(ax, up), __fmul_ru(ay, up)), 0x1p-125f);
}

/* True when compute_t_ext (src/topological.h:303-334) of the boundary
 * from pi to pe, ends moving at vi, ve, is certainly outside [0, dt]
 * (dt < 100), decided in binary32 so that the FP64 pipe stays free.
 *
 * With d = wrapped pe - pi and p = ve - vi, the reference's t_ext is
 * -|d|^2 / (d.p) up to relative rounding of order 1e-15 (the unit
 * tangent comes from atan2/cos/sin), and 100 when d.p rounds to 0; it is
 * a candidate only if s + |d|^2/dt <= 0 for s = d.p, within that
 * rounding.  Every input is cut to binary32 (f32_cut, relative error
 * below 2^-23, plus 2^-126 absolute for tiny values), and each binary32
 * quantity carries a bound on its distance from the exact value:
 *   |X - dx| <= ex = 2.5e-7 (|pe.x| + |pi.x| + D) + 1e-37 (two cuts,
 *     the rounded difference and, after a wrap, the cut D and one more
 *     rounding: at most 1.5 * 2^-23 of the same sum), same for y;
 *   |P - px| <= 2.5e-7 (|ve.x| + |vi.x|) + 1e-37, same for y;
 *   |S - s| <= A Ep + B Ex and |N - |d|^2| <= 2 A Ex, with Ex, Ep the
 *     summed bounds, A = |X| + |Y| + Ex >= |dx| + |dy| and
 *     B = |P| + |Q| + Ep >= |px| + |py|.
 * The rounding of the binary32 evaluation itself (a few 2^-24 of
 * A B + N/dt) and the reference's own rounding fit in the further
 * 1e-6 (A B + (N + 2 A Ex)/dt), and 1.001 covers the rounding of the bound.
 * The wrap (wrap_dist, |d| > D/2) is decided the reference's way only
 * outside a band of relative width 1e-5 plus ex around D/2; inside it,
 * for |d|^2 below 1e-30 and for NaN or overflow the answer is false, and
 * the caller computes t_ext exactly. */
__device__ __forceinline__ bool text_outside_dt(double2 pi, double2 pe, double2 vi, double2 ve, float Df, float hDf,
                                                float inv_dt)
{
    float ax = f32_cut(pe.x), bx = f32_cut(pi.x), ay = f32_cut(pe.y), by = f32_cut(pi.y);
    float X = ax - bx, Y = ay - by;
    float ex = 2.5e-7f * (fabsf(ax) + fabsf(bx) + Df) + 1e-37f;
    float ey = 2.5e-7f * (fabsf(ay) + fabsf(by) + Df) + 1e-37f;
    float lo = 0.99999f * hDf, hi = 1.00001f * hDf, aX = fabsf(X), aY = fabsf(Y);
    if ((aX > lo - ex && aX < hi + ex) || (aY > lo - ey && aY < hi + ey)) return false;
    if (X > hDf) X = X - Df; else if (X < -hDf) X = X + Df;
    if (Y > hDf) Y = Y - Df; else if (Y < -hDf) Y = Y + Df;
    float vex = f32_cut(ve.x), vix = f32_cut(vi.x), vey = f32_cut(ve.y), viy = f32_cut(vi.y);
    float P = vex - vix, Q = vey - viy;
    float Ex = ex + ey, Ep = 2.5e-7f * (fabsf(vex) + fabsf(vix) + fabsf(vey) + fabsf(viy)) + 2e-37f;
    float A = fabsf(X) + fabsf(Y) + Ex, B = fabsf(P) + fabsf(Q) + Ep;
    float S = X * P + Y * Q, N = X * X + Y * Y;
    float ni = N * inv_dt, ai = 2.0f * A * Ex * inv_dt;
    float E = A * Ep + B * Ex + ai + 1e-6f * (A * B + ni + ai);
    return N > 1e-30f && S + ni > 1.001f * E;
}

/* compute_dAdt (src/geometry.h:779-787) of grain g over its list; get(v,
 * r, w) gives vertex v's position and velocity */
template <class Get> __device__ __forceinline__ double dadt_over(const DevMesh &m, int g, Get get)
{
    const int *L = m.glist + (size_t)SEVC_MAXV * g;
    int n = m.gvlen[g];
    double d = 0;
    if (n > 0) {
        double2 r0, v0;
        get(L[0], r0, v0);
        double ax = 0, ay = 0, rx = r0.x, ry = r0.y, vxk = v0.x, vyk = v0.y;
        for (int k = 1; k < n; k++) {
            double2 r, w;
            get(L[k], r, w);
            double nx = ax + wrapd(r.x, rx, m.D);
            double ny = ay + wrapd(r.y, ry, m.D);
            d += (vxk * ny + ax * w.y);
            d -= (vyk * nx + ay * w.x);
            ax = nx; ay = ny; rx = r.x; ry = r.y; vxk = w.x; vyk = w.y;
        }
        d += (vxk * 0.0 + ax * v0.y);
        d -= (vyk * 0.0 + ay * v0.x);
    }
    return d;
}
__device__ __forceinline__ double dadt_from(const DevMesh &m, int g, const double2 *pos, const double2 *vel)
{
    return dadt_over(m, g, [&](int v, double2 &r, double2 &w) { r = pos[v]; w = vel[v]; });
}

/* an event is about to overwrite vertex v's position or velocity: keep
 * the step's starting values (once per step) */
__device__ __forceinline__ void save_vertex(const DevMesh &m, int v)
{
    unsigned st = *m.stamp;
    if (m.vstamp[v] == st) return;
    m.pos0[v] = m.pos[v];
    m.vel0[v] = m.vel[v];
    m.vstamp[v] = st;
}
/* an event is about to change boundary b's ends */
__device__ __forceinline__ void save_ends(const DevMesh &m, int b)
{
    unsigned st = *m.stamp;
    if (m.bstamp[b] == st) return;
    m.bv0[b] = m.bv[b];
    m.bstamp[b] = st;
}
/* position and velocity of vertex v when the step's events began */
__device__ __forceinline__ void start_state(const DevMesh &m, int v, unsigned st, double2 &p, double2 &w)
{
    bool saved = m.vstamp[v] == st;
    p = saved ? m.pos0[v] : m.pos[v];
    w = saved ? m.vel0[v] : m.vel[v];
}

/* an event is about to disable boundary b: make its extinction time the
 * value the step's labels would have computed */
__device__ __forceinline__ void finalize_boundary(const DevMesh &m, int b)
{
    if (m.bexact[b]) return;
    unsigned st = *m.stamp;
    int2 e = m.bstamp[b] == st ? m.bv0[b] : m.bv[b];
    double2 pi, pe, vi, ve;
    start_state(m, e.x, st, pi, vi);
    start_state(m, e.y, st, pe, ve);
    m.btext[b] = text_exact(pi, pe, vi, ve, m.D);
    m.bexact[b] = 1;
}
/* an event is about to edit grain g's list (or disable it): its dA/dt as
 * the step computed it before any event.  The list itself is still the
 * step's: lists change only in the fix-up pass, after mark_fix has
 * settled every grain it edits. */
__device__ __forceinline__ void finalize_grain(const DevMesh &m, int g)
{
    if (m.gexact[g]) return;
    unsigned st = *m.stamp;
    m.gdadt[g] = dadt_over(m, g, [&](int v, double2 &r, double2 &w) { start_state(m, v, st, r, w); });
    m.gexact[g] = 1;
}

/* first position of an ascending list whose value is >= x */
__device__ __forceinline__ int lower_bound_i(const int *a, int n, int x)
{
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (a[mid] < x) lo = mid + 1; else hi = mid;
    }
    return lo;
}

#endif
