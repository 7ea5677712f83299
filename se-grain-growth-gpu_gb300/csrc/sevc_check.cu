/*
 * Mesh invariants on the device: the checks of check_data
 * (src/utils.h:85-336, the tests that set is_valid = false), one thread
 * per boundary, vertex and grain, counted into one integer.  The host
 * restatement in sevc_host.c (sevc_host_check) counts the same violations
 * in the same way.  An index outside its array counts as one violation and
 * is not followed, so a damaged mesh is reported, never read out of bounds.
 */
#include "sevc_internal.h"
#include "sevc_host.h"

namespace {

constexpr int TPB = 256;

__device__ __forceinline__ bool inr(int x, int n) { return (unsigned)x < (unsigned)n; }

__device__ __forceinline__ void add_count(int *out, int bad)
{
    int s = bad;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0 && s) atomicAdd(out, s);
}

__device__ __forceinline__ bool in_list(const DevMesh &m, int g, int v)
{
    const int *L = m.glist + (size_t)SEVC_MAXV * g;
    int n = min(max(m.gvlen[g], 0), SEVC_MAXV);
    for (int i = 0; i < n; i++)
        if (L[i] == v) return true;
    return false;
}

/* src/utils.h:85-158, per enabled boundary */
__global__ void k_check_boundaries(DevMesh m, int *out)
{
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    int bad = 0;
    if (b < m.nb && m.ben[b]) {
        int2 e = m.bv[b];
        if (!inr(e.x, m.nv) || !inr(e.y, m.nv)) {
            bad = 1;
        } else {
            int4 sa = m.vb[e.x], sc = m.vb[e.y];
            bad += e.x == e.y;
            bad += !m.ven[e.x] || !m.ven[e.y];
            bad += sa.x != b && sa.y != b && sa.z != b;
            bad += sc.x != b && sc.y != b && sc.z != b;
            int s[6] = { sc.x, sc.y, sc.z, sa.x, sa.y, sa.z };
            bool ok_c = true, ok_a = true;
            for (int j = 0; j < 6; j++) {
                bool ok = inr(s[j], m.nb) && m.ben[s[j]];
                if (j < 3) ok_c &= ok; else ok_a &= ok;
            }
            bad += !ok_c;
            bad += !ok_a;
            int gic[2];
            int k = gintersect(m.vg[e.x], m.vg[e.y], gic);
            bad += k < 2 || gic[0] == gic[1];
        }
    }
    add_count(out, bad);
}

/* src/utils.h:160-280, per enabled vertex */
__global__ void k_check_vertices(DevMesh m, int *out)
{
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    int bad = 0;
    if (v < m.nv && m.ven[v]) {
        int4 s4 = m.vb[v], g4 = m.vg[v];
        int s[3] = { s4.x, s4.y, s4.z }, g[3] = { g4.x, g4.y, g4.z }, nb[3] = { -1, -2, -3 };
        bad += s[0] == s[1] || s[1] == s[2] || s[2] == s[0];
        bad += g[0] == g[1] || g[1] == g[2] || g[2] == g[0];
        for (int j = 0; j < 3; j++) {
            bool gok = inr(g[j], m.ng);
            bad += !gok || !m.gen[g[j]];
            bad += !gok || !in_list(m, g[j], v);
            if (!inr(s[j], m.nb)) { bad += 1; continue; }
            int2 e = m.bv[s[j]];
            bad += !m.ben[s[j]];
            bad += e.x == e.y;
            nb[j] = e.x == v ? e.y : e.x;
            bad += e.x != v && e.y != v;
        }
        bad += nb[0] == nb[1] || nb[1] == nb[2] || nb[2] == nb[0];
    }
    add_count(out, bad);
}

/* src/utils.h:282-336, per enabled grain */
__global__ void k_check_grains(DevMesh m, int *out)
{
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    int bad = 0;
    if (g < m.ng && m.gen[g]) {
        const int *L = m.glist + (size_t)SEVC_MAXV * g;
        int n = m.gvlen[g];
        if (n < 0 || n > SEVC_MAXV) {
            bad = 1;
        } else {
            bool listed = true;
            for (int j = 0; j < n; j++) {
                if (!inr(L[j], m.nv)) { bad++; listed = false; continue; }
                bad += !m.ven[L[j]];
            }
            for (int j = 0; j < n && listed; j++) {
                int4 s = m.vg[L[j]];
                if (s.x != g && s.y != g && s.z != g) { bad++; break; }
            }
            int cnt = 0;
            for (int j = 0; j < SEVC_MAXV; j++) cnt += L[j] != -1;
            bad += cnt != n;
        }
    }
    add_count(out, bad);
}

/* FP64 issue-rate probe: 8 independent fused multiply-add chains per
 * thread, so the pipe, not latency, limits the rate */
__global__ void k_fp64_rate(int iters, double a, double b, double *sink)
{
    double x[8];
    for (int k = 0; k < 8; k++) x[k] = threadIdx.x * 1e-3 + k;
    for (int i = 0; i < iters; i++)
#pragma unroll
        for (int k = 0; k < 8; k++) x[k] = fma(x[k], a, b);
    double s = 0;
    for (int k = 0; k < 8; k++) s += x[k];
    if (s == 12345.678) *sink = s;   /* keeps the chains live */
}


/* ---- state digests (sevc_state_digest) ---- */
__device__ __forceinline__ unsigned long long digest_mix(unsigned long long z)   /* splitmix64 finaliser */
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
__device__ __forceinline__ unsigned long long ubits(int v) { return (unsigned long long)(unsigned)v; }
__device__ __forceinline__ unsigned long long ubits(double v) { return (unsigned long long)__double_as_longlong(v); }

/* elements of field f in the layout of sevc_get_state */
__device__ long long digest_len(const DevMesh &m, int f)
{
    if (f < 5) return m.nv;
    if (f < 7) return 3LL * m.nv;
    if (f < 13) return m.nb;
    if (f == 13) return (long long)SEVC_MAXV * m.ng;
    return m.ng;
}
__device__ unsigned long long digest_bits(const DevMesh &m, int f, long long i)
{
    switch (f) {
    case 0: return ubits(m.pos[i].x);
    case 1: return ubits(m.pos[i].y);
    case 2: return ubits(m.vel[i].x);
    case 3: return ubits(m.vel[i].y);
    case 4: return m.ven[i];
    case 5: return ubits(slot3(m.vb[i / 3], (int)(i % 3)));
    case 6: return ubits(slot3(m.vg[i / 3], (int)(i % 3)));
    case 7: return ubits(m.bv[i].x);
    case 8: return ubits(m.bv[i].y);
    case 9: return ubits(m.benergy[i]);
    case 10: return ubits(m.blen[i]);
    case 11: return m.ben[i];
    case 12: return m.bcand[i];
    case 13: return ubits(m.glist[i]);
    case 14: return ubits(m.gvlen[i]);
    case 15: return ubits(m.garea[i]);
    case 16: return ubits(m.gori[i]);
    case 17: return ubits(m.gse[i]);
    case 18: return m.gen[i];
    default: return m.gtype[i];
    }
}
/* blockIdx.y = field; the sum is order-independent, so the result does
 * not depend on the launch shape */
__global__ void k_digest(DevMesh m, unsigned long long *out)
{
    const int f = blockIdx.y;
    const long long n = digest_len(m, f);
    const unsigned long long salt = (unsigned long long)f << 56;
    unsigned long long acc = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        acc += digest_mix(salt + (unsigned long long)i * 0x9E3779B97F4A7C15ULL + digest_bits(m, f, i));
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out + f, acc);
}

} // namespace

/* FP64 multiply-add instructions (thread operations) per second on the
 * current device, measured with CUDA events */
extern "C" sevc_status sevc_measure_fp64_rate(double *ops_per_s)
{
    if (!ops_per_s) return SEVC_ERR_ARG;
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return SEVC_ERR_CUDA;
    double *sink = nullptr;
    cudaEvent_t e0, e1;
    if (cudaMalloc(&sink, sizeof(double)) != cudaSuccess) return SEVC_ERR_CUDA;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int blocks = nsm * 8, threads = 256, iters = 4096;
    COUNT_LAUNCHES(1), k_fp64_rate<<<blocks, threads>>>(64, 1.0000001, 1e-9, sink);   /* warm-up */
    cudaEventRecord(e0);
    COUNT_LAUNCHES(1), k_fp64_rate<<<blocks, threads>>>(iters, 1.0000001, 1e-9, sink);
    cudaEventRecord(e1);
    float ms = 0;
    bool ok = cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess && ms > 0;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    if (!ok) return SEVC_ERR_CUDA;
    *ops_per_s = (double)blocks * threads * iters * 8 / (ms * 1e-3);
    return SEVC_OK;
}

/* ---- self-test of the certified division / square root (vmag) ---- */
__device__ __forceinline__ unsigned long long mix64(unsigned long long z)   /* splitmix64 finaliser */
{
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
/* a double in [1, 2) from 52 random bits, times 2^k */
__device__ __forceinline__ double unit_pow2(unsigned long long u, int k)
{
    return __longlong_as_double((long long)((u & 0x000FFFFFFFFFFFFFULL) | ((unsigned long long)(1023 + k) << 52)));
}

/* counts: 0 divisions, 1 division mismatches, 2 divisions not certified,
 * 3 square roots, 4 square-root mismatches, 5 not certified, 6 vmag
 * evaluations, 7 vmag mismatches (a mismatch is a certified result whose
 * bits differ from the native operation's) */
__global__ void k_selftest_arith(long long n, unsigned long long seed, unsigned long long *counts)
{
    unsigned long long c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        unsigned long long a = mix64(seed ^ (2 * i)), b = mix64(seed ^ (2 * i + 1)), kind = (a >> 60) & 7;
        /* division q / p with 0 <= q <= p */
        int kp = (int)((b >> 56) % 121) - 60;
        double p = unit_pow2(b, kp), q;
        if (kind < 4) {
            q = p * unit_pow2(a, -1 - (int)((a >> 52) & 7));          /* a general ratio */
        } else if (kind < 7) {
            /* q = RN(p m) for a rounding midpoint m = k 2^-53 + 2^-54 of (1/2, 1) */
            double kd = __longlong_as_double((long long)((a & 0x000FFFFFFFFFFFFFULL) | (1022ULL << 52)));
            q = __fma_rn(p, kd, p * 0x1p-54);
            if (kind == 6) q = __longlong_as_double(dbits(q) + (((a >> 59) & 1) ? 1 : -1));
            if (dbits(q) > dbits(p)) q = p;
        } else {
            int w = (int)((a >> 40) & 3);
            q = w == 0 ? p : (w == 1 ? 0.0 : p * 0x1p-1040);            /* r = 1, 0, subnormal q */
        }
        double r;
        c[0]++;
        if (div_fast(q, p, r)) { if (dbits(r) != dbits(q / p)) c[1]++; }
        else c[2]++;
        /* square root of t in [1, 2) */
        double t;
        if (kind < 4) {
            t = unit_pow2(a, 0);
        } else {
            /* t = RN(m^2) next to the square of a midpoint m = s + 2^-53 */
            double s = unit_pow2(a, 0);
            if (s > 1.4142135623730950) s = s - 0.4142135623730950;
            t = __fma_rn(s, s, s * 0x1p-52);
            if (kind == 6) t = __longlong_as_double(dbits(t) + (((a >> 59) & 1) ? 1 : -1));
            if ((dbits(t) >> 52) != 1023) t = 1.5;
        }
        c[3]++;
        if (sqrt_fast(t, r)) { if (dbits(r) != dbits(sqrt(t))) c[4]++; }
        else c[5]++;
        /* whole vector2_mag on coordinates of random sign and scale */
        double x = unit_pow2(mix64(a), (int)(b & 63) - 32), y = unit_pow2(mix64(b), (int)((a >> 8) & 63) - 32);
        if (kind == 7) y = ((a >> 44) & 1) ? x : 0.0;
        if ((a >> 48) & 1) x = -x;
        if ((b >> 48) & 1) y = -y;
        c[6]++;
        if (dbits(vmag(x, y)) != dbits(vmag_native(x, y))) c[7]++;
    }
    for (int k = 0; k < 8; k++) {
        unsigned long long v = c[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0 && v) atomicAdd(counts + k, v);
    }
}

extern "C" sevc_status sevc_selftest_arith(long long n, unsigned long long seed, long long *counts)
{
    if (!counts || n < 0) return SEVC_ERR_ARG;
    unsigned long long *d = nullptr;
    if (cudaMalloc(&d, 8 * sizeof(unsigned long long)) != cudaSuccess) return SEVC_ERR_CUDA;
    bool ok = cudaMemset(d, 0, 8 * sizeof(unsigned long long)) == cudaSuccess;
    if (ok) {
        COUNT_LAUNCHES(1), k_selftest_arith<<<152 * 8, 256>>>(n, seed, d);
        unsigned long long h[8];
        ok = cudaGetLastError() == cudaSuccess && cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost) == cudaSuccess;
        for (int k = 0; ok && k < 8; k++) counts[k] = (long long)h[k];
    }
    cudaFree(d);
    return ok ? SEVC_OK : SEVC_ERR_CUDA;
}

void launch_check(const DevMesh &m, int *out, cudaStream_t s)
{
    cudaMemsetAsync(out, 0, sizeof(int), s);
    COUNT_LAUNCHES(1), k_check_boundaries<<<(m.nb + TPB - 1) / TPB, TPB, 0, s>>>(m, out);
    COUNT_LAUNCHES(1), k_check_vertices<<<(m.nv + TPB - 1) / TPB, TPB, 0, s>>>(m, out);
    COUNT_LAUNCHES(1), k_check_grains<<<(m.ng + TPB - 1) / TPB, TPB, 0, s>>>(m, out);
}

void launch_digest(const DevMesh &m, unsigned long long *out, cudaStream_t s)
{
    long long n = (long long)SEVC_MAXV * m.ng;
    long long gx = (n + TPB - 1) / TPB;
    if (gx > 4 * 152) gx = 4 * 152;
    if (gx < 1) gx = 1;
    COUNT_LAUNCHES(1), k_digest<<<dim3((unsigned)gx, SEVC_DIGEST_FIELDS), TPB, 0, s>>>(m, out);
}
