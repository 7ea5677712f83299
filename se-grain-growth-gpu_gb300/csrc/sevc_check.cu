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

void launch_check(const DevMesh &m, int *out, cudaStream_t s)
{
    cudaMemsetAsync(out, 0, sizeof(int), s);
    COUNT_LAUNCHES(1), k_check_boundaries<<<(m.nb + TPB - 1) / TPB, TPB, 0, s>>>(m, out);
    COUNT_LAUNCHES(1), k_check_vertices<<<(m.nv + TPB - 1) / TPB, TPB, 0, s>>>(m, out);
    COUNT_LAUNCHES(1), k_check_grains<<<(m.ng + TPB - 1) / TPB, TPB, 0, s>>>(m, out);
}
