/*
 * Topological transitions of one time step (src/topological.h of the
 * reference): candidate compaction, the polling system, conflict
 * resolution, removal of adjacent 3-sided pairs, 3-sided grain removal,
 * T1 flips and the deferred grain-list edits.
 *
 * Candidates are gathered by an order-preserving warp-ballot compaction,
 * so every later pass touches only the few boundaries and grains that can
 * change.  Edits whose order is observable run in ascending index order,
 * like the reference's single-thread kernels; the list edits
 * (ADD -> REMOVE -> REPLACE) touch only the grain being edited and run one
 * thread per grain, which gives the reference's serial result.
 */
#include "sevc_internal.h"

namespace {

constexpr int TPB = 256;
constexpr int CT_ITEMS = 16;
constexpr int CT_TILE = TPB * CT_ITEMS;
constexpr int WL_BLOCKS = 152;

/* ------------------------------------------------------------------ */
/* grain-list primitives, src/geometry.h:614-734                       */
/* ------------------------------------------------------------------ */
__device__ int glist_find(const DevMesh &m, int g, int v)          /* grain_contains_vertex :703 */
{
    const int *L = m.glist + (size_t)SEVC_MAXV * g;
    int n = m.gvlen[g];
    for (int i = 0; i < n; i++)
        if (L[i] == v) return i;
    return -1;
}
__device__ int glist_consecutive(const DevMesh &m, int g, int A, int B) /* :724 */
{
    const int *L = m.glist + (size_t)SEVC_MAXV * g;
    int n = m.gvlen[g];
    for (int i = 0; i < n; i++) {
        if (L[i] == A && L[(i + 1) % n] == B) return 1;
        if (L[i] == B && L[(i + 1) % n] == A) return 2;
    }
    return -1;
}
__device__ void glist_add_after(const DevMesh &m, int g, int v, int prev) /* :629 */
{
    int *L = m.glist + (size_t)SEVC_MAXV * g;
    int n = m.gvlen[g], pos = -1;
    for (int i = 0; i < n; i++)
        if (L[i] == prev) { pos = i + 1; break; }
    if (pos < 0) { raise_err(m, ERRB_TOPOLOGY); return; }
    if (n >= SEVC_MAXV) { raise_err(m, ERRB_CAPACITY); return; }
    for (int i = n; i > pos; i--) L[i] = L[i - 1];
    L[pos] = v;
    m.gvlen[g] = n + 1;
}
__device__ void glist_remove(const DevMesh &m, int g, int v)      /* :653 */
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
__device__ void glist_replace(const DevMesh &m, int g, int oldv, int newv) /* :686 */
{
    int *L = m.glist + (size_t)SEVC_MAXV * g;
    int n = m.gvlen[g];
    for (int i = 0; i < n; i++)
        if (L[i] == oldv) { L[i] = newv; return; }
}

/* Set flags[i] (a 0/1 byte) to 1; true for the one caller that changed
 * it.  Events that run concurrently may queue the same grain. */
__device__ __forceinline__ bool claim_byte(uint8_t *flags, int i)
{
    uintptr_t a = (uintptr_t)(flags + i);
    unsigned bit = 1u << (8 * (unsigned)(a & 3));
    return !(atomicOr((unsigned *)(a & ~(uintptr_t)3), bit) & bit);
}
/* queue a grain for the fix-up pass (grain.fix = true); its list is
 * about to change, so its dA/dt for this step is settled first */
__device__ void mark_fix(const DevMesh &m, int g)
{
    finalize_grain(m, g);
    if (!claim_byte(m.gfix, g)) return;
    int i = atomicAdd(m.nfix, 1);
    if (i < m.fixcap) m.fixlist[i] = g; else raise_err(m, ERRB_WORKLIST);
}
/* write a deferred edit into vertex v's mod slot (mod_t, src/geometry.h:26);
 * prev < -1 keeps the slot's previous vrt_prev_id, as the reference does
 * when it only assigns fix/vrt/grn */
__device__ void set_mod(const DevMesh &m, int v, int slot, int fix, int grn, int vrt, int prev)
{
    int4 *md = m.vmod + 4 * (size_t)v + slot;
    int4 x = *md;
    x.x = grn; x.y = vrt; if (prev >= -1) x.z = prev; x.w = fix;
    *md = x;
    if (!m.vmodmark[v]) {
        m.vmodmark[v] = 1;
        int i = atomicAdd(m.nmod, 1);
        if (i < m.modcap) m.modlist[i] = v; else raise_err(m, ERRB_WORKLIST);
    }
}

/* ------------------------------------------------------------------ */
/* order-preserving compaction                                         */
/* ------------------------------------------------------------------ */
template <int KIND>
__device__ __forceinline__ bool pred(const DevMesh &m, int i)
{
    if (KIND == CK_CAND) return m.ben[i] && m.bcand[i];
    if (KIND == CK_GRAIN_CAND) return m.gen[i] && m.gcand[i];
    if (KIND == CK_GVLEN3) return m.gvlen[i] == 3;
    if (KIND == CK_MARKED) return m.bmark[i] != 0;
    /* CK_TWO_THREE: enabled boundary whose two common grains both have
     * three vertices (src/topological.h:31-35, :970-974) */
    if (!m.ben[i]) return false;
    int2 e = m.bv[i];
    int gic[2];
    if (gintersect(m.vg[e.x], m.vg[e.y], gic) < 2) return false;
    return m.gvlen[gic[0]] == 3 && m.gvlen[gic[1]] == 3;
}

template <int KIND>
__global__ void k_compact_count(DevMesh m, int n, int *blockcnt)
{
    int base = blockIdx.x * CT_TILE, c = 0;
    for (int k = 0; k < CT_ITEMS; k++) {
        int i = base + k * TPB + threadIdx.x;
        if (i < n && pred<KIND>(m, i)) c++;
    }
    __shared__ int s[TPB / 32];
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < TPB / 32; w++) t += s[w];
        blockcnt[blockIdx.x] = t;
    }
}

template <int KIND>
__global__ void k_compact_scatter(DevMesh m, int n, const int *blockcnt, int *out, int *n_out)
{
    __shared__ int s[TPB / 32 + 1];
    __shared__ int base_off;
    int part = 0;
    for (int j = threadIdx.x; j < (int)blockIdx.x; j += TPB) part += blockcnt[j];
    for (int o = 16; o > 0; o >>= 1) part += __shfl_down_sync(0xffffffffu, part, o);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = part;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < TPB / 32; w++) t += s[w];
        base_off = t;
    }
    __syncthreads();
    int off = base_off;
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int k = 0; k < CT_ITEMS; k++) {
        int i = blockIdx.x * CT_TILE + k * TPB + threadIdx.x;
        bool f = i < n && pred<KIND>(m, i);
        unsigned bal = __ballot_sync(0xffffffffu, f);
        __syncthreads();
        if (lane == 0) s[warp] = __popc(bal);
        __syncthreads();
        if (threadIdx.x == 0) {
            int acc = 0;
            for (int w = 0; w < TPB / 32; w++) { int t = s[w]; s[w] = acc; acc += t; }
            s[TPB / 32] = acc;
        }
        __syncthreads();
        if (f) out[off + s[warp] + __popc(bal & ((1u << lane) - 1))] = i;
        off += s[TPB / 32];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) *n_out = off;
}

/* The same compaction for the kinds whose predicate is a byte flag (or the
 * AND of two): each thread owns 16 consecutive items, read as one 16-byte
 * word per flag array, so a tile costs one round trip to memory instead of
 * sixteen.  Items keep ascending order (thread order, then bit order).
 * Flag arrays are allocated in 256-byte multiples, so the word of the last
 * partial group stays inside its allocation; items >= n are masked off. */
template <int KIND>
__device__ __forceinline__ unsigned flag_mask16(const DevMesh &m, int i0, int n)
{
    const uint8_t *a = KIND == CK_CAND ? m.ben : (KIND == CK_GRAIN_CAND ? m.gen : m.bmark);
    uint4 w = *reinterpret_cast<const uint4 *>(a + i0);
    if constexpr (KIND == CK_CAND || KIND == CK_GRAIN_CAND) {
        const uint8_t *b = KIND == CK_CAND ? m.bcand : m.gcand;
        uint4 v = *reinterpret_cast<const uint4 *>(b + i0);
        w.x &= v.x; w.y &= v.y; w.z &= v.z; w.w &= v.w;   /* flags are 0 / 1 */
    }
    unsigned q[4] = { w.x, w.y, w.z, w.w }, mask = 0;
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
        for (int k = 0; k < 4; k++)
            mask |= (((q[j] >> (8 * k)) & 0xffu) != 0u ? 1u : 0u) << (4 * j + k);
    int valid = n - i0;
    return valid >= 16 ? mask : (mask & ((1u << valid) - 1u));
}
template <int KIND>
__global__ void k_flag_count(DevMesh m, int n, int *blockcnt)
{
    griddep_wait();
    int i0 = (blockIdx.x * TPB + threadIdx.x) * CT_ITEMS;
    int c = i0 < n ? __popc(flag_mask16<KIND>(m, i0, n)) : 0;
    __shared__ int s[TPB / 32];
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < TPB / 32; w++) t += s[w];
        blockcnt[blockIdx.x] = t;
    }
}
template <int KIND>
__global__ void k_flag_scatter(DevMesh m, int n, const int *blockcnt, int *out, int *n_out)
{
    griddep_wait();
    __shared__ int s[TPB / 32];
    __shared__ int base_off, tot;
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int part = 0;
    for (int j = threadIdx.x; j < (int)blockIdx.x; j += TPB) part += blockcnt[j];
    for (int o = 16; o > 0; o >>= 1) part += __shfl_down_sync(0xffffffffu, part, o);
    if (lane == 0) s[warp] = part;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < TPB / 32; w++) t += s[w];
        base_off = t;
    }
    __syncthreads();
    int i0 = (blockIdx.x * TPB + threadIdx.x) * CT_ITEMS;
    unsigned mask = i0 < n ? flag_mask16<KIND>(m, i0, n) : 0u;
    int c = __popc(mask), incl = c;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) s[warp] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int w = 0; w < TPB / 32; w++) { int t = s[w]; s[w] = acc; acc += t; }
        tot = acc;
    }
    __syncthreads();
    int pos = base_off + s[warp] + incl - c;
    while (mask) {
        int k = __ffs(mask) - 1;
        mask &= mask - 1;
        out[pos++] = i0 + k;
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) *n_out = base_off + tot;
}

/* ------------------------------------------------------------------ */
/* polling system, src/topological.h:362-578                           */
/* ------------------------------------------------------------------ */
/* vertices_vote (:362) for the endpoints of listed boundaries; it also
 * zeroes the iteration's count of unconverged instances (the previous
 * iteration's was read before this kernel starts) */
__global__ void k_poll_vote(DevMesh m, const int *list, const int *n, int *nrun)
{
    griddep_wait();
    if (blockIdx.x == 0 && threadIdx.x == 0) *nrun = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < *n; i += gridDim.x * blockDim.x) {
    if (m.pdone[m.binst[list[i]]]) continue;
    int2 e = m.bv[list[i]];
    for (int k = 0; k < 2; k++) {
        int v = k == 0 ? e.x : e.y;
        if (!m.ven[v]) continue;
        int4 sb = m.vb[v];
        double mt = 99999999;
        int am = 0;
        for (int j = 0; j < 3; j++) {
            int b = slot3(sb, j);
            if (m.btext[b] <= mt && m.bcand[b]) { mt = m.btext[b]; am = j; }
        }
        m.voted[v] = slot3(sb, am);
    }
    }
}
/* count_boundaries_votes (:406) */
__global__ void k_poll_count(DevMesh m, const int *list, const int *n)
{
    griddep_wait();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < *n; i += gridDim.x * blockDim.x) {
        int b = list[i];
        if (!(m.ben[b] && m.bcand[b]) || m.pdone[m.binst[b]]) continue;
        int2 e = m.bv[b];
        m.bvotes[b] = (m.voted[e.x] == b) + (m.voted[e.y] == b);
    }
}
/* unlabel (:441).  A two-vote candidate is never adjacent to another
 * two-vote candidate (their shared vertex votes once), so the parallel
 * writes cannot change any thread's decision. */
__global__ void k_poll_unlabel(DevMesh m, const int *list, const int *n)
{
    griddep_wait();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < *n; i += gridDim.x * blockDim.x) {
        int b = list[i];
        if (!(m.ben[b] && m.bcand[b] && m.bvotes[b] == 2) || m.pdone[m.binst[b]]) continue;
        int2 e = m.bv[b];
        int4 si = m.vb[e.x], se = m.vb[e.y];
        for (int j = 0; j < 3; j++) {
            int x = slot3(si, j), y = slot3(se, j);
            if (x != b) m.bcand[x] = 0;
            if (y != b) m.bcand[y] = 0;
        }
    }
}
/* flips_per_block (:486-511) part one: a mismatch of boundary b marks
 * grid thread (b mod grid) as failed, b counted within its instance; then
 * write_candidate_results (:466-477) for the same element. */
__global__ void k_poll_compare_write(DevMesh m, int *threadfail, int grid)
{
    griddep_wait();
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= m.nb) return;
    int inst = m.binst[b];
    if (m.pdone[inst]) return;
    uint8_t en = m.ben[b], c = m.bcand[b];
    if (en && c != m.bcandbuf[b]) threadfail[(size_t)inst * grid + (b - m.boff[inst]) % grid] = 1;
    m.bcandbuf[b] = en ? c : 0;
}
/* The same for a single instance: 16 consecutive boundaries per thread,
 * the three flag arrays read and the buffer written as 16-byte words
 * (allocations are 256-byte multiples; bytes past nb are written back
 * unchanged).  grid >= 16. */
__global__ void k_poll_compare_write16(DevMesh m, int *threadfail, int grid)
{
    griddep_wait();
    int b0 = (blockIdx.x * blockDim.x + threadIdx.x) * 16;
    if (b0 >= m.nb || m.pdone[0]) return;
    uint4 we = *reinterpret_cast<const uint4 *>(m.ben + b0);
    uint4 wc = *reinterpret_cast<const uint4 *>(m.bcand + b0);
    uint4 wb = *reinterpret_cast<const uint4 *>(m.bcandbuf + b0);
    unsigned e4[4] = { we.x, we.y, we.z, we.w }, c4[4] = { wc.x, wc.y, wc.z, wc.w }, b4[4] = { wb.x, wb.y, wb.z, wb.w };
    int slot = b0 % grid;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        unsigned nb4 = 0;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            int i = 4 * j + k;
            unsigned e = (e4[j] >> (8 * k)) & 0xffu, c = (c4[j] >> (8 * k)) & 0xffu, o = (b4[j] >> (8 * k)) & 0xffu;
            unsigned nbyte = o;
            if (b0 + i < m.nb) {
                if (e && c != o) {
                    int t = slot + i;
                    threadfail[t >= grid ? t - grid : t] = 1;
                }
                nbyte = e ? c : 0u;
            }
            nb4 |= nbyte << (8 * k);
        }
        b4[j] = nb4;
    }
    *reinterpret_cast<uint4 *>(m.bcandbuf + b0) = make_uint4(b4[0], b4[1], b4[2], b4[3]);
}
/* part two, on the reference's grid (blockIdx.y = instance): per thread
 * AND over its stride set (already folded into threadfail), per block the
 * shared-memory tree whose bool += acts as OR (compare_candidates
 * :526-537); then, in the instance's last block to finish, the host's AND
 * over blocks (:533-535): an instance whose blocks all passed has
 * converged and takes no further iteration this step */
__global__ void k_poll_final(DevMesh m, int *threadfail, int *pblock, int *pcnt, int *piters, int *nrun)
{
    griddep_wait();
    __shared__ int t[256];
    __shared__ int last;
    int inst = blockIdx.y;
    if (m.pdone[inst]) return;                       /* uniform over the instance's blocks */
    size_t tid = (size_t)inst * gridDim.x * blockDim.x + blockIdx.x * blockDim.x + threadIdx.x;
    t[threadIdx.x] = threadfail[tid] ? 0 : 1;
    threadfail[tid] = 0;
    __syncthreads();
    for (int i = blockDim.x / 2; i != 0; i /= 2) {
        if ((int)threadIdx.x < i) t[threadIdx.x] = (t[threadIdx.x] || t[threadIdx.x + i]) ? 1 : 0;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        pblock[(size_t)inst * gridDim.x + blockIdx.x] = t[0];
        __threadfence();
        last = atomicAdd(pcnt + inst, 1) == (int)gridDim.x - 1;
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    pcnt[inst] = 0;
    __threadfence();
    piters[inst]++;
    int ok = 1;
    for (int i = 0; i < (int)gridDim.x; i++) ok &= __ldcg(pblock + (size_t)inst * gridDim.x + i) != 0;
    if (ok) m.pdone[inst] = 1;
    else atomicAdd(nrun, 1);
}

/* ------------------------------------------------------------------ */
/* conflicts, src/topological.h:83-155                                 */
/* ------------------------------------------------------------------ */
__device__ void conflict_check_one(const DevMesh &m, int b)
{
    if (!(m.ben[b] && !m.bcand[b])) return;
    int2 e = m.bv[b];
    int4 si = m.vb[e.x], se = m.vb[e.y];
    int bi = -1, be = -1;
    for (int j = 0; j < 3; j++) {
        int x = slot3(si, j);
        if (x != b && m.bcand[x]) { bi = x; break; }
    }
    for (int j = 0; j < 3; j++) {
        int x = slot3(se, j);
        if (x != b && m.bcand[x]) { be = x; break; }
    }
    if (bi >= 0 && be >= 0) {
        double ti = m.btext[bi], te = m.btext[be];
        int w;
        if (ti == te) w = bi < be ? bi : be;
        else w = ti < te ? bi : be;
        /* b is reached from each candidate next to it and every visit writes
         * the same w; the first writer (bconf was -1) counts the mark */
        if (atomicExch(&m.bconf[b], w) == -1) atomicAdd(&m.evt[EVT_COUNT * m.binst[b] + EVT_CONFLICTS], 1);
    }
}
/* check_conflictive_boundaries for every non-candidate boundary adjacent
 * to a candidate (the only ones it can mark); one thread per candidate and
 * slot of its ends, so the six neighbours' load chains run side by side
 * (every visit of a boundary writes the same winner) */
__global__ void k_conflict_check(DevMesh m, const int *list, const int *n)
{
    griddep_wait();
    const int total = 6 * *n;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        int i = t / 6, r = t - 6 * i;
        int c = list[i];
        if (!(m.ben[c] && m.bcand[c])) continue;
        int2 e = m.bv[c];
        int b = slot3(m.vb[r < 3 ? e.x : e.y], r < 3 ? r : r - 3);
        if (b != c) conflict_check_one(m, b);
    }
}
__global__ void k_conflict_unlabel(DevMesh m, const int *list, const int *n)
{
    griddep_wait();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < *n; i += gridDim.x * blockDim.x) {
        int b = list[i];
        if (!(m.ben[b] && m.bcand[b])) continue;
        int2 e = m.bv[b];
        int4 si = m.vb[e.x], se = m.vb[e.y];
        bool drop = false;
        for (int j = 0; j < 3; j++) {
            int x = slot3(si, j);
            if (b != x && m.bconf[x] != -1) { if (m.bconf[x] != b) { drop = true; break; } }
        }
        for (int j = 0; j < 3; j++) {
            int x = slot3(se, j);
            if (b != x && m.bconf[x] != -1) { if (m.bconf[x] != b) { drop = true; break; } }
        }
        if (drop) m.bcand[b] = 0;
    }
}

/* ------------------------------------------------------------------ */
/* removal of two adjacent 3-sided grains, src/topological.h:840-985   */
/* ------------------------------------------------------------------ */
/* remove_two_grains (:840-955); returns the rewired boundary CE or -1 */
__device__ int remove_two_grains_dev(const DevMesh &m, int bnd, const int *gnic)
{
    int2 eb = m.bv[bnd];
    int A = eb.x, B = eb.y;
    int4 sa = m.vb[A], sbv = m.vb[B];
    int AC = -1, BD = -1;
    for (int i = 0; i < 3; i++) if (slot3(sa, i) == bnd) { AC = slot3(sa, (i + 1) % 3); break; }
    for (int j = 0; j < 3; j++) if (slot3(sbv, j) == bnd) { BD = slot3(sbv, (j + 1) % 3); break; }
    if (AC < 0 || BD < 0) { raise_err(m, ERRB_TOPOLOGY); return -1; }
    int C = other_end(m.bv[AC], A);
    int D = other_end(m.bv[BD], B);
    int4 sc = m.vb[C], sd = m.vb[D];
    int CE = -1, DF = -1;
    for (int k = 0; k < 3; k++) if (slot3(sc, k) == AC) { CE = slot3(sc, (k + 2) % 3); break; }
    for (int l = 0; l < 3; l++) if (slot3(sd, l) == BD) { DF = slot3(sd, (l + 2) % 3); break; }
    if (CE < 0 || DF < 0) { raise_err(m, ERRB_TOPOLOGY); return -1; }
    int F = other_end(m.bv[DF], D);
    int2 ce = m.bv[CE];
    if (ce.x == C) ce.x = F; else ce.y = F;
    save_ends(m, CE);
    m.bv[CE] = ce;
    int4 sf = m.vb[F];
    for (int p = 0; p < 3; p++) if (slot3(sf, p) == DF) { set_slot3(sf, p, CE); break; }
    m.vb[F] = sf;
    if (gnic[0] < 0 || gnic[1] < 0) { raise_err(m, ERRB_TOPOLOGY); return -1; }
    int G3, G4;
    if (glist_find(m, gnic[0], A) >= 0) { G3 = gnic[0]; G4 = gnic[1]; } else { G3 = gnic[1]; G4 = gnic[0]; }
    set_mod(m, A, 0, FIX_REMOVE, G3, A, -2); mark_fix(m, G3);
    set_mod(m, A, 1, FIX_REMOVE, G3, C, -2);
    set_mod(m, A, 2, FIX_REMOVE, G3, D, -2);
    set_mod(m, B, 0, FIX_REMOVE, G4, B, -2); mark_fix(m, G4);
    set_mod(m, B, 1, FIX_REMOVE, G4, C, -2);
    set_mod(m, B, 2, FIX_REMOVE, G4, D, -2);
    sa = m.vb[A]; sbv = m.vb[B];
    for (int i = 0; i < 3; i++) {
        finalize_boundary(m, slot3(sa, i));
        finalize_boundary(m, slot3(sbv, i));
        m.ben[slot3(sa, i)] = 0;
        m.ben[slot3(sbv, i)] = 0;
    }
    finalize_boundary(m, DF);
    finalize_boundary(m, bnd);
    m.ben[DF] = 0;
    m.ben[bnd] = 0;
    m.ven[A] = 0; m.ven[D] = 0; m.ven[C] = 0; m.ven[B] = 0;
    return CE;
}

__device__ bool two_three_qualifies(const DevMesh &m, int b, int *gic)
{
    if (!m.ben[b]) return false;
    int2 e = m.bv[b];
    if (gintersect(m.vg[e.x], m.vg[e.y], gic) < 2) return false;
    return m.gvlen[gic[0]] == 3 && m.gvlen[gic[1]] == 3;
}

/* The step's first 2x3 count: a qualifying boundary lies on two 3-sided
 * grains, so only the boundaries at the vertices of the 3-sided grains
 * (bucket 3 of this step's side-count order) are tested; the ordered
 * compaction of the marks then gives the same ascending list as testing
 * every boundary. */
__global__ void k_mark_two_three(DevMesh m, const int *perm, const int *vbucket)
{
    int n3 = vbucket[VB_COUNT(3)], start = vbucket[VB_START(3)];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += gridDim.x * blockDim.x) {
        const int *L = m.glist + (size_t)SEVC_MAXV * perm[start + i];
        for (int k = 0; k < 3; k++) {
            int4 s = m.vb[L[k]];
            for (int j = 0; j < 3; j++) {
                int b = slot3(s, j), gic[2];
                if (two_three_qualifies(m, b, gic)) m.bmark[b] = 1;
            }
        }
    }
}

__device__ bool sorted_contains(const int *a, int lo, int hi, int x)
{
    int end = hi;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (a[mid] < x) lo = mid + 1; else hi = mid;
    }
    return lo < end && a[lo] == x;
}

/* remove_two_grains_configurations (:965-985) is one thread scanning every
 * boundary in index order.  Only listed boundaries (those qualifying at the
 * count) and boundaries re-wired during the scan (CE) can qualify, so the
 * scan visits exactly those, in index order, re-testing each on visit. */
/* One thread per instance, each over its own part of the ascending list. */
__global__ void k_remove_two_three(DevMesh m, const int *list, const int *n, int *extra, int *segcnt,
                                   const int *pass_dev)
{
    int inst = blockIdx.x * blockDim.x + threadIdx.x;
    if (inst >= m.ninst) return;
    if (pass_dev) segcnt += (size_t)*pass_dev * m.ninst;
    int i = lower_bound_i(list, *n, m.boff[inst]);
    int N = lower_bound_i(list, *n, m.boff[inst + 1]);
    segcnt[inst] = N - i;
    extra += (size_t)inst * EXTRA_CAP;
    int *evt = m.evt + EVT_COUNT * inst;
    int ne = 0;
    while (i < N || ne > 0) {
        int b;
        if (ne > 0 && (i >= N || extra[0] < list[i])) {
            b = extra[0];
            for (int k = 1; k < ne; k++) extra[k - 1] = extra[k];
            ne--;
        } else {
            b = list[i++];
        }
        int gic[2];
        if (!two_three_qualifies(m, b, gic)) continue;
        int2 e = m.bv[b];
        int gnic[2];
        gsymdiff(m.vg[e.x], m.vg[e.y], gnic);
        int CE = remove_two_grains_dev(m, b, gnic);
        m.gen[gic[0]] = 0;
        m.gen[gic[1]] = 0;
        evt[EVT_TWO_THREE]++;
        if (CE > b && !sorted_contains(list, i, N, CE)) {
            int g2[2];
            if (two_three_qualifies(m, CE, g2)) {
                bool dup = false;
                for (int k = 0; k < ne; k++) dup |= extra[k] == CE;
                if (!dup) {
                    if (ne >= EXTRA_CAP) { raise_err(m, ERRB_WORKLIST); continue; }
                    int k = ne++;
                    while (k > 0 && extra[k - 1] > CE) { extra[k] = extra[k - 1]; k--; }
                    extra[k] = CE;
                }
            }
        }
    }
}

/* ------------------------------------------------------------------ */
/* 3-sided grain removal, src/topological.h:614-822, :994-1004         */
/* ------------------------------------------------------------------ */
/* label_3sided_grains (:994-1004) for one 3-sided grain */
__device__ uint8_t label3_cand(const DevMesh &m, int g, double dt)
{
    /* The reference breaks out of a vertex's boundary loop once a flip
     * candidate inside the grain is found; that sets the result to 1 for
     * good, so testing every boundary gives the same answer and lets all
     * nine records load at once. */
    const int *L = m.glist + (size_t)SEVC_MAXV * g;
    int l0 = L[0], l1 = L[1], l2 = L[2];
    int4 s[3] = { m.vb[l0], m.vb[l1], m.vb[l2] };
    int bs[9];
    int2 e[9];
#pragma unroll
    for (int j = 0; j < 9; j++) bs[j] = slot3(s[j / 3], j % 3);
#pragma unroll
    for (int j = 0; j < 9; j++) e[j] = m.bv[bs[j]];
    bool cand = false;
    int ans = 0;
#pragma unroll
    for (int j = 0; j < 9; j++) {
        bool ii = e[j].x == l0 || e[j].x == l1 || e[j].x == l2;
        bool ee = e[j].y == l0 || e[j].y == l1 || e[j].y == l2;
        if (ii && ee) {
            int b = bs[j];
            uint8_t en = m.ben[b], ca = m.bcand[b];
            double t = m.btext[b];
            cand |= ca && en;
            ans += (t >= 0 && t <= dt) && en;
        }
    }
    return cand || ans / 2 == 3;
}
/* clear_grains_state + label_3sided_grains for enabled grains */
__global__ void k_label_3sided(DevMesh m, double dt)
{
    griddep_wait();
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= m.ng || !m.gen[g]) return;
    m.gcand[g] = m.gvlen[g] == 3 ? label3_cand(m, g, dt) : 0;
}
/* The same when no list changed since this step's side-count order: only
 * the grains of its 3-sided bucket are visited.  Every other enabled grain
 * already has gcand = 0, because each step clears the flag of every grain
 * it listed as a candidate (k_remove_reserve). */
__global__ void k_label_3sided_bucket(DevMesh m, double dt, const int *perm, const int *vbucket)
{
    griddep_wait();
    int n3 = vbucket[VB_COUNT(3)], start = vbucket[VB_START(3)];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += gridDim.x * blockDim.x) {
        int g = perm[start + i];
        m.gcand[g] = label3_cand(m, g, dt);
    }
}
/* either of the two above, as the step's first 2x3 count says: no 2x3
 * removal (count 0) leaves every list as the side-count order saw it */
__global__ void k_label_3sided_auto(DevMesh m, double dt, const int *perm, const int *vbucket, const int *tt_first)
{
    griddep_wait();
    if (*tt_first == 0) {
        int n3 = vbucket[VB_COUNT(3)], start = vbucket[VB_START(3)];
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += gridDim.x * blockDim.x) {
            int g = perm[start + i];
            m.gcand[g] = label3_cand(m, g, dt);
        }
    } else {
        for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.ng; g += gridDim.x * blockDim.x)
            if (m.gen[g]) m.gcand[g] = m.gvlen[g] == 3 ? label3_cand(m, g, dt) : 0;
    }
}
/* loop control of the whole-step graph (one thread) */
__global__ void k_poll_cond(cudaGraphConditionalHandle hnd, const int *nrun, int *ptot, int cap, int *err)
{
    if (threadIdx.x) return;
    int it = ++*ptot;
    bool run = *nrun > 0;
    if (run && it >= cap) {
        atomicOr(err, ERRB_NONCONVERGED);
        run = false;
    }
    cudaGraphSetConditional(hnd, run ? 1u : 0u);
}
__global__ void k_tt_init(cudaGraphConditionalHandle hnd, const int *n, int *first, int *pass)
{
    if (threadIdx.x) return;
    *first = *n;
    *pass = 0;
    cudaGraphSetConditional(hnd, *n > 0 ? 1u : 0u);
}
__global__ void k_tt_cond(cudaGraphConditionalHandle hnd, const int *n, int *pass)
{
    if (threadIdx.x) return;
    int p = ++*pass;
    cudaGraphSetConditional(hnd, (*n > 0 && p < TWO_THREE_PASSES) ? 1u : 0u);
}

/* remove_grain (:687-822) */
__device__ void remove_grain_dev(const DevMesh &m, int grn)
{
    const int *L = m.glist + (size_t)SEVC_MAXV * grn;
    int A = L[0], B = L[1], C = L[2];
    double D = m.D;
    double2 pa = m.pos[A], pb = m.pos[B], pc = m.pos[C];
    log_event(m, EV_REMOVE, A, B, C, pa, pb, pc);
    double nAB = arclen(pa, pb, D), nBC = arclen(pb, pc, D), nCA = arclen(pc, pa, D);
    double denom = nAB + nBC + nCA;
    double x0 = 0, y0 = 0;                                      /* adjust_origin_for_points, 3 points */
    double x1 = x0 + wrapd(pb.x, pa.x, D), y1 = y0 + wrapd(pb.y, pa.y, D);
    double x2 = x1 + wrapd(pc.x, pb.x, D), y2 = y1 + wrapd(pc.y, pb.y, D);
    pa.x += (nBC * x0 + nCA * x1 + nAB * x2) / denom;
    pa.y += (nBC * y0 + nCA * y1 + nAB * y2) / denom;
    pa.x = dmod(pa.x, D);
    pa.y = dmod(pa.y, D);
    save_vertex(m, A);
    m.pos[A] = pa;
    int gbc[2], gab[2], gac[2];
    gintersect(m.vg[B], m.vg[C], gbc);
    int G3 = gbc[0] == grn ? gbc[1] : gbc[0];
    gintersect(m.vg[A], m.vg[B], gab);
    int G2 = gab[0] == grn ? gab[1] : gab[0];
    gintersect(m.vg[A], m.vg[C], gac);
    int G1 = gac[0] == grn ? gac[1] : gac[0];
    if (G1 < 0 || G2 < 0 || G3 < 0) { raise_err(m, ERRB_TOPOLOGY); return; }
    m.vel[A] = make_double2(0.0, 0.0);
    int4 sc = m.vb[C], sb = m.vb[B];
    for (int i = 0; i < 3; i++) {
        int x = slot3(sc, i);
        int2 e = m.bv[x];
        if ((e.x == B && e.y == C) || (e.y == B && e.x == C)) { finalize_boundary(m, x); m.ben[x] = 0; break; }
    }
    int BE = -1, CF = -1;
    for (int i = 0; i < 3; i++) {
        int x = slot3(sb, i);
        int2 e = m.bv[x];
        if (!(e.x == A || e.y == A) && !(e.x == C || e.y == C)) { BE = x; break; }
    }
    for (int i = 0; i < 3; i++) {
        int x = slot3(sc, i);
        int2 e = m.bv[x];
        if (!(e.x == A || e.y == A) && !(e.x == B || e.y == B)) { CF = x; break; }
    }
    if (BE < 0 || CF < 0) { raise_err(m, ERRB_TOPOLOGY); return; }
    int2 e;
    save_ends(m, BE);
    save_ends(m, CF);
    e = m.bv[BE]; if (e.x == B) e.x = A; else e.y = A; m.bv[BE] = e;
    e = m.bv[CF]; if (e.x == C) e.x = A; else e.y = A; m.bv[CF] = e;
    int4 sa = m.vb[A];
    for (int i = 0; i < 3; i++) {
        int x = slot3(sa, i);
        int2 f = m.bv[x];
        if (f.x == B || f.y == B) { finalize_boundary(m, x); m.ben[x] = 0; set_slot3(sa, i, BE); break; }
    }
    for (int i = 0; i < 3; i++) {
        int x = slot3(sa, i);
        int2 f = m.bv[x];
        if (f.x == C || f.y == C) { finalize_boundary(m, x); m.ben[x] = 0; set_slot3(sa, i, CF); break; }
    }
    m.vb[A] = sa;
    m.ven[B] = 0;
    m.ven[C] = 0;
    m.gen[grn] = 0;
    set_mod(m, B, 0, FIX_REMOVE, G2, B, -2); mark_fix(m, G2);
    set_mod(m, C, 0, FIX_REMOVE, G1, C, -2); mark_fix(m, G1);
    set_mod(m, B, 1, FIX_REMOVE, G3, B, -2); mark_fix(m, G3);
    set_mod(m, C, 1, FIX_REPLACE, G3, A, C);
    int4 ga = m.vg[A];
    for (int i = 0; i < 3; i++) if (slot3(ga, i) == grn) set_slot3(ga, i, G3);
    m.vg[A] = ga;
}

/* ------------------------------------------------------------------ */
/* Events in parallel with the serial order's result                    */
/* ------------------------------------------------------------------ */
/* The reference applies the 3-sided removals one at a time in ascending
 * grain order (remove_grains <<<1,1>>>, :994) and defines no order for the
 * flips; here both phases follow ascending list order.  An event reads and
 * writes only its footprint (its vertices and the boundaries in their
 * slots) plus grain-level records that commute: queueing a grain for the
 * fix-up (an atomic claim of its flag), its mod slots (per vertex) and the
 * dA/dt settled from the step's starting values (settled before any event
 * of the phase runs).  Two events with disjoint footprints therefore
 * commute, and the serial result is obtained by deterministic reservation:
 *   reserve  every event writes its key into each footprint record
 *            (atomicMin); the key orders events by list position;
 *   apply    an event that holds every one of its records shares none
 *            with an earlier event: it runs at once, all such in parallel;
 *            any other is deferred;
 *   deferred the deferred events run one at a time in list order, after
 *            the parallel ones; each shares records only with earlier
 *            events, which have all run (in parallel or before it here),
 *            and commutes with every later parallel one.
 * Keys carry a per-phase epoch in their high half that grows every step,
 * so records never need clearing: an earlier step's key is larger and is
 * replaced by the first reservation of a later step. */
__device__ __forceinline__ unsigned long long resv_key(unsigned epoch, int pos)
{
    return ((unsigned long long)(0xFFFFFFFFu - epoch) << 32) | (unsigned)pos;
}
__device__ __forceinline__ bool valid_v(const DevMesh &m, int v) { return (unsigned)v < (unsigned)m.nv; }
__device__ __forceinline__ bool valid_b(const DevMesh &m, int b) { return (unsigned)b < (unsigned)m.nb; }
__device__ __forceinline__ bool valid_g(const DevMesh &m, int g) { return (unsigned)g < (unsigned)m.ng; }

/* bring a record into this SM's L1 (no register result, no wait) */
__device__ __forceinline__ void l1_touch(const void *p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }
/* An event's warp reserves its vertices and the boundaries in their slots
 * (lane 3j + k: vertex j, slot k) and settles the dA/dt of every grain
 * around them, one grain per lane (a grain an earlier lane also sees is
 * left to that lane), so the settling runs side by side instead of one
 * grain after another.  With `internal`, the extinction times of the
 * boundaries joining two of the event's vertices (the ones a 3-sided
 * removal disables) are settled too, each by the lane at its first end.
 * Settling reads only the step's starting values, which nothing changes
 * before the events apply, and is idempotent (an event that defers and
 * then finds other boundaries settles those itself).  Warp-uniform
 * arguments; every lane calls it. */
__device__ void reserve_warp(const DevMesh &m, const DevScratch &x, const int *verts, int nverts,
                             unsigned long long key, int lane, bool internal)
{
    int j = lane / 3, k = lane - 3 * j, h = -1;
    if (lane < 3 * nverts) {
        int v = verts[j];
        if (valid_v(m, v)) {
            if (k == 0) atomicMin(x.vown + v, key);
            int b = slot3(m.vb[v], k);
            if (valid_b(m, b)) {
                atomicMin(x.bown + b, key);
                if (internal) {
                    int2 e = m.bv[b];
                    bool in = false;
                    for (int q = 0; q < nverts; q++) in |= verts[q] != v && (verts[q] == e.x || verts[q] == e.y);
                    if (in && e.x == v) finalize_boundary(m, b);
                }
            }
            h = slot3(m.vg[v], k);
            if (!valid_g(m, h)) h = -1;
        }
    }
    bool first = h >= 0;
    for (int q = 0; q < 9; q++) {
        int hq = __shfl_sync(0xffffffffu, h, q);
        if (q < lane && hq == h) first = false;
    }
    /* settling walks the grain's list with three dependent loads per
     * vertex: the lanes first bring their grains' lists and vertex records
     * into L1, every load of a list issued at once */
    if (first && !m.gexact[h]) {
        const int *L = m.glist + (size_t)SEVC_MAXV * h;
        int n = m.gvlen[h];
        n = n < SEVC_MAXV ? n : SEVC_MAXV;
#pragma unroll 4
        for (int k = 0; k < n; k++) {
            int v = L[k];
            if (valid_v(m, v)) { l1_touch(m.pos + v); l1_touch(m.vel + v); l1_touch(m.vstamp + v); }
        }
    }
    __syncwarp();
    if (first) finalize_grain(m, h);
}
/* the records an event's single-thread code reads, brought into L1 by
 * the warp in two parallel rounds: the vertices' own records, then the
 * boundaries in their slots and the grains around them */
__device__ void prefetch_event(const DevMesh &m, const int *verts, int nverts, int lane)
{
    int j = lane / 3, k = lane - 3 * j;
    if (lane >= 3 * nverts) return;
    int v = verts[j];
    if (!valid_v(m, v)) return;
    if (k == 0) {
        l1_touch(m.pos + v); l1_touch(m.vel + v); l1_touch(m.vstamp + v); l1_touch(m.pos0 + v);
        l1_touch(m.vmod + 4 * (size_t)v); l1_touch(m.vmodmark + v);
    }
    int b = slot3(m.vb[v], k), h = slot3(m.vg[v], k);
    if (valid_b(m, b)) { l1_touch(m.bv + b); l1_touch(m.bstamp + b); l1_touch(m.bexact + b); l1_touch(m.ben + b); }
    if (valid_g(m, h)) { l1_touch(m.gfix + h); l1_touch(m.gexact + h); l1_touch(m.gvlen + h); }
}
/* whether v and every boundary in its slots hold key; nothing but the
 * event holding v writes its slots, so they are the reserved ones */
__device__ bool holds_vertex(const DevMesh &m, const DevScratch &x, int v, unsigned long long key)
{
    if (x.vown[v] != key) return false;
    int4 s = m.vb[v];
    for (int j = 0; j < 3; j++) {
        int b = slot3(s, j);
        if (!valid_b(m, b) || x.bown[b] != key) return false;
    }
    return true;
}

/* 3-sided removals (remove_grains, :994): a listed grain that is enabled
 * and a candidate is removed; a removal disables only its own grain, so
 * the set is known up front.  One warp per listed grain, which also
 * clears the grain's candidate flag (src/main.cu:260; nothing after this
 * test reads it this step). */
__global__ void k_remove_reserve(DevMesh m, DevScratch x, const int *list, const int *n)
{
    griddep_wait();
    const unsigned ep = 2u * *m.stamp;
    const int lane = threadIdx.x & 31, nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < *n; i += nw) {
        int g = list[i];
        bool rm = m.gen[g] && m.gcand[g];
        __syncwarp();
        if (lane == 0) m.gcand[g] = 0;
        if (!rm) continue;
        const int *L = m.glist + (size_t)SEVC_MAXV * g;
        int verts[3] = { L[0], L[1], L[2] };
        reserve_warp(m, x, verts, 3, resv_key(ep, i), lane, true);
        if (lane == 0) {
            int p = atomicAdd(x.n_ehits, 1);
            x.ehits[p] = i;
        }
    }
}
/* one warp per removal: its records are brought into L1, then lane 0
 * applies it (or defers it when an earlier removal holds a record) */
__global__ void k_remove_apply(DevMesh m, DevScratch x, const int *list)
{
    griddep_wait();
    const unsigned ep = 2u * *m.stamp;
    const int nh = *x.n_ehits;
    const int lane = threadIdx.x & 31, nw = (gridDim.x * blockDim.x) >> 5;
    for (int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < nh; t += nw) {
        int i = x.ehits[t], g = list[i];
        const int *L = m.glist + (size_t)SEVC_MAXV * g;
        int verts[3] = { L[0], L[1], L[2] };
        unsigned long long key = resv_key(ep, i);
        bool own = true;
        if (lane == 0)
            for (int k = 0; k < 3 && own; k++) own = valid_v(m, verts[k]) && holds_vertex(m, x, verts[k], key);
        own = __shfl_sync(0xffffffffu, own, 0);
        if (own) prefetch_event(m, verts, 3, lane);
        __syncwarp();
        if (lane == 0) {
            if (own) {
                remove_grain_dev(m, g);
                atomicAdd(&m.evt[EVT_COUNT * m.ginst[g] + EVT_REMOVALS], 1);
            } else {
                x.edefer[i] = 1;
                atomicAdd(&x.ndefer[m.ginst[g]], 1);
            }
        }
        __syncwarp();
    }
}
/* one warp per instance: its deferred removals in list order */
__global__ void k_remove_deferred(DevMesh m, DevScratch x, const int *list, const int *n)
{
    griddep_wait();
    int inst = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (inst == 0 && lane == 0) *x.n_ehits = 0;
    if (inst >= m.ninst || x.ndefer[inst] == 0) return;
    int lo = lower_bound_i(list, *n, m.goff[inst]);
    int hi = lower_bound_i(list, *n, m.goff[inst + 1]);
    for (int base = lo; base < hi; base += 32) {
        int i = base + lane;
        bool f = i < hi && x.edefer[i];
        unsigned hits = __ballot_sync(0xffffffffu, f);
        if (lane == 0)
            while (hits) {
                int j = __ffs(hits) - 1;
                hits &= hits - 1;
                x.edefer[base + j] = 0;
                remove_grain_dev(m, list[base + j]);
                m.evt[EVT_COUNT * inst + EVT_REMOVALS]++;
            }
        __syncwarp();
    }
    if (lane == 0) x.ndefer[inst] = 0;
}

/* unlabel_boundaries_st2 (:588-606) for an enabled candidate b: it stays
 * a candidate unless a grain on either side has 3 sides.  It reads and
 * writes only b's own flags, so it runs inside the flip reservation (one
 * warp per candidate, warp-uniform result). */
__device__ bool unlabel_st2_keeps(const DevMesh &m, int b)
{
    int2 e = m.bv[b];
    int gic[2];
    if (gintersect(m.vg[e.x], m.vg[e.y], gic) < 2) {       /* the step fails */
        if ((threadIdx.x & 31) == 0) raise_err(m, ERRB_TOPOLOGY);
        return false;
    }
    bool keep = !(m.gvlen[gic[0]] == 3 || m.gvlen[gic[1]] == 3);
    __syncwarp();
    if (!keep && (threadIdx.x & 31) == 0) m.bcand[b] = 0;
    return keep;
}

/* ------------------------------------------------------------------ */
/* T1 flip, src/topological.h:174-291                                  */
/* ------------------------------------------------------------------ */
__device__ void flip_dev(const DevMesh &m, int bnd, double eps)
{
    int2 eb = m.bv[bnd];
    int A = eb.x, B = eb.y;
    int gic[2], gnic[2];
    if (gintersect(m.vg[A], m.vg[B], gic) < 2) { raise_err(m, ERRB_TOPOLOGY); return; }
    gsymdiff(m.vg[A], m.vg[B], gnic);
    int4 sa = m.vb[A], sb = m.vb[B];
    int i = -1, j = -1, AC = -1, BE = -1;
    for (int k = 0; k < 3; k++) if (slot3(sa, k) == bnd) { i = (k + 1) % 3; AC = slot3(sa, i); break; }
    for (int k = 0; k < 3; k++) if (slot3(sb, k) == bnd) { j = (k + 1) % 3; BE = slot3(sb, j); break; }
    if (AC < 0 || BE < 0 || gnic[0] < 0 || gnic[1] < 0) { raise_err(m, ERRB_TOPOLOGY); return; }
    set_slot3(sa, i, BE);
    set_slot3(sb, j, AC);
    m.vb[A] = sa;
    m.vb[B] = sb;
    save_ends(m, AC);
    save_ends(m, BE);
    int2 e = m.bv[AC]; if (e.x == A) e.x = B; else e.y = B; m.bv[AC] = e;
    e = m.bv[BE]; if (e.x == B) e.x = A; else e.y = A; m.bv[BE] = e;
    int g1, g2, g3, g4;
    for (g2 = 0; g2 < 2; g2++) if (glist_consecutive(m, gic[g2], A, B) == 1) break;
    for (g4 = 0; g4 < 2; g4++) if (glist_consecutive(m, gic[g4], B, A) == 1) break;
    for (g3 = 0; g3 < 2; g3++) if (glist_find(m, gnic[g3], A) >= 0) break;
    for (g1 = 0; g1 < 2; g1++) if (glist_find(m, gnic[g1], B) >= 0) break;
    if (g2 < 2) { set_mod(m, A, 0, FIX_REMOVE, gic[g2], A, -2); mark_fix(m, gic[g2]); }
    if (g4 < 2) { set_mod(m, B, 0, FIX_REMOVE, gic[g4], B, -2); mark_fix(m, gic[g4]); }
    if (g3 < 2) { set_mod(m, A, 1, FIX_ADD, gnic[g3], B, A); mark_fix(m, gnic[g3]); }
    if (g1 < 2) { set_mod(m, B, 1, FIX_ADD, gnic[g1], A, B); mark_fix(m, gnic[g1]); }
    if (g1 == 2 || g2 == 2 || g3 == 2 || g4 == 2) { raise_err(m, ERRB_TOPOLOGY); return; }
    int4 ga = m.vg[A], gb = m.vg[B];
    for (int k = 0; k < 3; k++) {
        if (slot3(ga, k) == gic[g2]) set_slot3(ga, k, gnic[g1]);
        if (slot3(gb, k) == gic[g4]) set_slot3(gb, k, gnic[g3]);
    }
    m.vg[A] = ga;
    m.vg[B] = gb;
    double2 pa = m.pos[A], pb = m.pos[B];                 /* vector2_mean, src/geometry.h:311 */
    log_event(m, EV_FLIP, A, B, -1, pa, pb, pb);
    double2 c = pa;
    c.x += wrapd(pb.x, pa.x, m.D) / 2;
    c.y += wrapd(pb.y, pa.y, m.D) / 2;
    c.x = dmod(c.x, m.D);
    c.y = dmod(c.y, m.D);
    save_vertex(m, A);
    save_vertex(m, B);
    m.pos[A] = c;
    m.pos[B] = c;
    sa = m.vb[A]; { int t = sa.y; sa.y = sa.x; sa.x = t; } m.vb[A] = sa; /* vertex_invert_boundary_order */
    sb = m.vb[B]; { int t = sb.y; sb.y = sb.x; sb.x = t; } m.vb[B] = sb;
    /* boundary_compute_energy (no GB scaling here, as in the reference) */
    if (eps == 0.0) {
        m.benergy[bnd] = 1.0;
    } else {
        int g2c[2];
        if (gintersect(m.vg[A], m.vg[B], g2c) < 2) { raise_err(m, ERRB_TOPOLOGY); return; }
        m.benergy[bnd] = gb_energy(m.gori[g2c[0]] - m.gori[g2c[1]], eps);
    }
    m.vel[A] = make_double2(0, 0);
    m.vel[B] = make_double2(0, 0);
}

/* Before lane 0 applies a flip (one long chain of dependent loads), the
 * warp brings the flip's neighbourhood into the SM's L1 in a few parallel
 * rounds: the two vertices' slots, positions and velocities; the boundary
 * ends and grain records around them; the lists of those grains; and the
 * positions, velocities and save stamps of the listed vertices (read by
 * finalize_grain).  Loads only, every index checked against its array. */
__device__ __forceinline__ void touch(const void *p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }
__device__ void prefetch_flip(const DevMesh &m, int bnd, int lane)
{
    int2 e = m.bv[bnd];
    if (e.x < 0 || e.x >= m.nv || e.y < 0 || e.y >= m.nv) return;
    int4 gA = m.vg[e.x], gB = m.vg[e.y], bA = m.vb[e.x], bB = m.vb[e.y];
    int gs[6] = { gA.x, gA.y, gA.z, gB.x, gB.y, gB.z }, bs[6] = { bA.x, bA.y, bA.z, bB.x, bB.y, bB.z };
    if (lane < 6) {
        int g = gs[lane];
        if (g >= 0 && g < m.ng) { touch(m.gvlen + g); touch(m.gexact + g); touch(m.gfix + g); }
        int b = bs[lane];
        if (b >= 0 && b < m.nb) touch(m.bv + b);
    } else if (lane < 8) {
        int v = lane == 6 ? e.x : e.y;
        touch(m.pos + v); touch(m.vel + v); touch(m.vstamp + v); touch(m.vmod + 4 * (size_t)v);
    }
    /* lists of the grains: lane 5k + j reads entries j, j + 5, ... of grain k */
    int k = lane / 5, j = lane % 5;
    if (k < 6) {
        int g = gs[k];
        if (g >= 0 && g < m.ng) {
            int n = m.gvlen[g];
            n = n < SEVC_MAXV ? n : SEVC_MAXV;
            const int *L = m.glist + (size_t)SEVC_MAXV * g;
            for (int i = j; i < n; i += 5) {
                int v = L[i];
                if (v >= 0 && v < m.nv) { touch(m.pos + v); touch(m.vel + v); touch(m.vstamp + v); }
            }
        }
    }
}

/* What flip_dev derives before it writes anything: the two ends, their
 * other boundaries AC and BE (the successors of bnd in their slot
 * orders, at slots i and j), the grains on both sides (gic) and at the
 * ends (gnic), the ends' slot and grain records, and which of those grains
 * get which list edit (g1..g4, as flip_dev names them). */
struct FlipPlan {
    int A, B, AC, BE, i, j, g1, g2, g3, g4;
    int gic[2], gnic[2];
    int4 sa, sb, ga, gb;
};

/* Every lane of the warp derives the flip's plan; lanes 0-7 scan the four
 * grain lists at once (a flip edits no list, so the answers are the ones
 * flip_dev's own scans give).  The four grains the flip queues for the
 * fix-up pass (mark_fix) then have their dA/dt settled, each by its own
 * lane: finalize_grain reads only the grain's list and its vertices'
 * positions and velocities at the start of the step, which nothing in a
 * flip changes before those calls, so the values are the ones the flip
 * would compute.  Returns false (nothing settled) on any inconsistency;
 * the flip then runs its own checks and reports it. */
__device__ bool flip_plan(const DevMesh &m, int bnd, int lane, FlipPlan &P)
{
    int2 eb = m.bv[bnd];
    int A = eb.x, B = eb.y;
    if (A < 0 || A >= m.nv || B < 0 || B >= m.nv || A == B) return false;
    P.A = A; P.B = B;
    P.ga = m.vg[A]; P.gb = m.vg[B]; P.sa = m.vb[A]; P.sb = m.vb[B];
    if (gintersect(P.ga, P.gb, P.gic) < 2) return false;
    gsymdiff(P.ga, P.gb, P.gnic);
    P.i = P.j = P.AC = P.BE = -1;
    for (int k = 0; k < 3; k++) if (slot3(P.sa, k) == bnd) { P.i = (k + 1) % 3; P.AC = slot3(P.sa, P.i); break; }
    for (int k = 0; k < 3; k++) if (slot3(P.sb, k) == bnd) { P.j = (k + 1) % 3; P.BE = slot3(P.sb, P.j); break; }
    if (P.AC < 0 || P.BE < 0 || P.gnic[0] < 0 || P.gnic[1] < 0) return false;
    bool hit = false;
    if (lane < 4) hit = glist_consecutive(m, P.gic[lane & 1], lane < 2 ? A : B, lane < 2 ? B : A) == 1;
    else if (lane < 8) hit = glist_find(m, P.gnic[lane & 1], lane < 6 ? A : B) >= 0;
    unsigned h = __ballot_sync(0xffffffffu, hit);
    P.g2 = (h & 1) ? 0 : (h & 2) ? 1 : 2;
    P.g4 = (h & 4) ? 0 : (h & 8) ? 1 : 2;
    P.g3 = (h & 16) ? 0 : (h & 32) ? 1 : 2;
    P.g1 = (h & 64) ? 0 : (h & 128) ? 1 : 2;
    if (P.g1 == 2 || P.g2 == 2 || P.g3 == 2 || P.g4 == 2) return false;
    int G[4] = { P.gic[P.g2], P.gic[P.g4], P.gnic[P.g3], P.gnic[P.g1] };
    if (lane < 4) {
        int g = G[lane];
        bool dup = false;
        for (int k = 0; k < lane; k++) dup |= G[k] == g;
        if (!dup) finalize_grain(m, g);
    }
    return true;
}

/* flip_dev from a plan, for the usual case AC != BE: the same writes with
 * the same values, but every record the flip reads is loaded up front in
 * one round trip instead of behind the writes that precede it, and the
 * work-list appends of the mod slots and of the fix-up grains take one
 * atomic each (the fix-up pass edits each queued grain on its own, so the
 * order of the entries does not matter). */
__device__ void flip_planned(const DevMesh &m, int bnd, double eps, const FlipPlan &P)
{
    const int A = P.A, B = P.B, AC = P.AC, BE = P.BE;
    const int G[4] = { P.gic[P.g2], P.gic[P.g4], P.gnic[P.g3], P.gnic[P.g1] };
    unsigned st = *m.stamp;
    unsigned sAC = m.bstamp[AC], sBE = m.bstamp[BE], stA = m.vstamp[A], stB = m.vstamp[B];
    int2 eAC = m.bv[AC], eBE = m.bv[BE];
    int4 mA0 = m.vmod[4 * (size_t)A], mB0 = m.vmod[4 * (size_t)B];
    uint8_t mkA = m.vmodmark[A], mkB = m.vmodmark[B];
    double2 pa = m.pos[A], pb = m.pos[B], va = m.vel[A], vb = m.vel[B];
    log_event(m, EV_FLIP, A, B, -1, pa, pb, pb);
    /* boundary slots, then vertex_invert_boundary_order */
    int4 sa = P.sa, sb = P.sb;
    set_slot3(sa, P.i, BE);
    set_slot3(sb, P.j, AC);
    { int t = sa.y; sa.y = sa.x; sa.x = t; }
    { int t = sb.y; sb.y = sb.x; sb.x = t; }
    m.vb[A] = sa;
    m.vb[B] = sb;
    if (sAC != st) { m.bv0[AC] = eAC; m.bstamp[AC] = st; }      /* save_ends */
    if (sBE != st) { m.bv0[BE] = eBE; m.bstamp[BE] = st; }
    if (eAC.x == A) eAC.x = B; else eAC.y = B;
    if (eBE.x == B) eBE.x = A; else eBE.y = A;
    m.bv[AC] = eAC;
    m.bv[BE] = eBE;
    /* set_mod(A, 0, REMOVE), (B, 0, REMOVE), (A, 1, ADD), (B, 1, ADD) */
    mA0.x = G[0]; mA0.y = A; mA0.w = FIX_REMOVE;
    mB0.x = G[1]; mB0.y = B; mB0.w = FIX_REMOVE;
    m.vmod[4 * (size_t)A] = mA0;
    m.vmod[4 * (size_t)B] = mB0;
    m.vmod[4 * (size_t)A + 1] = make_int4(G[2], B, A, FIX_ADD);
    m.vmod[4 * (size_t)B + 1] = make_int4(G[3], A, B, FIX_ADD);
    int nm = (mkA ? 0 : 1) + (mkB ? 0 : 1);
    if (nm) {
        int i0 = atomicAdd(m.nmod, nm);
        if (!mkA) {
            m.vmodmark[A] = 1;
            if (i0 < m.modcap) m.modlist[i0] = A; else raise_err(m, ERRB_WORKLIST);
            i0++;
        }
        if (!mkB) {
            m.vmodmark[B] = 1;
            if (i0 < m.modcap) m.modlist[i0] = B; else raise_err(m, ERRB_WORKLIST);
        }
    }
    /* mark_fix of the four grains (their dA/dt is settled); flips running
     * at the same time may queue the same grain, the claim decides */
    bool nf[4];
    int nfix = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        nf[k] = claim_byte(m.gfix, G[k]);
        nfix += nf[k];
    }
    if (nfix) {
        int i0 = atomicAdd(m.nfix, nfix);
#pragma unroll
        for (int k = 0; k < 4; k++)
            if (nf[k]) {
                if (i0 < m.fixcap) m.fixlist[i0] = G[k]; else raise_err(m, ERRB_WORKLIST);
                i0++;
            }
    }
    int4 ga = P.ga, gb = P.gb;
    for (int k = 0; k < 3; k++) {
        if (slot3(ga, k) == G[0]) set_slot3(ga, k, G[3]);
        if (slot3(gb, k) == G[1]) set_slot3(gb, k, G[2]);
    }
    m.vg[A] = ga;
    m.vg[B] = gb;
    double2 c = pa;                                         /* vector2_mean, src/geometry.h:311 */
    c.x += wrapd(pb.x, pa.x, m.D) / 2;
    c.y += wrapd(pb.y, pa.y, m.D) / 2;
    c.x = dmod(c.x, m.D);
    c.y = dmod(c.y, m.D);
    if (stA != st) { m.pos0[A] = pa; m.vel0[A] = va; m.vstamp[A] = st; }   /* save_vertex */
    if (stB != st) { m.pos0[B] = pb; m.vel0[B] = vb; m.vstamp[B] = st; }
    m.pos[A] = c;
    m.pos[B] = c;
    if (eps == 0.0) {
        m.benergy[bnd] = 1.0;
    } else {
        int g2c[2];
        if (gintersect(ga, gb, g2c) < 2) { raise_err(m, ERRB_TOPOLOGY); return; }
        m.benergy[bnd] = gb_energy(m.gori[g2c[0]] - m.gori[g2c[1]], eps);
    }
    m.vel[A] = make_double2(0, 0);
    m.vel[B] = make_double2(0, 0);
}

/* apply_flippings (:1016-1026): the reference flips every remaining
 * candidate in parallel, with unsynchronised writes when two share
 * records; here flips follow ascending list (boundary) order, which is
 * every race-free outcome.  A flip changes no boundary's enabled or
 * candidate flag, so the flips are known up front.  Reservation, parallel
 * application and the deferred pass as for the removals (epoch 2 * stamp
 * + 1); the footprint is both ends with their slots. */
__global__ void k_flip_reserve(DevMesh m, DevScratch x, const int *list, const int *n)
{
    griddep_wait();
    const unsigned ep = 2u * *m.stamp + 1u;
    const int lane = threadIdx.x & 31, nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < *n; i += nw) {
        int b = list[i];
        if (!(m.ben[b] && m.bcand[b])) continue;
        if (!unlabel_st2_keeps(m, b)) continue;
        int2 e = m.bv[b];
        int verts[2] = { e.x, e.y };
        reserve_warp(m, x, verts, 2, resv_key(ep, i), lane, false);
        if (lane == 0) {
            int p = atomicAdd(x.n_ehits, 1);
            x.ehits[p] = i;
        }
    }
}
/* one warp per flip: lanes prefetch its neighbourhood and derive the
 * plan, lane 0 applies it */
__global__ void k_flip_apply(DevMesh m, DevScratch x, double eps, const int *list)
{
    griddep_wait();
    const unsigned ep = 2u * *m.stamp + 1u;
    const int nh = *x.n_ehits;
    const int lane = threadIdx.x & 31, nw = (gridDim.x * blockDim.x) >> 5;
    for (int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < nh; t += nw) {
        int i = x.ehits[t], b = list[i];
        int2 e = m.bv[b];
        unsigned long long key = resv_key(ep, i);
        bool own = false;
        if (lane == 0)
            own = valid_v(m, e.x) && valid_v(m, e.y) && holds_vertex(m, x, e.x, key) && holds_vertex(m, x, e.y, key);
        own = __shfl_sync(0xffffffffu, own, 0);
        if (own) {
            prefetch_flip(m, b, lane);
            FlipPlan P;
            bool planned = flip_plan(m, b, lane, P) && P.AC != P.BE;
            __syncwarp();
            if (lane == 0) {
                if (planned) flip_planned(m, b, eps, P);
                else flip_dev(m, b, eps);
                atomicAdd(&m.evt[EVT_COUNT * m.binst[b] + EVT_FLIPS], 1);
            }
        } else if (lane == 0) {
            x.edefer[i] = 1;
            atomicAdd(&x.ndefer[m.binst[b]], 1);
        }
        __syncwarp();
    }
}
/* One block per instance: its deferred flips in list order.  The block
 * tests FLIP_TPB entries at a time and warp 0 applies the deferred ones,
 * its lanes prefetching each flip's records. */
constexpr int FLIP_TPB = 512;
__global__ void __launch_bounds__(FLIP_TPB) k_flip_deferred(DevMesh m, DevScratch x, double eps, const int *list,
                                                            const int *n)
{
    griddep_wait();
    __shared__ unsigned hitmask[FLIP_TPB / 32];
    int inst = blockIdx.x, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (inst == 0 && threadIdx.x == 0) *x.n_ehits = 0;
    if (x.ndefer[inst] == 0) return;
    int lo = 0, hi = *n;
    if (m.ninst > 1) {
        lo = lower_bound_i(list, hi, m.boff[inst]);
        hi = lower_bound_i(list, hi, m.boff[inst + 1]);
    }
    for (int base = lo; base < hi; base += FLIP_TPB) {
        int i = base + (int)threadIdx.x;
        bool f = i < hi && x.edefer[i];
        unsigned w = __ballot_sync(0xffffffffu, f);
        if (lane == 0) hitmask[warp] = w;
        if (!__syncthreads_or(f)) continue;           /* the barrier also publishes hitmask */
        if (warp == 0) {
            for (int k = 0; k < FLIP_TPB / 32; k++) {
                unsigned hits = hitmask[k];
                while (hits) {
                    int j = __ffs(hits) - 1;
                    hits &= hits - 1;
                    int b = list[base + 32 * k + j];
                    prefetch_flip(m, b, lane);
                    FlipPlan P;
                    bool planned = flip_plan(m, b, lane, P) && P.AC != P.BE;
                    __syncwarp();
                    if (lane == 0) {
                        x.edefer[base + 32 * k + j] = 0;
                        if (planned) flip_planned(m, b, eps, P);
                        else flip_dev(m, b, eps);
                        m.evt[EVT_COUNT * inst + EVT_FLIPS]++;
                    }
                    __syncwarp();
                }
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) x.ndefer[inst] = 0;
}

/* ------------------------------------------------------------------ */
/* fix_grain_lists, src/topological.h:1035-1227                        */
/* ------------------------------------------------------------------ */
/* perform_ADD_ops, perform_REMOVE_ops, perform_REPLACE_ops
 * (src/topological.h:1035-1148) for one queued grain.  The reference runs
 * each over all grains before the next; an edit only touches its own
 * grain's list and only reads the mods, which nothing writes meanwhile, so
 * running the three for one grain back to back gives the same lists.
 *
 * One warp per grain.  The lanes copy the list to shared memory and read
 * the four mod slots of every listed vertex at once, recording for each
 * entry whether one of them is an ADD, REMOVE or REPLACE for this grain;
 * lane 0 then runs the three passes exactly as written (same visiting
 * order, same first-match searches, same shifts and -1 fills) on the
 * shared copy, reading the mods again only for the entries that hold an
 * edit (and the flags of a vertex an edit brings into the list), and the
 * lanes write back every entry the passes touched.  The long chain of
 * dependent global reads of one thread per grain becomes one parallel
 * round and a few L1 hits. */
constexpr int FIX_TPB = 256, FIX_WARPS = FIX_TPB / 32;
__device__ __forceinline__ unsigned mod_ops_for(const DevMesh &m, int v, int g)
{
    if ((unsigned)v >= (unsigned)m.nv) return 0;
    const int4 *md = m.vmod + 4 * (size_t)v;
    unsigned f = 0;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        int4 x = md[j];
        if (x.x == g) f |= x.w == FIX_ADD ? 1u : x.w == FIX_REMOVE ? 2u : x.w == FIX_REPLACE ? 4u : 0u;
    }
    return f;
}
__device__ void fix_grain_serial(const DevMesh &m, int g, int *Ls, unsigned char *Fs, int *Ss, unsigned char *SFs,
                                 int &n, int &hi)
{
    for (int i = 0; i < n; i++) {                        /* ADD */
        if (!(Fs[i] & 1u)) continue;
        const int v = Ls[i];
        for (int j = 0; j < 4; j++) {
            int4 md = m.vmod[4 * (size_t)v + j];
            if (!(md.w == FIX_ADD && md.x == g)) continue;
            int pos = -1;                                /* glist_add_after(g, md.y, md.z) */
            for (int k = 0; k < n; k++)
                if (Ls[k] == md.z) { pos = k + 1; break; }
            if (pos < 0) { raise_err(m, ERRB_TOPOLOGY); continue; }
            if (n >= SEVC_MAXV) { raise_err(m, ERRB_CAPACITY); continue; }
            for (int k = n; k > pos; k--) { Ls[k] = Ls[k - 1]; Fs[k] = Fs[k - 1]; }
            Ls[pos] = md.y;
            Fs[pos] = (unsigned char)mod_ops_for(m, md.y, g);
            n++;
            hi = n > hi ? n : hi;
        }
    }
    const int n0 = n;                                    /* REMOVE over the list as it stood */
    for (int i = 0; i < n0; i++) { Ss[i] = Ls[i]; SFs[i] = Fs[i]; }
    for (int i = 0; i < n0; i++) {
        if (!(SFs[i] & 2u)) continue;
        const int v = Ss[i];
        for (int j = 0; j < 4; j++) {
            int4 md = m.vmod[4 * (size_t)v + j];
            if (!(md.w == FIX_REMOVE && md.x == g)) continue;
            for (int k = 0; k < n; k++)                  /* glist_remove(g, md.y) */
                if (Ls[k] == md.y) {
                    for (int q = k; q < n - 1; q++) { Ls[q] = Ls[q + 1]; Fs[q] = Fs[q + 1]; }
                    n--;
                    Ls[n] = -1;
                    Fs[n] = 0;
                    break;
                }
        }
    }
    for (int i = 0; i < n; i++) {                        /* REPLACE */
        if (!(Fs[i] & 4u)) continue;
        const int v = Ls[i];
        for (int j = 0; j < 4; j++) {
            int4 md = m.vmod[4 * (size_t)v + j];
            if (!(md.w == FIX_REPLACE && md.x == g)) continue;
            for (int k = 0; k < n; k++)                  /* glist_replace(g, md.z, md.y) */
                if (Ls[k] == md.z) {
                    Ls[k] = md.y;
                    Fs[k] = (unsigned char)mod_ops_for(m, md.y, g);
                    break;
                }
        }
    }
}
__global__ void __launch_bounds__(FIX_TPB) k_fix_edit(DevMesh m)
{
    griddep_wait();
    __shared__ int Ls[FIX_WARPS][SEVC_MAXV], Ss[FIX_WARPS][SEVC_MAXV];
    __shared__ unsigned char Fs[FIX_WARPS][SEVC_MAXV], SFs[FIX_WARPS][SEVC_MAXV];
    __shared__ int Nw[FIX_WARPS][2];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int nf = min(*m.nfix, m.fixcap), nw = (gridDim.x * blockDim.x) >> 5;
    for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nf; w += nw) {
        const int g = m.fixlist[w];
        if (!(m.gen[g] && m.gfix[g])) continue;
        int *L = m.glist + (size_t)SEVC_MAXV * g;
        const int n = m.gvlen[g];
        for (int i = lane; i < n; i += 32) {
            int v = L[i];
            Ls[wib][i] = v;
            Fs[wib][i] = (unsigned char)mod_ops_for(m, v, g);
        }
        __syncwarp();
        if (lane == 0) {
            int nn = n, hi = n;
            fix_grain_serial(m, g, Ls[wib], Fs[wib], Ss[wib], SFs[wib], nn, hi);
            Nw[wib][0] = nn;
            Nw[wib][1] = hi;
            if (nn != n) m.gvlen[g] = nn;
        }
        __syncwarp();
        const int hi = Nw[wib][1];
        for (int i = lane; i < hi; i += 32) L[i] = Ls[wib][i];
        __syncwarp();
    }
}
/* clear_grains_fix_state (:1150-1163): fix = false for enabled grains and
 * reset the mods of every vertex listed by an enabled grain.  Only queued
 * grains can have fix set and only marked vertices can hold mods.
 *
 * areas: compute_grain_areas after the removals (src/main.cu:266) for the
 * grains this fix-up edited.  Only a grain whose list changed since the
 * grain pass can have a new area (the vertex a 3-sided removal moves
 * belongs only to grains that removal queues), and its list and vertices
 * are final for the step here; a grain edited by several fix-ups (2x3
 * passes, then the removals) is computed again by each, the last one on
 * the final positions.  The flips' fix-up comes after the counts and needs
 * none (the next step's grain pass computes every area). */
__global__ void k_fix_clear(DevMesh m, int areas)
{
    griddep_wait();
    int nf = min(*m.nfix, m.fixcap), nm = min(*m.nmod, m.modcap);
    for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < nf; w += gridDim.x * blockDim.x) {
        int g = m.fixlist[w];
        if (m.gen[g]) {
            m.gfix[g] = 0;
            if (areas) {
                double2 none = make_double2(0, 0);
                m.garea[g] = area_stream(m.glist + (size_t)SEVC_MAXV * g, m.gvlen[g], m.pos, -1, none, m.D);
            }
        }
    }
    for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < nm; w += gridDim.x * blockDim.x) {
        int v = m.modlist[w];
        m.vmodmark[v] = 0;
        int4 sg = m.vg[v];
        bool listed = false;
        for (int j = 0; j < 3 && !listed; j++) {
            int g = slot3(sg, j);
            if (g >= 0 && m.gen[g] && glist_find(m, g, v) >= 0) listed = true;
        }
        if (listed)
            for (int j = 0; j < 4; j++) m.vmod[4 * (size_t)v + j] = make_int4(-1, -1, -1, FIX_NONE);
    }
    /* empty both work lists once every block has read their lengths */
    if (last_block(m.lastblk + 0) && threadIdx.x == 0) {
        *m.nfix = 0;
        *m.nmod = 0;
    }
}

/* instance of every boundary and grain from the offset tables */
__global__ void k_fill_instance_ids(DevMesh m)
{
    int stride = gridDim.x * blockDim.x;
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < m.nb; b += stride)
        m.binst[b] = lower_bound_i(m.boff, m.ninst + 1, b + 1) - 1;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.ng; g += stride)
        m.ginst[g] = lower_bound_i(m.goff, m.ninst + 1, g + 1) - 1;
}

template <int KIND>
void compact_impl(const DevMesh &m, const DevScratch &x, int n, int *out, int *n_out, cudaStream_t s)
{
    int tiles = (n + CT_TILE - 1) / CT_TILE;
    if (tiles == 0) { cudaMemsetAsync(n_out, 0, sizeof(int), s); return; }
    /* the 16-byte flag reads need 16-byte aligned arrays (the handle's
     * allocation gives 256) */
    uintptr_t al = KIND == CK_CAND ? ((uintptr_t)m.ben | (uintptr_t)m.bcand)
                 : KIND == CK_GRAIN_CAND ? ((uintptr_t)m.gen | (uintptr_t)m.gcand) : (uintptr_t)m.bmark;
    bool flags16 = (KIND == CK_CAND || KIND == CK_GRAIN_CAND || KIND == CK_MARKED) && (al & 15u) == 0;
    if (flags16) {
        launch_dep(k_flag_count<KIND>, tiles, TPB, s, m, n, x.blockcnt);
        launch_dep(k_flag_scatter<KIND>, tiles, TPB, s, m, n, x.blockcnt, out, n_out);
    } else {
        COUNT_LAUNCHES(1), k_compact_count<KIND><<<tiles, TPB, 0, s>>>(m, n, x.blockcnt);
        COUNT_LAUNCHES(1), k_compact_scatter<KIND><<<tiles, TPB, 0, s>>>(m, n, x.blockcnt, out, n_out);
    }
}

inline int listgrid(int cap) { int g = (cap + TPB - 1) / TPB; return g < 4 * WL_BLOCKS ? g : 4 * WL_BLOCKS; }

} // namespace

void launch_compact(const DevMesh &m, const DevScratch &x, CompactKind kind, int *out, int *n_out, cudaStream_t s)
{
    switch (kind) {
    case CK_CAND: compact_impl<CK_CAND>(m, x, m.nb, out, n_out, s); break;
    case CK_TWO_THREE: compact_impl<CK_TWO_THREE>(m, x, m.nb, out, n_out, s); break;
    case CK_GRAIN_CAND: compact_impl<CK_GRAIN_CAND>(m, x, m.ng, out, n_out, s); break;
    case CK_GVLEN3: compact_impl<CK_GVLEN3>(m, x, m.ng, out, n_out, s); break;
    case CK_MARKED: compact_impl<CK_MARKED>(m, x, m.nb, out, n_out, s); break;
    }
}

void launch_two_three_first(const DevMesh &m, const DevScratch &x, int *out, int *n_out, cudaStream_t s)
{
    cudaMemsetAsync(m.bmark, 0, (size_t)m.nb, s);
    int g = (m.ng + TPB - 1) / TPB;
    COUNT_LAUNCHES(1), k_mark_two_three<<<g < 4 * WL_BLOCKS ? g : 4 * WL_BLOCKS, TPB, 0, s>>>(m, x.perm, x.vbucket);
    compact_impl<CK_MARKED>(m, x, m.nb, out, n_out, s);
}

void launch_poll_iteration(const DevMesh &m, const DevScratch &x, const int *cand, const int *ncand,
                           const StepParams &p, cudaStream_t s)
{
    int g = listgrid(m.nb);
    launch_dep(k_poll_vote, g, TPB, s, m, cand, ncand, x.nrun);
    launch_dep(k_poll_count, g, TPB, s, m, cand, ncand);
    launch_dep(k_poll_unlabel, g, TPB, s, m, cand, ncand);
    int grid = p.n_blocks * p.n_threads;
    bool aligned = (((uintptr_t)m.ben | (uintptr_t)m.bcand | (uintptr_t)m.bcandbuf) & 15u) == 0;
    if (p.ninst == 1 && grid >= 16 && aligned) {
        int th = (m.nb + 15) / 16;
        launch_dep(k_poll_compare_write16, (th + TPB - 1) / TPB, TPB, s, m, x.threadfail, grid);
    } else {
        launch_dep(k_poll_compare_write, (m.nb + TPB - 1) / TPB, TPB, s, m, x.threadfail, grid);
    }
    launch_dep(k_poll_final, dim3(p.n_blocks, p.ninst), p.n_threads, s, m, x.threadfail, x.pblock, x.pcnt, x.piters,
               x.nrun);
}

void launch_conflicts(const DevMesh &m, const int *cand, const int *ncand, cudaStream_t s)
{
    int g = listgrid(m.nb);
    launch_dep(k_conflict_check, g, TPB, s, m, cand, ncand);
    launch_dep(k_conflict_unlabel, g, TPB, s, m, cand, ncand);
}

inline int instgrid(const DevMesh &m) { return (m.ninst + 31) / 32; }

void launch_remove_two_three(const DevMesh &m, const DevScratch &x, const int *list, const int *n, int pass,
                             cudaStream_t s)
{
    COUNT_LAUNCHES(1), k_remove_two_three<<<instgrid(m), 32, 0, s>>>(m, list, n, x.extra,
                                                                     x.segcnt + (size_t)pass * m.ninst, nullptr);
}
void launch_remove_two_three_dev(const DevMesh &m, const DevScratch &x, const int *list, const int *n, cudaStream_t s)
{
    COUNT_LAUNCHES(1), k_remove_two_three<<<instgrid(m), 32, 0, s>>>(m, list, n, x.extra, x.segcnt, x.tt_pass);
}
void launch_poll_cond(const DevMesh &m, const DevScratch &x, cudaGraphConditionalHandle hnd, int cap, cudaStream_t s)
{
    COUNT_LAUNCHES(1), k_poll_cond<<<1, 32, 0, s>>>(hnd, x.nrun, x.ptot, cap, m.err);
}
void launch_tt_init(const DevScratch &x, cudaGraphConditionalHandle hnd, cudaStream_t s)
{
    COUNT_LAUNCHES(1), k_tt_init<<<1, 32, 0, s>>>(hnd, x.n_b, x.tt_first, x.tt_pass);
}
void launch_tt_cond(const DevScratch &x, cudaGraphConditionalHandle hnd, cudaStream_t s)
{
    COUNT_LAUNCHES(1), k_tt_cond<<<1, 32, 0, s>>>(hnd, x.n_b, x.tt_pass);
}
void launch_label_3sided_auto(const DevMesh &m, const DevScratch &x, double dt, cudaStream_t s)
{
    int g = (m.ng + TPB - 1) / TPB;
    launch_dep(k_label_3sided_auto, g < 4 * 152 ? g : 4 * 152, TPB, s, m, dt, x.perm, x.vbucket, x.tt_first);
}

void launch_label_3sided(const DevMesh &m, const DevScratch &x, double dt, bool bucket, cudaStream_t s)
{
    if (bucket) {
        int g = (m.ng + TPB - 1) / TPB;
        launch_dep(k_label_3sided_bucket, g < 4 * 152 ? g : 4 * 152, TPB, s, m, dt, x.perm, x.vbucket);
    } else {
        launch_dep(k_label_3sided, (m.ng + TPB - 1) / TPB, TPB, s, m, dt);
    }
}

void launch_remove_grains(const DevMesh &m, const DevScratch &x, const int *list, const int *n, cudaStream_t s)
{
    launch_dep(k_remove_reserve, 4 * WL_BLOCKS, TPB, s, m, x, list, n);
    launch_dep(k_remove_apply, 4 * WL_BLOCKS, TPB, s, m, x, list);
    launch_dep(k_remove_deferred, (m.ninst + 3) / 4, 128, s, m, x, list, n);
}


void launch_flips(const DevMesh &m, double eps, const int *cand, const int *ncand, const DevScratch &x,
                  cudaStream_t s)
{
    launch_dep(k_flip_reserve, 4 * WL_BLOCKS, TPB, s, m, x, cand, ncand);
    launch_dep(k_flip_apply, 4 * WL_BLOCKS, TPB, s, m, x, eps, cand);
    launch_dep(k_flip_deferred, m.ninst, FLIP_TPB, s, m, x, eps, cand, ncand);
}

void launch_fix_lists(const DevMesh &m, cudaStream_t s, bool areas)
{
    launch_dep(k_fix_edit, WL_BLOCKS, FIX_TPB, s, m);
    launch_dep(k_fix_clear, WL_BLOCKS, TPB, s, m, (int)areas);
}

void launch_fill_instance_ids(const DevMesh &m, cudaStream_t s)
{
    COUNT_LAUNCHES(1), k_fill_instance_ids<<<4 * WL_BLOCKS, TPB, 0, s>>>(m);
}
