/*
 * Engine: device memory, the order of one time step, and the C ABI of
 * include/sevc.h.
 *
 * The step follows src/main.cu:120-394 of the reference phase by phase;
 * the kernels live in sevc_geometry.cu, sevc_topology.cu and
 * sevc_nucleation.cu.  All work of a handle is enqueued on its own CUDA
 * stream; the host reads back only small counters (polling convergence,
 * 2x3 counts, the step summary).
 */
#include "sevc_internal.h"
#include "sevc_host.h"

#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <ftw.h>
#include <map>
#include <string>
#include <sys/stat.h>
#include <unistd.h>
#include <vector>

long long sevc_kernel_launches = 0;

struct ProfEntry { double ms = 0; int64_t launches = 0; };

struct sevc_handle {
    sevc_options opt;
    int nv = 0, nb = 0, ng = 0;
    cudaStream_t stream = nullptr;
    void *dblock = nullptr;
    DevMesh m{};
    DevScratch x{};
    StepParams p{};
    /* run state, src/main.cu:29-113 */
    int n = 0, curr_n_grains = 0, allow_nucleation = 0;
    double t = 0, nucleated_area = 0;
    int polling_cap = 100000;
    int exact_all = 0;
    /* pinned readback */
    int *h_ctr = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    bool profiling = false;
    std::map<std::string, ProfEntry> prof;
    std::vector<std::pair<std::string, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
    std::vector<cudaEvent_t> evpool;
};

namespace {

bool cuda_ok(cudaError_t e, const char *what)
{
    if (e == cudaSuccess) return true;
    sevc_set_error("%s: %s", what, cudaGetErrorString(e));
    return false;
}

cudaEvent_t pool_event(sevc_handle *h)
{
    if (!h->evpool.empty()) { cudaEvent_t e = h->evpool.back(); h->evpool.pop_back(); return e; }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}

/* time a group of launches when profiling is on */
struct Prof {
    sevc_handle *h;
    const char *name;
    cudaEvent_t a = nullptr;
    Prof(sevc_handle *hh, const char *n) : h(hh), name(n)
    {
        if (h->profiling) { a = pool_event(h); cudaEventRecord(a, h->stream); }
    }
    ~Prof()
    {
        if (!h->profiling) return;
        cudaEvent_t b = pool_event(h);
        cudaEventRecord(b, h->stream);
        h->pending.push_back({ name, { a, b } });
    }
};

void prof_collect(sevc_handle *h)
{
    for (auto &pe : h->pending) {
        float ms = 0;
        cudaEventElapsedTime(&ms, pe.second.first, pe.second.second);
        auto &e = h->prof[pe.first];
        e.ms += ms;
        e.launches += 1;
        h->evpool.push_back(pe.second.first);
        h->evpool.push_back(pe.second.second);
    }
    h->pending.clear();
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

/* one device allocation carved into every array */
bool alloc_device(sevc_handle *h)
{
    size_t V = h->nv, B = h->nb, G = h->ng;
    int grid = h->p.n_blocks * h->p.n_threads;
    size_t maxn = B > G ? B : G;
    size_t tiles = (maxn + 4095) / 4096 + 1;
    struct Req { void **p; size_t bytes; };
    DevMesh &m = h->m;
    DevScratch &x = h->x;
    std::vector<Req> r = {
        { (void **)&m.pos, V * 16 }, { (void **)&m.vel, V * 16 }, { (void **)&m.terms, V * 32 },
        { (void **)&m.contrib, V * 48 }, { (void **)&m.venergy, V * 8 }, { (void **)&m.ven, V },
        { (void **)&m.vb, V * 16 }, { (void **)&m.vg, V * 16 }, { (void **)&m.vmod, V * 64 },
        { (void **)&m.voted, V * 4 }, { (void **)&m.vmodmark, V }, { (void **)&m.modlist, V * 4 },
        { (void **)&m.bv, B * 8 }, { (void **)&m.benergy, B * 8 }, { (void **)&m.blen, B * 8 },
        { (void **)&m.btext, B * 8 }, { (void **)&m.ben, B }, { (void **)&m.bcand, B },
        { (void **)&m.bcandbuf, B }, { (void **)&m.bvotes, B * 4 }, { (void **)&m.bconf, B * 4 },
        { (void **)&m.glist, G * SEVC_MAXV * 4 }, { (void **)&m.gvlen, G * 4 }, { (void **)&m.garea, G * 8 },
        { (void **)&m.gdadt, G * 8 }, { (void **)&m.gori, G * 8 }, { (void **)&m.gse, G * 8 },
        { (void **)&m.gq, G * 8 }, { (void **)&m.gen, G }, { (void **)&m.gcand, G }, { (void **)&m.gfix, G },
        { (void **)&m.gtype, G }, { (void **)&m.fixlist, G * 4 }, { (void **)&m.nfix, 4 }, { (void **)&m.nmod, 4 },
        { (void **)&m.err, 16 }, { (void **)&m.evt, 16 },
        { (void **)&x.list_a, maxn * 4 }, { (void **)&x.list_b, maxn * 4 }, { (void **)&x.list_c, maxn * 4 },
        { (void **)&x.n_a, 4 }, { (void **)&x.n_b, 4 }, { (void **)&x.n_c, 4 }, { (void **)&x.blockcnt, tiles * 4 },
        { (void **)&x.extra, 1024 * 4 }, { (void **)&x.threadfail, (size_t)grid * 4 },
        { (void **)&x.block_area, (size_t)h->p.n_blocks * 8 }, { (void **)&x.counters, CTR_COUNT * 4 },
        { (void **)&x.rng, 8192 * sizeof(curandState) }, { (void **)&x.rng_saved, 8192 * sizeof(curandState) },
        { (void **)&x.nucl_buf, 64 * 4 }, { (void **)&x.vbucket, 64 * 4 }, { (void **)&x.perm, G * 4 },
        { (void **)&x.n_perm, 4 }, { (void **)&m.adirty, G * 4 }, { (void **)&m.nadirty, 4 }, { (void **)&m.gadirty, G },
        { (void **)&m.nlist, G * 4 }, { (void **)&m.nnlist, 4 }, { (void **)&m.bforce, B },
    };
    size_t total = 0;
    for (auto &q : r) total += align256(q.bytes);
    char *base = nullptr;
    if (!cuda_ok(cudaMalloc(&base, total), "cudaMalloc mesh")) return false;
    if (!cuda_ok(cudaMemsetAsync(base, 0, total, h->stream), "memset")) return false;
    h->dblock = base;
    for (auto &q : r) { *q.p = base; base += align256(q.bytes); }
    m.nv = h->nv; m.nb = h->nb; m.ng = h->ng; m.D = h->opt.domain_bound;
    return true;
}

bool upload(sevc_handle *h, const sevc_mesh_host &hm)
{
    size_t V = h->nv, B = h->nb, G = h->ng;
    std::vector<double2> d2(V);
    std::vector<int4> i4(V);
    cudaStream_t s = h->stream;
    auto put = [&](void *dst, const void *src, size_t bytes) {
        return cuda_ok(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s), "upload") &&
               cuda_ok(cudaStreamSynchronize(s), "upload sync");
    };
    for (size_t i = 0; i < V; i++) d2[i] = make_double2(hm.px[i], hm.py[i]);
    if (!put(h->m.pos, d2.data(), V * 16)) return false;
    for (size_t i = 0; i < V; i++) d2[i] = make_double2(hm.vx[i], hm.vy[i]);
    if (!put(h->m.vel, d2.data(), V * 16)) return false;
    for (size_t i = 0; i < V; i++) i4[i] = make_int4(hm.vb[3 * i], hm.vb[3 * i + 1], hm.vb[3 * i + 2], -1);
    if (!put(h->m.vb, i4.data(), V * 16)) return false;
    for (size_t i = 0; i < V; i++) i4[i] = make_int4(hm.vg[3 * i], hm.vg[3 * i + 1], hm.vg[3 * i + 2], -1);
    if (!put(h->m.vg, i4.data(), V * 16)) return false;
    if (!put(h->m.ven, hm.ven, V) || !put(h->m.venergy, hm.venergy, V * 8)) return false;
    {
        std::vector<int4> md(4 * V, make_int4(-1, -1, -1, FIX_NONE));
        if (!put(h->m.vmod, md.data(), 4 * V * 16)) return false;
        std::vector<int> neg(V, -1);
        if (!put(h->m.voted, neg.data(), V * 4)) return false;
    }
    std::vector<int2> bv(B);
    for (size_t i = 0; i < B; i++) bv[i] = make_int2(hm.bini[i], hm.bend[i]);
    if (!put(h->m.bv, bv.data(), B * 8)) return false;
    if (!put(h->m.benergy, hm.benergy, B * 8) || !put(h->m.blen, hm.blen, B * 8) ||
        !put(h->m.btext, hm.btext, B * 8) || !put(h->m.ben, hm.ben, B) || !put(h->m.bcand, hm.bcand, B))
        return false;
    {
        std::vector<int> neg(B, -1);
        if (!put(h->m.bconf, neg.data(), B * 4)) return false;
    }
    if (!put(h->m.glist, hm.glist, G * SEVC_MAXV * 4) || !put(h->m.gvlen, hm.gvlen, G * 4) ||
        !put(h->m.garea, hm.garea, G * 8) || !put(h->m.gdadt, hm.gdadt, G * 8) || !put(h->m.gori, hm.gori, G * 8) ||
        !put(h->m.gse, hm.gse, G * 8) || !put(h->m.gen, hm.gen, G) || !put(h->m.gtype, hm.gtype, G))
        return false;
    return true;
}

sevc_status validate(const sevc_options *o)
{
    if (!(o->dt > 0)) { sevc_set_error("dt must be > 0"); return SEVC_ERR_ARG; }
    if (o->n_threads < 1 || o->n_threads > 256 || o->n_blocks < 1) {
        sevc_set_error("n_threads must be in [1,256] and n_blocks >= 1 (src/utils.h:4-5 sizes)");
        return SEVC_ERR_ARG;
    }
    if (o->do_nucleation && (o->n_blocks != 32 || o->n_threads != 256)) {
        sevc_set_error("nucleation needs n_blocks=32 and n_threads=256 (src/nucleation2.cu:295-396)");
        return SEVC_ERR_ARG;
    }
    if (o->do_nucleation && o->nucleation_gap <= 0) {
        sevc_set_error("dtau/dt < 1 makes nucleation_gap 0 (src/main.cu:141 would divide by zero)");
        return SEVC_ERR_ARG;
    }
    return SEVC_OK;
}

sevc_status require_device()
{
    int dev = 0;
    if (cudaGetDeviceCount(&dev) != cudaSuccess || dev == 0) {
        sevc_set_error("no CUDA device");
        return SEVC_ERR_CUDA;
    }
    return SEVC_OK;
}

sevc_status create_from_host(const sevc_options *opt, sevc_hmesh *hm, sevc_handle **out)
{
    *out = nullptr;
    if (require_device()) return SEVC_ERR_CUDA;
    sevc_handle *h = new sevc_handle();
    h->opt = *opt;
    h->nv = hm->m.nv; h->nb = hm->m.nb; h->ng = hm->m.ng;
    h->p.dt = opt->dt; h->p.eps = opt->GB_eps; h->p.scaling = opt->GB_scaling; h->p.MC_k = opt->MC_k;
    h->p.n_blocks = opt->n_blocks; h->p.n_threads = opt->n_threads;
    h->curr_n_grains = h->ng;
    if (!cuda_ok(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking), "stream") ||
        !cuda_ok(cudaMallocHost(&h->h_ctr, 256), "pinned") || !alloc_device(h) || !upload(h, hm->m)) {
        sevc_destroy(h);
        return SEVC_ERR_CUDA;
    }
    cudaEventCreate(&h->ev0);
    cudaEventCreate(&h->ev1);
    launch_rng_init(h->x.rng, 8192, h->stream);                           /* src/main.cu:81 */
    if (!cuda_ok(cudaStreamSynchronize(h->stream), "init")) { sevc_destroy(h); return SEVC_ERR_CUDA; }
    *out = h;
    return SEVC_OK;
}

sevc_status read_ints(sevc_handle *h, const int *dsrc, int n, int *dst)
{
    if (!cuda_ok(cudaMemcpyAsync(h->h_ctr, dsrc, n * sizeof(int), cudaMemcpyDeviceToHost, h->stream), "readback") ||
        !cuda_ok(cudaStreamSynchronize(h->stream), "readback sync"))
        return SEVC_ERR_CUDA;
    memcpy(dst, h->h_ctr, n * sizeof(int));
    return SEVC_OK;
}

sevc_status err_bits_to_status(int bits)
{
    if (bits & ERRB_CAPACITY) { sevc_set_error("a grain list exceeded %d vertices", SEVC_MAXV); return SEVC_ERR_CAPACITY; }
    if (bits & ERRB_TOPOLOGY) { sevc_set_error("inconsistent mesh met by an event kernel"); return SEVC_ERR_TOPOLOGY; }
    if (bits & ERRB_RNG) { sevc_set_error("nucleation picked no valid vertex (the reference reads stale data here)"); return SEVC_ERR_TOPOLOGY; }
    if (bits & ERRB_WORKLIST) { sevc_set_error("internal worklist overflow"); return SEVC_ERR_CAPACITY; }
    return SEVC_OK;
}

} // namespace

/* ================================================================== */
/* C ABI                                                               */
/* ================================================================== */
extern "C" {

sevc_status sevc_create(const sevc_options *opt, sevc_handle **out)
{
    if (!opt || !out) return SEVC_ERR_ARG;
    if (require_device()) return SEVC_ERR_CUDA;
    sevc_status st = validate(opt);
    if (st) return st;
    sevc_hmesh hm;
    int rc = sevc_host_load_files(opt, &hm);
    if (rc) return (sevc_status)rc;
    st = create_from_host(opt, &hm, out);
    sevc_hmesh_free(&hm);
    return st;
}

sevc_status sevc_create_from_arrays(const sevc_options *opt, int nv, const double *xy, int nb, const int32_t *ridges,
                                    int ng, const double *oris, const double *se, sevc_handle **out)
{
    if (!opt || !out || !xy || !ridges || !oris || !se) return SEVC_ERR_ARG;
    if (require_device()) return SEVC_ERR_CUDA;
    sevc_status st = validate(opt);
    if (st) return st;
    if (ng != opt->n_grains) { sevc_set_error("ng != opt->n_grains"); return SEVC_ERR_ARG; }
    sevc_hmesh hm;
    int rc = sevc_host_build(opt, nv, xy, nb, ridges, ng, oris, ng, se, &hm);
    if (rc) return (sevc_status)rc;
    st = create_from_host(opt, &hm, out);
    sevc_hmesh_free(&hm);
    return st;
}

void sevc_destroy(sevc_handle *h)
{
    if (!h) return;
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->dblock) cudaFree(h->dblock);
    if (h->h_ctr) cudaFreeHost(h->h_ctr);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    for (auto e : h->evpool) cudaEventDestroy(e);
    for (auto &pe : h->pending) { cudaEventDestroy(pe.second.first); cudaEventDestroy(pe.second.second); }
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

int sevc_should_continue(const sevc_handle *h)
{
    const sevc_options &o = h->opt;
    int mg = o.min_grains;
    return ((h->t <= o.tmax && o.tmax > 0) || (h->n <= o.nmax && o.nmax > 0)) &&
           (h->curr_n_grains >= mg && mg > 0);
}

sevc_status sevc_step(sevc_handle *h, sevc_step_info *info)
{
    if (!h) return SEVC_ERR_ARG;
    cudaStream_t s = h->stream;
    const sevc_options &o = h->opt;
    DevMesh &m = h->m;
    DevScratch &x = h->x;
    sevc_step_info loc;
    memset(&loc, 0, sizeof loc);
    loc.n = h->n;
    loc.t = h->t;
    long long launches0 = sevc_kernel_launches;
    cudaEventRecord(h->ev0, s);
    cudaMemsetAsync(m.err, 0, 16, s);
    cudaMemsetAsync(m.evt, 0, 16, s);
    launch_area_dirty(m, 0, s);   /* drop the previous step's post-area marks */

    { Prof pr(h, "boundary_geometry"); launch_boundary_geometry(m, o.GB_eps, o.GB_scaling, s); } /* :124-130 */
    if (h->curr_n_grains <= 5 * o.n_grains / 6) h->allow_nucleation = 1;                        /* :137 */
    if (o.do_nucleation && o.nucleation_gap > 0 && (h->n % o.nucleation_gap) == 0 && h->allow_nucleation) {
        loc.nucleation_attempted = 1;
        { Prof pr(h, "nucleation"); launch_nucleation(m, x, h->p, s); }                           /* :144-168 */
        { Prof pr(h, "boundary_geometry"); launch_boundary_geometry(m, o.GB_eps, o.GB_scaling, s); } /* :171-181 */
    }
    { Prof pr(h, "grain_fd"); launch_grain_fd(m, x, s); }                                         /* :127,:203 */
    { Prof pr(h, "vertex_fd"); launch_vertex_fd(m, s); }                                          /* :133,:203 */
    /* The first count of the 2x3 loop (:228) depends only on the topology,
     * which nothing changes before that loop: count now, and learn whether
     * this step can disable boundaries other than 3-sided grains' or export.
     * Otherwise only 3-sided grains' dA/dt and the extinction times that
     * matter are computed (see k_text_label). */
    int c23 = 0, n3 = 0;
    { Prof pr(h, "two_three_count"); launch_compact(m, x, CK_TWO_THREE, x.list_b, x.n_b, s); }
    if (!cuda_ok(cudaMemcpyAsync(h->h_ctr, x.n_b, 4, cudaMemcpyDeviceToHost, s), "readback") ||
        !cuda_ok(cudaMemcpyAsync(h->h_ctr + 1, x.vbucket + VB_COUNT(3), 4, cudaMemcpyDeviceToHost, s), "readback") ||
        !cuda_ok(cudaStreamSynchronize(s), "sync"))
        return SEVC_ERR_CUDA;
    c23 = h->h_ctr[0];
    n3 = h->h_ctr[1];
    int mg = o.min_grains;
    int full = h->exact_all || o.dt >= 100 || (o.snap_gap > 0 && h->n % o.snap_gap == 0) || c23 > 0 ||
               (mg > 0 && h->curr_n_grains + 1 - n3 <= mg);
    loc.outputs_complete = full;
    if (!full) { Prof pr(h, "text_label"); launch_mark_force(m, x, n3, s); }
    { Prof pr(h, "grain_dadt"); launch_grain_dadt(m, x, full, n3, s); }                           /* :206 */
    { Prof pr(h, "text_label"); launch_text_label(m, o.dt, full, s); }                            /* :212-216 */
    { Prof pr(h, "compact"); launch_compact(m, x, CK_CAND, x.list_a, x.n_a, s); }

    int conv = 0, it = 0;                                                                          /* :219 */
    while (!conv) {
        if (it >= h->polling_cap) { sevc_set_error("polling did not converge"); return SEVC_ERR_NONCONVERGED; }
        it++;
        { Prof pr(h, "polling"); launch_poll_iteration(m, x, x.list_a, x.n_a, h->p, s); }
        if (read_ints(h, x.counters + CTR_CONVERGED, 1, &conv)) return SEVC_ERR_CUDA;
    }
    loc.polling_iters = it;
    { Prof pr(h, "conflicts"); launch_conflicts(m, x.list_a, x.n_a, s); }                         /* :222-225 */

    for (int k = 0; k < 20; k++) {                                                                 /* :227-250 */
        int c = c23;
        if (k > 0) {
            { Prof pr(h, "two_three_count"); launch_compact(m, x, CK_TWO_THREE, x.list_b, x.n_b, s); }
            if (read_ints(h, x.n_b, 1, &c)) return SEVC_ERR_CUDA;
        }
        loc.two_three_counts[k] = c;
        loc.n_two_three_iters = k + 1;
        if (c == 0) break;
        { Prof pr(h, "two_three_remove"); launch_remove_two_three(m, x, x.list_b, x.n_b, s); }
        { Prof pr(h, "fix_lists"); launch_fix_lists(m, s); }
    }
    { Prof pr(h, "label_3sided"); launch_label_3sided(m, o.dt, s); }                              /* :252-255 */
    { Prof pr(h, "compact"); launch_compact(m, x, CK_GRAIN_CAND, x.list_c, x.n_c, s); }
    { Prof pr(h, "remove_grains"); launch_remove_grains(m, x.list_c, x.n_c, s); }                 /* :259 */
    { Prof pr(h, "fix_lists"); launch_fix_lists(m, s); }                                          /* :262 */
    { Prof pr(h, "grain_area"); launch_area_dirty(m, 1, s); }                                     /* :266 */
    { Prof pr(h, "unlabel_st2"); launch_unlabel_st2(m, x.list_a, x.n_a, s); }                     /* :282 */
    { Prof pr(h, "flips"); launch_flips(m, o.GB_eps, x.list_a, x.n_a, x, s); }                     /* :289 */
    { Prof pr(h, "fix_lists"); launch_fix_lists(m, s); }                                          /* :294 */
    { Prof pr(h, "update"); launch_update_positions(m, o.dt, s); }                                /* :314 */
    { Prof pr(h, "counts"); launch_counts(m, x, h->p, s); }                                       /* :317-325 */
    cudaEventRecord(h->ev1, s);

    int ctr[CTR_COUNT];
    if (read_ints(h, x.counters, CTR_COUNT, ctr)) return SEVC_ERR_CUDA;
    int ev[8];
    if (read_ints(h, m.err, 4, ev) || read_ints(h, m.evt, 4, ev + 4)) return SEVC_ERR_CUDA;
    float ms = 0;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    if (h->profiling) prof_collect(h);
    h->curr_n_grains = ctr[CTR_NGRAINS];
    double na;
    memcpy(&na, ctr + CTR_NUCL_AREA_SLOT, sizeof(double));
    h->nucleated_area = na;
    loc.curr_n_grains = h->curr_n_grains;
    loc.nucleated_area = na;
    loc.n_two_three = ev[4 + EVT_TWO_THREE];
    loc.n_removals = ev[4 + EVT_REMOVALS];
    loc.n_flips = ev[4 + EVT_FLIPS];
    loc.n_nucleations = ev[4 + EVT_NUCLEATIONS];
    loc.nucleation_candidate = loc.nucleation_attempted ? ctr[CTR_CANDIDATE] : -1;
    loc.gpu_ms = ms;
    loc.kernel_launches = (int)(sevc_kernel_launches - launches0);
    loc.export_due = (o.snap_gap > 0 && h->n % o.snap_gap == 0) || (h->curr_n_grains <= mg && mg > 0); /* :328 */
    h->n++;                                                                                         /* :388-389 */
    h->t = h->n * o.dt;
    loc.keep_going = (h->curr_n_grains <= mg && mg > 0) ? 0 : sevc_should_continue(h);             /* :391 */
    if (info) *info = loc;
    return err_bits_to_status(ev[0]);
}

sevc_status sevc_run_steps(sevc_handle *h, int nsteps, int *done, sevc_step_info *last)
{
    sevc_step_info inf;
    memset(&inf, 0, sizeof inf);
    int k = 0;
    sevc_status st = SEVC_OK;
    while (k < nsteps) {
        st = sevc_step(h, &inf);
        k++;
        if (st || !inf.keep_going) break;
    }
    if (done) *done = k;
    if (last) *last = inf;
    return st;
}

sevc_status sevc_mesh_sizes(const sevc_handle *h, int *nv, int *nb, int *ng)
{
    if (!h) return SEVC_ERR_ARG;
    if (nv) *nv = h->nv;
    if (nb) *nb = h->nb;
    if (ng) *ng = h->ng;
    return SEVC_OK;
}

sevc_status sevc_get_state(sevc_handle *h, sevc_mesh_host *o)
{
    if (!h || !o) return SEVC_ERR_ARG;
    size_t V = h->nv, B = h->nb, G = h->ng;
    cudaStream_t s = h->stream;
    std::vector<double2> d2(V);
    std::vector<DevMesh::FdTerms> d4(V);
    std::vector<int4> i4(V);
    std::vector<int2> i2(B);
    auto get = [&](void *dst, const void *src, size_t bytes) {
        return cuda_ok(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s), "download");
    };
    bool ok = get(d2.data(), h->m.pos, V * 16) && cuda_ok(cudaStreamSynchronize(s), "sync");
    if (!ok) return SEVC_ERR_CUDA;
    for (size_t i = 0; i < V; i++) { o->px[i] = d2[i].x; o->py[i] = d2[i].y; }
    if (!get(d2.data(), h->m.vel, V * 16) || !cuda_ok(cudaStreamSynchronize(s), "sync")) return SEVC_ERR_CUDA;
    for (size_t i = 0; i < V; i++) { o->vx[i] = d2[i].x; o->vy[i] = d2[i].y; }
    if (!get(d4.data(), h->m.terms, V * 32) || !cuda_ok(cudaStreamSynchronize(s), "sync")) return SEVC_ERR_CUDA;
    for (size_t i = 0; i < V; i++) {            /* src/calculus.h:63-69: -term / grad_eps */
        o->vel_bnd_x[i] = -d4[i].bx / SEVC_GRAD_EPS;
        o->vel_grn_x[i] = -d4[i].gx / SEVC_GRAD_EPS;
        o->vel_bnd_y[i] = -d4[i].by / SEVC_GRAD_EPS;
        o->vel_grn_y[i] = -d4[i].gy / SEVC_GRAD_EPS;
    }
    if (!get(i4.data(), h->m.vb, V * 16) || !cuda_ok(cudaStreamSynchronize(s), "sync")) return SEVC_ERR_CUDA;
    for (size_t i = 0; i < V; i++) { o->vb[3 * i] = i4[i].x; o->vb[3 * i + 1] = i4[i].y; o->vb[3 * i + 2] = i4[i].z; }
    if (!get(i4.data(), h->m.vg, V * 16) || !cuda_ok(cudaStreamSynchronize(s), "sync")) return SEVC_ERR_CUDA;
    for (size_t i = 0; i < V; i++) { o->vg[3 * i] = i4[i].x; o->vg[3 * i + 1] = i4[i].y; o->vg[3 * i + 2] = i4[i].z; }
    if (!get(i2.data(), h->m.bv, B * 8) || !cuda_ok(cudaStreamSynchronize(s), "sync")) return SEVC_ERR_CUDA;
    for (size_t i = 0; i < B; i++) { o->bini[i] = i2[i].x; o->bend[i] = i2[i].y; }
    ok = get(o->venergy, h->m.venergy, V * 8) && get(o->ven, h->m.ven, V) && get(o->benergy, h->m.benergy, B * 8) &&
         get(o->blen, h->m.blen, B * 8) && get(o->btext, h->m.btext, B * 8) && get(o->ben, h->m.ben, B) &&
         get(o->bcand, h->m.bcand, B) && get(o->glist, h->m.glist, G * SEVC_MAXV * 4) &&
         get(o->gvlen, h->m.gvlen, G * 4) && get(o->garea, h->m.garea, G * 8) && get(o->gdadt, h->m.gdadt, G * 8) &&
         get(o->gori, h->m.gori, G * 8) && get(o->gse, h->m.gse, G * 8) && get(o->gen, h->m.gen, G) &&
         get(o->gtype, h->m.gtype, G) && cuda_ok(cudaStreamSynchronize(s), "sync");
    return ok ? SEVC_OK : SEVC_ERR_CUDA;
}

sevc_status sevc_export_text(sevc_handle *h, const char *path, double time)
{
    if (!h || !path) return SEVC_ERR_ARG;
    sevc_hmesh hm;
    if (sevc_hmesh_alloc(&hm, h->nv, h->nb, h->ng)) return SEVC_ERR_CAPACITY;
    sevc_status st = sevc_get_state(h, &hm.m);
    if (!st) st = (sevc_status)sevc_host_export(&hm.m, &h->opt, path, time);
    sevc_hmesh_free(&hm);
    return st;
}

sevc_status sevc_check_data(sevc_handle *h, int *n_bad)
{
    if (!h || !n_bad) return SEVC_ERR_ARG;
    sevc_hmesh hm;
    if (sevc_hmesh_alloc(&hm, h->nv, h->nb, h->ng)) return SEVC_ERR_CAPACITY;
    sevc_status st = sevc_get_state(h, &hm.m);
    if (!st) *n_bad = sevc_host_check(&hm.m);
    sevc_hmesh_free(&hm);
    return st;
}

sevc_status sevc_rng_record(int nstreams, int ndraws, double *out)
{
    if (nstreams <= 0 || ndraws <= 0 || !out) return SEVC_ERR_ARG;
    int dev = 0;
    if (cudaGetDeviceCount(&dev) != cudaSuccess || dev == 0) { sevc_set_error("no CUDA device"); return SEVC_ERR_CUDA; }
    return rng_record(nstreams, ndraws, out) ? SEVC_ERR_CUDA : SEVC_OK;
}

sevc_status sevc_set_exact_all(sevc_handle *h, int on)
{
    if (!h) return SEVC_ERR_ARG;
    h->exact_all = on != 0;
    return SEVC_OK;
}

sevc_status sevc_set_profiling(sevc_handle *h, int on)
{
    if (!h) return SEVC_ERR_ARG;
    h->profiling = on != 0;
    if (!on) h->prof.clear();
    return SEVC_OK;
}

sevc_status sevc_get_profile(sevc_handle *h, int max_entries, char (*names)[48], double *ms, int64_t *launches,
                             int *n_entries)
{
    if (!h || !n_entries) return SEVC_ERR_ARG;
    int k = 0;
    for (auto &e : h->prof) {
        if (k < max_entries) {
            snprintf(names[k], 48, "%s", e.first.c_str());
            ms[k] = e.second.ms;
            launches[k] = e.second.launches;
        }
        k++;
    }
    *n_entries = k;
    return SEVC_OK;
}

/* ------------------------------------------------------------------ */
/* the program, src/main.cu:21-424                                     */
/* ------------------------------------------------------------------ */
static int rm_entry(const char *p, const struct stat *, int, struct FTW *) { return remove(p); }

/* create_folders, src/io.h:21-52 */
static bool make_folders(sevc_options *o, int verbose)
{
    struct stat st;
    if (o->output_folder[0] == '\0') {
        time_t t = time(NULL);
        struct tm tm = *localtime(&t);
        strftime(o->output_folder, sizeof o->output_folder, "%Y%m%d_%H%M%S", &tm);
        if (verbose) printf("No folder was found in .ini\n");
    } else if (stat(o->output_folder, &st) != -1) {
        if (verbose) printf("Folder already exists. Overwritting...\n");
        nftw(o->output_folder, rm_entry, 16, FTW_DEPTH | FTW_PHYS);
        if (verbose) printf("rm -rf %s\n", o->output_folder);
    }
    mkdir(o->output_folder, 0775);
    char data[300];
    snprintf(data, sizeof data, "%s/DATA", o->output_folder);
    mkdir(data, 0775);
    snprintf(o->output_folder, sizeof o->output_folder, "%s", data);
    if (verbose) printf("mkdir %s\n", o->output_folder);
    return true;
}

sevc_status sevc_run_program(const sevc_options *opt_in, int verbose)
{
    sevc_options opt = *opt_in;
    make_folders(&opt, verbose);
    if (verbose && opt.min_grains > 0) printf("Saving up to %d grains.\n", opt.min_grains);
    sevc_handle *h = nullptr;
    sevc_status st = sevc_create(&opt, &h);
    if (st) return st;
    if (verbose) printf("%d grains loaded.\nData loaded.\n", h->ng);
    sevc_hmesh hm;
    if (sevc_hmesh_alloc(&hm, h->nv, h->nb, h->ng)) { sevc_destroy(h); return SEVC_ERR_CAPACITY; }
    int prog = 0;
    while (sevc_should_continue(h)) {
        if (verbose) printf("n = %d, t = %f\n", h->n, h->t);
        sevc_step_info inf;
        st = sevc_step(h, &inf);
        if (st) break;
        if (verbose) {
            for (int k = 0; k < inf.n_two_three_iters; k++)
                printf("%d configurations of two three sided grains\n", inf.two_three_counts[k]);
            printf("Number of grains: %d\n", inf.curr_n_grains);
            printf("Nucleated area %%: %.16f\n", inf.nucleated_area);
        }
        if (inf.export_due) {
            if (verbose)
                printf("Saving at n=%d, t=%.16f, n_grains=%d, nucl_area=%.16f\n", inf.n, inf.t, inf.curr_n_grains,
                       inf.nucleated_area);
            if ((st = sevc_get_state(h, &hm.m))) break;
            if (sevc_host_check(&hm.m)) {
                if (verbose) printf("Error while saving output file. Exiting...\n");
                break;
            }
            if (verbose) printf("Valid data. Saving...\n");
            char path[600];
            snprintf(path, sizeof path, "%s/%06d.txt", opt.output_folder, prog);
            if ((st = (sevc_status)sevc_host_export(&hm.m, &h->opt, path, inf.t))) break;
            prog++;
        }
        if (!inf.keep_going) break;
    }
    if (verbose) {
        printf("\nPerformed %d iterations.\n", h->n - 1);
        printf("Number of grains: %d\n", h->curr_n_grains);
        printf("Done.\n");
    }
    sevc_hmesh_free(&hm);
    sevc_destroy(h);
    return st;
}

} // extern "C"
