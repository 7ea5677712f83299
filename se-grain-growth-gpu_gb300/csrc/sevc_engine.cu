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

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <ftw.h>
#include <functional>
#include <map>
#include <string>
#include <thread>
#include <sys/stat.h>
#include <unistd.h>
#include <vector>

long long sevc_kernel_launches = 0;
thread_local bool sevc_pdl_off = false;
thread_local int sevc_pdl_skip = 0;

struct ProfEntry { double ms = 0; int64_t launches = 0; };

struct StepGraph {
    cudaGraphExec_t exec = nullptr;
    int kernels = 0;   /* kernels one replay launches */
};

/* host part of the run state (the device part is the handle's block) */
struct RunState {
    int n = 0, curr_n_grains = 0;
    double t = 0, nucleated_area = 0;
    std::vector<int> icurr, iallow;
    std::vector<double> iarea;
};

/* Adjoint tape: checkpoints of the whole device block every `every` steps;
 * the backward pass replays one segment at a time from its checkpoint,
 * recording what the adjoint of each step needs. */
struct Tape {
    int every = 0;                 /* 0: not taping */
    long long nsteps = 0;          /* steps taken since the tape started */
    bool replaying = false;
    std::vector<void *> ckpt;      /* device copies, state after k*every steps */
    std::vector<RunState> runs;
    void *rec = nullptr;           /* per-step records of one segment */
    size_t rec_step_bytes = 0;
    int rec_steps = 0, log_cap = 0;
    void *adj = nullptr;           /* AdjointBuffers storage */
    size_t adj_bytes = 0;
    double *separam = nullptr;     /* the stored energies when the tape started */
    /* set while a segment is replayed: after a step's nucleation kernels,
     * copies the mesh (as the velocities will see it) into that step's
     * record */
    std::function<void(cudaStream_t)> after_nucleation;
};

struct sevc_handle {
    sevc_options opt;
    int nv = 0, nb = 0, ng = 0;
    cudaStream_t stream = nullptr;
    void *dblock = nullptr;
    DevMesh m{};
    DevScratch x{};
    StepParams p{};
    /* run state, src/main.cu:29-113 */
    int n = 0, curr_n_grains = 0;
    double t = 0, nucleated_area = 0;
    int polling_cap = 100000;
    int exact_all = 0;
    int outputs_complete = 1;   /* the last step computed every output-only value */
    /* instances (one for a plain handle): entity offsets, initial grain
     * count (the n_grains of src/main.cu:137), per-instance run state and
     * the per-instance summary of the last step */
    int ninst = 1;
    std::vector<int> voff, boff, goff, ng0, icurr, iallow;
    std::vector<double> iarea;
    std::vector<sevc_step_info> iinfo;
    /* pinned readback / upload buffers */
    int *h_ctr = nullptr;
    int *h_big = nullptr;
    size_t h_big_ints = 0;
    int *h_on = nullptr;   /* per instance: nucleation attempt this step */
    int *h_flags = nullptr;/* host part of the step's output decision (x.flags) */
    size_t dbytes = 0;     /* size of the device block */
    Tape tape;
    /* CUDA graphs of the step's fixed launch sequences: the first half
     * without / with a nucleation attempt, one polling iteration, and the
     * second half of a step without 2x3 pairs */
    StepGraph g_pre[2], g_poll, g_post;
    /* the whole step as one graph (without / with a nucleation attempt):
     * the polling and 2x3 loops are conditional WHILE nodes driven by the
     * device, so a step is one graph launch and one readback */
    StepGraph g_step[2];
    bool device_loops = true;
    bool use_graphs = true;
    bool force_direct = false;   /* this step launches directly (an adjoint replay records inside it) */
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    /* sevc_run keeps two steps in flight, each with its own pinned upload
     * and readback buffers and its events (allocated on first use) */
    struct RunSlot {
        int *big = nullptr, *on = nullptr, *flags = nullptr;
        cudaEvent_t ev0 = nullptr, ev1 = nullptr, done = nullptr;
        sevc_step_info loc;
        long long launches = 0;
    } rslot[2];
    bool rslot_ready = false;
    /* side streams of the step (branches that do not depend on each other
     * run concurrently; captured as graph branches) and the fork / join
     * events between them: 0-5 in the first half, 6-7 in the tail */
    cudaStream_t side[3] = { nullptr, nullptr, nullptr };   /* [2]: capture of loop bodies */
    cudaEvent_t evfork[10] = {};
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
    size_t V = h->nv, B = h->nb, G = h->ng, I = h->ninst;
    size_t grid = (size_t)h->p.n_blocks * h->p.n_threads;
    size_t maxn = B > G ? B : G;
    size_t tiles = (maxn + 4095) / 4096 + 1;
    size_t nrng = h->opt.do_nucleation ? (size_t)RNG_GRID * I : RNG_GRID;
    struct Req { void **p; size_t bytes; };
    DevMesh &m = h->m;
    DevScratch &x = h->x;
    std::vector<Req> r = {
        { (void **)&m.voff, (I + 1) * 4 }, { (void **)&m.boff, (I + 1) * 4 }, { (void **)&m.goff, (I + 1) * 4 },
        { (void **)&m.binst, B * 4 }, { (void **)&m.ginst, G * 4 }, { (void **)&m.pdone, I * 4 },
        { (void **)&x.pblock, I * h->p.n_blocks * 4 }, { (void **)&x.piters, I * 4 }, { (void **)&x.nrun, 4 },
        { (void **)&x.pcnt, I * 4 },
        { (void **)&x.segcnt, I * TWO_THREE_PASSES * 4 }, { (void **)&x.nucl_on, I * 4 }, { (void **)&x.flags, 16 },
        { (void **)&x.summary, h->h_big_ints * 4 }, { (void **)&m.elog, sizeof(EventLog) },
        { (void **)&m.pos, V * 16 }, { (void **)&m.vel, V * 16 }, { (void **)&m.terms, V * 32 },
        { (void **)&m.contrib, V * 48 }, { (void **)&m.venergy, V * 8 }, { (void **)&m.ven, V },
        { (void **)&m.vspd, V * 4 },
        { (void **)&m.vb, V * 16 }, { (void **)&m.vg, V * 16 }, { (void **)&m.vmod, V * 64 },
        { (void **)&m.voted, V * 4 }, { (void **)&m.vmodmark, V }, { (void **)&m.modlist, V * 4 },
        { (void **)&m.bv, B * 8 }, { (void **)&m.benergy, B * 8 }, { (void **)&m.blen, B * 8 },
        { (void **)&m.btext, B * 8 }, { (void **)&m.ben, B }, { (void **)&m.bcand, B },
        { (void **)&m.bcandbuf, B }, { (void **)&m.bvotes, B * 4 }, { (void **)&m.bconf, B * 4 },
        { (void **)&m.glist, G * SEVC_MAXV * 4 }, { (void **)&m.gvlen, G * 4 }, { (void **)&m.garea, G * 8 },
        { (void **)&m.gdadt, G * 8 }, { (void **)&m.gori, G * 8 }, { (void **)&m.gse, G * 8 },
        { (void **)&m.gq, G * 8 }, { (void **)&m.gen, G }, { (void **)&m.gcand, G }, { (void **)&m.gfix, G },
        { (void **)&m.gtype, G }, { (void **)&m.fixlist, G * 4 }, { (void **)&m.nfix, 4 }, { (void **)&m.nmod, 4 },
        { (void **)&m.err, 16 }, { (void **)&m.evt, I * EVT_COUNT * 4 },
        { (void **)&x.list_a, maxn * 4 }, { (void **)&x.list_b, maxn * 4 }, { (void **)&x.list_c, maxn * 4 },
        { (void **)&x.n_a, 4 }, { (void **)&x.n_b, 4 }, { (void **)&x.n_c, 4 }, { (void **)&x.blockcnt, tiles * 4 },
        { (void **)&x.extra, I * EXTRA_CAP * 4 }, { (void **)&x.threadfail, I * grid * 4 },
        { (void **)&x.block_area, I * h->p.n_blocks * 8 }, { (void **)&x.counters, I * CTR_COUNT * 4 },
        { (void **)&x.rng, nrng * sizeof(curandState) }, { (void **)&x.rng_saved, nrng * sizeof(curandState) },
        { (void **)&x.nucl_buf, I * 96 * 4 }, { (void **)&x.vbucket, 64 * 4 }, { (void **)&x.perm, G * 4 },
        { (void **)&x.n_perm, 4 }, { (void **)&m.nlist, G * 4 }, { (void **)&m.nnlist, I * 4 }, { (void **)&m.pos0, V * 16 },
        { (void **)&m.vel0, V * 16 }, { (void **)&m.bv0, B * 8 }, { (void **)&m.vstamp, V * 4 },
        { (void **)&m.bstamp, B * 4 }, { (void **)&m.stamp, 4 }, { (void **)&m.bexact, B }, { (void **)&m.gexact, G },
        { (void **)&m.bmark, B }, { (void **)&m.lastblk, 8 * 4 },
        { (void **)&x.digest, SEVC_DIGEST_FIELDS * 8 },
        { (void **)&x.vown, V * 8 }, { (void **)&x.bown, B * 8 }, { (void **)&x.ehits, maxn * 4 },
        { (void **)&x.n_ehits, 4 }, { (void **)&x.edefer, maxn }, { (void **)&x.ndefer, I * 4 },
        { (void **)&x.ptot, 4 }, { (void **)&x.tt_first, 4 }, { (void **)&x.tt_pass, 4 },
    };
    size_t total = 0;
    for (auto &q : r) total += align256(q.bytes);
    char *base = nullptr;
    if (!cuda_ok(cudaMalloc(&base, total), "cudaMalloc mesh")) return false;
    if (!cuda_ok(cudaMemsetAsync(base, 0, total, h->stream), "memset")) return false;
    h->dblock = base;
    h->dbytes = total;
    for (auto &q : r) { *q.p = base; base += align256(q.bytes); }
    /* reservation keys start above every key an event writes */
    if (!cuda_ok(cudaMemsetAsync(x.vown, 0xFF, V * 8, h->stream), "memset") ||
        !cuda_ok(cudaMemsetAsync(x.bown, 0xFF, B * 8, h->stream), "memset"))
        return false;
    m.nv = h->nv; m.nb = h->nb; m.ng = h->ng; m.D = h->opt.domain_bound;
    m.ninst = h->ninst;
    m.fixcap = h->ng;
    m.modcap = h->nv;
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
    size_t I1 = h->ninst + 1;
    return put(h->m.voff, h->voff.data(), I1 * 4) && put(h->m.boff, h->boff.data(), I1 * 4) &&
           put(h->m.goff, h->goff.data(), I1 * 4);
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

/* `offs` = 3 x (ninst + 1) entity offsets (vertices, boundaries, grains)
 * and `ng0` the initial grain count of each instance; NULL for a plain
 * handle (one instance holding everything, n_grains from the options). */
sevc_status create_from_host(const sevc_options *opt, sevc_hmesh *hm, sevc_handle **out, int ninst = 1,
                             const std::vector<int> *offs = nullptr, const std::vector<int> *ng0 = nullptr)
{
    *out = nullptr;
    if (require_device()) return SEVC_ERR_CUDA;
    sevc_handle *h = new sevc_handle();
    h->opt = *opt;
    h->nv = hm->m.nv; h->nb = hm->m.nb; h->ng = hm->m.ng;
    h->ninst = ninst;
    if (offs) {
        h->voff.assign(offs->begin(), offs->begin() + ninst + 1);
        h->boff.assign(offs->begin() + ninst + 1, offs->begin() + 2 * (ninst + 1));
        h->goff.assign(offs->begin() + 2 * (ninst + 1), offs->end());
        h->ng0 = *ng0;
    } else {
        h->voff = { 0, h->nv };
        h->boff = { 0, h->nb };
        h->goff = { 0, h->ng };
        h->ng0 = { opt->n_grains };
    }
    h->icurr.resize(ninst);
    h->iallow.assign(ninst, 0);
    h->iarea.assign(ninst, 0.0);
    h->iinfo.assign(ninst, sevc_step_info{});
    int max_ng = 0;
    for (int i = 0; i < ninst; i++) {
        h->icurr[i] = h->goff[i + 1] - h->goff[i];
        if (h->icurr[i] > max_ng) max_ng = h->icurr[i];
    }
    h->p.dt = opt->dt; h->p.eps = opt->GB_eps; h->p.scaling = opt->GB_scaling; h->p.MC_k = opt->MC_k;
    h->p.n_blocks = opt->n_blocks; h->p.n_threads = opt->n_threads;
    h->p.ninst = ninst;
    h->p.max_inst_ng = max_ng;
    h->p.mu = 1.0;
    h->curr_n_grains = h->ng;
    /* readback: counters, events, polling iterations, 2x3 counts per instance */
    h->h_big_ints = (size_t)ninst * (CTR_COUNT + EVT_COUNT + 1 + TWO_THREE_PASSES) + 64;
    bool streams_ok = cuda_ok(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking), "stream");
    for (int k = 0; streams_ok && k < 3; k++)
        streams_ok = cuda_ok(cudaStreamCreateWithFlags(&h->side[k], cudaStreamNonBlocking), "stream");
    for (int k = 0; streams_ok && k < 10; k++)
        streams_ok = cuda_ok(cudaEventCreateWithFlags(&h->evfork[k], cudaEventDisableTiming), "event");
    if (!streams_ok || !cuda_ok(cudaMallocHost(&h->h_ctr, 256), "pinned") ||
        !cuda_ok(cudaMallocHost(&h->h_big, h->h_big_ints * sizeof(int)), "pinned") ||
        !cuda_ok(cudaMallocHost(&h->h_on, ninst * sizeof(int)), "pinned") ||
        !cuda_ok(cudaMallocHost(&h->h_flags, 4 * sizeof(int)), "pinned") || !alloc_device(h) ||
        !upload(h, hm->m)) {
        sevc_destroy(h);
        return SEVC_ERR_CUDA;
    }
    cudaEventCreate(&h->ev0);
    cudaEventCreate(&h->ev1);
    launch_fill_instance_ids(h->m, h->stream);
    launch_rng_init(h->x.rng, RNG_GRID, h->stream);                       /* src/main.cu:81 */
    if (h->opt.do_nucleation)                                             /* every instance gets the same streams */
        for (int i = 1; i < ninst; i++)
            if (!cuda_ok(cudaMemcpyAsync(h->x.rng + (size_t)i * RNG_GRID, h->x.rng, RNG_GRID * sizeof(curandState),
                                         cudaMemcpyDeviceToDevice, h->stream), "rng copy")) {
                sevc_destroy(h);
                return SEVC_ERR_CUDA;
            }
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

RunState save_run(const sevc_handle *h)
{
    RunState r;
    r.n = h->n;
    r.curr_n_grains = h->curr_n_grains;
    r.t = h->t;
    r.nucleated_area = h->nucleated_area;
    r.icurr = h->icurr;
    r.iallow = h->iallow;
    r.iarea = h->iarea;
    return r;
}
void load_run(sevc_handle *h, const RunState &r)
{
    h->n = r.n;
    h->curr_n_grains = r.curr_n_grains;
    h->t = r.t;
    h->nucleated_area = r.nucleated_area;
    h->icurr = r.icurr;
    h->iallow = r.iallow;
    h->iarea = r.iarea;
}
bool tape_checkpoint(sevc_handle *h)
{
    void *ck = nullptr;
    if (!cuda_ok(cudaMalloc(&ck, h->dbytes), "cudaMalloc checkpoint")) return false;
    if (!cuda_ok(cudaMemcpyAsync(ck, h->dblock, h->dbytes, cudaMemcpyDeviceToDevice, h->stream), "checkpoint")) {
        cudaFree(ck);
        return false;
    }
    h->tape.ckpt.push_back(ck);
    h->tape.runs.push_back(save_run(h));
    return true;
}
void tape_free(sevc_handle *h)
{
    Tape &tp = h->tape;
    if (h->stream) cudaStreamSynchronize(h->stream);
    for (void *p : tp.ckpt) cudaFree(p);
    if (tp.rec) cudaFree(tp.rec);
    if (tp.adj) cudaFree(tp.adj);
    if (tp.separam) cudaFree(tp.separam);
    tp = Tape();
}

void drop_graphs(sevc_handle *h)
{
    StepGraph *gs[] = { &h->g_pre[0], &h->g_pre[1], &h->g_poll, &h->g_post, &h->g_step[0], &h->g_step[1] };
    for (StepGraph *g : gs) {
        if (g->exec) cudaGraphExecDestroy(g->exec);
        *g = StepGraph();
    }
}

/* Graphs replay launches with their captured arguments: not while
 * profiling (events between groups), nor while a tape records events
 * (the log pointers are arguments). */
bool graphs_on(const sevc_handle *h)
{
    return h->use_graphs && !h->profiling && !h->force_direct;
}

/* Run a fixed launch sequence: replay its graph (captured on first use) or
 * enqueue it directly. */
template <class F> bool run_seq(sevc_handle *h, StepGraph &g, F &&enqueue)
{
    if (!graphs_on(h)) { enqueue(); return true; }
    if (!g.exec) {
        long long k0 = sevc_kernel_launches;
        cudaGraph_t graph = nullptr;
        if (!cuda_ok(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal), "capture")) return false;
        enqueue();
        if (!cuda_ok(cudaStreamEndCapture(h->stream, &graph), "capture")) return false;
        bool ok = cuda_ok(cudaGraphInstantiate(&g.exec, graph, 0), "graph instantiate");
        cudaGraphDestroy(graph);
        g.kernels = (int)(sevc_kernel_launches - k0);
        sevc_kernel_launches = k0;
        if (!ok) { g = StepGraph(); return false; }
    }
    sevc_kernel_launches += g.kernels;
    return cuda_ok(cudaGraphLaunch(g.exec, h->stream), "graph launch");
}

/* first half of the step, up to the candidate list (src/main.cu:121-216) */
void enqueue_pre(sevc_handle *h, bool nucleation)
{
    cudaStream_t s = h->stream;
    const sevc_options &o = h->opt;
    DevMesh &m = h->m;
    DevScratch &x = h->x;
    size_t I = h->ninst;
    /* the per-step records (event counts, error bits, 2x3 pass counts,
     * polling state, dA/dt exactness marks) are zero here: the previous
     * step's summary kernel cleared them as it read them (a new handle's
     * block starts zeroed, and checkpoints are taken between steps) */
    if (nucleation) {   /* :124-130 for the attempt's vertex (k_nucl_finish), then :144-168 */
        { Prof pr(h, "nucleation"); launch_nucleation(m, x, h->p, s); }
        if (h->tape.after_nucleation) h->tape.after_nucleation(s);
    }
    /* From here three branches that share no written data run concurrently
     * (side streams, graph branches when captured):
     *   main   side-count order, thread-per-grain grain pass
     *   side0  boundary arclengths and energies (:124-130 / :171-181)
     *   side1  warp-per-grain grain pass of the widest grains; the first
     *          2x3 count (:228), which depends only on the topology that
     *          nothing changes before that loop; the device-side decision
     *          whether this step computes every output-only value
     * and join before the vertex pass, which reads all of them.  After it,
     * dA/dt of the 3-sided grains (side0) runs beside the t_ext labels.
     * While profiling everything stays on the main stream, in order. */
    /* every boundary energy this step is 1 * 1 exactly (k_boundary_geometry) */
    const bool unit_gamma = o.GB_eps == 0.0 && o.GB_scaling == 1.0;
    if (h->profiling) {
        { Prof pr(h, "boundary_geometry"); launch_boundary_geometry(m, o.GB_eps, o.GB_scaling, h->p.shape, s); }
        {
            Prof pr(h, "grain_fd");
            launch_grain_sort(m, x, s);
            launch_grain_fd_wide(m, x, h->p.shape, s);
            launch_grain_fd_sorted(m, x, h->p.shape, s);
        }
        { Prof pr(h, "two_three_count"); launch_two_three_first(m, x, x.list_b, x.n_b, s); }
        launch_full_flag(m, x, s);
        { Prof pr(h, "vertex_fd"); launch_vertex_fd(m, h->p.mu, unit_gamma, h->p.shape, s); }
        { Prof pr(h, "grain_dadt"); launch_grain_dadt(m, x, s); }
        { Prof pr(h, "text_label"); launch_text_label(m, x, o.dt, h->p.shape, s); }
        { Prof pr(h, "compact"); launch_compact(m, x, CK_CAND, x.list_a, x.n_a, s); }
    } else {
        cudaStream_t s0 = h->side[0], s1 = h->side[1];
        cudaEvent_t *ev = h->evfork;
        cudaEventRecord(ev[0], s);
        cudaStreamWaitEvent(s0, ev[0], 0);
        launch_boundary_geometry(m, o.GB_eps, o.GB_scaling, h->p.shape, s0);          /* :124-130, :171-181 */
        cudaEventRecord(ev[1], s0);
        launch_grain_sort(m, x, s);
        cudaEventRecord(ev[2], s);
        cudaStreamWaitEvent(s1, ev[2], 0);
        launch_grain_fd_wide(m, x, h->p.shape, s1);                                    /* :127,:203 */
        launch_two_three_first(m, x, x.list_b, x.n_b, s1);                             /* :228 */
        launch_full_flag(m, x, s1);
        cudaEventRecord(ev[3], s1);
        launch_grain_fd_sorted(m, x, h->p.shape, s);                                   /* :127,:203 */
        cudaStreamWaitEvent(s, ev[1], 0);
        cudaStreamWaitEvent(s, ev[3], 0);
        launch_vertex_fd(m, h->p.mu, unit_gamma, h->p.shape, s);                       /* :133,:203 */
        cudaEventRecord(ev[4], s);
        cudaStreamWaitEvent(s0, ev[4], 0);
        launch_grain_dadt(m, x, s0);                                                   /* :206 */
        cudaEventRecord(ev[5], s0);
        launch_text_label(m, x, o.dt, h->p.shape, s);                                  /* :212-216 */
        launch_compact(m, x, CK_CAND, x.list_a, x.n_a, s);
        cudaStreamWaitEvent(s, ev[5], 0);
    }
}

void enqueue_poll(sevc_handle *h)
{
    Prof pr(h, "polling");
    launch_poll_iteration(h->m, h->x, h->x.list_a, h->x.n_a, h->p, h->stream);
}

/* from the 3-sided labels to the end of the step (src/main.cu:252-325);
 * lists_unchanged: no 2x3 removal edited a list since the side-count order
 * (1), some did (0), the device knows (-1: the step's first 2x3 count
 * recorded by the whole-step graph decides) */
void enqueue_tail(sevc_handle *h, int lists_unchanged)
{
    cudaStream_t s = h->stream;
    const sevc_options &o = h->opt;
    DevMesh &m = h->m;
    DevScratch &x = h->x;
    if (lists_unchanged < 0) {                                                                    /* :252-255 */
        sevc_pdl_skip = 1;       /* the first kernel after a conditional node */
        launch_label_3sided_auto(m, x, o.dt, s);
        sevc_pdl_skip = 0;
    } else {
        Prof pr(h, "label_3sided");
        launch_label_3sided(m, x, o.dt, lists_unchanged != 0, s);
    }
    { Prof pr(h, "compact"); launch_compact(m, x, CK_GRAIN_CAND, x.list_c, x.n_c, s); }
    { Prof pr(h, "remove_grains"); launch_remove_grains(m, x, x.list_c, x.n_c, s); }              /* :259 */
    { Prof pr(h, "fix_lists"); launch_fix_lists(m, s); }                                          /* :262 */
    /* The counts (:317-325) read only grain flags, types and areas, which
     * are final here (the flips and the list fix-up after them change
     * none): side0 computes them beside the flips, the fix-up and the
     * position update, joining before the summary. */
    if (!h->profiling) {
        cudaEventRecord(h->evfork[6], s);
        cudaStreamWaitEvent(h->side[0], h->evfork[6], 0);
        launch_counts(m, x, h->p, h->side[0]);
        cudaEventRecord(h->evfork[7], h->side[0]);
    }
    { Prof pr(h, "flips"); launch_flips(m, o.GB_eps, x.list_a, x.n_a, x, s); }             /* :282, :289 */
    if (h->profiling) {
        { Prof pr(h, "fix_lists"); launch_fix_lists(m, s, false); }                               /* :294 */
        { Prof pr(h, "update"); launch_update_positions(m, o.dt, s); }                            /* :314 */
        { Prof pr(h, "counts"); launch_counts(m, x, h->p, s); }
    } else {
        /* the position update reads positions and velocities, final once
         * the flips are applied; the fix-up after them edits only lists
         * and mods: side1 updates beside it */
        cudaEventRecord(h->evfork[8], s);
        cudaStreamWaitEvent(h->side[1], h->evfork[8], 0);
        sevc_pdl_skip = 1;
        launch_update_positions(m, o.dt, h->side[1]);                                             /* :314 */
        sevc_pdl_skip = 0;
        cudaEventRecord(h->evfork[9], h->side[1]);
        launch_fix_lists(m, s, false);                                                            /* :294 */
        cudaStreamWaitEvent(s, h->evfork[9], 0);
        cudaStreamWaitEvent(s, h->evfork[7], 0);
    }
    launch_pack_summary(m, x, h->ninst, x.summary, s);
}

/* second half of a step without 2x3 pairs: conflicts, then the tail */
void enqueue_post(sevc_handle *h)
{
    { Prof pr(h, "conflicts"); launch_conflicts(h->m, h->x.list_a, h->x.n_a, h->stream); }         /* :222-225 */
    enqueue_tail(h, 1);
}

/* Add a WHILE conditional node at the current point of the capture on the
 * handle's stream.  pre(handle) enqueues on that stream what runs just
 * before the node (it may set the condition); body(stream, handle)
 * enqueues the loop body onto the given stream, captured into the node's
 * body graph.  The body's first kernel goes without programmatic
 * serialisation (nothing precedes it in the body); the others keep it. */
template <class Pre, class Body>
bool capture_while(sevc_handle *h, unsigned dflt, unsigned flags, Pre &&pre, Body &&body)
{
    cudaStream_t s = h->stream;
    cudaStreamCaptureStatus st;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    const cudaGraphEdgeData *ed = nullptr;
    size_t nd = 0;
    if (!cuda_ok(cudaStreamGetCaptureInfo(s, &st, nullptr, &cg, &deps, &ed, &nd), "capture info")) return false;
    cudaGraphConditionalHandle hnd;
    if (!cuda_ok(cudaGraphConditionalHandleCreate(&hnd, cg, dflt, flags), "conditional handle")) return false;
    pre(hnd);
    if (!cuda_ok(cudaStreamGetCaptureInfo(s, &st, nullptr, &cg, &deps, &ed, &nd), "capture info")) return false;
    std::vector<cudaGraphNode_t> dv(deps, deps + nd);
    cudaGraphNodeParams np = { cudaGraphNodeTypeConditional };
    np.conditional.handle = hnd;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    if (!cuda_ok(cudaGraphAddNode(&node, cg, dv.data(), nullptr, dv.size(), &np), "conditional node")) return false;
    cudaGraph_t bodyg = np.conditional.phGraph_out[0];
    if (!cuda_ok(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies),
                 "capture dependencies"))
        return false;
    cudaStream_t bs = h->side[2];
    bool ok = cuda_ok(cudaStreamBeginCaptureToGraph(bs, bodyg, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal),
                      "body capture");
    if (ok) {
        sevc_pdl_skip = 1;       /* the body's first kernel has no kernel before it */
        body(bs, hnd);
        sevc_pdl_skip = 0;
        cudaGraph_t out = nullptr;
        ok = cuda_ok(cudaStreamEndCapture(bs, &out), "body capture");
    }
    return ok;
}

/* The whole step as one launch sequence for a graph (src/main.cu:121-325):
 * the first half, the polling loop and the 2x3 loop as device-driven
 * WHILE nodes with the conflicts in between, then the tail.  Only while
 * capturing. */
bool enqueue_step_graph(sevc_handle *h, bool nucleation)
{
    cudaStream_t s = h->stream;
    DevMesh &m = h->m;
    DevScratch &x = h->x;
    enqueue_pre(h, nucleation);
    bool ok = capture_while(h, 1u, cudaGraphCondAssignDefault, [](cudaGraphConditionalHandle) {},   /* :219 */
                            [&](cudaStream_t bs, cudaGraphConditionalHandle hnd) {
                                launch_poll_iteration(m, x, x.list_a, x.n_a, h->p, bs);
                                launch_poll_cond(m, x, hnd, h->polling_cap, bs);
                            });
    if (!ok) return false;
    sevc_pdl_skip = 1;           /* the first kernel after a conditional node */
    launch_conflicts(m, x.list_a, x.n_a, s);                                                        /* :222-225 */
    sevc_pdl_skip = 0;
    ok = capture_while(h, 0u, 0u, [&](cudaGraphConditionalHandle hnd) { launch_tt_init(x, hnd, s); },  /* :227-250 */
                       [&](cudaStream_t bs, cudaGraphConditionalHandle hnd) {
                           launch_remove_two_three_dev(m, x, x.list_b, x.n_b, bs);
                           launch_fix_lists(m, bs);
                           launch_compact(m, x, CK_TWO_THREE, x.list_b, x.n_b, bs);
                           launch_tt_cond(x, hnd, bs);
                       });
    if (!ok) return false;
    enqueue_tail(h, -1);
    return true;
}

sevc_status err_bits_to_status(int bits)
{
    if (bits & ERRB_CAPACITY) { sevc_set_error("a grain list exceeded %d vertices", SEVC_MAXV); return SEVC_ERR_CAPACITY; }
    if (bits & ERRB_TOPOLOGY) { sevc_set_error("inconsistent mesh met by an event kernel"); return SEVC_ERR_TOPOLOGY; }
    if (bits & ERRB_RNG) { sevc_set_error("nucleation picked no valid vertex (the reference reads stale data here)"); return SEVC_ERR_TOPOLOGY; }
    if (bits & ERRB_WORKLIST) { sevc_set_error("internal worklist overflow"); return SEVC_ERR_CAPACITY; }
    if (bits & ERRB_NONCONVERGED) { sevc_set_error("polling did not converge"); return SEVC_ERR_NONCONVERGED; }
    return SEVC_OK;
}

} // namespace

/* ================================================================== */
/* C ABI                                                               */
/* ================================================================== */
namespace {
/* bytes of the packed step summary (k_pack_summary's layout) */
size_t summary_bytes(const sevc_handle *h)
{
    size_t I = h->ninst;
    return (I * CTR_COUNT + I * EVT_COUNT + 4 + I + I * TWO_THREE_PASSES + 1) * sizeof(int);
}
/* The step's summary (hb: counters, events, error bits, polling
 * iterations and 2x3 counts of every instance; h_on: the instances that
 * attempted a nucleation) into the run state and `info`; then n++ and
 * t = n dt (src/main.cu:388-391).  loc carries n, t and the attempt flag of
 * the step. */
sevc_status finish_step(sevc_handle *h, const int *hb, const int *h_on, bool whole, float ms, int launches,
                        sevc_step_info loc, sevc_step_info *info)
{
    const sevc_options &o = h->opt;
    const int I = h->ninst;
    const bool batch = I > 1;
    const int mg = o.min_grains;
    const size_t o_evt = (size_t)I * CTR_COUNT, o_err = o_evt + (size_t)I * EVT_COUNT, o_pit = o_err + 4,
                 o_seg = o_pit + I, o_full = o_seg + (size_t)I * TWO_THREE_PASSES;
    const int full = hb[o_full] != 0;
    loc.outputs_complete = full;
    h->outputs_complete = full;
    int total = 0;
    double area_sum = 0;
    for (int i = 0; i < I; i++) {
        const int *ctr = hb + (size_t)i * CTR_COUNT, *ev = hb + o_evt + (size_t)i * EVT_COUNT;
        double na;
        memcpy(&na, ctr + CTR_NUCL_AREA_SLOT, sizeof(double));
        h->icurr[i] = ctr[CTR_NGRAINS];
        h->iarea[i] = na;
        total += h->icurr[i];
        area_sum += na;
        sevc_step_info &ii = h->iinfo[i];
        memset(&ii, 0, sizeof ii);
        ii.n = loc.n;
        ii.t = loc.t;
        ii.curr_n_grains = h->icurr[i];
        ii.nucleated_area = na;
        ii.polling_iters = hb[o_pit + i];
        for (int k = 0; k < TWO_THREE_PASSES; k++) {
            int c = hb[o_seg + (size_t)k * I + i];
            ii.two_three_counts[k] = c;
            ii.n_two_three_iters = k + 1;
            if (c == 0) break;
        }
        ii.n_two_three = ev[EVT_TWO_THREE];
        ii.n_removals = ev[EVT_REMOVALS];
        ii.n_flips = ev[EVT_FLIPS];
        ii.n_nucleations = ev[EVT_NUCLEATIONS];
        ii.n_conflicts = ev[EVT_CONFLICTS];
        ii.nucleation_attempted = h_on[i];
        /* reported in the instance's own vertex indices */
        ii.nucleation_candidate = (h_on[i] && ctr[CTR_CANDIDATE] >= 0) ? ctr[CTR_CANDIDATE] - h->voff[i] : -1;
        ii.gpu_ms = ms;
        ii.outputs_complete = full;
        ii.kernel_launches = launches;
        ii.export_due = (o.snap_gap > 0 && h->n % o.snap_gap == 0) || (h->icurr[i] <= mg && mg > 0); /* :328 */
        loc.n_two_three += ii.n_two_three;
        loc.n_removals += ii.n_removals;
        loc.n_flips += ii.n_flips;
        loc.n_nucleations += ii.n_nucleations;
        loc.n_conflicts += ii.n_conflicts;
    }
    if (whole) {        /* the loops' counts, as the host loops report them */
        loc.polling_iters = 0;
        for (int i = 0; i < I; i++) loc.polling_iters = std::max(loc.polling_iters, h->iinfo[i].polling_iters);
        for (int k = 0; k < TWO_THREE_PASSES; k++) {
            int c = 0;
            for (int i = 0; i < I; i++) c += hb[o_seg + (size_t)k * I + i];
            loc.two_three_counts[k] = c;
            loc.n_two_three_iters = k + 1;
            if (c == 0) break;
        }
    }
    h->curr_n_grains = total;
    h->nucleated_area = batch ? area_sum / I : area_sum;
    loc.curr_n_grains = total;
    loc.nucleated_area = h->nucleated_area;
    loc.nucleation_candidate = (!batch && loc.nucleation_attempted) ? h->iinfo[0].nucleation_candidate : -1;
    loc.gpu_ms = ms;
    loc.kernel_launches = launches;
    loc.export_due = (o.snap_gap > 0 && h->n % o.snap_gap == 0) || (!batch && h->curr_n_grains <= mg && mg > 0);
    h->n++;                                                                                         /* :388-389 */
    h->t = h->n * o.dt;
    for (int i = 0; i < I; i++) {
        int cont = ((h->t <= o.tmax && o.tmax > 0) || (h->n <= o.nmax && o.nmax > 0)) && (h->icurr[i] >= mg && mg > 0);
        h->iinfo[i].keep_going = (h->icurr[i] <= mg && mg > 0) ? 0 : cont;                          /* :391 */
    }
    loc.keep_going = batch ? sevc_should_continue(h) : h->iinfo[0].keep_going;
    if (info) *info = loc;
    sevc_status st = err_bits_to_status(hb[o_err]);
    if (!st && h->tape.every > 0 && !h->tape.replaying) {
        h->tape.nsteps++;
        if (h->tape.nsteps % h->tape.every == 0 && !tape_checkpoint(h)) return SEVC_ERR_CUDA;
    }
    return st;
}

} // namespace

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

sevc_status sevc_create_batch(const sevc_options *opt, int ninst, const int *nv, const double *const *xy,
                              const int *nb, const int32_t *const *ridges, const int *ng, const double *const *oris,
                              const double *const *se, sevc_handle **out)
{
    if (!opt || !out || ninst < 1 || !nv || !xy || !nb || !ridges || !ng || !oris || !se) return SEVC_ERR_ARG;
    if (require_device()) return SEVC_ERR_CUDA;
    sevc_status st = validate(opt);
    if (st) return st;
    std::vector<sevc_hmesh> parts(ninst);
    int built = 0;
    auto free_parts = [&]() { for (int i = 0; i < built; i++) sevc_hmesh_free(&parts[i]); };
    std::vector<int> offs(3 * (ninst + 1), 0), ng0(ninst);
    int *vo = offs.data(), *bo = vo + ninst + 1, *go = bo + ninst + 1;
    for (int i = 0; i < ninst; i++) {
        if (!xy[i] || !ridges[i] || !oris[i] || !se[i]) { free_parts(); return SEVC_ERR_ARG; }
        sevc_options oi = *opt;
        oi.n_grains = ng[i];
        int rc = sevc_host_build(&oi, nv[i], xy[i], nb[i], ridges[i], ng[i], oris[i], ng[i], se[i], &parts[i]);
        if (rc) {
            std::string why = sevc_last_error();
            free_parts();
            sevc_set_error("instance %d: %s", i, why.c_str());
            return (sevc_status)rc;
        }
        built++;
        const sevc_mesh_host &p = parts[i].m;
        if ((long long)vo[i] + p.nv > 0x7fffffffLL || (long long)bo[i] + p.nb > 0x7fffffffLL ||
            (long long)go[i] + p.ng > 0x7fffffffLL / SEVC_MAXV) {
            free_parts();
            sevc_set_error("batch too large for 32-bit indices");
            return SEVC_ERR_ARG;
        }
        vo[i + 1] = vo[i] + p.nv;
        bo[i + 1] = bo[i] + p.nb;
        go[i + 1] = go[i] + p.ng;
        ng0[i] = ng[i];
    }
    sevc_hmesh all;
    if (sevc_hmesh_alloc(&all, vo[ninst], bo[ninst], go[ninst])) { free_parts(); return SEVC_ERR_CAPACITY; }
    sevc_mesh_host &a = all.m;
    auto shift = [](int32_t *dst, const int32_t *src, size_t n, int off) {
        for (size_t k = 0; k < n; k++) dst[k] = src[k] >= 0 ? src[k] + off : src[k];
    };
    for (int i = 0; i < ninst; i++) {
        const sevc_mesh_host &p = parts[i].m;
        size_t v = vo[i], b = bo[i], g = go[i], V = p.nv, B = p.nb, G = p.ng;
        double *vd[] = { a.px, a.py, a.vx, a.vy, a.venergy, a.vel_bnd_x, a.vel_grn_x, a.vel_bnd_y, a.vel_grn_y };
        const double *vs[] = { p.px, p.py, p.vx, p.vy, p.venergy, p.vel_bnd_x, p.vel_grn_x, p.vel_bnd_y, p.vel_grn_y };
        for (int f = 0; f < 9; f++) memcpy(vd[f] + v, vs[f], V * 8);
        memcpy(a.ven + v, p.ven, V);
        shift(a.vb + 3 * v, p.vb, 3 * V, bo[i]);
        shift(a.vg + 3 * v, p.vg, 3 * V, go[i]);
        shift(a.bini + b, p.bini, B, vo[i]);
        shift(a.bend + b, p.bend, B, vo[i]);
        double *bd[] = { a.benergy, a.blen, a.btext };
        const double *bs[] = { p.benergy, p.blen, p.btext };
        for (int f = 0; f < 3; f++) memcpy(bd[f] + b, bs[f], B * 8);
        memcpy(a.ben + b, p.ben, B);
        memcpy(a.bcand + b, p.bcand, B);
        shift(a.glist + SEVC_MAXV * g, p.glist, SEVC_MAXV * G, vo[i]);
        memcpy(a.gvlen + g, p.gvlen, G * 4);
        double *gd[] = { a.garea, a.gdadt, a.gori, a.gse };
        const double *gs[] = { p.garea, p.gdadt, p.gori, p.gse };
        for (int f = 0; f < 4; f++) memcpy(gd[f] + g, gs[f], G * 8);
        memcpy(a.gen + g, p.gen, G);
        memcpy(a.gtype + g, p.gtype, G);
    }
    free_parts();
    st = create_from_host(opt, &all, out, ninst, &offs, &ng0);
    sevc_hmesh_free(&all);
    return st;
}

sevc_status sevc_instance_count(const sevc_handle *h, int *ninst)
{
    if (!h || !ninst) return SEVC_ERR_ARG;
    *ninst = h->ninst;
    return SEVC_OK;
}

sevc_status sevc_instance_ranges(const sevc_handle *h, int32_t *voff, int32_t *boff, int32_t *goff)
{
    if (!h) return SEVC_ERR_ARG;
    for (int i = 0; i <= h->ninst; i++) {
        if (voff) voff[i] = h->voff[i];
        if (boff) boff[i] = h->boff[i];
        if (goff) goff[i] = h->goff[i];
    }
    return SEVC_OK;
}

sevc_status sevc_instance_info(const sevc_handle *h, int inst, sevc_step_info *info)
{
    if (!h || !info || inst < 0 || inst >= h->ninst) return SEVC_ERR_ARG;
    *info = h->iinfo[inst];
    return SEVC_OK;
}

void sevc_destroy(sevc_handle *h)
{
    if (!h) return;
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->dblock) cudaFree(h->dblock);
    if (h->h_ctr) cudaFreeHost(h->h_ctr);
    if (h->h_big) cudaFreeHost(h->h_big);
    if (h->h_on) cudaFreeHost(h->h_on);
    if (h->h_flags) cudaFreeHost(h->h_flags);
    for (auto &sl : h->rslot) {
        if (sl.big) cudaFreeHost(sl.big);
        if (sl.on) cudaFreeHost(sl.on);
        if (sl.flags) cudaFreeHost(sl.flags);
        if (sl.ev0) cudaEventDestroy(sl.ev0);
        if (sl.ev1) cudaEventDestroy(sl.ev1);
        if (sl.done) cudaEventDestroy(sl.done);
    }
    tape_free(h);
    drop_graphs(h);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    for (auto e : h->evfork) if (e) cudaEventDestroy(e);
    for (auto sd : h->side) if (sd) { cudaStreamSynchronize(sd); cudaStreamDestroy(sd); }
    for (auto e : h->evpool) cudaEventDestroy(e);
    for (auto &pe : h->pending) { cudaEventDestroy(pe.second.first); cudaEventDestroy(pe.second.second); }
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

int sevc_should_continue(const sevc_handle *h)
{
    const sevc_options &o = h->opt;
    int mg = o.min_grains;
    bool time_left = (h->t <= o.tmax && o.tmax > 0) || (h->n <= o.nmax && o.nmax > 0);
    if (h->ninst > 1) return time_left;   /* a batch runs to the shared tmax / nmax */
    return time_left && (h->curr_n_grains >= mg && mg > 0);
}

sevc_status sevc_step(sevc_handle *h, sevc_step_info *info)
{
    if (!h) return SEVC_ERR_ARG;
    cudaStream_t s = h->stream;
    const sevc_options &o = h->opt;
    DevMesh &m = h->m;
    DevScratch &x = h->x;
    const int I = h->ninst;
    const bool batch = I > 1;
    sevc_step_info loc;
    memset(&loc, 0, sizeof loc);
    loc.n = h->n;
    loc.t = h->t;
    long long launches0 = sevc_kernel_launches;
    cudaEventRecord(h->ev0, s);
    int n_on = 0;                                                                                  /* :137-141 */
    for (int i = 0; i < I; i++) {
        if (h->icurr[i] <= 5 * h->ng0[i] / 6) h->iallow[i] = 1;
        h->h_on[i] = o.do_nucleation && o.nucleation_gap > 0 && (h->n % o.nucleation_gap) == 0 && h->iallow[i];
        n_on += h->h_on[i];
    }
    if (n_on) {
        loc.nucleation_attempted = 1;
        if (!cuda_ok(cudaMemcpyAsync(x.nucl_on, h->h_on, I * sizeof(int), cudaMemcpyHostToDevice, s), "upload"))
            return SEVC_ERR_CUDA;
    }
    /* host part of the output decision (k_full_flag): steps that can export,
     * long steps, exact_all, and every step of a batch */
    int mg = o.min_grains;
    h->h_flags[1] = h->exact_all || o.dt >= 100 || (o.snap_gap > 0 && h->n % o.snap_gap == 0);
    h->h_flags[2] = batch ? 0 : mg;   /* a batch does not stop at min_grains */
    h->h_flags[3] = h->curr_n_grains;
    if (!cuda_ok(cudaMemcpyAsync(x.flags + 1, h->h_flags + 1, 3 * sizeof(int), cudaMemcpyHostToDevice, s), "upload"))
        return SEVC_ERR_CUDA;
    h->force_direct = n_on > 0 && (bool)h->tape.after_nucleation;
    const bool whole = graphs_on(h) && h->device_loops;
    if (whole) {
        /* one graph: the loops run on the device, their counts come back
         * with the step summary */
        bool cap_ok = true;
        if (!run_seq(h, h->g_step[n_on ? 1 : 0], [&] { cap_ok = enqueue_step_graph(h, n_on > 0); }) || !cap_ok)
            return SEVC_ERR_CUDA;
    } else {
    if (!run_seq(h, h->g_pre[n_on ? 1 : 0], [&] { enqueue_pre(h, n_on > 0); })) return SEVC_ERR_CUDA;

    /* polling (:219); the first readback also brings the 2x3 count */
    int running = 1, it = 0, c23 = 0;
    while (running) {
        if (it >= h->polling_cap) { sevc_set_error("polling did not converge"); return SEVC_ERR_NONCONVERGED; }
        it++;
        if (!run_seq(h, h->g_poll, [&] { enqueue_poll(h); })) return SEVC_ERR_CUDA;
        if (!cuda_ok(cudaMemcpyAsync(h->h_ctr, x.nrun, 4, cudaMemcpyDeviceToHost, s), "readback") ||
            (it == 1 && !cuda_ok(cudaMemcpyAsync(h->h_ctr + 1, x.n_b, 4, cudaMemcpyDeviceToHost, s), "readback")) ||
            !cuda_ok(cudaStreamSynchronize(s), "sync"))
            return SEVC_ERR_CUDA;
        running = h->h_ctr[0];
        if (it == 1) c23 = h->h_ctr[1];
    }
    loc.polling_iters = it;

    if (c23 == 0) {                                  /* the usual step: no 2x3 pair */
        loc.two_three_counts[0] = 0;
        loc.n_two_three_iters = 1;
        if (!run_seq(h, h->g_post, [&] { enqueue_post(h); })) return SEVC_ERR_CUDA;
    } else {
        { Prof pr(h, "conflicts"); launch_conflicts(m, x.list_a, x.n_a, s); }                     /* :222-225 */
        for (int k = 0; k < TWO_THREE_PASSES; k++) {                                               /* :227-250 */
            int c = c23;
            if (k > 0) {
                { Prof pr(h, "two_three_count"); launch_compact(m, x, CK_TWO_THREE, x.list_b, x.n_b, s); }
                if (read_ints(h, x.n_b, 1, &c)) return SEVC_ERR_CUDA;
            }
            loc.two_three_counts[k] = c;
            loc.n_two_three_iters = k + 1;
            if (c == 0) break;
            { Prof pr(h, "two_three_remove"); launch_remove_two_three(m, x, x.list_b, x.n_b, k, s); }
            { Prof pr(h, "fix_lists"); launch_fix_lists(m, s); }
        }
        enqueue_tail(h, 0);
    }
    }
    cudaEventRecord(h->ev1, s);

    /* one readback: counters, events, error bits, polling iterations and
     * 2x3 counts of every instance */
    int *hb = h->h_big;
    if (!cuda_ok(cudaMemcpyAsync(hb, x.summary, summary_bytes(h), cudaMemcpyDeviceToHost, s), "readback") ||
        !cuda_ok(cudaStreamSynchronize(s), "readback sync"))
        return SEVC_ERR_CUDA;
    float ms = 0;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    if (h->profiling) prof_collect(h);
    int launches = (int)(sevc_kernel_launches - launches0);
    return finish_step(h, hb, h->h_on, whole, ms, launches, loc, info);
}

sevc_status sevc_run(sevc_handle *h, int nsteps, sevc_step_info *infos, int *done)
{
    if (!h || nsteps < 0) return SEVC_ERR_ARG;
    if (done) *done = 0;
    const sevc_options &o = h->opt;
    const int I = h->ninst;
    const bool batch = I > 1;
    const int mg = o.min_grains;
    /* pipelined: one graph per step, nothing read inside a step, and no
     * input of a step that depends on the previous step's counts (a single
     * mesh with a grain-count stop feeds its count to the output decision) */
    const bool pipe = graphs_on(h) && h->device_loops && !h->profiling && h->tape.every <= 0 && (batch || mg <= 0);
    if (!pipe) {
        for (int k = 0; k < nsteps; k++) {
            sevc_step_info inf;
            sevc_status st = sevc_step(h, &inf);
            if (infos) infos[k] = inf;
            if (done) *done = k + 1;
            if (st) return st;
        }
        return SEVC_OK;
    }
    cudaStream_t s = h->stream;
    DevScratch &x = h->x;
    if (!h->rslot_ready) {
        for (auto &sl : h->rslot)
            if (!cuda_ok(cudaMallocHost(&sl.big, h->h_big_ints * sizeof(int)), "pinned") ||
                !cuda_ok(cudaMallocHost(&sl.on, I * sizeof(int)), "pinned") ||
                !cuda_ok(cudaMallocHost(&sl.flags, 4 * sizeof(int)), "pinned") || !cuda_ok(cudaEventCreate(&sl.ev0), "event") ||
                !cuda_ok(cudaEventCreate(&sl.ev1), "event") ||
                !cuda_ok(cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming), "event"))
                return SEVC_ERR_CUDA;
        h->rslot_ready = true;
    }
    int launched = 0, finished = 0;
    sevc_status st = SEVC_OK;
    auto finish_one = [&]() -> sevc_status {
        sevc_handle::RunSlot &sl = h->rslot[finished % 2];
        if (!cuda_ok(cudaEventSynchronize(sl.done), "readback sync")) return SEVC_ERR_CUDA;
        float ms = 0;
        cudaEventElapsedTime(&ms, sl.ev0, sl.ev1);
        sevc_step_info inf;
        sevc_status r = finish_step(h, sl.big, sl.on, true, ms, (int)sl.launches, sl.loc, &inf);
        if (infos) infos[finished] = inf;
        finished++;
        if (done) *done = finished;
        return r;
    };
    /* step `launched` goes in while the one before it runs; what it needs
     * of the host is known in advance (its index, hence its snapshot and
     * attempt decisions) except whether an instance has just passed the
     * 5/6 gate (src/main.cu:137-139), so an attempt step waits for the step
     * before it unless every instance has already passed */
    while (finished < nsteps && !st) {
        bool can_launch = launched < nsteps && launched - finished < 2;
        const int nk = h->n + (launched - finished);
        const bool attempt = o.do_nucleation && o.nucleation_gap > 0 && (nk % o.nucleation_gap) == 0;
        if (can_launch && attempt && launched > finished)
            for (int i = 0; i < I; i++) can_launch = can_launch && h->iallow[i];
        if (!can_launch) {
            st = finish_one();
            continue;
        }
        sevc_handle::RunSlot &sl = h->rslot[launched % 2];
        memset(&sl.loc, 0, sizeof sl.loc);
        sl.loc.n = nk;
        sl.loc.t = nk * o.dt;
        int n_on = 0;                                                                              /* :137-141 */
        for (int i = 0; i < I; i++) {
            if (h->icurr[i] <= 5 * h->ng0[i] / 6) h->iallow[i] = 1;
            sl.on[i] = attempt && h->iallow[i];
            n_on += sl.on[i];
        }
        sl.loc.nucleation_attempted = n_on > 0;
        sl.flags[1] = h->exact_all || o.dt >= 100 || (o.snap_gap > 0 && nk % o.snap_gap == 0);
        sl.flags[2] = batch ? 0 : mg;
        sl.flags[3] = h->curr_n_grains;   /* read only when min_grains > 0: not here */
        if ((n_on && !cuda_ok(cudaMemcpyAsync(x.nucl_on, sl.on, I * sizeof(int), cudaMemcpyHostToDevice, s), "upload")) ||
            !cuda_ok(cudaMemcpyAsync(x.flags + 1, sl.flags + 1, 3 * sizeof(int), cudaMemcpyHostToDevice, s), "upload")) {
            st = SEVC_ERR_CUDA;
            break;
        }
        cudaEventRecord(sl.ev0, s);
        long long k0 = sevc_kernel_launches;
        bool cap_ok = true;
        if (!run_seq(h, h->g_step[n_on ? 1 : 0], [&] { cap_ok = enqueue_step_graph(h, n_on > 0); }) || !cap_ok) {
            st = SEVC_ERR_CUDA;
            break;
        }
        sl.launches = sevc_kernel_launches - k0;
        cudaEventRecord(sl.ev1, s);
        if (!cuda_ok(cudaMemcpyAsync(sl.big, x.summary, summary_bytes(h), cudaMemcpyDeviceToHost, s), "readback") ||
            !cuda_ok(cudaEventRecord(sl.done, s), "event")) {
            st = SEVC_ERR_CUDA;
            break;
        }
        launched++;
    }
    if (launched > finished) cudaStreamSynchronize(s);   /* after a failure: let the step in flight end */
    return st;
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

/* a snapshot after a step that skipped output-only values would not be
 * the reference's: refuse it */
static bool export_allowed(const sevc_handle *h)
{
    if (h->outputs_complete) return true;
    sevc_set_error("the last step computed only the output values it could observe: export after steps with "
                   "export_due (snap_gap) or enable sevc_set_exact_all");
    return false;
}

sevc_status sevc_export_text(sevc_handle *h, const char *path, double time)
{
    if (!h || !path) return SEVC_ERR_ARG;
    if (!export_allowed(h)) return SEVC_ERR_ARG;
    sevc_hmesh hm;
    if (sevc_hmesh_alloc(&hm, h->nv, h->nb, h->ng)) return SEVC_ERR_CAPACITY;
    sevc_status st = sevc_get_state(h, &hm.m);
    if (!st) st = (sevc_status)sevc_host_export(&hm.m, &h->opt, path, time);
    sevc_hmesh_free(&hm);
    return st;
}

sevc_status sevc_export_instance_text(sevc_handle *h, int inst, const char *path, double time)
{
    if (!h || !path || inst < 0 || inst >= h->ninst) return SEVC_ERR_ARG;
    if (!export_allowed(h)) return SEVC_ERR_ARG;
    sevc_hmesh all, one;
    if (sevc_hmesh_alloc(&all, h->nv, h->nb, h->ng)) return SEVC_ERR_CAPACITY;
    sevc_status st = sevc_get_state(h, &all.m);
    int vo = h->voff[inst], bo = h->boff[inst], go = h->goff[inst];
    size_t V = h->voff[inst + 1] - vo, B = h->boff[inst + 1] - bo, G = h->goff[inst + 1] - go;
    if (!st && sevc_hmesh_alloc(&one, (int)V, (int)B, (int)G)) st = SEVC_ERR_CAPACITY;
    if (!st) {
        const sevc_mesh_host &a = all.m;
        sevc_mesh_host &p = one.m;
        auto unshift = [](int32_t *dst, const int32_t *src, size_t n, int off) {
            for (size_t k = 0; k < n; k++) dst[k] = src[k] >= 0 ? src[k] - off : src[k];
        };
        double *vd[] = { p.px, p.py, p.vx, p.vy, p.venergy, p.vel_bnd_x, p.vel_grn_x, p.vel_bnd_y, p.vel_grn_y };
        const double *vs[] = { a.px, a.py, a.vx, a.vy, a.venergy, a.vel_bnd_x, a.vel_grn_x, a.vel_bnd_y, a.vel_grn_y };
        for (int f = 0; f < 9; f++) memcpy(vd[f], vs[f] + vo, V * 8);
        memcpy(p.ven, a.ven + vo, V);
        unshift(p.vb, a.vb + 3 * (size_t)vo, 3 * V, bo);
        unshift(p.vg, a.vg + 3 * (size_t)vo, 3 * V, go);
        unshift(p.bini, a.bini + bo, B, vo);
        unshift(p.bend, a.bend + bo, B, vo);
        double *bd[] = { p.benergy, p.blen, p.btext };
        const double *bs[] = { a.benergy, a.blen, a.btext };
        for (int f = 0; f < 3; f++) memcpy(bd[f], bs[f] + bo, B * 8);
        memcpy(p.ben, a.ben + bo, B);
        memcpy(p.bcand, a.bcand + bo, B);
        unshift(p.glist, a.glist + (size_t)SEVC_MAXV * go, SEVC_MAXV * G, vo);
        memcpy(p.gvlen, a.gvlen + go, G * 4);
        double *gd[] = { p.garea, p.gdadt, p.gori, p.gse };
        const double *gs[] = { a.garea, a.gdadt, a.gori, a.gse };
        for (int f = 0; f < 4; f++) memcpy(gd[f], gs[f] + go, G * 8);
        memcpy(p.gen, a.gen + go, G);
        memcpy(p.gtype, a.gtype + go, G);
        sevc_options oi = h->opt;
        oi.n_grains = h->ng0[inst];
        st = (sevc_status)sevc_host_export(&p, &oi, path, time);
        sevc_hmesh_free(&one);
    }
    sevc_hmesh_free(&all);
    return st;
}

sevc_status sevc_check_data(sevc_handle *h, int *n_bad)
{
    if (!h || !n_bad) return SEVC_ERR_ARG;
    launch_check(h->m, h->x.nrun, h->stream);   /* nrun is free between steps */
    if (read_ints(h, h->x.nrun, 1, n_bad)) return SEVC_ERR_CUDA;
    return SEVC_OK;
}

sevc_status sevc_state_digest(sevc_handle *h, uint64_t *out)
{
    if (!h || !out) return SEVC_ERR_ARG;
    cudaStream_t s = h->stream;
    if (!cuda_ok(cudaMemsetAsync(h->x.digest, 0, SEVC_DIGEST_FIELDS * 8, s), "memset")) return SEVC_ERR_CUDA;
    launch_digest(h->m, h->x.digest, s);
    if (!cuda_ok(cudaMemcpyAsync(out, h->x.digest, SEVC_DIGEST_FIELDS * 8, cudaMemcpyDeviceToHost, s), "readback") ||
        !cuda_ok(cudaStreamSynchronize(s), "sync"))
        return SEVC_ERR_CUDA;
    return SEVC_OK;
}

sevc_status sevc_check_data_host(sevc_handle *h, int *n_bad)
{
    if (!h || !n_bad) return SEVC_ERR_ARG;
    sevc_hmesh hm;
    if (sevc_hmesh_alloc(&hm, h->nv, h->nb, h->ng)) return SEVC_ERR_CAPACITY;
    sevc_status st = sevc_get_state(h, &hm.m);
    if (!st) *n_bad = sevc_host_check(&hm.m);
    sevc_hmesh_free(&hm);
    return st;
}

sevc_status sevc_check_mesh(const sevc_mesh_host *hm, int *n_bad)
{
    if (!hm || !n_bad || hm->nv < 0 || hm->nb < 0 || hm->ng < 0) return SEVC_ERR_ARG;
    if (require_device()) return SEVC_ERR_CUDA;
    size_t V = hm->nv, B = hm->nb, G = hm->ng;
    std::vector<int4> vb(V), vg(V);
    std::vector<int2> bv(B);
    for (size_t i = 0; i < V; i++) {
        vb[i] = make_int4(hm->vb[3 * i], hm->vb[3 * i + 1], hm->vb[3 * i + 2], -1);
        vg[i] = make_int4(hm->vg[3 * i], hm->vg[3 * i + 1], hm->vg[3 * i + 2], -1);
    }
    for (size_t i = 0; i < B; i++) bv[i] = make_int2(hm->bini[i], hm->bend[i]);
    DevMesh m{};
    m.nv = (int)V; m.nb = (int)B; m.ng = (int)G;
    size_t off[9], total = 0;
    size_t sz[9] = { V * 16, V * 16, V, B * 8, B, G * SEVC_MAXV * 4, G * 4, G, 4 };
    for (int i = 0; i < 9; i++) { off[i] = total; total += align256(sz[i]); }
    char *d = nullptr;
    if (!cuda_ok(cudaMalloc(&d, total), "cudaMalloc")) return SEVC_ERR_CUDA;
    m.vb = (int4 *)(d + off[0]); m.vg = (int4 *)(d + off[1]); m.ven = (uint8_t *)(d + off[2]);
    m.bv = (int2 *)(d + off[3]); m.ben = (uint8_t *)(d + off[4]); m.glist = (int *)(d + off[5]);
    m.gvlen = (int *)(d + off[6]); m.gen = (uint8_t *)(d + off[7]);
    int *cnt = (int *)(d + off[8]);
    bool ok = cuda_ok(cudaMemcpy(m.vb, vb.data(), V * 16, cudaMemcpyHostToDevice), "upload") &&
              cuda_ok(cudaMemcpy(m.vg, vg.data(), V * 16, cudaMemcpyHostToDevice), "upload") &&
              cuda_ok(cudaMemcpy(m.ven, hm->ven, V, cudaMemcpyHostToDevice), "upload") &&
              cuda_ok(cudaMemcpy(m.bv, bv.data(), B * 8, cudaMemcpyHostToDevice), "upload") &&
              cuda_ok(cudaMemcpy(m.ben, hm->ben, B, cudaMemcpyHostToDevice), "upload") &&
              cuda_ok(cudaMemcpy(m.glist, hm->glist, G * SEVC_MAXV * 4, cudaMemcpyHostToDevice), "upload") &&
              cuda_ok(cudaMemcpy(m.gvlen, hm->gvlen, G * 4, cudaMemcpyHostToDevice), "upload") &&
              cuda_ok(cudaMemcpy(m.gen, hm->gen, G, cudaMemcpyHostToDevice), "upload");
    if (ok) {
        launch_check(m, cnt, 0);
        ok = cuda_ok(cudaMemcpy(n_bad, cnt, 4, cudaMemcpyDeviceToHost), "readback");
    }
    cudaFree(d);
    return ok ? SEVC_OK : SEVC_ERR_CUDA;
}

sevc_status sevc_rng_record(int nstreams, int ndraws, double *out)
{
    if (nstreams <= 0 || ndraws <= 0 || !out) return SEVC_ERR_ARG;
    int dev = 0;
    if (cudaGetDeviceCount(&dev) != cudaSuccess || dev == 0) { sevc_set_error("no CUDA device"); return SEVC_ERR_CUDA; }
    return rng_record(nstreams, ndraws, out) ? SEVC_ERR_CUDA : SEVC_OK;
}

/* ---------------- parameters and the adjoint ---------------- */
sevc_status sevc_set_mobility(sevc_handle *h, double mu)
{
    if (!h || !(mu > 0) || h->tape.every > 0) return SEVC_ERR_ARG;
    h->p.mu = mu;
    drop_graphs(h);              /* mu is a captured kernel argument */
    return SEVC_OK;
}

sevc_status sevc_set_gb_scaling(sevc_handle *h, double s)
{
    if (!h || h->tape.every > 0) return SEVC_ERR_ARG;
    h->opt.GB_scaling = s;
    h->p.scaling = s;
    drop_graphs(h);
    return SEVC_OK;
}

/* Launch-shape autotuner: coordinate search over the vertex-pass block
 * size, the per-boundary block size and the side count from which grains
 * get a warp each, timing `steps` steps (device time) per candidate from
 * the same saved state; the state is restored afterwards, and results do
 * not depend on the shapes. */
sevc_status sevc_autotune(sevc_handle *h, int steps, int *chosen)
{
    if (!h || steps < 1 || h->tape.every > 0) return SEVC_ERR_ARG;
    void *saved = nullptr;
    if (!cuda_ok(cudaMalloc(&saved, h->dbytes), "cudaMalloc") ||
        !cuda_ok(cudaMemcpyAsync(saved, h->dblock, h->dbytes, cudaMemcpyDeviceToDevice, h->stream), "copy"))
        return SEVC_ERR_CUDA;
    RunState r0 = save_run(h);
    int oc = h->outputs_complete;
    auto trial = [&](double *ms) -> sevc_status {
        drop_graphs(h);
        if (!cuda_ok(cudaMemcpyAsync(h->dblock, saved, h->dbytes, cudaMemcpyDeviceToDevice, h->stream), "copy"))
            return SEVC_ERR_CUDA;
        load_run(h, r0);
        sevc_step_info inf;
        sevc_status st = sevc_step(h, &inf);          /* captures the graphs */
        *ms = 0;
        for (int k = 0; k < steps && !st; k++) {
            st = sevc_step(h, &inf);
            *ms += inf.gpu_ms;
        }
        return st;
    };
    LaunchShape &sh = h->p.shape;
    int *fields[4] = { &sh.tpb_vertex, &sh.tpb_boundary, &sh.wide_sides, &sh.grain_occ };
    const std::vector<int> cands[4] = { { 128, 256, 512 }, { 128, 256, 512 }, { 9, 10, 11, 12 }, { 4, 5, 6, 8 } };
    sevc_status st = SEVC_OK;
    for (int f = 0; f < 4 && !st; f++) {
        int best = *fields[f];
        double best_ms = 1e300;
        for (int v : cands[f]) {
            *fields[f] = v;
            double ms = 0;
            st = trial(&ms);
            if (st) break;
            if (ms < best_ms) { best_ms = ms; best = v; }
        }
        *fields[f] = best;
    }
    drop_graphs(h);
    bool ok = cuda_ok(cudaMemcpyAsync(h->dblock, saved, h->dbytes, cudaMemcpyDeviceToDevice, h->stream), "copy") &&
              cuda_ok(cudaStreamSynchronize(h->stream), "sync");
    cudaFree(saved);
    load_run(h, r0);
    h->outputs_complete = oc;
    if (st) return st;
    if (!ok) return SEVC_ERR_CUDA;
    if (chosen) { chosen[0] = sh.tpb_vertex; chosen[1] = sh.tpb_boundary; chosen[2] = sh.wide_sides; chosen[3] = sh.grain_occ; }
    return SEVC_OK;
}

sevc_status sevc_set_limits(sevc_handle *h, int polling_cap, int worklist_cap)
{
    if (!h || polling_cap < 0 || worklist_cap < 0) return SEVC_ERR_ARG;
    if (polling_cap > 0) h->polling_cap = polling_cap;
    if (worklist_cap > 0) {
        h->m.fixcap = worklist_cap < h->ng ? worklist_cap : h->ng;
        h->m.modcap = worklist_cap < h->nv ? worklist_cap : h->nv;
    }
    drop_graphs(h);   /* captured launches carry both by value */
    return SEVC_OK;
}

sevc_status sevc_set_graphs(sevc_handle *h, int on)
{
    if (!h || on < 0 || on > 2) return SEVC_ERR_ARG;
    h->use_graphs = on != 0;
    h->device_loops = on == 1;
    drop_graphs(h);
    return SEVC_OK;
}

sevc_status sevc_set_stored_energy(sevc_handle *h, const double *se)
{
    if (!h || !se || h->tape.every > 0) return SEVC_ERR_ARG;
    if (!cuda_ok(cudaMemcpyAsync(h->m.gse, se, (size_t)h->ng * 8, cudaMemcpyHostToDevice, h->stream), "upload") ||
        !cuda_ok(cudaStreamSynchronize(h->stream), "sync"))
        return SEVC_ERR_CUDA;
    return SEVC_OK;
}

sevc_status sevc_tape_start(sevc_handle *h, int checkpoint_every)
{
    if (!h || checkpoint_every < 1) return SEVC_ERR_ARG;
    tape_free(h);
    h->tape.every = checkpoint_every;
    if (!cuda_ok(cudaMalloc(&h->tape.separam, (size_t)h->ng * 8), "cudaMalloc tape") ||
        !cuda_ok(cudaMemcpyAsync(h->tape.separam, h->m.gse, (size_t)h->ng * 8, cudaMemcpyDeviceToDevice, h->stream),
                 "tape copy"))
        return SEVC_ERR_CUDA;
    return tape_checkpoint(h) ? SEVC_OK : SEVC_ERR_CUDA;
}

sevc_status sevc_tape_stop(sevc_handle *h)
{
    if (!h) return SEVC_ERR_ARG;
    tape_free(h);
    return SEVC_OK;
}

sevc_status sevc_area_histogram(sevc_handle *h, int nbins, double amax, double *hist)
{
    if (!h || nbins < 1 || nbins > 1024 || !(amax > 0) || !hist) return SEVC_ERR_ARG;
    int nb = histogram_blocks(h->m);
    double *d = nullptr;
    if (!cuda_ok(cudaMalloc(&d, ((size_t)nb + 1) * nbins * 8), "cudaMalloc")) return SEVC_ERR_CUDA;
    double nnorm = h->curr_n_grains, sc = nnorm / (h->ninst * h->opt.domain_bound * h->opt.domain_bound);
    launch_histogram(h->m, nbins, amax, sc, nnorm, d + nbins, d, h->stream);
    bool ok = cuda_ok(cudaMemcpyAsync(hist, d, nbins * 8, cudaMemcpyDeviceToHost, h->stream), "readback") &&
              cuda_ok(cudaStreamSynchronize(h->stream), "sync");
    cudaFree(d);
    return ok ? SEVC_OK : SEVC_ERR_CUDA;
}

sevc_status sevc_adjoint_histogram(sevc_handle *h, int nbins, double amax, const double *dloss_dhist,
                                   double *grad_se, double *grad_gb_scaling, double *grad_mu)
{
    if (!h || nbins < 1 || nbins > 1024 || !(amax > 0) || !dloss_dhist) return SEVC_ERR_ARG;
    Tape &tp = h->tape;
    if (tp.every <= 0) { sevc_set_error("no tape: call sevc_tape_start before the steps"); return SEVC_ERR_ARG; }
    cudaStream_t s = h->stream;
    size_t V = h->nv, B = h->nb, G = h->ng;
    /* adjoint buffers */
    AdjointBuffers a{};
    double *d_dldh = nullptr;
    {
        struct Req { void **p; size_t bytes; };
        std::vector<Req> r = { { (void **)&a.lam, V * 16 }, { (void **)&a.lx, V * 16 }, { (void **)&a.lv, V * 16 },
                               { (void **)&a.mark, V }, { (void **)&a.sgn, G * 8 }, { (void **)&a.gse, G * 8 },
                               { (void **)&a.gmu, V * 8 }, { (void **)&a.ggam, V * 8 }, { (void **)&a.dlda, G * 8 },
                               { (void **)&a.scalars, 16 }, { (void **)&d_dldh, 1024 * 8 } };
        size_t total = 0;
        for (auto &q : r) total += align256(q.bytes);
        if (!tp.adj) {
            if (!cuda_ok(cudaMalloc(&tp.adj, total), "cudaMalloc adjoint")) return SEVC_ERR_CUDA;
            tp.adj_bytes = total;
        }
        char *base = (char *)tp.adj;
        for (auto &q : r) { *q.p = base; base += align256(q.bytes); }
    }
    /* per-step records of one segment */
    tp.log_cap = 4096 + (int)(V / 16);
    size_t off_pos = 0, off_vb = off_pos + align256(V * 16), off_vg = off_vb + align256(V * 16),
           off_vel1 = off_vg + align256(V * 16), off_ven = off_vel1 + align256(V * 16), off_ven1 = off_ven + align256(V),
           off_bv = off_ven1 + align256(V), off_ben = off_bv + align256(B * 8), off_gl = off_ben + align256(B),
           off_gvl = off_gl + align256(G * SEVC_MAXV * 4), off_gen = off_gvl + align256(G * 4),
           off_gty = off_gen + align256(G), off_log = off_gty + align256(G),
           off_nlog = off_log + align256((size_t)tp.log_cap * sizeof(EventRec)), step_bytes = off_nlog + 256;
    if (!tp.rec || tp.rec_step_bytes != step_bytes || tp.rec_steps < tp.every) {
        if (tp.rec) cudaFree(tp.rec);
        tp.rec = nullptr;
        if (!cuda_ok(cudaMalloc(&tp.rec, step_bytes * tp.every), "cudaMalloc tape records")) return SEVC_ERR_CUDA;
        tp.rec_step_bytes = step_bytes;
        tp.rec_steps = tp.every;
    }
    auto rec = [&](int k, size_t off) { return (char *)tp.rec + (size_t)k * step_bytes + off; };
    auto d2d = [&](void *dst, const void *src, size_t n) {
        return cuda_ok(cudaMemcpyAsync(dst, src, n, cudaMemcpyDeviceToDevice, s), "tape copy");
    };

    /* seed: dL/dx of the statistic at the final state */
    if (!cuda_ok(cudaMemcpyAsync(d_dldh, dloss_dhist, nbins * 8, cudaMemcpyHostToDevice, s), "upload")) return SEVC_ERR_CUDA;
    cudaMemsetAsync(a.gse, 0, G * 8, s);
    cudaMemsetAsync(a.gmu, 0, V * 8, s);
    cudaMemsetAsync(a.ggam, 0, V * 8, s);
    double nnorm = h->curr_n_grains, sc = nnorm / (h->ninst * h->opt.domain_bound * h->opt.domain_bound);
    launch_hist_seed(h->m, nbins, amax, sc, nnorm, d_dldh, a.dlda, a.lam, s);

    void *fin = nullptr;
    if (!cuda_ok(cudaMalloc(&fin, h->dbytes), "cudaMalloc") || !d2d(fin, h->dblock, h->dbytes)) return SEVC_ERR_CUDA;
    RunState rfin = save_run(h);
    sevc_status st = SEVC_OK;
    tp.replaying = true;
    long long nseg = (tp.nsteps + tp.every - 1) / tp.every;
    for (long long seg = nseg - 1; seg >= 0 && !st; seg--) {
        if (!d2d(h->dblock, tp.ckpt[seg], h->dbytes)) { st = SEVC_ERR_CUDA; break; }
        load_run(h, tp.runs[seg]);
        int K = (int)std::min<long long>(tp.every, tp.nsteps - seg * tp.every);
        for (int k = 0; k < K && !st; k++) {
            DevMesh &m = h->m;
            /* the mesh the step's velocities are computed on: at its start,
             * or after its nucleation (recorded again from inside the step) */
            auto record = [&, k](cudaStream_t rs) {
                auto cp = [&](size_t off, const void *src, size_t n) {
                    return cudaMemcpyAsync(rec(k, off), src, n, cudaMemcpyDeviceToDevice, rs) == cudaSuccess;
                };
                return cp(off_pos, m.pos, V * 16) && cp(off_vb, m.vb, V * 16) && cp(off_vg, m.vg, V * 16) &&
                       cp(off_ven, m.ven, V) && cp(off_bv, m.bv, B * 8) && cp(off_ben, m.ben, B) &&
                       cp(off_gl, m.glist, G * SEVC_MAXV * 4) && cp(off_gvl, m.gvlen, G * 4) &&
                       cp(off_gen, m.gen, G) && cp(off_gty, m.gtype, G);
            };
            bool ok = record(s) && cuda_ok(cudaMemsetAsync(rec(k, off_nlog), 0, 4, s), "memset");
            if (!ok) { st = SEVC_ERR_CUDA; break; }
            tp.after_nucleation = [&, record](cudaStream_t rs) { if (!record(rs)) sevc_set_error("tape copy"); };
            EventLog on = { (EventRec *)rec(k, off_log), (int *)rec(k, off_nlog), tp.log_cap }, off = { nullptr, nullptr, 0 };
            if (!cuda_ok(cudaMemcpyAsync(m.elog, &on, sizeof on, cudaMemcpyHostToDevice, s), "upload")) {
                st = SEVC_ERR_CUDA;
                break;
            }
            st = sevc_step(h, nullptr);
            tp.after_nucleation = nullptr;
            h->force_direct = false;
            if (!cuda_ok(cudaMemcpyAsync(m.elog, &off, sizeof off, cudaMemcpyHostToDevice, s), "upload"))
                st = SEVC_ERR_CUDA;
            if (!st && !(d2d(rec(k, off_vel1), m.vel, V * 16) && d2d(rec(k, off_ven1), m.ven, V))) st = SEVC_ERR_CUDA;
        }
        for (int k = K - 1; k >= 0 && !st; k--) {
            DevMesh view = h->m;
            view.pos = (double2 *)rec(k, off_pos);
            view.vb = (int4 *)rec(k, off_vb);
            view.vg = (int4 *)rec(k, off_vg);
            view.ven = (uint8_t *)rec(k, off_ven);
            view.bv = (int2 *)rec(k, off_bv);
            view.ben = (uint8_t *)rec(k, off_ben);
            view.glist = (int *)rec(k, off_gl);
            view.gvlen = (int *)rec(k, off_gvl);
            view.gen = (uint8_t *)rec(k, off_gen);
            view.gtype = (uint8_t *)rec(k, off_gty);
            view.gse = tp.separam;           /* a nucleated grain's 0 is applied by its type */
            launch_adjoint_step(view, a, h->opt.dt, h->p.mu, h->opt.GB_eps, h->opt.GB_scaling,
                                (const EventRec *)rec(k, off_log), (const int *)rec(k, off_nlog),
                                (const uint8_t *)rec(k, off_ven1), (const double2 *)rec(k, off_vel1), s);
        }
    }
    tp.replaying = false;
    tp.after_nucleation = nullptr;
    h->force_direct = false;
    if (!d2d(h->dblock, fin, h->dbytes)) st = SEVC_ERR_CUDA;
    load_run(h, rfin);
    launch_sum_ordered(a.gmu, (int)V, a.scalars, s);
    launch_sum_ordered(a.ggam, (int)V, a.scalars + 1, s);
    double sc2[2] = { 0, 0 };
    if (!st && grad_se && !cuda_ok(cudaMemcpyAsync(grad_se, a.gse, G * 8, cudaMemcpyDeviceToHost, s), "readback"))
        st = SEVC_ERR_CUDA;
    if (!st && !cuda_ok(cudaMemcpyAsync(sc2, a.scalars, 16, cudaMemcpyDeviceToHost, s), "readback")) st = SEVC_ERR_CUDA;
    if (!cuda_ok(cudaStreamSynchronize(s), "sync") && !st) st = SEVC_ERR_CUDA;
    cudaFree(fin);
    if (st) return st;
    if (grad_mu) *grad_mu = sc2[0];
    if (grad_gb_scaling) *grad_gb_scaling = sc2[1];
    return SEVC_OK;
}

/* ---------------- checkpoint files ---------------- */
namespace {
const char CKPT_MAGIC[8] = { 'S', 'E', 'V', 'C', 'C', 'K', 'P', '1' };
struct CkptHeader {
    char magic[8];
    int32_t nv, nb, ng, ninst;
    uint64_t dbytes;
    int32_t n, curr_n_grains;
    double t, nucleated_area, mu, gb_scaling;
    int32_t outputs_complete, reserved;
};
} // namespace

sevc_status sevc_checkpoint_save(sevc_handle *h, const char *path)
{
    if (!h || !path) return SEVC_ERR_ARG;
    std::vector<char> blk(h->dbytes);
    if (!cuda_ok(cudaMemcpyAsync(blk.data(), h->dblock, h->dbytes, cudaMemcpyDeviceToHost, h->stream), "download") ||
        !cuda_ok(cudaStreamSynchronize(h->stream), "sync"))
        return SEVC_ERR_CUDA;
    CkptHeader hd{};
    memcpy(hd.magic, CKPT_MAGIC, 8);
    hd.nv = h->nv; hd.nb = h->nb; hd.ng = h->ng; hd.ninst = h->ninst;
    hd.dbytes = h->dbytes;
    hd.n = h->n; hd.curr_n_grains = h->curr_n_grains;
    hd.t = h->t; hd.nucleated_area = h->nucleated_area; hd.mu = h->p.mu; hd.gb_scaling = h->opt.GB_scaling;
    hd.outputs_complete = h->outputs_complete;
    FILE *f = fopen(path, "wb");
    if (!f) { sevc_set_error("cannot write %s", path); return SEVC_ERR_IO; }
    size_t I = h->ninst;
    bool ok = fwrite(&hd, sizeof hd, 1, f) == 1 && fwrite(h->icurr.data(), 4, I, f) == I &&
              fwrite(h->iallow.data(), 4, I, f) == I && fwrite(h->iarea.data(), 8, I, f) == I &&
              fwrite(blk.data(), 1, blk.size(), f) == blk.size();
    ok = (fclose(f) == 0) && ok;
    if (!ok) { sevc_set_error("short write to %s", path); return SEVC_ERR_IO; }
    return SEVC_OK;
}

sevc_status sevc_checkpoint_load(sevc_handle *h, const char *path)
{
    if (!h || !path) return SEVC_ERR_ARG;
    if (h->tape.every > 0) { sevc_set_error("stop the adjoint tape before loading a checkpoint"); return SEVC_ERR_ARG; }
    FILE *f = fopen(path, "rb");
    if (!f) { sevc_set_error("cannot read %s", path); return SEVC_ERR_IO; }
    CkptHeader hd{};
    size_t I = h->ninst;
    std::vector<int> icurr(I), iallow(I);
    std::vector<double> iarea(I);
    std::vector<char> blk(h->dbytes);
    bool ok = fread(&hd, sizeof hd, 1, f) == 1;
    if (ok && (memcmp(hd.magic, CKPT_MAGIC, 8) || hd.nv != h->nv || hd.nb != h->nb || hd.ng != h->ng ||
               hd.ninst != h->ninst || hd.dbytes != h->dbytes)) {
        fclose(f);
        sevc_set_error("%s is not a checkpoint of a handle of this shape", path);
        return SEVC_ERR_PARSE;
    }
    ok = ok && fread(icurr.data(), 4, I, f) == I && fread(iallow.data(), 4, I, f) == I &&
         fread(iarea.data(), 8, I, f) == I && fread(blk.data(), 1, blk.size(), f) == blk.size();
    fclose(f);
    if (!ok) { sevc_set_error("truncated checkpoint %s", path); return SEVC_ERR_PARSE; }
    if (!cuda_ok(cudaMemcpyAsync(h->dblock, blk.data(), h->dbytes, cudaMemcpyHostToDevice, h->stream), "upload") ||
        !cuda_ok(cudaStreamSynchronize(h->stream), "sync"))
        return SEVC_ERR_CUDA;
    h->n = hd.n; h->curr_n_grains = hd.curr_n_grains; h->t = hd.t; h->nucleated_area = hd.nucleated_area;
    h->p.mu = hd.mu; h->opt.GB_scaling = hd.gb_scaling; h->p.scaling = hd.gb_scaling;
    h->outputs_complete = hd.outputs_complete;
    drop_graphs(h);
    h->icurr = icurr; h->iallow = iallow; h->iarea = iarea;
    return SEVC_OK;
}

sevc_status sevc_grain_stats(sevc_handle *h, int inst, sevc_grain_stats_t *out)
{
    if (!h || !out || inst < -1 || inst >= h->ninst) return SEVC_ERR_ARG;
    int lo = inst < 0 ? 0 : h->goff[inst], hi = inst < 0 ? h->ng : h->goff[inst + 1];
    double *d = nullptr;
    if (!cuda_ok(cudaMalloc(&d, 8 * 8), "cudaMalloc")) return SEVC_ERR_CUDA;
    launch_grain_stats(h->m, lo, hi, d, h->stream);
    double r[8];
    bool ok = cuda_ok(cudaMemcpyAsync(r, d, sizeof r, cudaMemcpyDeviceToHost, h->stream), "readback") &&
              cuda_ok(cudaStreamSynchronize(h->stream), "sync");
    cudaFree(d);
    if (!ok) return SEVC_ERR_CUDA;
    double n = r[0];
    out->n_grains = (int)n;
    out->mean_area = n > 0 ? r[1] / n : 0;
    out->std_area = n > 1 ? sqrt(std::max(0.0, r[2] / n - out->mean_area * out->mean_area)) : 0;
    out->mean_sides = n > 0 ? r[3] / n : 0;
    out->n_three_sided = (int)r[4];
    out->min_area = r[5];
    out->max_area = r[6];
    return SEVC_OK;
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
    char data[sizeof o->output_folder];
    snprintf(data, sizeof data, "%.250s/DATA", o->output_folder);
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
    /* Snapshots are written by a host thread while the next steps run: the
     * state is downloaded into one of two host copies, the previous writer
     * is joined, and a new one formats and writes the copy.  The validity
     * check that gates a save (src/main.cu:331-338) runs on the device
     * before the download, with the same rules as the host check. */
    sevc_hmesh hm[2];
    if (sevc_hmesh_alloc(&hm[0], h->nv, h->nb, h->ng)) { sevc_destroy(h); return SEVC_ERR_CAPACITY; }
    if (sevc_hmesh_alloc(&hm[1], h->nv, h->nb, h->ng)) { sevc_hmesh_free(&hm[0]); sevc_destroy(h); return SEVC_ERR_CAPACITY; }
    std::thread writer;
    int wstat = 0;
    std::string wpath;
    auto join_writer = [&]() -> sevc_status {
        if (writer.joinable()) writer.join();
        if (wstat) { sevc_set_error("write error on %s", wpath.c_str()); return (sevc_status)wstat; }
        return SEVC_OK;
    };
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
            int bad = 0;
            if ((st = sevc_check_data(h, &bad))) break;
            if (bad) {
                if (verbose) printf("Error while saving output file. Exiting...\n");
                break;
            }
            if (verbose) printf("Valid data. Saving...\n");
            sevc_hmesh &buf = hm[prog & 1];
            if ((st = sevc_get_state(h, &buf.m))) break;
            if ((st = join_writer())) break;
            char path[600];
            snprintf(path, sizeof path, "%s/%06d.txt", opt.output_folder, prog);
            wpath = path;
            sevc_options o = h->opt;
            double t = inf.t;
            std::string p = path;
            writer = std::thread([&wstat, &buf, o, p, t]() { wstat = sevc_host_export(&buf.m, &o, p.c_str(), t); });
            prog++;
        }
        if (!inf.keep_going) break;
    }
    sevc_status ws = join_writer();
    if (!st) st = ws;
    if (verbose) {
        printf("\nPerformed %d iterations.\n", h->n - 1);
        printf("Number of grains: %d\n", h->curr_n_grains);
        printf("Done.\n");
    }
    sevc_hmesh_free(&hm[0]);
    sevc_hmesh_free(&hm[1]);
    sevc_destroy(h);
    return st;
}

} // extern "C"
