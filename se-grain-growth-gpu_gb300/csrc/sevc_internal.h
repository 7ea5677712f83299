/*
 * Internal launch interface between the engine (sevc_engine.cu) and the
 * kernel translation units.  Every launcher enqueues on `s` and returns
 * without synchronising.
 */
#ifndef SEVC_INTERNAL_H
#define SEVC_INTERNAL_H

#include "sevc_device.cuh"
#include <curand_kernel.h>

/* Scratch shared by launches of one handle.  Arrays marked "per instance"
 * hold one block for each instance of a batched handle. */
struct DevScratch {
    int *list_a, *list_b, *list_c;   /* ordered index lists (capacity max(nb, ng)) */
    int *n_a, *n_b, *n_c;            /* their lengths */
    int *blockcnt;                   /* per-tile counts for ordered compaction */
    int *extra;                      /* dynamic insertions of the 2x3 pass, EXTRA_CAP per instance */
    int *threadfail;                 /* polling predicate: one flag per grid thread, per instance */
    int *pblock;                     /* polling predicate: one result per grid block, per instance */
    int *pcnt;                       /* per instance: blocks of k_poll_final done (zero between launches) */
    int *piters;                     /* polling iterations this step, per instance */
    int *nrun;                       /* instances whose polling has not converged */
    int *segcnt;                     /* 2x3 count of each pass (20), per instance */
    double *block_area;              /* nucleated-area partial per block, per instance */
    int *counters;                   /* CTR_COUNT device counters per instance, see CTR_* */
    curandState *rng, *rng_saved;    /* 8192 cuRAND states + pre-attempt copy, per instance */
    int *nucl_buf;                   /* 96 ints per instance: per-block pick, alive count, pick's rank */
    int *nucl_on;                    /* per instance: attempt a nucleation this step */
    int *vbucket;                    /* 64 ints: side-count histogram + cursors */
    int *flags;                      /* 4 ints: the step's output decision, see launch_full_flag */
    int *summary;                    /* the step's summary packed for one readback */
    int *perm, *n_perm;              /* enabled grains ordered by side count */
    unsigned long long *digest;      /* SEVC_DIGEST_FIELDS sums of sevc_state_digest */
    /* events applied in parallel (removals, flips): reservation keys of
     * every vertex and boundary, the events of the phase (list positions),
     * the deferred ones (flag per list position, count per instance) */
    unsigned long long *vown, *bown;
    int *ehits, *n_ehits;
    uint8_t *edefer;
    int *ndefer;
    /* device-driven loops of a whole-step graph: polling iterations taken
     * (all instances), the first 2x3 count and the 2x3 pass index */
    int *ptot, *tt_first, *tt_pass;
};
constexpr int EXTRA_CAP = 1024;
constexpr int TWO_THREE_PASSES = 20;  /* src/main.cu:227 */
constexpr int RNG_GRID = 8192;        /* the reference's 32 x 256 nucleation grid */

enum {
    CTR_NGRAINS = 0,     /* current_n_grains */
    CTR_CONVERGED = 1,   /* polling predicate result */
    CTR_FLIPS = 2,
    CTR_REMOVALS = 3,
    CTR_TWO_THREE = 4,
    CTR_NUCLEATIONS = 5,
    CTR_CANDIDATE = 6,   /* vrt_id_candidate (persists across attempts) */
    CTR_NUCL_ATTEMPT = 7,
    CTR_COUNT = 16
};
#define CTR_NUCL_AREA_SLOT 8 /* double stored at counters + 8 (two ints) */

/* launch shapes the autotuner may change (results do not depend on them);
 * the defaults are what it picked on the 1M-grain mesh */
struct LaunchShape {
    int tpb_vertex = 128;    /* threads per block of the vertex pass */
    int tpb_boundary = 128;  /* of the per-boundary passes (geometry, t_ext) */
    int wide_sides = 11;     /* grains of this many sides or more get a warp each */
    int grain_occ = 6;       /* resident blocks per SM of the thread-per-grain grain pass (4, 5, 6, 8) */
};

struct StepParams {
    double dt, eps, scaling, MC_k;
    int n_blocks, n_threads; /* reference launch grid, drives observable partitions */
    int ninst;               /* instances in the handle */
    int max_inst_ng;         /* grains of the largest instance */
    double mu;               /* mobility (velocity factor); 1 in the reference */
    LaunchShape shape;
};

/* geometry (sevc_geometry.cu) */
void launch_boundary_geometry(const DevMesh &m, double eps, double scaling, const LaunchShape &sh, cudaStream_t s);
/* grain pass: side-count order (x.perm / x.vbucket), then the warp-per-grain
 * kernel for grains of wide_sides or more and the thread-per-grain kernel
 * for the rest (disjoint grains: the two may run concurrently) */
void launch_grain_sort(const DevMesh &m, const DevScratch &x, cudaStream_t s);
void launch_grain_fd_wide(const DevMesh &m, const DevScratch &x, const LaunchShape &sh, cudaStream_t s);
void launch_grain_fd_sorted(const DevMesh &m, const DevScratch &x, const LaunchShape &sh, cudaStream_t s);
/* unit_gamma: every boundary energy is exactly 1 (GB_eps = 0, GB_scaling = 1) */
void launch_vertex_fd(const DevMesh &m, double mu, bool unit_gamma, const LaunchShape &sh, cudaStream_t s);
/* side-count histogram layout in DevScratch::vbucket */
#define VB_START(b) (32 + (b))
#define VB_COUNT(b) (48 + (b))
/* x.flags: [0] computed "full" decision, [1] host part of it, [2]
 * min_grains, [3] current grain count (see k_full_flag); also advances
 * the step stamp of the events' save-on-write (m.stamp) */
void launch_full_flag(const DevMesh &m, const DevScratch &x, cudaStream_t s);
void launch_grain_dadt(const DevMesh &m, const DevScratch &x, cudaStream_t s);
void launch_text_label(const DevMesh &m, const DevScratch &x, double dt, const LaunchShape &sh, cudaStream_t s);
void launch_update_positions(const DevMesh &m, double dt, cudaStream_t s);
void launch_counts(const DevMesh &m, const DevScratch &x, const StepParams &p, cudaStream_t s);
/* counters | events | error bits | polling iterations | 2x3 counts | output decision, into out */
void launch_pack_summary(const DevMesh &m, const DevScratch &x, int ninst, int *out, cudaStream_t s);

/* topology (sevc_topology.cu) */
enum CompactKind { CK_CAND = 0, CK_TWO_THREE = 1, CK_GRAIN_CAND = 2, CK_GVLEN3 = 3, CK_MARKED = 4 };
void launch_compact(const DevMesh &m, const DevScratch &x, CompactKind kind, int *out, int *n_out, cudaStream_t s);
/* the CK_TWO_THREE list from the 3-sided bucket of this step's grain pass */
void launch_two_three_first(const DevMesh &m, const DevScratch &x, int *out, int *n_out, cudaStream_t s);
/* one polling iteration for every instance not yet converged; leaves the
 * number still running in x.nrun */
void launch_poll_iteration(const DevMesh &m, const DevScratch &x, const int *cand, const int *ncand,
                           const StepParams &p, cudaStream_t s);
void launch_conflicts(const DevMesh &m, const int *cand, const int *ncand, cudaStream_t s);
/* pass `pass` of the 2x3 loop (per-instance counts go to x.segcnt) */
void launch_remove_two_three(const DevMesh &m, const DevScratch &x, const int *list, const int *n, int pass,
                             cudaStream_t s);
/* the same with the pass index read from x.tt_pass on the device */
void launch_remove_two_three_dev(const DevMesh &m, const DevScratch &x, const int *list, const int *n, cudaStream_t s);
/* Loop control of the whole-step graph (conditional WHILE nodes):
 * poll_cond after each polling iteration: continue while an instance has
 * not converged, up to `cap` iterations (past it: ERRB_NONCONVERGED);
 * tt_init before the 2x3 loop: record the first count, start while it is
 * nonzero; tt_cond after each pass: the next pass runs while the count
 * just compacted is nonzero and fewer than TWO_THREE_PASSES ran. */
void launch_poll_cond(const DevMesh &m, const DevScratch &x, cudaGraphConditionalHandle hnd, int cap, cudaStream_t s);
void launch_tt_init(const DevScratch &x, cudaGraphConditionalHandle hnd, cudaStream_t s);
void launch_tt_cond(const DevScratch &x, cudaGraphConditionalHandle hnd, cudaStream_t s);
/* the 3-sided labels, bucket or full as x.tt_first says (no 2x3 removal:
 * the bucket) */
void launch_label_3sided_auto(const DevMesh &m, const DevScratch &x, double dt, cudaStream_t s);
/* bucket: no grain list changed since this step's side-count order, so
 * only its 3-sided bucket is visited */
void launch_label_3sided(const DevMesh &m, const DevScratch &x, double dt, bool bucket, cudaStream_t s);
void launch_remove_grains(const DevMesh &m, const DevScratch &x, const int *list, const int *n, cudaStream_t s);
/* clears the candidate flag of every listed grain (after the removals) */
void launch_flips(const DevMesh &m, double eps, const int *cand, const int *ncand, const DevScratch &x,
                  cudaStream_t s);
void launch_fix_lists(const DevMesh &m, cudaStream_t s, bool areas = true);
void launch_fill_instance_ids(const DevMesh &m, cudaStream_t s);

/* check_data on the device (sevc_check.cu): violations counted into *out */
void launch_check(const DevMesh &m, int *out, cudaStream_t s);
/* per-field digests of the state (sevc_state_digest) into out[SEVC_DIGEST_FIELDS] */
void launch_digest(const DevMesh &m, unsigned long long *out, cudaStream_t s);

/* nucleation (sevc_nucleation.cu) */
void launch_rng_init(curandState *st, int n, cudaStream_t s);
void launch_nucleation(const DevMesh &m, const DevScratch &x, const StepParams &p, cudaStream_t s);
int rng_record(int nstreams, int ndraws, double *host_out);

/* adjoint (sevc_adjoint.cu) */
struct AdjointBuffers {
    double2 *lam;    /* adjoint of the positions (current step boundary) */
    double2 *lx, *lv;/* adjoint of the post-event positions / of the velocities */
    uint8_t *mark;   /* vertices moved by an event in the step */
    double *sgn;     /* sign of each grain's area at the step's start */
    double *gse;     /* dL/dSE per grain (accumulated) */
    double *gmu;     /* dL/dmu per vertex (accumulated) */
    double *ggam;    /* dL/dGB_scaling per vertex (accumulated) */
    double *dlda;    /* dL/dA per grain of the statistic */
    double *scalars; /* reduced dL/dmu, dL/dGB_scaling */
};
/* soft histogram of a_g = |A_g| sc over nbins bins of [0, amax), divided by nnorm */
void launch_histogram(const DevMesh &m, int nbins, double amax, double sc, double nnorm, double *blockbins,
                      double *hist, cudaStream_t s);
int histogram_blocks(const DevMesh &m);
/* lam = d(sum_k dldh_k h_k)/dx at the current state */
void launch_hist_seed(const DevMesh &m, int nbins, double amax, double sc, double nnorm, const double *dldh,
                      double *dlda, double2 *lam, cudaStream_t s);
/* one step backward: `rec` views the mesh as recorded at the step's start,
 * log / ven1 / vel1 its events and the enabled flags and velocities after it */
void launch_adjoint_step(const DevMesh &rec, const AdjointBuffers &a, double dt, double mu, double eps, double s_gb,
                         const EventRec *log, const int *nlog, const uint8_t *ven1, const double2 *vel1,
                         cudaStream_t s);
void launch_sum_ordered(const double *a, int n, double *out, cudaStream_t s);
/* out[0..6] = count, sum |A|, sum A^2, sum vlen, 3-sided count, min |A|, max |A| over grains [lo, hi) */
void launch_grain_stats(const DevMesh &m, int lo, int hi, double *out, cudaStream_t s);

#define SEVC_CUDA_OK(expr) ((expr) == cudaSuccess)

/* kernels launched by this process (reported per step) */
extern long long sevc_kernel_launches;
/* set while launches must go without the programmatic-serialisation
 * attribute (a whole stretch of capture); sevc_pdl_skip counts the next
 * launches that must (the first kernel of a conditional node's body and
 * the first kernel after a conditional node, whose predecessor is not a
 * kernel) */
extern thread_local bool sevc_pdl_off;
extern thread_local int sevc_pdl_skip;
#define COUNT_LAUNCHES(k) (sevc_kernel_launches += (k))

/* Launch with programmatic dependent launch allowed: the grid may be
 * scheduled while the previous kernel of the stream drains, which hides
 * most of the launch gap between the short kernels of the step's sparse
 * half.  Every kernel launched this way calls griddep_wait() before its
 * first global memory access; that returns once the previous kernel has
 * completed and its writes are visible, so only the scheduling overlaps. */
template <typename... P, typename... A>
inline void launch_dep(void (*k)(P...), dim3 grid, dim3 block, cudaStream_t s, A &&...args)
{
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cfg.attrs = at;
    bool plain = sevc_pdl_off || sevc_pdl_skip > 0;
    if (sevc_pdl_skip > 0) sevc_pdl_skip--;
    cfg.numAttrs = plain ? 0 : 1;
    COUNT_LAUNCHES(1);
    cudaLaunchKernelEx(&cfg, k, static_cast<A &&>(args)...);
}

#endif
