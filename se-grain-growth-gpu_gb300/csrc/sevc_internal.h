/*
 * Internal launch interface between the engine (sevc_engine.cu) and the
 * kernel translation units.  Every launcher enqueues on `s` and returns
 * without synchronising.
 */
#ifndef SEVC_INTERNAL_H
#define SEVC_INTERNAL_H

#include "sevc_device.cuh"
#include <curand_kernel.h>

/* scratch shared by launches of one handle */
struct DevScratch {
    int *list_a, *list_b, *list_c;   /* ordered index lists (capacity max(nb, ng)) */
    int *n_a, *n_b, *n_c;            /* their lengths */
    int *blockcnt;                   /* per-tile counts for ordered compaction */
    int *extra;                      /* dynamic insertions of the 2x3 pass */
    int *threadfail;                 /* polling predicate: one flag per grid thread */
    double *block_area;              /* nucleated-area partial per block */
    int *counters;                   /* small device counters, see CTR_* */
    curandState *rng, *rng_saved;    /* 8192 cuRAND states + pre-attempt copy */
    int *nucl_buf;                   /* 64 ints: per-block pick and alive count */
    int *vbucket;                    /* 32 ints: side-count histogram + cursors */
    int *perm, *n_perm;              /* enabled grains ordered by side count */
};

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

struct StepParams {
    double dt, eps, scaling, MC_k;
    int n_blocks, n_threads; /* reference launch grid, drives observable partitions */
};

/* geometry (sevc_geometry.cu) */
void launch_boundary_geometry(const DevMesh &m, double eps, double scaling, cudaStream_t s);
void launch_grain_fd(const DevMesh &m, const DevScratch &x, cudaStream_t s);
void launch_vertex_fd(const DevMesh &m, cudaStream_t s);
/* side-count histogram layout in DevScratch::vbucket */
#define VB_START(b) (32 + (b))
#define VB_COUNT(b) (48 + (b))
void launch_grain_dadt(const DevMesh &m, const DevScratch &x, int full, int n3, cudaStream_t s);
void launch_mark_force(const DevMesh &m, const DevScratch &x, int n3, cudaStream_t s);
void launch_text_label(const DevMesh &m, double dt, int full, cudaStream_t s);
void launch_grain_area(const DevMesh &m, cudaStream_t s);
void launch_area_dirty(const DevMesh &m, int compute, cudaStream_t s);
void launch_update_positions(const DevMesh &m, double dt, cudaStream_t s);
void launch_counts(const DevMesh &m, const DevScratch &x, const StepParams &p, cudaStream_t s);

/* topology (sevc_topology.cu) */
enum CompactKind { CK_CAND = 0, CK_TWO_THREE = 1, CK_GRAIN_CAND = 2, CK_GVLEN3 = 3 };
void launch_compact(const DevMesh &m, const DevScratch &x, CompactKind kind, int *out, int *n_out, cudaStream_t s);
void launch_poll_iteration(const DevMesh &m, const DevScratch &x, const int *cand, const int *ncand,
                           const StepParams &p, cudaStream_t s);
void launch_conflicts(const DevMesh &m, const int *cand, const int *ncand, cudaStream_t s);
void launch_remove_two_three(const DevMesh &m, const DevScratch &x, const int *list, const int *n, cudaStream_t s);
void launch_label_3sided(const DevMesh &m, double dt, cudaStream_t s);
void launch_remove_grains(const DevMesh &m, const int *list, const int *n, cudaStream_t s);
void launch_unlabel_st2(const DevMesh &m, const int *cand, const int *ncand, cudaStream_t s);
void launch_flips(const DevMesh &m, double eps, const int *cand, const int *ncand, const DevScratch &x,
                  cudaStream_t s);
void launch_fix_lists(const DevMesh &m, cudaStream_t s);

/* nucleation (sevc_nucleation.cu) */
void launch_rng_init(curandState *st, int n, cudaStream_t s);
void launch_nucleation(const DevMesh &m, const DevScratch &x, const StepParams &p, cudaStream_t s);
int rng_record(int nstreams, int ndraws, double *host_out);

#define SEVC_CUDA_OK(expr) ((expr) == cudaSuccess)

/* kernels launched by this process (reported per step) */
extern long long sevc_kernel_launches;
#define COUNT_LAUNCHES(k) (sevc_kernel_launches += (k))

#endif
