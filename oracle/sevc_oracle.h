/*
 * ORACLE — TEST INFRASTRUCTURE ONLY.
 *
 * A CPU restatement, in plain C, of the reference vertex-model time step
 * (tclaudioe/SE-grain-growth-GPU, "SEVC").  It exists so that tests, the
 * smoke check and the CPU-baseline leg of the benchmark can check the GPU
 * product against an independent implementation.  Nothing in the product
 * (the CUDA library, its C ABI or its CLI) may link, load or call it.
 *
 * Every function cites the reference file:line it restates.  Semantics are
 * the reference's, including its quirks, with these deliberate choices:
 *   - entities are int32 indices into structure-of-arrays (-1 is NULL);
 *   - kernels that run race-free in parallel in the reference are
 *     restated as loops in thread-id order (same result);
 *   - `apply_flippings` (src/topological.h:1016) runs flips in parallel
 *     with unsynchronised writes when two candidates share a vertex; here
 *     flips are applied in ascending boundary order, which equals every
 *     race-free outcome;
 *   - reductions whose floating-point order or grid partition is
 *     observable (polling convergence, nucleated area, nucleation vertex
 *     pick) emulate the n_blocks x n_threads grid-stride partition;
 *   - memory the reference leaves uninitialised (candidate buffer,
 *     nucleation candidate id) starts at zero, like a zero-filled
 *     allocation;
 *   - situations where the reference reads uninitialised data or writes
 *     out of bounds set an error status instead.
 * Floating point is IEEE binary64 without contraction (built with
 * -ffp-contract=off); atan2/cos/sin/pow/exp come from the C library.
 *
 * Parity of this oracle is pinned against the reference's own sources
 * executed on the CPU (oracle/ref builds them; tests/golden holds the
 * outputs), see tests/test_oracle_golden.py.
 */
#ifndef SEVC_ORACLE_H
#define SEVC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_VRT_PER_GRN 100  /* src/geometry.h:9 */
#define ORC_MAX_T_EXT 100000     /* src/geometry.h:11 */
#define ORC_NB_FIX 4

/* fix_t (src/geometry.h:17) */
enum { ORC_ADD = 0, ORC_REMOVE = 1, ORC_REPLACE = 2, ORC_NONE = 3 };
/* gtype_t (src/geometry.h:19) */
enum { ORC_COMMON = 0, ORC_NUCLEATED = 1 };

/* status codes */
enum {
    ORC_OK = 0,
    ORC_ERR_IO = 1,
    ORC_ERR_PARSE = 2,
    ORC_ERR_CAPACITY = 3,
    ORC_ERR_NONCONVERGED = 4,
    ORC_ERR_TOPOLOGY = 5,
    ORC_ERR_RNG = 6,
    ORC_ERR_ARG = 7
};

/* struct options (src/options.h:15-46) */
typedef struct orc_options {
    double dt, dtau;
    int nucleation_gap;
    double tmax;
    int nmax, snap_gap;
    double leave_percent;
    int n_grains;
    char vertex_fname[256], boundary_fname[256], orientation_fname[256], SE_fname[256];
    double GB_eps, GB_scaling, SE_eps, SE_min, SE_max, nucleation_scaling, domain_bound;
    int do_nucleation;
    double MC_k;
    int n_blocks, n_threads, debug_lvl;
    char output_folder[256];
    /* set by the caller: stop threshold (the reference hard-codes 5000 at
     * src/main.cu:49; -1 disables the grain-count stop) */
    int min_grains;
} orc_options;

typedef struct orc_mod { int grn, vrt, prev, fix; } orc_mod; /* mod_t, src/geometry.h:26 */

typedef struct orc_state {
    orc_options opt;
    int nv, nb, ng;
    /* vertices (src/geometry.h:39-59) */
    double *px, *py, *vx, *vy, *venergy;
    double *vel_bnd_x, *vel_grn_x, *vel_bnd_y, *vel_grn_y;
    double *nucl_r, *nucl_ori, *DeltaE, *nfactor;
    uint8_t *ven, *vnucleate;
    int *vb;      /* 3 per vertex: boundaries[3] */
    int *vg;      /* 3 per vertex: grains[3] */
    orc_mod *vmod;/* 4 per vertex */
    int *voted;
    /* boundaries (src/geometry.h:61-72) */
    int *bini, *bend;
    double *benergy, *blen, *btext;
    uint8_t *ben, *bcand;
    int *bvotes, *bconf;
    /* grains (src/geometry.h:74-86) */
    int *glist;   /* 100 per grain */
    int *gvlen;
    double *garea, *gdadt, *gori, *gse;
    uint8_t *gen, *gcand, *gfix, *gtype;
    /* run state (src/main.cu:29-113) */
    int n, prog, curr_n_grains, allow_nucleation;
    double t, nucleated_area;
    uint8_t *cand_buf;
    int vrt_id_candidate;
    int vertex_buffer[64];
    int vrt_ids[2], bnd_ids[3], grn_id;
    int polling_iters, polling_cap;
    int last_two_three[20];
    int n_two_three_iters;
    /* rng: per-thread stream of doubles in (0,1] */
    int rng_kind;               /* 0 synthetic, 1 table */
    uint64_t rng_seed;
    int rng_nstreams, rng_ndraws;
    const double *rng_table;    /* nstreams x ndraws, borrowed */
    int64_t *rng_pos;           /* per stream draw counter */
    /* per-step event log (counts) */
    int ev_flips, ev_removals, ev_two_three, ev_nucleations;
    int status;                 /* sticky error */
    int nthreads_omp;           /* >1: OpenMP for race-free loops */
    int ev_conflicts;           /* boundaries marked by check_conflictive_boundaries this step
                                   (one device printf each, src/topological.h:116) */
} orc_state;

/* options.h:69-206 restated.  Returns ORC_OK or ORC_ERR_IO. */
int orc_parse_ini(const char *path, orc_options *opt);
/* options.h:71-85 defaults + the derived fields of :172-181 */
void orc_default_options(orc_options *opt);
void orc_finish_options(orc_options *opt);

/* io.h:66-264 restated: load from the four input files. */
int orc_load_files(const orc_options *opt, orc_state **out);
/* Same as the loader but from in-memory arrays (positions in [0,1),
 * ridges, orientations in [0,1), stored energies).  The data go through
 * the same scaling and face traversal as the file loader. */
int orc_load_arrays(const orc_options *opt, int nv, const double *xy, int nb,
                    const int *ridges, int ng, const double *oris, const double *se,
                    orc_state **out);
void orc_free(orc_state *st);

void orc_rng_synthetic(orc_state *st, uint64_t seed);
void orc_rng_table(orc_state *st, int nstreams, int ndraws, const double *table);

/* One iteration of the main loop body src/main.cu:121-389 (without the
 * snapshot export).  Returns status. */
int orc_step(orc_state *st);
/* Loop condition of src/main.cu:120 for the current state. */
int orc_should_continue(const orc_state *st);
/* Snapshot condition of src/main.cu:328. */
int orc_should_export(const orc_state *st);
/* src/main.cu:388-393: n++, t = n*dt, then the stop tests; 1 = keep going */
int orc_finish_step(orc_state *st);

/* Field accessor for bindings: returns the array called `name` (e.g.
 * "px", "glist") and its element count; kind: 0 double, 1 int32,
 * 2 uint8, 3 int64, 4 orc_mod.  NULL if unknown. */
void *orc_field(orc_state *st, const char *name, int64_t *count, int *kind);
orc_state *orc_clone(const orc_state *st);

/* io.h:280-377 restated.  Writes one snapshot file. */
int orc_export(const orc_state *st, const char *path, double time);
/* utils.h:85-336 restated: number of violated invariants (0 = valid). */
int orc_check_data(const orc_state *st);

/* Individual phases (for fine-grained tests) */
void orc_compute_boundary_arclengths(orc_state *st);
void orc_compute_grain_areas(orc_state *st);
void orc_compute_boundary_energies(orc_state *st);
void orc_compute_vertex_energies(orc_state *st);
void orc_compute_vertex_velocities(orc_state *st);
void orc_compute_grain_dadts(orc_state *st);
void orc_compute_t_ext(orc_state *st);
int  orc_current_n_grains(const orc_state *st);
double orc_nucleated_fraction_area(const orc_state *st);

/* a blank state of the given sizes, to be filled through orc_field */
orc_state *orc_alloc_blank(const orc_options *opt, int nv, int nb, int ng);
/* per-field digests of the state, as the engine's sevc_state_digest */
void orc_state_digest(orc_state *st, uint64_t *out);

#ifdef __cplusplus
}
#endif

#endif
