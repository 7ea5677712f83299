/*
 * sevc.h — C ABI of the GB300 vertex-model grain-growth engine.
 *
 * The reference (tclaudioe/SE-grain-growth-GPU) has no library API: its
 * drop-in contract is the executable `SEVC -c file.ini`, its .ini keys,
 * its four input files and its `DATA/%06d.txt` snapshots.  Inside that
 * executable the hot path is the body of the main loop (src/main.cu:120-394)
 * operating on device arrays.  Each entry point below replaces one piece
 * of that program; the citation on each says which.  The `sevc` CLI in
 * se-grain-growth-gpu_gb300/cli is the drop-in executable built on them.
 *
 * Conventions: plain C types only; every call returns an sevc_status;
 * host buffers are owned by the caller; device memory is owned by the
 * handle; one handle = one CUDA stream on the current device; a handle is
 * not thread-safe.  There is no CPU fallback: without a CUDA device every
 * compute call returns SEVC_ERR_CUDA.
 */
#ifndef SEVC_H
#define SEVC_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SEVC_MAX_VRT_PER_GRN 100 /* src/geometry.h:9 */

typedef enum sevc_status {
    SEVC_OK = 0,
    SEVC_ERR_IO = 1,           /* a file could not be opened/written        */
    SEVC_ERR_PARSE = 2,        /* malformed input file or option            */
    SEVC_ERR_CAPACITY = 3,     /* a grain list would exceed 100 vertices    */
    SEVC_ERR_NONCONVERGED = 4, /* polling loop hit its iteration cap        */
    SEVC_ERR_TOPOLOGY = 5,     /* inconsistent mesh met by an event kernel  */
    SEVC_ERR_CUDA = 6,         /* CUDA runtime error / no device            */
    SEVC_ERR_ARG = 7           /* invalid argument                           */
} sevc_status;

/* struct options, src/options.h:15-46, plus the stop threshold that the
 * reference hard-codes at src/main.cu:49. */
typedef struct sevc_options {
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
    int min_grains; /* stop when fewer grains remain; <=0 disables.  The
                       reference always uses 5000 (src/main.cu:49). */
} sevc_options;

/* Host mirror of the mesh, structure-of-arrays, entity = index, -1 = NULL.
 * Field meanings follow src/geometry.h:39-86. */
typedef struct sevc_mesh_host {
    int nv, nb, ng;
    double *px, *py, *vx, *vy, *venergy;
    double *vel_bnd_x, *vel_grn_x, *vel_bnd_y, *vel_grn_y;
    uint8_t *ven;
    int32_t *vb;    /* 3 per vertex */
    int32_t *vg;    /* 3 per vertex */
    int32_t *bini, *bend;
    double *benergy, *blen, *btext;
    uint8_t *ben, *bcand;
    int32_t *glist; /* 100 per grain */
    int32_t *gvlen;
    double *garea, *gdadt, *gori, *gse;
    uint8_t *gen, *gtype;
} sevc_mesh_host;

/* What one loop iteration did (src/main.cu:121-325). */
typedef struct sevc_step_info {
    int n;                     /* iteration index of the step just run       */
    double t;                  /* its time n*dt                              */
    int curr_n_grains;         /* src/main.cu:317                            */
    double nucleated_area;     /* src/main.cu:321 (percent of domain)        */
    int export_due;            /* src/main.cu:328 condition                  */
    int keep_going;            /* src/main.cu:120 and :391 after n++         */
    int polling_iters;         /* iterations of src/topological.h:555        */
    int n_two_three_iters;     /* passes of src/main.cu:227-250              */
    int two_three_counts[20];  /* the count printed by each pass             */
    int n_flips, n_removals, n_two_three, n_nucleations;
    int nucleation_attempted;  /* src/main.cu:141 condition was true         */
    int nucleation_candidate;  /* vertex id kept by the Metropolis test, -1  */
    double gpu_ms;             /* device time of the step (CUDA events)      */
    int outputs_complete;      /* 1: every enabled boundary's t_ext and every
                                  enabled grain's dA/dt was computed this step
                                  (always so on steps that can export) */
    int kernel_launches;       /* CUDA kernels the step launched             */
    int n_conflicts;           /* boundaries marked conflictive, one device
                                  printf each in src/topological.h:116      */
} sevc_step_info;

typedef struct sevc_handle sevc_handle;

/* Defaults of src/options.h:71-85 (min_grains = 5000 as src/main.cu:49). */
sevc_status sevc_default_options(sevc_options *opt);
/* load_config_file, src/options.h:69-206 (same keys and parsing quirks). */
sevc_status sevc_load_ini(const char *path, sevc_options *opt);

/* load_from_files + host_to_device, src/io.h:66-264 and
 * src/translation.h:140-155: read the four input files named in `opt`,
 * build grains by face traversal, and upload the mesh. */
sevc_status sevc_create(const sevc_options *opt, sevc_handle **out);
/* Same from in-memory arrays: nv positions in [0,1) (xy interleaved),
 * nb ridges (pairs), ng orientations in [0,1) and stored energies. */
sevc_status sevc_create_from_arrays(const sevc_options *opt, int nv, const double *xy, int nb,
                                    const int32_t *ridges, int ng, const double *oris,
                                    const double *se, sevc_handle **out);
void sevc_destroy(sevc_handle *h);
/* load_from_files alone (src/io.h:66-264), on the host, no GPU needed:
 * call once with out == NULL to get the sizes, then with caller arrays. */
sevc_status sevc_load_mesh_host(const sevc_options *opt, sevc_mesh_host *out, int *nv, int *nb, int *ng);

/* One iteration of the loop body src/main.cu:121-389: geometry refresh,
 * optional nucleation, finite-difference velocities, extinction times,
 * polling, conflicts, 2x3 and 3-sided removal, T1 flips, grain-list
 * fix-ups, position update, grain count and nucleated area; then n++ and
 * t = n*dt.  `info` (may be NULL) describes the step that ran. */
sevc_status sevc_step(sevc_handle *h, sevc_step_info *info);
/* Run up to `nsteps` iterations, as many calls of sevc_step would: it
 * stops early after a step whose keep_going is 0 (the reference's loop
 * condition, src/main.cu:120) or that fails.  `done` = steps run, `last`
 * (may be NULL) the last step's info.  Each step's stop test needs that
 * step's grain count, so the steps are not pipelined: every step reads its
 * summary back before the next is launched. */
sevc_status sevc_run_steps(sevc_handle *h, int nsteps, int *done, sevc_step_info *last);
/* Run `nsteps` iterations of the loop body src/main.cu:120-394 (fewer only
 * on a failure) and write each step's info to infos[k] (may be NULL);
 * `done` = steps run.  It does not stop at the reference's stop criterion
 * (src/main.cu:120, :391): the caller reads keep_going and the
 * counts from `infos`.  With one graph per step (sevc_set_graphs(h, 1), the
 * default), no profiling or tape, and no grain-count stop (min_grains <= 0,
 * or a batch), the steps are pipelined: each step is launched while the one
 * before it runs and its summary is read back afterwards, so the GPU does
 * not wait on the host between steps (an attempt step waits for the step
 * before it until every instance has passed the 5/6 gate, whose count it
 * needs); otherwise it steps as sevc_step does.  Results are those of
 * nsteps calls of sevc_step. */
sevc_status sevc_run(sevc_handle *h, int nsteps, sevc_step_info *infos, int *done);
/* Loop condition of src/main.cu:120 for the current state. */
int sevc_should_continue(const sevc_handle *h);

/* export_data, src/io.h:280-377: write one snapshot with the reference's
 * exact text format; `time` is printed as TIME.  Allowed before the first
 * step and after steps whose outputs are complete (export_due steps, or
 * every step with sevc_set_exact_all); SEVC_ERR_ARG otherwise. */
sevc_status sevc_export_text(sevc_handle *h, const char *path, double time);
/* The same text for a mesh held in host arrays (export_data's format,
 * src/io.h:280-377), on the host only: the lines are formatted by all host
 * threads in chunks and written in order, so the file is the one a serial
 * writer produces. */
sevc_status sevc_write_snapshot(const sevc_mesh_host *mesh, const sevc_options *opt, const char *path, double time);
/* device_to_host, src/translation.h:184-199 (without freeing anything):
 * copy the mesh into caller-owned arrays sized like sevc_mesh_sizes. */
sevc_status sevc_get_state(sevc_handle *h, sevc_mesh_host *out);
sevc_status sevc_mesh_sizes(const sevc_handle *h, int *nv, int *nb, int *ng);
/* check_data, src/utils.h:85-336: number of violated invariants (>= 0),
 * counted on the device (one thread per boundary, vertex and grain). */
sevc_status sevc_check_data(sevc_handle *h, int *n_bad);
/* The same count on the host after a download of the mesh. */
sevc_status sevc_check_data_host(sevc_handle *h, int *n_bad);
/* The device count for a mesh held in host arrays (uploaded to temporary
 * device memory); indices outside their arrays count as violations. */
sevc_status sevc_check_mesh(const sevc_mesh_host *mesh, int *n_bad);

/* Digests of the mesh state, computed on the device without a download:
 * out[f] = sum over the elements i of field f (in the layout that
 * sevc_get_state returns) of mix(salt_f + i * 0x9E3779B97F4A7C15 + bits_i)
 * mod 2^64, where bits_i is the element's IEEE-754 bit pattern (doubles),
 * its value as an unsigned 32-bit integer (int32) or its byte (uint8), and
 * mix is the splitmix64 finaliser.  Two states with equal digests are
 * equal field by field with overwhelming probability, so a long run can be
 * compared with a reference run every step at the cost of one small
 * readback.  Fields f (SEVC_DIGEST_FIELDS of them, salt_f = f << 56): px, py,
 * vx, vy, ven, vb, vg, bini, bend, benergy, blen, ben, bcand, glist (all
 * 100 slots per grain), gvlen, garea, gori, gse, gen, gtype.  No
 * counterpart in the reference (whose only check is check_data,
 * src/utils.h:85-336). */
#define SEVC_DIGEST_FIELDS 20
sevc_status sevc_state_digest(sevc_handle *h, uint64_t *out);

/* The whole program of src/main.cu:21-424 after option loading: create
 * DATA folder, load, loop with snapshots and the reference's log lines.
 * `log` (may be NULL) receives stdout-style lines. */
sevc_status sevc_run_program(const sevc_options *opt, int verbose);

/* The reference seeds 8192 cuRAND XORWOW states with curand_init(32, tid,
 * 0) (src/nucleation2.cu:12-16) and draws curand_uniform_double.  This
 * records the first `ndraws` draws of streams 0..nstreams-1 into `out`
 * (stream-major), for replay by an independent checker. */
sevc_status sevc_rng_record(int nstreams, int ndraws, double *out);

/* The same record without any allocation.  No counterpart in the
 * reference.  For callers that cannot let a library call cudaMalloc: a
 * host framework that hands out device memory only from its own pool, a
 * process whose device-memory budget is already taken by the simulation,
 * or code that must not trigger the implicit synchronisation cudaMalloc
 * can cause.  The caller passes the output: d_out is DEVICE memory for
 * nstreams x ndraws doubles (stream-major); work is enqueued on `stream`
 * (a cudaStream_t, NULL = default stream) and the call returns without
 * waiting.  Scratch is a fixed device array of 8192 generator states
 * (384 KiB per GPU, kept until exit); nstreams > 8192 is rejected with
 * SEVC_ERR_ARG.  The first call on each device resolves that array's
 * device address (with the device current); make that first call before
 * any stream capture.  With CUDA's lazy module loading (the default) that
 * first call is also when the 384 KiB are committed on the device (set
 * CUDA_MODULE_LOADING=EAGER to commit them when the library is loaded);
 * later calls take no device memory.  The address is kept for the life of
 * the process: after cudaDeviceReset on a device, do not call this entry
 * point on that device again.  All calls share the array: calls that
 * overlap on the GPU race and must be serialised by the caller. */
sevc_status sevc_rng_record_noalloc(int nstreams, int ndraws, double *d_out, void *stream);

/* ---- batched ensembles (no counterpart in the reference) ----
 *
 * One handle advancing `ninst` independent microstructures together: the
 * meshes are stored one after another in every device array and each
 * kernel launch of a step covers all of them, so hundreds of small runs
 * cost one run's launches and host round trips.  Every instance follows
 * exactly the plain method: instance i, stepped in a batch, produces bit
 * for bit what a plain handle created from the same arrays produces (its
 * own polling convergence, 2x3 loop, event order and its own copy of the
 * 8192 random streams).  Options are shared except n_grains, which is
 * each instance's grain count.  The batch runs until the shared tmax /
 * nmax; min_grains is reported per instance (keep_going of
 * sevc_instance_info) but stops nothing.  Output-only values follow the
 * plain rule (complete on snapshot steps, see sevc_set_exact_all).
 *
 * Arrays of instance i: nv[i] positions xy[i] (interleaved), nb[i] ridges
 * ridges[i] (pairs), ng[i] orientations oris[i] and stored energies se[i],
 * as in sevc_create_from_arrays. */
sevc_status sevc_create_batch(const sevc_options *opt, int ninst, const int *nv, const double *const *xy,
                              const int *nb, const int32_t *const *ridges, const int *ng, const double *const *oris,
                              const double *const *se, sevc_handle **out);
sevc_status sevc_instance_count(const sevc_handle *h, int *ninst);
/* ninst+1 offsets each: instance i owns global vertex indices
 * [voff[i], voff[i+1]) etc. of sevc_get_state (any pointer may be NULL) */
sevc_status sevc_instance_ranges(const sevc_handle *h, int32_t *voff, int32_t *boff, int32_t *goff);
/* the summary of the last step for one instance */
sevc_status sevc_instance_info(const sevc_handle *h, int inst, sevc_step_info *info);
/* export_data (src/io.h:280-377) of one instance, in its own indices */
sevc_status sevc_export_instance_text(sevc_handle *h, int inst, const char *path, double time);

/* ---- checkpoint files and statistics (no counterpart in the reference) ----
 *
 * A checkpoint is the handle's whole device state (mesh, scratch, random
 * streams, polling buffers) plus its host run state, in one binary file;
 * loading it into a handle created from the same inputs and options
 * resumes the run bit for bit. */
sevc_status sevc_checkpoint_save(sevc_handle *h, const char *path);
sevc_status sevc_checkpoint_load(sevc_handle *h, const char *path);

typedef struct sevc_grain_stats_t {
    int n_grains;        /* enabled grains (current_n_grains, src/calculus.h:264) */
    int n_three_sided;
    double mean_area, std_area, min_area, max_area;   /* of |A| */
    double mean_sides;
} sevc_grain_stats_t;
/* grain-size statistics of one instance (inst = -1: all grains) */
sevc_status sevc_grain_stats(sevc_handle *h, int inst, sevc_grain_stats_t *out);

/* ---- parameters and the adjoint (no counterpart in the reference) ----
 *
 * Mobility mu multiplies every vertex velocity (the reference has none:
 * mu = 1, which changes no bit).  GB_scaling and the per-grain stored
 * energies (after the loader's scaling) can be replaced between runs.
 * None of the three may change while a tape is recording. */
sevc_status sevc_set_mobility(sevc_handle *h, double mu);
sevc_status sevc_set_gb_scaling(sevc_handle *h, double gb_scaling);
sevc_status sevc_set_stored_energy(sevc_handle *h, const double *se /* ng values */);

/* Gradients of a grain-size statistic with respect to the per-grain stored
 * energies, GB_scaling and the mobility, by a hand-written adjoint of the
 * velocity, event and translation kernels.  sevc_tape_start checkpoints
 * the whole device state now and every `checkpoint_every` steps after; the
 * adjoint replays one segment at a time from its checkpoint, recording the
 * mesh and the position-moving events of each step, and runs the steps
 * backward.  Topology changes are followed (flips, 2x3 and 3-sided
 * removals move or disable vertices; a nucleation moves its vertex and
 * places the new triangle by a map of the neighbours' positions, with the
 * replayed random draws).  Discrete decisions carry no gradient, and a
 * nucleated grain's stored energy (0) is not a parameter.
 * Memory: one copy of the device state per checkpoint plus about 600 bytes
 * per grain per step of one segment. */
sevc_status sevc_tape_start(sevc_handle *h, int checkpoint_every);
sevc_status sevc_tape_stop(sevc_handle *h);
/* Smoothed histogram of normalised grain areas a = |A| N / (domain area)
 * (N enabled grains, so a has mean 1 when all grains are counted):
 * hist[k] = (1/N) sum_g B2(a_g / w - k - 1/2), w = amax / nbins, B2 the
 * quadratic B-spline; nbins <= 1024. */
sevc_status sevc_area_histogram(sevc_handle *h, int nbins, double amax, double *hist);
/* Given dloss/dhist (nbins values) at the current state, write dloss/dSE
 * (ng values, may be NULL), dloss/dGB_scaling and dloss/dmu, for the steps
 * taken since sevc_tape_start.  The handle's state is left unchanged. */
sevc_status sevc_adjoint_histogram(sevc_handle *h, int nbins, double amax, const double *dloss_dhist,
                                   double *grad_se, double *grad_gb_scaling, double *grad_mu);

/* Output-only fields (extinction times of boundaries that cannot flip,
 * dA/dt of grains that cannot vanish) are computed for every entity only
 * on steps that can export a snapshot (sevc_step_info.outputs_complete);
 * on other steps only the values that can ever be exported are (those of
 * entities the step disables).  sevc_export_text after a step that was
 * not complete is refused (SEVC_ERR_ARG).  on = 1 computes every value on
 * every step. */
sevc_status sevc_set_exact_all(sevc_handle *h, int on);

/* Limits of the step's bounded loops and work lists, for exercising the
 * failure paths (0 keeps a value): polling_cap bounds the iterations of
 * the polling loop (src/topological.h:555 has no bound; default 100000),
 * past which sevc_step returns SEVC_ERR_NONCONVERGED; worklist_cap lowers
 * the capacity of the grain-list fix-up work lists (default: every grain
 * and every vertex, which cannot overflow), past which sevc_step returns
 * SEVC_ERR_CAPACITY ("internal worklist overflow").  After a step that
 * returned an error the mesh is in an undefined state: destroy the handle
 * or load a checkpoint.  No counterpart in the reference. */
sevc_status sevc_set_limits(sevc_handle *h, int polling_cap, int worklist_cap);

/* Launch mode.  on = 1 (the default): a step is one CUDA graph, captured
 * on first use and replayed, whose polling and 2x3 loops are conditional
 * nodes driven from the device; on = 2: the step's fixed launch sequences
 * (its first half, one polling iteration, the second half of a step
 * without 2x3 pairs) are graphs and the loops run on the host; on = 0
 * launches every kernel directly.  Results are identical in every mode.
 * Profiling and adjoint replays always launch directly. */
sevc_status sevc_set_graphs(sevc_handle *h, int on);

/* Launch-shape autotuner (no counterpart in the reference): times `steps`
 * steps from the current state for each candidate block size of the
 * vertex pass (128/256/512) and of the per-boundary passes, each side
 * count from which grains get a warp each (9..12), and the resident blocks
 * per SM of the thread-per-grain grain pass (4, 5, 6, 8), one parameter at a
 * time, keeps the fastest and restores the state.  chosen (4 ints, may be
 * NULL) receives them in that order.  Results never depend on these
 * shapes. */
sevc_status sevc_autotune(sevc_handle *h, int steps, int *chosen);

/* Per-kernel device time accumulated while profiling is on (CUDA events
 * around each launch on the handle's stream). */
sevc_status sevc_set_profiling(sevc_handle *h, int on);
sevc_status sevc_get_profile(sevc_handle *h, int max_entries, char (*names)[48], double *ms,
                             int64_t *launches, int *n_entries);

/* Initial microstructure: the job of the reference's generator
 * voronoi/voronoi.py:12-169 (a periodic Voronoi diagram of n seeds drawn
 * uniformly in the unit square, vertices on the 2^-32 grid of [0, 1), only
 * triple junctions; a degenerate sample is drawn again, up to 20 times),
 * in C on every host core.  Outputs: xy 2n vertices (interleaved), ridges
 * 3n pairs of vertex indices, oris n orientations U[0,1) and se n stored
 * energies (se_dist 0: U[0,1), 1: triangular(3, 6, 6) as voronoi.py
 * --sedist triangular); oris and se may be NULL.  The random stream is
 * this library's (xoshiro256** seeded by `seed`), not numpy's: meshes
 * agree with voronoi.py's in distribution.  n >= 64.  SEVC_ERR_TOPOLOGY if
 * no sample gave a triple-junction mesh. */
sevc_status sevc_voronoi_generate(int n, uint64_t seed, int se_dist, double *xy, int32_t *ridges, double *oris,
                                  double *se);
/* The four input files of voronoi.py:141-164 (vertices "%.16f %.16f",
 * ridges "%d %d", orientations and stored energies "%.16f"). */
sevc_status sevc_voronoi_write(int n, const double *xy, const int32_t *ridges, const double *oris, const double *se,
                               const char *vertex_file, const char *ridge_file, const char *ori_file,
                               const char *se_file);

/* The number formatting of the snapshots: writes x as printf("%.16f")
 * does (correctly rounded, ties to even) into out (at least 48 bytes),
 * returns the length.  Integer arithmetic only, several times faster
 * than printf; used by sevc_export_text. */
int sevc_format_fixed16(double x, char *out);

/* The FP64 multiply-add issue rate of the current device, in thread
 * operations per second (independent chains, CUDA events); the roofline
 * that binds the finite-difference kernels.  No counterpart in the
 * reference. */
sevc_status sevc_measure_fp64_rate(double *ops_per_s);

/* Self-test of the device arithmetic behind every arclength: the
 * certified fast division and square root that replace the binary64
 * operations in vector2_mag (src/geometry.h:217).  Runs n random cases
 * (general operands, operands whose exact result lies next to a rounding
 * midpoint, special operands) on the current device and compares each
 * certified result, and each whole vector2_mag, bit for bit with the
 * native operation.  counts[8]: divisions, division mismatches, divisions
 * not certified (these fall back to the native division), square roots,
 * square-root mismatches, square roots not certified, vector2_mag
 * evaluations, vector2_mag mismatches.  No counterpart in the reference. */
sevc_status sevc_selftest_arith(long long n, unsigned long long seed, long long *counts);

/* Text of the last error on this thread. */
const char *sevc_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
