/*
 * Host-side helpers of the engine (C): option parsing, mesh loading and
 * snapshot text.  Internal header; the public API is include/sevc.h.
 */
#ifndef SEVC_HOST_H
#define SEVC_HOST_H

#include "../../include/sevc.h"
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SEVC_MAX_T_EXT 100000.0 /* src/geometry.h:11 */
#define SEVC_GRAD_EPS 1e-8      /* src/calculus.h:7 */

/* A host mesh with owned storage. */
typedef struct sevc_hmesh {
    sevc_mesh_host m;
    void *block; /* single allocation backing every array */
} sevc_hmesh;

int sevc_hmesh_alloc(sevc_hmesh *hm, int nv, int nb, int ng);
void sevc_hmesh_free(sevc_hmesh *hm);

/* Loader of src/io.h:66-264 from arrays.  n_ori / n_se values are
 * assigned to the first grains (the rest stay 0, as the reference leaves
 * them). */
int sevc_host_build(const sevc_options *opt, int nv, const double *xy, int nb, const int *ridges,
                    int n_ori, const double *oris, int n_se, const double *se, sevc_hmesh *out);
/* Same, reading the four files named in opt. */
int sevc_host_load_files(const sevc_options *opt, sevc_hmesh *out);

/* export_data, src/io.h:280-377. */
int sevc_host_export(const sevc_mesh_host *m, const sevc_options *opt, const char *path, double time);
/* check_data, src/utils.h:85-336: count of violated invariants. */
int sevc_host_check(const sevc_mesh_host *m);

void sevc_set_error(const char *fmt, ...);

#ifdef __cplusplus
}
#endif
#endif
