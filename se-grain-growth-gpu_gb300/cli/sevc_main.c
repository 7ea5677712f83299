/*
 * sevc — drop-in replacement for the reference executable `SEVC -c file.ini`
 * (src/main.cu:21-424): same options file, same input files, same
 * DATA/%06d.txt snapshots and the same host log lines, on the GB300 engine.
 *
 *   sevc -c file.ini [--honor-leave-percent] [--quiet]
 *
 * --honor-leave-percent stops at floor(leave_percent * n_grains) grains;
 * without it the stop threshold is 5000 grains, the constant the reference
 * hard-codes at src/main.cu:49.
 */
#include "../../include/sevc.h"

#include <math.h>
#include <stdio.h>
#include <string.h>

static void print_options(const sevc_options *o)  /* src/options.h:173-204 */
{
    if (o->tmax > 0 && o->nmax == -1) printf("Running until t = %.16f\n", o->tmax);
    else printf("Running until iteration #%d\n", o->nmax);
    printf("Grain Boundary Energy Info:\n\tUsing GB epsilon: %.16f\n\tGB energy scaling: %.16f\n", o->GB_eps,
           o->GB_scaling);
    printf("Stored Energy Info:\n\tSE scaling: %.16f\n", o->SE_eps);
    if (o->SE_min == 999 && o->SE_max == 999) printf("\tMin and max values of SE will be obtained from data\n");
    else if (o->SE_min == o->SE_max) printf("\tMin SE = Max SE: %.16f\n", o->SE_max);
    else printf("\tMin SE: %.16f\n\tMax SE: %.16f\n", o->SE_min, o->SE_max);
    printf("\tMC k: %.16f\n", o->MC_k);
    if (o->do_nucleation)
        printf("Perform nucleation: True\n\tNucleating each %d steps\n\tNucleation scaling: %.16f\n",
               o->nucleation_gap, o->nucleation_scaling);
    else printf("Perform nucleation: False\n");
    printf("Domain bound [0 x %.2f][0 x %.2f]\n", o->domain_bound, o->domain_bound);
    printf("Configuration file loaded.\n");
}

int main(int argc, char **argv)
{
    const char *ini = NULL;
    int honor = 0, verbose = 1;
    for (int i = 1; i < argc; i++) {
        if (!strcmp(argv[i], "-c") && i + 1 < argc) ini = argv[++i];
        else if (!strcmp(argv[i], "--honor-leave-percent")) honor = 1;
        else if (!strcmp(argv[i], "--quiet")) verbose = 0;
    }
    if (!ini) {
        fprintf(stderr, "usage: %s -c file.ini [--honor-leave-percent] [--quiet]\n", argv[0]);
        return 1;
    }
    sevc_options opt;
    if (verbose) printf("Loading %s ...\n", ini);
    if (sevc_load_ini(ini, &opt) != SEVC_OK) {
        fprintf(stderr, "%s\n", sevc_last_error());
        return 1;
    }
    if (honor) opt.min_grains = opt.leave_percent < 0 ? -1 : (int)floor(opt.leave_percent * opt.n_grains);
    if (verbose) print_options(&opt);
    sevc_status st = sevc_run_program(&opt, verbose);
    if (st != SEVC_OK) {
        fprintf(stderr, "sevc: error %d: %s\n", (int)st, sevc_last_error());
        return 1;
    }
    return 0;
}
