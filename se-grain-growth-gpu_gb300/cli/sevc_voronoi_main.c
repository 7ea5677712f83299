/*
 * sevc-voronoi — the reference's input generator voronoi/voronoi.py:112-169
 * as a C program on the library's generator (sevc_voronoi_generate):
 *
 *   sevc-voronoi <N> <seed> <file vertices> <file ridges> <file orientations> <file_SE> [--sedist DIST]
 *
 * DIST is uniform (default) or triangular; the files have voronoi.py's
 * formats and its periodic triple-junction mesh of N grains (2N vertices,
 * 3N ridges).
 */
#include "../../include/sevc.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

int main(int argc, char **argv)
{
    if (argc != 7 && argc != 9) {
        fprintf(stderr, "Usage:\n\t%s <N> <seed> <file vertices> <file ridges> <file orientations> <file_SE> "
                        "[--sedist DIST]\n", argv[0]);
        return 1;
    }
    int n = atoi(argv[1]);
    unsigned long long seed = strtoull(argv[2], NULL, 10);
    int dist = 0;
    if (argc == 9) {
        if (strcmp(argv[7], "--sedist")) { fprintf(stderr, "unknown option %s\n", argv[7]); return 1; }
        dist = !strcmp(argv[8], "triangular");
    }
    double *xy = malloc(sizeof(double) * 4 * (size_t)n), *oris = malloc(sizeof(double) * (size_t)n);
    double *se = malloc(sizeof(double) * (size_t)n);
    int32_t *ridges = malloc(sizeof(int32_t) * 6 * (size_t)n);
    if (!xy || !oris || !se || !ridges) { fprintf(stderr, "out of memory\n"); return 1; }
    if (sevc_voronoi_generate(n, seed, dist, xy, ridges, oris, se) != SEVC_OK ||
        sevc_voronoi_write(n, xy, ridges, oris, se, argv[3], argv[4], argv[5], argv[6]) != SEVC_OK) {
        fprintf(stderr, "%s\n", sevc_last_error());
        return 1;
    }
    printf("Vertices: %d\nRidges: %d\nOrientations: %d\nSE %s: %d\n", 2 * n, 3 * n, n,
           dist ? "triangular" : "uniform", n);
    free(xy); free(oris); free(se); free(ridges);
    return 0;
}
