/*
 * mks_oracle_main.c — command-line driver for the oracle (test
 * infrastructure): runs a start.dat the way mulskips.e does, in the current
 * directory.  Usage: mks_oracle LENX LENY LENZ [numbers.txt] [num_mc_max]
 * [geo.bin [temp.bin]]; with both, the InitSt LA input of
 * ora_set_la_input as raw int8 / int16 arrays; with geo.bin alone, the
 * InitSt IN per-site geometry of ora_set_geometry (raw int8).
 */
#include <stdio.h>
#include <stdint.h>
#include <stdlib.h>
#include "mks_oracle.h"

int main(int argc, char **argv)
{
    if (argc < 4) {
        fprintf(stderr, "usage: %s LENX LENY LENZ [numbers.txt] [num_mc_max] [geo.bin [temp.bin]]\n", argv[0]);
        return 2;
    }
    const char *numbers = argc > 4 ? argv[4] : NULL;
    int mcmax = argc > 5 ? atoi(argv[5]) : 0;
    printf(" KMC box size: %d %d %d\n", atoi(argv[1]), atoi(argv[2]), atoi(argv[3]));
    ora_t *o = ora_create("start.dat", numbers, atoi(argv[1]), atoi(argv[2]), atoi(argv[3]), mcmax);
    if (!o) {
        printf("%s\n", ora_last_error());
        return 1;
    }
    if (argc == 7) {
        size_t n = (size_t)atoi(argv[1]) * atoi(argv[2]) * atoi(argv[3]);
        int8_t *geo = (int8_t *)malloc(n);
        FILE *fg = fopen(argv[6], "rb");
        int ok = geo && fg && fread(geo, 1, n, fg) == n;
        if (fg) fclose(fg);
        if (!ok || ora_set_geometry(o, geo)) {
            printf("cannot load the geometry %s\n", argv[6]);
            return 1;
        }
        free(geo);
    } else if (argc > 7) {
        size_t nz = (size_t)atoi(argv[3]);
        size_t nt = (size_t)(atoi(argv[1]) / 3) * (atoi(argv[2]) / 3) * (atoi(argv[3]) / 3);
        int8_t *geo = (int8_t *)malloc(nz);
        int16_t *t = (int16_t *)malloc(nt * sizeof(int16_t));
        FILE *fg = fopen(argv[6], "rb"), *ft = fopen(argv[7], "rb");
        int ok = geo && t && fg && ft && fread(geo, 1, nz, fg) == nz && fread(t, sizeof(int16_t), nt, ft) == nt;
        if (fg) fclose(fg);
        if (ft) fclose(ft);
        if (!ok || ora_set_la_input(o, geo, t)) {
            printf("cannot load the LA input %s %s\n", argv[6], argv[7]);
            return 1;
        }
        free(geo);
        free(t);
    }
    int r = ora_main(o, ".");
    if (r) printf("%s\n", ora_last_error());
    ora_destroy(o);
    return r ? 1 : 0;
}
