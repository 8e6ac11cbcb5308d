/*
 * mks_oracle_main.c — command-line driver for the oracle (test
 * infrastructure): runs a start.dat the way mulskips.e does, in the current
 * directory.  Usage: mks_oracle LENX LENY LENZ [numbers.txt] [num_mc_max]
 */
#include <stdio.h>
#include <stdlib.h>
#include "mks_oracle.h"

int main(int argc, char **argv)
{
    if (argc < 4) {
        fprintf(stderr, "usage: %s LENX LENY LENZ [numbers.txt] [num_mc_max]\n", argv[0]);
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
    int r = ora_main(o, ".");
    if (r) printf("%s\n", ora_last_error());
    ora_destroy(o);
    return r ? 1 : 0;
}
