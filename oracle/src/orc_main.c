/*
 * orc_main.c -- "orcflow <file.in> [threads]": the CPU oracle run as a
 * command, writing the same output files as ompVC (test infrastructure).
 */
#include <stdio.h>
#include <stdlib.h>

#include "orc.h"

int main(int argc, char **argv)
{
    if (argc < 2) {
        fprintf(stderr, "usage: %s inputfile [threads]\n", argv[0]);
        return 1;
    }
    char err[1024] = {0};
    double secs = 0;
    long long steps = 0;
    int rc = orc_run(argv[1], argc > 2 ? atoi(argv[2]) : 0, &secs, &steps, err, (int)sizeof(err));
    if (rc) {
        fprintf(stderr, "ERROR: %s (code %d)\n", err, rc);
        return 1;
    }
    printf("{\"advect_seconds\": %.6f, \"steps\": %lld}\n", secs, steps);
    return 0;
}
