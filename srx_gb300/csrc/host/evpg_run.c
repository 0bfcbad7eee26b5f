/*
 * evpg_run: command-line drop-in for the reference's `trial <input>`
 * (evp.c:7-32). Reads the same namelist, slip and microstructure files and
 * writes vm.out, dd.out, err.out, iters.txt and, with --iout, the .iout dumps.
 *
 *   evpg_run <input> [--outdir D] [--steps K] [--rho0 FILE]
 *                    [--fp32] [--line-search] [--gnd] [--iout]
 *
 * --gnd: first-order GND densities, as the reference built with DD_GND.
 */
#include "evpg.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

int main(int argc, char **argv)
{
    const char *input = 0, *outdir = ".", *rho0 = 0;
    int steps = -1, prec = EVPG_FP64, mode = EVPG_NR_PLAIN, iout = 0, opts = 0, a, st;
    void *job = 0;
    for (a = 1; a < argc; a++) {
        if (!strcmp(argv[a], "--outdir") && a + 1 < argc) outdir = argv[++a];
        else if (!strcmp(argv[a], "--steps") && a + 1 < argc) steps = atoi(argv[++a]);
        else if (!strcmp(argv[a], "--rho0") && a + 1 < argc) rho0 = argv[++a];
        else if (!strcmp(argv[a], "--fp32")) prec = EVPG_FP32_BULK;
        else if (!strcmp(argv[a], "--line-search")) mode = EVPG_NR_LINESEARCH;
        else if (!strcmp(argv[a], "--iout")) iout = 1;
        else if (!strcmp(argv[a], "--gnd")) opts |= EVPG_JOB_GND;
        else if (argv[a][0] == '-') { fprintf(stderr, "evpg_run: unknown option %s\n", argv[a]); return 2; }
        else input = argv[a];
    }
    if (!input) {
        fprintf(stderr, "usage: evpg_run <input> [--outdir D] [--steps K] [--rho0 F] [--fp32] [--line-search] [--gnd] [--iout]\n");
        return 2;
    }
    st = evpg_job_open_opts(input, rho0, prec, mode, opts, &job);
    if (st) {
        fprintf(stderr, "evpg_run: %s: %s\n", evpg_status_string(st), evpg_last_error());
        return 1;
    }
    st = evpg_job_run(job, outdir, steps, iout);
    if (st) fprintf(stderr, "evpg_run: %s: %s\n", evpg_status_string(st), evpg_last_error());
    evpg_job_close(job);
    return st ? 1 : 0;
}
