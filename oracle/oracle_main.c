/*
 * Command-line driver for the C restatement (TEST INFRASTRUCTURE ONLY).
 *
 *   evp_oracle <namelist> [-t threads] [-n increments] [-trace file]
 *
 * Runs the job like the reference's main (evp.c:7-32), writes vm.out and
 * err.out lines in the reference's formats (evolution.c:427,563) next to
 * the namelist's current directory, and prints one JSON line with the wall
 * time of the increment loop and the voxel-iteration count.
 */
#include "evp_oracle.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

int main(int argc, char **argv)
{
    if (argc < 2) {
        fprintf(stderr, "usage: %s <namelist> [-t threads] [-n incr] [-trace f]\n", argv[0]);
        return 2;
    }
    int nt = 1, ninc = -1;
    const char *trace = NULL;
    for (int i = 2; i < argc; ++i) {
        if (!strcmp(argv[i], "-t") && i + 1 < argc) nt = atoi(argv[++i]);
        else if (!strcmp(argv[i], "-n") && i + 1 < argc) ninc = atoi(argv[++i]);
        else if (!strcmp(argv[i], "-trace") && i + 1 < argc) trace = argv[++i];
    }
    char err[256] = {0};
    struct timespec t0, t1, t2;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    oracle_job *j = oracle_create(argv[1], nt, trace, err);
    if (!j) { fprintf(stderr, "oracle: %s\n", err); return 1; }
    clock_gettime(CLOCK_MONOTONIC, &t1);
    if (ninc < 0) {
        /* N_steps from the namelist is not exposed; run until asked */
        ninc = 1;
    }
    oracle_run(j, ninc);
    clock_gettime(CLOCK_MONOTONIC, &t2);
    FILE *vm = fopen("vm.out", "w"), *er = fopen("err.out", "w");
    fprintf(vm, "EVM\tEVMP\tDVM\tDVMP\tSVM\tSVMSVM_1\tIteration_tot\n");
    fprintf(er, "IT\tERRE\tERRS\tSVM\n");
    long vit = 0;
    for (int k = 0; k < oracle_n_increments(j); ++k) {
        oracle_incr r;
        oracle_get_increment(j, k, &r);
        fprintf(vm, "%e\t%e\t%e\t%e\t%e\t%e\t%d\n", r.e_vm, r.evmp, r.d_vm, r.dvmp,
                r.s_vm, r.s_vm1, r.iter_total);
        double *a = malloc(sizeof(double) * 3 * (r.iters + 1));
        oracle_get_iter_log(j, k, a, a + r.iters + 1, a + 2 * (r.iters + 1));
        fprintf(er, "STEP = %d\n", r.istep);
        for (int i = 0; i < r.iters; ++i)
            fprintf(er, "%d\t%e\t%e\t%e\n", i + 1, a[i], a[r.iters + 1 + i], a[2 * (r.iters + 1) + i]);
        free(a);
        vit += (long)r.iters;
    }
    fclose(vm);
    fclose(er);
    double su = (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec);
    double ev = (t2.tv_sec - t1.tv_sec) + 1e-9 * (t2.tv_nsec - t1.tv_nsec);
    printf("{\"setup_s\": %.6f, \"evolution_s\": %.6f, \"voxel_iters\": %ld, \"threads\": %d}\n",
           su, ev, vit * oracle_nvox(j), nt);
    oracle_destroy(j);
    return 0;
}
