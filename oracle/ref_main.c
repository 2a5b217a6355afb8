/*
 * Driver for the UNMODIFIED reference sources built as the parity oracle
 * (TEST INFRASTRUCTURE ONLY).  It replaces the reference's evp.c (evp.c:7-32)
 * with the same call sequence -- GetNameList, MPI_Init, OpenFiles (rank 0),
 * SetupJob, Evolution -- and adds a wall-clock timer around Evolution().
 * VOCE_REF_RANKS=P runs P ranks (the shim's forked processes), each with
 * its x slab of the grid, as the reference's MPI build does.  It does not
 * call DestroyJob(): that function frees gammatotal and then indexes it, and
 * frees tau_x once per voxel (init.c:874,883,885).
 *
 * The reference's globals are defined in ref_globals.c.
 *
 * usage: evp_ref <namelist> [timing-json-out]
 */
#include "evp.h"

#include <stdio.h>
#include <time.h>

int main(int argc, char **argv)
{
    if (argc < 2) {
        fprintf(stderr, "usage: %s <namelist> [timing.json]\n", argv[0]);
        return 2;
    }
    GetNameList(argv);
    /* the slab FFT's shared exchange buffer: one complex field of the grid */
    shim_mpi_reserve(sizeof(fftw_complex) * (size_t)CellDim[0] * CellDim[1] * CellDim[2]);
    MPI_Init(&argc, &argv);
    MPI_Comm_size(MPI_COMM_WORLD, &NumPE);
    MPI_Comm_rank(MPI_COMM_WORLD, &rank);
    if (rank == 0) PrintNameList();
    if (rank == 0) OpenFiles();

    struct timespec t0, t1, t2;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    SetupJob();
    clock_gettime(CLOCK_MONOTONIC, &t1);
    Evolution();
    clock_gettime(CLOCK_MONOTONIC, &t2);
    if (rank == 0) CloseFiles();

    double setup_s = (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec);
    double evo_s = (t2.tv_sec - t1.tv_sec) + 1e-9 * (t2.tv_nsec - t1.tv_nsec);
    if (argc > 2 && rank == 0) {
        FILE *f = fopen(argv[2], "w");
        if (f) {
            fprintf(f, "{\"setup_s\": %.9f, \"evolution_s\": %.9f, \"nxyz\": %d}\n",
                    setup_s, evo_s, Nxyz);
            fclose(f);
        }
    }
    MPI_Finalize();
    return 0;
}
