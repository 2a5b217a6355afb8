/*
 * FFTW-2 MPI API stand-in on top of fft_core (see fftw_mpi.h).
 * TEST INFRASTRUCTURE ONLY.
 */
#include "fftw_mpi.h"
#include "fft_core.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

struct shim_fftwnd_plan {
    int nx, ny, nz, sign;
    int rank, np;                      /* slab of this rank: x in [rank nx/np, (rank+1) nx/np) */
    fftc_plan1d *px, *py, *pz;         /* line plans of the slab transform (np > 1) */
};

/* the most recent plan's dims size the padding of fftw_malloc (below) */
static int g_last_ny = 0, g_last_nz = 0;
static int g_threads = 1;

fftwnd_mpi_plan fftw3d_mpi_create_plan(MPI_Comm comm, int nx, int ny, int nz,
                                       fftw_direction dir, int flags)
{
    (void)comm; (void)flags;
    struct shim_fftwnd_plan *p = (struct shim_fftwnd_plan *)calloc(1, sizeof(*p));
    p->nx = nx; p->ny = ny; p->nz = nz;
    p->sign = (dir == FFTW_FORWARD) ? -1 : 1;
    MPI_Comm_rank(MPI_COMM_WORLD, &p->rank);
    MPI_Comm_size(MPI_COMM_WORLD, &p->np);
    if (p->np > 1) {
        if (nx % p->np != 0 || !shim_mpi_shared_buffer()) {
            fprintf(stderr, "shim fftw: %d ranks do not divide nx = %d (or no shared buffer)\n", p->np, nx);
            MPI_Abort(MPI_COMM_WORLD, 92);
        }
        p->px = fftc_plan1d_create(nx, p->sign);
        p->py = fftc_plan1d_create(ny, p->sign);
        p->pz = fftc_plan1d_create(nz, p->sign);
    }
    g_last_ny = ny;
    g_last_nz = nz;
    const char *t = getenv("VOCE_REF_FFT_THREADS");
    if (t && *t) g_threads = atoi(t);
    return p;
}

void fftwnd_mpi_local_sizes(fftwnd_mpi_plan p, int *local_nx,
                            int *local_x_start, int *local_ny_after_transpose,
                            int *local_y_start_after_transpose,
                            int *total_local_size)
{
    const int lnx = p->nx / p->np;
    *local_nx = lnx;
    *local_x_start = p->rank * lnx;
    *local_ny_after_transpose = p->ny / p->np;
    *local_y_start_after_transpose = p->rank * (p->ny / p->np);
    *total_local_size = lnx * p->ny * p->nz;
}

/* With several ranks the transform runs on the shared buffer: each rank puts
 * its x slab there and transforms its own z and y lines, then a share of the
 * x lines, then takes its slab back.  Every line gets the same 1-D transform
 * with the same stride as in fftc_3d, so the result has the same bits as the
 * one-rank transform. */
static void slab_fft(fftwnd_mpi_plan p, double *local)
{
    const int nx = p->nx, ny = p->ny, nz = p->nz, lnx = nx / p->np, x0 = p->rank * lnx;
    const long plane = (long)ny * nz, slab = (long)lnx * plane;
    double *g = (double *)shim_mpi_shared_buffer();
    int nmax = nx > ny ? nx : ny;
    if (nz > nmax) nmax = nz;
    double *scr = (double *)malloc(sizeof(double) * 4 * (size_t)nmax);
    memcpy(g + 2 * x0 * plane, local, sizeof(double) * 2 * slab);
    for (long l = 0; l < (long)lnx * ny; ++l)                       /* z lines */
        fftc_line(p->pz, g + 2 * (x0 * plane + l * nz), 1, scr);
    for (long l = 0; l < (long)lnx * nz; ++l) {                     /* y lines */
        const long x = x0 + l / nz, z = l % nz;
        fftc_line(p->py, g + 2 * (x * plane + z), nz, scr);
    }
    shim_mpi_barrier();
    const long l0 = plane * p->rank / p->np, l1 = plane * (p->rank + 1) / p->np;
    for (long l = l0; l < l1; ++l)                                 /* x lines */
        fftc_line(p->px, g + 2 * l, plane, scr);
    shim_mpi_barrier();
    memcpy(local, g + 2 * x0 * plane, sizeof(double) * 2 * slab);
    shim_mpi_barrier();   /* the buffer is free for the next transform */
    free(scr);
}

void fftwnd_mpi(fftwnd_mpi_plan p, int n_fields, fftw_complex *local_data,
                fftw_complex *work, fftwnd_mpi_output_order output_order)
{
    (void)work; (void)output_order;
    long n = (long)(p->nx / p->np) * p->ny * p->nz;
    for (int f = 0; f < n_fields; ++f) {
        if (p->np > 1) slab_fft(p, (double *)(local_data + f * n));
        else fftc_3d(p->nx, p->ny, p->nz, p->sign, (double *)(local_data + f * n), g_threads);
    }
}

void fftwnd_mpi_destroy_plan(fftwnd_mpi_plan p)
{
    if (p) {
        fftc_plan1d_destroy(p->px);
        fftc_plan1d_destroy(p->py);
        fftc_plan1d_destroy(p->pz);
    }
    free(p);
}

/* The reference writes one element past its fft_data slab after the
 * displacement-fluctuation loop (evolution.c:552-553: pIDX evaluated after
 * local_loop has run to completion, i.e. (ny+1)*nz elements past the end).
 * Pad every allocation so that this lands in owned, zeroed memory. */
void *fftw_malloc(size_t n)
{
    size_t pad = ((size_t)(g_last_ny + 1) * (size_t)g_last_nz + 16) * sizeof(fftw_complex);
    void *p = calloc(1, n + pad);
    return p;
}

void fftw_free(void *p) { free(p); }
