/*
 * FFTW-2 MPI API stand-in on top of fft_core (see fftw_mpi.h).
 * TEST INFRASTRUCTURE ONLY.
 */
#include "fftw_mpi.h"
#include "fft_core.h"

#include <stdlib.h>
#include <string.h>

struct shim_fftwnd_plan {
    int nx, ny, nz, sign;
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
    *local_nx = p->nx;
    *local_x_start = 0;
    *local_ny_after_transpose = p->ny;
    *local_y_start_after_transpose = 0;
    *total_local_size = p->nx * p->ny * p->nz;
}

void fftwnd_mpi(fftwnd_mpi_plan p, int n_fields, fftw_complex *local_data,
                fftw_complex *work, fftwnd_mpi_output_order output_order)
{
    (void)work; (void)output_order;
    long n = (long)p->nx * p->ny * p->nz;
    for (int f = 0; f < n_fields; ++f)
        fftc_3d(p->nx, p->ny, p->nz, p->sign, (double *)(local_data + f * n),
                g_threads);
}

void fftwnd_mpi_destroy_plan(fftwnd_mpi_plan p) { free(p); }

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
