/*
 * Stand-in for the FFTW 2.x MPI API that the Voce reference calls
 * (init.c:640-649, evolution.c:356,389,542,555).  TEST INFRASTRUCTURE ONLY.
 *
 * FFTW 2.1.x itself is not vendored with the reference (Makefile:9-12 link
 * -lfftw_mpi -lfftw from an external prefix) and is not installed here, so
 * this shim restates its published contract for the calls used:
 *   - fftw3d_mpi_create_plan(comm, nx, ny, nz, dir, flags): complex 3-D
 *     transform of an nx*ny*nz row-major array (z fastest);
 *     FFTW_FORWARD uses exp(-2*pi*i*jk/n), FFTW_BACKWARD exp(+2*pi*i*jk/n);
 *     neither direction is normalised;
 *   - fftwnd_mpi(plan, 1, data, work, FFTW_NORMAL_ORDER): in-place
 *     transform, output in normal (untransposed) order;
 *   - fftwnd_mpi_local_sizes: rank r of P holds the x slab
 *     [r nx/P, (r+1) nx/P) (one rank: the whole grid); with P > 1 the
 *     transform runs on a shared buffer (shim_fftw.c, shim_mpi.c).
 * The transform itself is oracle/shim/fft_core.c (own mixed-radix code).
 *
 * Like FFTW 2's header this one includes <stdio.h>: evp.h:168 uses FILE
 * without including it.
 */
#ifndef VOCE_SHIM_FFTW_MPI_H
#define VOCE_SHIM_FFTW_MPI_H

#include <stdio.h>
#include <stddef.h>
#include "mpi.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_real;
typedef struct { fftw_real re, im; } fftw_complex;
typedef enum { FFTW_FORWARD = -1, FFTW_BACKWARD = 1 } fftw_direction;
typedef enum { FFTW_NORMAL_ORDER, FFTW_TRANSPOSED_ORDER } fftwnd_mpi_output_order;
#define FFTW_ESTIMATE (0)
#define FFTW_MEASURE (1)

typedef struct shim_fftwnd_plan *fftwnd_mpi_plan;

fftwnd_mpi_plan fftw3d_mpi_create_plan(MPI_Comm comm, int nx, int ny, int nz,
                                       fftw_direction dir, int flags);
void fftwnd_mpi_local_sizes(fftwnd_mpi_plan p, int *local_nx,
                            int *local_x_start, int *local_ny_after_transpose,
                            int *local_y_start_after_transpose,
                            int *total_local_size);
void fftwnd_mpi(fftwnd_mpi_plan p, int n_fields, fftw_complex *local_data,
                fftw_complex *work, fftwnd_mpi_output_order output_order);
void fftwnd_mpi_destroy_plan(fftwnd_mpi_plan p);
void *fftw_malloc(size_t n);
void fftw_free(void *p);

#ifdef __cplusplus
}
#endif
#endif
