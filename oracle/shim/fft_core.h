/*
 * Own mixed-radix complex FFT used by the oracle (TEST INFRASTRUCTURE ONLY):
 * both by the FFTW-2 shim that lets the reference sources run, and by the
 * C restatement in oracle/evp_oracle.c.  Sharing one transform between the
 * two makes their results comparable bit for bit.
 *
 * Convention (FFTW's): sign = -1 is exp(-2*pi*i*j*k/n), sign = +1 is
 * exp(+2*pi*i*j*k/n), unnormalised, natural order in and out.
 * Supported lengths: any n >= 1 whose prime factors are 2, 3, 5 or 7.
 */
#ifndef VOCE_FFT_CORE_H
#define VOCE_FFT_CORE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fftc_plan1d fftc_plan1d;

/* 1-D plan for length n and direction sign (-1 or +1); NULL if n unsupported */
fftc_plan1d *fftc_plan1d_create(int n, int sign);
void fftc_plan1d_destroy(fftc_plan1d *p);
/* transform one line of n complex values (interleaved re,im) with stride
 * `stride` complex elements; scratch holds 2*n doubles */
void fftc_line(const fftc_plan1d *p, double *data, long stride, double *scratch);

/* in-place 3-D transform of an nx*ny*nz row-major complex array (z fastest),
 * axes done in the order z, y, x.  nthreads <= 1 runs serially; the result
 * does not depend on nthreads. */
int fftc_3d(int nx, int ny, int nz, int sign, double *data, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
