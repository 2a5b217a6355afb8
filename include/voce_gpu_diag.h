/*
 * voce_gpu_diag.h -- measurement and diagnostic entry points of
 * libvoce_gpu.so.  None of these has a counterpart in the reference (it has
 * no timers, evolution.c); they exist so that a caller can time the solver
 * step on the RVE's own CUDA stream and attribute time to kernels.
 */
#ifndef VOCE_GPU_DIAG_H
#define VOCE_GPU_DIAG_H

#include "voce_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Kernel ids for voce_rve_get_kernel_time (in launch order). */
enum {
    VOCE_K_FFT_Z_FWD = 0,  /* r2c along z of the 6 stress components */
    VOCE_K_FFT_Y_FWD = 1,  /* c2c along y */
    VOCE_K_FFT_X_GREEN = 2,/* c2c along x, Green operator, inverse along x */
    VOCE_K_FFT_Y_INV = 3,  /* c2c along y, inverse */
    VOCE_K_FFT_Z_INV = 4,  /* c2r along z + displacement-gradient update */
    VOCE_K_NR = 5,         /* per-voxel Newton-Raphson stress update */
    VOCE_K_FIN_ITER = 6,   /* error norms, averages, mixed-BC update */
    VOCE_K_PRELUDE = 7,    /* increment prelude */
    VOCE_K_INC_FFT = 8,    /* antisymmetric update back to real space (3 launches) */
    VOCE_K_INCR_END = 9,   /* strain update, reorientation, Voce hardening */
    VOCE_K_FIN_INCR = 10,  /* increment averages */
    VOCE_K_COUNT = 11
};

/* voce_rve_run bracketed by CUDA events on the RVE's stream; device_ms is
 * the elapsed time between them. */
int voce_rve_run_timed(voce_rve *r, int n_increments, double *device_ms);
/* Execution strategy of voce_rve_run: 1 (default) runs each increment as one
 * CUDA graph whose Green-iteration loop is a device-side conditional WHILE
 * node; 0 lets the host read the convergence flag after every iteration.
 * Results are identical. */
int voce_rve_set_graph(voce_rve *r, int on);
/* When on, every kernel launch is bracketed by an event pair; the totals
 * accumulate until reset.  Profiling runs the host-driven loop. */
int voce_rve_set_profiling(voce_rve *r, int on);
int voce_rve_get_kernel_time(const voce_rve *r, int kernel, double *ms_total,
                             long long *timed_launches);
int voce_rve_reset_kernel_times(voce_rve *r);
/* Number of kernels this RVE has launched so far. */
long long voce_rve_kernel_launches(const voce_rve *r);
/* Write `bytes` of scratch on the RVE's stream (evicts the L2), then wait. */
int voce_rve_flush_l2(voce_rve *r, long long bytes);
/* Pinned host memory for inputs and results. */
void *voce_host_alloc(long long bytes);
void voce_host_free(void *p);
/* FP64 FMA throughput of the current device, TFLOP/s (FMA = 2 flops). */
double voce_measure_fp64_tflops(void);
/* Free and total memory of the current device, bytes (cudaMemGetInfo). */
int voce_device_memory(long long *free_bytes, long long *total_bytes);
/* out[i] = the reciprocal the FP64 Newton step and the Green operator use
 * (a hardware seed refined by two Newton-Raphson steps, plain division
 * outside 2^-99 <= |x| < 2^99), computed on the current device for n host
 * values: a check of that reciprocal against 1/x. */
int voce_diag_rcp(const double *x, double *out, int n);
/* out[i] = the square root the mixed_ir form's per-voxel error norms use (a
 * hardware reciprocal-square-root seed refined by one Newton-Raphson step;
 * sqrt itself outside 2^-99 <= x < 2^99), on the current device for n host
 * values: a check of that square root against sqrt.  No counterpart in the
 * reference. */
int voce_diag_sqrt(const double *x, double *out, int n);
/* The single-precision line FFT of the spectrum passes on the current
 * device: nlines lines of length L, in and out [nlines][L] complex values as
 * interleaved (re, im) doubles (rounded to float on the way in), transformed
 * by candidate `schedule` of a single-precision axis of length L (see the
 * schedules below; 0 is the default), sign -1 forward, +1 inverse,
 * unnormalised.  2 L (nlines | 1) complex floats must fit in 200 KB. */
int voce_diag_fft(int L, int nlines, int sign, int schedule, const double *in, double *out);

/* FFT tile tuning.  voce_rve_create times the forward-pass FFT phases with
 * a few tile sizes (lines per block) on the new RVE and keeps the fastest,
 * once per grid shape and spectrum precision per process (results do not
 * depend on the tile).  voce_set_autotune(0) keeps the fixed-budget choice.
 * voce_rve_get_tiles: the z-forward, y, x/Green, z-inverse tiles and the two
 * antisymmetric back-transform tiles of r. */
int voce_set_autotune(int on);
/* With VOCE_TILE_CACHE=<file> in the environment the choices are read from
 * that file first and new ones appended to it (one line per shape), so that
 * other processes on the machine use the same tiles. */
int voce_rve_get_tiles(const voce_rve *r, int tiles[6]);
/* Force the tiles (each divides the dimension it splits: ny, nx, ny, ny, ny,
 * ny; all phases fit in shared memory); between calls, outside a batch. */
int voce_rve_set_tiles(voce_rve *r, const int tiles[6]);

/* FFT radix schedules (no counterpart in the reference, which leaves its
 * transforms to FFTW).  Each axis of length L = 2^a 3^b can run as Stockham
 * passes of radix 4, 2 and 3; the candidate schedules are their stage orders
 * 4s-2-3s, 3s-4s-2, 2-4s-3s and 3s-2-4s, duplicates dropped.  In the
 * single-precision spectrum forms (VOCE_PREC_MIXED, VOCE_PREC_MIXED_NR32,
 * VOCE_PREC_MIXED_IR) an axis of length 16, 24, 32, 48, 64, 96, 128, 192 or
 * 256 has one more candidate, placed first: the register FFT, two passes of
 * small DFTs of lengths N1 x N2 = L held in registers (4x4, 4x6, 4x8, 6x8,
 * 8x8, 8x12, 8x16, 12x16, 16x16).  Candidate 0 is the default.
 * Unlike the tiles, the schedule changes results in the last bits (a
 * different order of roundings).  So the FP64 form never tunes it: its RVEs
 * run the default schedule of every axis unless the caller sets one, and its
 * results are the same bits in every process.  For the single-precision
 * spectrum forms, with tuning on,
 * voce_rve_create times the candidates of each axis on the forward pass that
 * transforms it (with the tuned tile) and keeps one only when it is more than
 * 3 % faster than the default; the choice is cached with the tiles (and in
 * VOCE_TILE_CACHE).  Their bits can therefore differ between processes whose
 * tuning timed differently (within the form's single-precision error), but
 * not within a process: an RVE keeps its schedule for life, alone, in a
 * batch, in the server and through snapshots.
 * voce_fft_schedule_count: Stockham candidates for length L (the FP64 form's
 * list; 0 if L is not 2^a 3^b).
 * voce_rve_fft_schedule_count: the candidates of axis (0 x, 1 y, 2 z) of r.
 * voce_rve_get_fft_schedule: the radices of axis in stage order (the
 * register FFT: its two lengths N1, N2); returns the number of stages (at
 * most max written), < 0 on error.
 * voce_rve_set_fft_schedule: use candidate k of axis; between calls,
 * outside a batch. */
int voce_fft_schedule_count(int L);
int voce_rve_fft_schedule_count(const voce_rve *r, int axis);
/* Chord steps in the FP64 Newton of the VOCE_PREC_MIXED form (no
 * counterpart in the reference, which refreshes the Jacobian every Newton
 * iteration, evolution.c:85-110): once a step has moved the stress by less
 * than 1e-4 relative, the next one reuses its factored Jacobian.  The
 * residual and the stop test are the reference's, and the converged stress
 * moves by ~1e-14; but a chord step can add a Newton iteration, and the
 * reference evaluates the strain rate and the error norms at the stress
 * before the last update, so those move by up to ~1e-8 relative.  That is
 * far inside the mixed form's error (single-precision spectrum) and outside
 * the FP64 form's parity bound, so the FP64 form never takes chord steps.
 * On (1) by default; applies to RVEs created afterwards. */
int voce_set_newton_chord(int on);
/* Start of the VOCE_PREC_MIXED_IR Newton (no counterpart in the reference):
 * before its FP64-residual iterations, each voxel's stress is moved from the
 * Green iterate by Newton steps computed on the FP32 pipe -- single-precision
 * steps to a relative update of 1e-4, then one step on a float-float residual
 * (about 48 bits) -- to within about 1e-9 relative of the FP64 residual's
 * root.  The FP64-residual steps and their stop test (evolution.c:112) then
 * run unchanged, so every accepted stress is a root of the FP64 residual to
 * the same test, and the strain rate is evaluated at the FP64 iteration's
 * start; the start only shortens the FP64 iterations (usually to one step).
 * Off, every Newton step of the form evaluates its residual in FP64 from the
 * Green iterate.  On (1) by default; applies to RVEs created afterwards. */
int voce_set_ir_predictor(int on);
int voce_rve_get_fft_schedule(const voce_rve *r, int axis, int *radices, int max);
int voce_rve_set_fft_schedule(voce_rve *r, int axis, int k);

#ifdef __cplusplus
}
#endif
#endif
