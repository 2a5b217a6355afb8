/*
 * voce_batch.h -- batched RVEs: many RVEs of any grid size advanced
 * together, one kernel launch per phase for the whole batch.
 *
 * There is no counterpart in the reference, which runs one RVE per MPI job
 * (evp.c:7-32).  Every RVE keeps its own state, convergence and increment
 * count; a batch "tick" advances each RVE that still has work by one
 * Green-operator iteration (plus its increment end when it converges in
 * that tick).  Per-RVE sums use the same fixed-order reductions as a lone
 * RVE, so an RVE gives bit-identical results alone and in any batch.
 * The tick loop runs on the device as a CUDA graph with a conditional WHILE
 * node; the host returns when every RVE has done its increments or the
 * tick budget is spent.
 */
#ifndef VOCE_BATCH_H
#define VOCE_BATCH_H

#include "voce_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct voce_batch voce_batch;

/* All RVEs of a batch have the batch's precision (VOCE_PREC_*). */
int voce_batch_create(int precision, voce_batch **out);
/* Schedule n_increments more increments of r (created with
 * voce_rve_create*) inside the batch.  While it belongs to a batch an RVE is
 * advanced only by voce_batch_run. */
int voce_batch_add(voce_batch *b, voce_rve *r, int n_increments);
/* Take r out after any voce_batch_run; it keeps its state and can run alone
 * again, be snapshotted or join another batch.  Taken out in the middle of
 * an increment it continues that increment where it stopped (voce_rve_run(n)
 * and voce_batch_add(.., n) count it as the first of their n). */
int voce_batch_remove(voce_batch *b, voce_rve *r);
int voce_batch_size(const voce_batch *b);
/* Run up to max_ticks ticks; *active_left receives the number of RVEs that
 * still have increments to do.  Increment records of every RVE are
 * available afterwards through voce_rve_get_increment. */
int voce_batch_run(voce_batch *b, int max_ticks, int *active_left);
/* voce_batch_run in two halves, so that the host can work while the GPU
 * runs the ticks (no counterpart in the reference).  voce_batch_launch
 * enqueues up to max_ticks ticks and returns at once; voce_batch_wait waits
 * for them and takes in the increment records, as voce_batch_run does.
 * In between, the caller may create RVEs and add them to this batch (they
 * join at the next launch) or do unrelated host and GPU work; it must not
 * read or change the state of the batch's RVEs (fields, snapshots, runs).
 * voce_batch_remove, voce_batch_run, voce_batch_launch and
 * voce_batch_destroy wait for outstanding ticks first. */
int voce_batch_launch(voce_batch *b, int max_ticks);
int voce_batch_wait(voce_batch *b, int *active_left);
/* Ticks run so far. */
long long voce_batch_ticks(const voce_batch *b);
/* Detaches the RVEs (they are not destroyed) and frees the batch. */
int voce_batch_destroy(voce_batch *b);

/* Diagnostics.  With profiling on, voce_batch_run drives the ticks from the
 * host instead of the graph (same kernels, same results) and brackets every
 * launch with CUDA events; voce_batch_get_kernel_time then gives the summed
 * milliseconds and the launch count of kernel k (the VOCE_K_* ids of
 * voce_gpu_diag.h). */
int voce_batch_set_profiling(voce_batch *b, int on);
int voce_batch_get_kernel_time(const voce_batch *b, int k, double *ms, long long *launches);
int voce_batch_reset_kernel_times(voce_batch *b);

#ifdef __cplusplus
}
#endif
#endif
