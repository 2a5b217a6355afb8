/*
 * voce_serve.h -- serving RVE solve requests with continuous batching.
 *
 * There is no counterpart in the reference (one RVE per MPI job).  A
 * request is one RVE (namelist, slip data, mesh) and a number of strain
 * increments, as a multiscale or microstructure-screening caller would send
 * it.  The server keeps one batch (voce_batch.h) running on the GPU.  Each
 * voce_server_poll() is one round: admit queued requests first-in first-out
 * while their device footprint (voce_rve_footprint) fits the HBM budget;
 * advance the batch by at most ticks_per_round ticks; retire the requests
 * whose increments are done, which frees their memory for the next
 * admissions.  Requests that arrive while others run join the running batch
 * at the next round; fields and hardening state stay on the device between
 * increments.  Times are seconds on the server's monotonic clock.
 *
 * A request can be cancelled, and given a deadline, at any time between
 * calls: a cancelled request leaves the queue, or the running batch between
 * two ticks, and its device memory is freed at once; a request that is not
 * done by its deadline is ended the same way at the start of the next
 * voce_server_poll, with the error VOCE_ERR_DEADLINE.  Neither changes the
 * other requests' results (each RVE's arithmetic is independent of what else
 * is in the batch).
 */
#ifndef VOCE_SERVE_H
#define VOCE_SERVE_H

#include "voce_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct voce_server voce_server;

enum { VOCE_REQ_QUEUED = 0, VOCE_REQ_RUNNING = 1, VOCE_REQ_DONE = 2, VOCE_REQ_FAILED = 3,
       VOCE_REQ_CANCELLED = 4 };

typedef struct {
    long long id;
    int status;                 /* VOCE_REQ_* */
    int error;                  /* VOCE_ERR_* when failed */
    int increments_done, increments_wanted;
    int dims[3];
    double t_submit, t_admit, t_done;
    long long voxel_iterations; /* sum over its increments of voxels x Green iterations */
    voce_increment last;        /* record of its last increment */
    int preemptions;            /* times it was suspended to make room */
    double t_deadline;          /* server time by which it must be done (0: none) */
} voce_request_info;

/* keep_fields: keep the final stress and strain-rate fields (Voigt order,
 * io.c:321-397) of finished requests on the host. */
int voce_server_create(int precision, long long hbm_budget_bytes,
                       int ticks_per_round, int keep_fields, voce_server **out);
/* Copies the inputs; the request is queued at the current server time. */
int voce_server_submit(voce_server *s, const voce_namelist *nl,
                       const voce_slip *slip[2], const voce_mesh *mesh,
                       int n_increments, long long *id_out);
/* Time slicing under a full budget: when the request at the head of the
 * queue does not fit, a running request that has run at least `ticks` batch
 * ticks since its admission (the longest-running first) is suspended -- its
 * state goes to host memory as a snapshot, it frees its device memory and
 * rejoins the back of the queue -- until the head fits.  A suspended request
 * resumes exactly where it stopped (bit-identical results).  0 (the
 * default): no suspension, first in first out. */
int voce_server_set_quantum(voce_server *s, int ticks);
/* Active limit: admit the queue head only while the voxels of the admitted
 * requests, with it, stay at or under `voxels` (a request is always admitted
 * when nothing runs).  Once the batch holds enough voxels to keep the GPU
 * busy, more requests in flight only share it: each tick takes longer and
 * every request finishes later.  A limit near that point keeps throughput
 * and lets requests finish in arrival order, which lowers p50 and p99
 * latency.  0 (the default): admission by HBM footprint alone. */
int voce_server_set_active_limit(voce_server *s, long long voxels);
/* Cancel request id (queued or running): it leaves the queue or the batch,
 * its device memory is freed, its status becomes VOCE_REQ_CANCELLED (error
 * VOCE_ERR_CANCELLED) and t_done the cancellation time.  VOCE_ERR_STATE if it
 * has already ended. */
int voce_server_cancel(voce_server *s, long long id);
/* Deadline of request id: server time t (voce_server_now's clock; 0 clears
 * it).  A request not done when a voce_server_poll starts at or after t is
 * ended there: status VOCE_REQ_FAILED, error VOCE_ERR_DEADLINE, its device
 * memory freed.  VOCE_ERR_STATE if it has already ended. */
int voce_server_set_deadline(voce_server *s, long long id, double t);
/* One round; *running and *queued receive the counts afterwards.  Expired
 * deadlines are handled first.  The running requests' ticks are then
 * launched, and admission (reading inputs, creating RVEs) runs while they
 * are on the GPU; the admitted requests join the batch at the next round.
 * With nothing running, or when the queue head is the first request of its
 * grid shape (its FFT tiles are timed on an idle GPU), admission comes
 * first and the ticks are launched after it.  The round ends when the ticks
 * are done; finished requests are retired.  A request that fails on
 * admission, or cannot be suspended, ends with that error (VOCE_REQ_FAILED)
 * and the other requests go on. */
int voce_server_poll(voce_server *s, int *running, int *queued);
double voce_server_now(const voce_server *s);
int voce_server_info(const voce_server *s, long long id, voce_request_info *out);
/* Final fields of a finished request kept with keep_fields:
 * which = 20 (stress) or 21 (plastic strain rate), 6 x nvox doubles. */
int voce_server_result(const voce_server *s, long long id, int which, double *host_out);
/* Bytes of device memory the admitted requests hold. */
long long voce_server_bytes_in_use(const voce_server *s);
int voce_server_destroy(voce_server *s);

#ifdef __cplusplus
}
#endif
#endif
