// Continuous-batching request server over the public C ABI (voce_serve.h).
#include "voce_batch.h"
#include "voce_gpu.h"
#include "voce_serve.h"
#include "voce_internal.h"
#include "voce_trace.h"

#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace {

struct Request {
    voce_request_info info;
    voce_namelist nl;
    voce_slip slip[2];
    bool has_slip[2] = {false, false};
    std::vector<double> euler;
    std::vector<int> grain, phase;
    voce_rve *rve = nullptr;
    long long footprint = 0;
    std::vector<double> sig, edot;  // kept fields (Voigt, 6 x nvox)
    std::vector<char> snap;         // state while suspended (voce_rve_snapshot)
    long long ticks_run = 0;        // batch ticks since its last admission
};

}  // namespace

struct voce_server {
    int precision = 0;
    long long budget = 0, in_use = 0;
    int ticks_per_round = 1;
    int quantum = 0;                // ticks before a running request may be suspended
    long long max_active = 0;       // voxels of the admitted requests at most (0: no limit)
    long long active = 0;           // voxels of the admitted requests
    bool keep_fields = false;
    voce_batch *batch = nullptr;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    long long next_id = 1;
    std::map<long long, std::unique_ptr<Request>> reqs;
    std::deque<long long> queue;
    std::vector<long long> running;
    double now() const
    {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
};

namespace {

long long voxels(const Request &q)
{
    return (long long)q.info.dims[0] * q.info.dims[1] * q.info.dims[2];
}

// Move a running request's state to host memory (a snapshot) and free its
// device memory; it goes to the back of the queue and resumes, bit for bit,
// when admitted again.
int suspend(voce_server *s, Request &q)
{
    int rc = voce_batch_remove(s->batch, q.rve);
    if (rc) return rc;
    const long long n = voce_rve_snapshot_size(q.rve);
    if (n < 0) return (int)-n;
    q.snap.resize((size_t)n);
    rc = voce_rve_snapshot(q.rve, q.snap.data(), n);
    if (rc) return rc;
    q.info.increments_done = voce_rve_increments_done(q.rve);
    voce_rve_destroy(q.rve);
    q.rve = nullptr;
    s->in_use -= q.footprint;
    s->active -= voxels(q);
    q.info.status = VOCE_REQ_QUEUED;
    q.info.preemptions += 1;
    q.ticks_run = 0;
    s->running.erase(std::find(s->running.begin(), s->running.end(), q.info.id));
    s->queue.push_back(q.info.id);
    return VOCE_OK;
}

// End a request: done (error 0), failed (a VOCE_ERR_* code) or cancelled
// (VOCE_ERR_CANCELLED).  Its RVE leaves the batch and its device memory is
// freed; a finished request's record and (with keep_fields) fields are kept.
void retire(voce_server *s, Request &q, int error)
{
    if (q.rve) {
        if (!error) {
            int n = voce_rve_increments_done(q.rve);
            q.info.increments_done = n;
            long long vi = 0;
            const long long nv = (long long)q.info.dims[0] * q.info.dims[1] * q.info.dims[2];
            for (int k = 0; k < n; ++k) {
                voce_increment rec;
                if (voce_rve_get_increment(q.rve, k, &rec) == VOCE_OK) {
                    vi += nv * rec.iters;
                    q.info.last = rec;
                }
            }
            q.info.voxel_iterations = vi;
            if (s->keep_fields) {
                q.sig.resize(6 * nv);
                q.edot.resize(6 * nv);
                voce_rve_get_field(q.rve, VOCE_FIELD_SIG_VOIGT, q.sig.data());
                voce_rve_get_field(q.rve, VOCE_FIELD_EDOT_VOIGT, q.edot.data());
            }
        }
        if (s->batch) voce_batch_remove(s->batch, q.rve);
        voce_rve_destroy(q.rve);
        q.rve = nullptr;
        s->in_use -= q.footprint;
        s->active -= voxels(q);
    }
    q.info.status = error == VOCE_ERR_CANCELLED ? VOCE_REQ_CANCELLED : error ? VOCE_REQ_FAILED : VOCE_REQ_DONE;
    q.info.error = error;
    q.info.t_done = s->now();
    // inputs are no longer needed
    std::vector<double>().swap(q.euler);
    std::vector<int>().swap(q.grain);
    std::vector<int>().swap(q.phase);
    std::vector<char>().swap(q.snap);
}

bool ended(const Request &q)
{
    return q.info.status == VOCE_REQ_DONE || q.info.status == VOCE_REQ_FAILED ||
           q.info.status == VOCE_REQ_CANCELLED;
}

// End request q with `error`, wherever it is (queue or batch).
void end_request(voce_server *s, Request &q, int error)
{
    if (q.info.status == VOCE_REQ_QUEUED) {
        auto it = std::find(s->queue.begin(), s->queue.end(), q.info.id);
        if (it != s->queue.end()) s->queue.erase(it);
    } else if (q.info.status == VOCE_REQ_RUNNING) {
        auto it = std::find(s->running.begin(), s->running.end(), q.info.id);
        if (it != s->running.end()) s->running.erase(it);
    }
    retire(s, q, error);
}

// The device batch, made at the first admission (a server that has admitted
// nothing needs no GPU).
int ensure_batch(voce_server *s)
{
    return s->batch ? VOCE_OK : voce_batch_create(s->precision, &s->batch);
}

}  // namespace

extern "C" {

int voce_server_create(int precision, long long budget, int ticks_per_round, int keep_fields,
                       voce_server **out)
{
    if (!out || budget <= 0 || ticks_per_round < 1) return VOCE_ERR_ARG;
    voce_server *s = new voce_server();
    s->precision = (precision == VOCE_PREC_MIXED || precision == VOCE_PREC_MIXED_NR32 ||
                    precision == VOCE_PREC_MIXED_IR) ? precision
                                                                                      : VOCE_PREC_FP64;
    s->budget = budget;
    s->ticks_per_round = ticks_per_round;
    s->keep_fields = keep_fields != 0;
    *out = s;
    return VOCE_OK;
}

int voce_server_submit(voce_server *s, const voce_namelist *nl, const voce_slip *slip[2],
                       const voce_mesh *mesh, int n_increments, long long *id_out)
{
    if (!s || !nl || !mesh || !mesh->euler_deg || !mesh->phase || n_increments < 1) return VOCE_ERR_ARG;
    auto q = std::make_unique<Request>();
    std::memset(&q->info, 0, sizeof(q->info));
    q->nl = *nl;
    for (int p = 0; p < 2; ++p)
        if (slip && slip[p]) { q->slip[p] = *slip[p]; q->has_slip[p] = true; }
    const long long nv = (long long)mesh->dims[0] * mesh->dims[1] * mesh->dims[2];
    q->euler.assign(mesh->euler_deg, mesh->euler_deg + 3 * nv);
    q->phase.assign(mesh->phase, mesh->phase + nv);
    if (mesh->grain) q->grain.assign(mesh->grain, mesh->grain + nv);
    else q->grain.assign(nv, 1);
    std::memcpy(q->info.dims, mesh->dims, sizeof(q->info.dims));
    q->info.id = s->next_id++;
    q->info.status = VOCE_REQ_QUEUED;
    q->info.increments_wanted = n_increments;
    q->info.t_submit = s->now();
    q->footprint = voce_rve_footprint(mesh->dims, s->precision);
    if (id_out) *id_out = q->info.id;
    s->queue.push_back(q->info.id);
    s->reqs[q->info.id] = std::move(q);
    return VOCE_OK;
}

int voce_server_cancel(voce_server *s, long long id)
{
    if (!s) return VOCE_ERR_ARG;
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return VOCE_ERR_ARG;
    Request &q = *it->second;
    if (ended(q)) return VOCE_ERR_STATE;
    end_request(s, q, VOCE_ERR_CANCELLED);
    return VOCE_OK;
}

int voce_server_set_deadline(voce_server *s, long long id, double t)
{
    if (!s || !(t >= 0.0)) return VOCE_ERR_ARG;
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return VOCE_ERR_ARG;
    if (ended(*it->second)) return VOCE_ERR_STATE;
    it->second->info.t_deadline = t;
    return VOCE_OK;
}

int voce_server_poll(voce_server *s, int *running, int *queued)
{
    VOCE_TRACE("voce_server_poll");
    if (!s) return VOCE_ERR_ARG;
    // requests past their deadline end first (queued or running; between
    // ticks, so none of their kernels is in flight)
    {
        const double now = s->now();
        std::vector<long long> late;
        for (long long id : s->queue)
            if (s->reqs[id]->info.t_deadline > 0.0 && now >= s->reqs[id]->info.t_deadline) late.push_back(id);
        for (long long id : s->running)
            if (s->reqs[id]->info.t_deadline > 0.0 && now >= s->reqs[id]->info.t_deadline) late.push_back(id);
        for (long long id : late) end_request(s, *s->reqs[id], VOCE_ERR_DEADLINE);
    }
    // the running requests' ticks go to the GPU first; admission (reading
    // inputs, allocating and setting up new RVEs) then overlaps them, and the
    // new requests join the batch at the next round.  A server with nothing
    // running admits first and launches at once, and so does one whose next
    // request is the first of its grid shape (its FFT tiles are timed on an
    // otherwise idle GPU).
    std::vector<long long> launched;
    long long t0 = 0;
    const bool tune_next = !s->queue.empty() && !voce::tiles_known(s->reqs[s->queue.front()]->info.dims, s->precision);
    if (!s->running.empty() && !tune_next) {
        t0 = voce_batch_ticks(s->batch);
        int rc = voce_batch_launch(s->batch, s->ticks_per_round);
        if (rc) return rc;
        launched = s->running;
    }
    // admission: first in, first out, while the footprint fits (and the
    // voxels in flight stay under the active limit, when one is set: a lone
    // request is always admitted); with a quantum, requests that have run
    // that long make room by suspending
    while (!s->queue.empty()) {
        Request &q = *s->reqs[s->queue.front()];
        if (q.footprint > s->budget) {
            s->queue.pop_front();
            retire(s, q, VOCE_ERR_NOMEM);
            continue;
        }
        if (s->max_active > 0 && !s->running.empty() && s->active + voxels(q) > s->max_active) break;
        if (s->in_use + q.footprint > s->budget) {
            Request *victim = nullptr;
            if (s->quantum > 0)
                for (long long id : s->running) {
                    Request &c = *s->reqs[id];
                    if (c.ticks_run >= s->quantum && (!victim || c.ticks_run > victim->ticks_run)) victim = &c;
                }
            if (!victim) break;
            // a request that cannot be suspended ends with the error (its
            // memory is freed all the same) instead of staying half out of
            // the batch
            int rc = suspend(s, *victim);
            if (rc) end_request(s, *victim, rc);
            continue;
        }
        s->queue.pop_front();
        int rc = ensure_batch(s);
        if (rc != VOCE_OK) {
            retire(s, q, rc);
            continue;
        }
        if (!q.snap.empty()) {
            // a suspended request: its state comes back from the snapshot
            rc = voce_rve_restore(q.snap.data(), (long long)q.snap.size(), &q.rve);
            if (rc == VOCE_OK) std::vector<char>().swap(q.snap);
        } else {
            voce_mesh m;
            std::memcpy(m.dims, q.info.dims, sizeof(m.dims));
            m.euler_deg = q.euler.data();
            m.grain = q.grain.data();
            m.phase = q.phase.data();
            const voce_slip *sp[2] = {q.has_slip[0] ? &q.slip[0] : nullptr,
                                      q.has_slip[1] ? &q.slip[1] : nullptr};
            rc = voce_rve_create(&q.nl, sp, &m, s->precision, &q.rve);
        }
        // increments still to do (one in progress counts as the first)
        if (rc == VOCE_OK)
            rc = voce_batch_add(s->batch, q.rve, q.info.increments_wanted - voce_rve_increments_done(q.rve));
        if (rc != VOCE_OK) {
            if (q.rve) { voce_rve_destroy(q.rve); q.rve = nullptr; }
            retire(s, q, rc);
            continue;
        }
        s->in_use += q.footprint;
        s->active += voxels(q);
        q.info.status = VOCE_REQ_RUNNING;
        if (q.info.preemptions == 0) q.info.t_admit = s->now();
        q.ticks_run = 0;
        s->running.push_back(q.info.id);
    }
    if (launched.empty() && !s->running.empty()) {
        t0 = voce_batch_ticks(s->batch);
        int rc = voce_batch_launch(s->batch, s->ticks_per_round);
        if (rc) return rc;
        launched = s->running;
    }
    if (!launched.empty()) {
        int left = 0;
        int rc = voce_batch_wait(s->batch, &left);
        if (rc) return rc;
        const long long ran = voce_batch_ticks(s->batch) - t0;
        // the requests that were in the batch when it launched (one suspended
        // meanwhile has left the running list)
        for (long long id : launched)
            if (s->reqs[id]->info.status == VOCE_REQ_RUNNING) s->reqs[id]->ticks_run += ran;
        std::vector<long long> still;
        for (long long id : s->running) {
            Request &q = *s->reqs[id];
            int done = voce_rve_increments_done(q.rve);
            q.info.increments_done = done;
            if (done >= q.info.increments_wanted) retire(s, q, 0);
            else still.push_back(id);
        }
        s->running.swap(still);
    }
    if (running) *running = (int)s->running.size();
    if (queued) *queued = (int)s->queue.size();
    return VOCE_OK;
}

double voce_server_now(const voce_server *s) { return s ? s->now() : -1.0; }

int voce_server_set_quantum(voce_server *s, int ticks)
{
    if (!s || ticks < 0) return VOCE_ERR_ARG;
    s->quantum = ticks;
    return VOCE_OK;
}

int voce_server_set_active_limit(voce_server *s, long long voxels)
{
    if (!s || voxels < 0) return VOCE_ERR_ARG;
    s->max_active = voxels;
    return VOCE_OK;
}

int voce_server_info(const voce_server *s, long long id, voce_request_info *out)
{
    if (!s || !out) return VOCE_ERR_ARG;
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return VOCE_ERR_ARG;
    *out = it->second->info;
    if (it->second->rve) out->increments_done = voce_rve_increments_done(it->second->rve);
    return VOCE_OK;
}

int voce_server_result(const voce_server *s, long long id, int which, double *host_out)
{
    if (!s || !host_out) return VOCE_ERR_ARG;
    auto it = s->reqs.find(id);
    if (it == s->reqs.end() || it->second->info.status != VOCE_REQ_DONE) return VOCE_ERR_STATE;
    const std::vector<double> &v = which == VOCE_FIELD_EDOT_VOIGT ? it->second->edot : it->second->sig;
    if (v.empty()) return VOCE_ERR_STATE;
    std::memcpy(host_out, v.data(), sizeof(double) * v.size());
    return VOCE_OK;
}

long long voce_server_bytes_in_use(const voce_server *s) { return s ? s->in_use : -1; }

int voce_server_destroy(voce_server *s)
{
    if (!s) return VOCE_OK;
    for (auto &kv : s->reqs)
        if (kv.second->rve) {
            if (s->batch) voce_batch_remove(s->batch, kv.second->rve);
            voce_rve_destroy(kv.second->rve);
        }
    if (s->batch) voce_batch_destroy(s->batch);
    delete s;
    return VOCE_OK;
}

}  // extern "C"
