"""Serving with continuous batching (include/voce_serve.h): requests that
arrive while others run join the running batch; admission respects the HBM
budget; every result equals the same RVE solved alone, bit for bit."""
import os
import tempfile

import numpy as np
import pytest

from voce_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def _inputs(case):
    d = tempfile.mkdtemp(prefix="serve_")
    nlp = case.write(d)
    return nlp, capi.read_namelist(nlp), capi.read_slip(os.path.join(d, "mat.sx"))


def test_requests_alone_and_in_the_mix(voce_lib):
    rng = np.random.Generator(np.random.PCG64(77))
    cases = []
    for i, (n, g, inc) in enumerate([(16, 10, 2), (8, 4, 3), (24, 20, 1), (12, 6, 2), (16, 30, 2), (8, 3, 1)]):
        c = synth.small_case(n, g, 500 + i, n_steps=inc, load=synth.random_traceless_load(rng))
        c.iter_max = 40
        cases.append((c, inc))
    alone = []
    for c, n in cases:
        nlp, _, _ = _inputs(c)
        with capi.Rve.from_files(nlp) as r:
            r.run(n)
            alone.append((r.increment(n - 1), r.field("sig_voigt"), r.field("edot_voigt")))
    budget = 2 * capi.footprint((24, 24, 24))      # forces queueing
    with capi.Server(capi.PREC_FP64, budget, ticks_per_round=5, keep_fields=True) as s:
        ids = []
        for k, (c, n) in enumerate(cases):
            _, nl, sx = _inputs(c)
            ids.append(s.submit(nl, sx, c.mesh.euler_deg, c.mesh.grain, c.mesh.phase, n))
            if k % 2:                                # arrivals while others run
                s.poll()
                assert s.bytes_in_use <= budget
        for _ in range(100000):
            run, que = s.poll()
            assert s.bytes_in_use <= budget
            if run == 0 and que == 0:
                break
        for rid, (c, n), (inc, sig, edot) in zip(ids, cases, alone):
            info = s.info(rid)
            assert info.status == capi.REQ_DONE and info.increments_done == n
            assert info.t_submit <= info.t_admit <= info.t_done
            assert info.last.iters == inc["iters"] and list(info.last.sig_avg) == inc["sig_avg"]
            assert np.array_equal(s.result(rid, "sig_voigt", c.mesh.nvox), sig)
            assert np.array_equal(s.result(rid, "edot_voigt", c.mesh.nvox), edot)


def test_request_larger_than_budget_fails(voce_lib):
    c = synth.small_case(16, 5, 9, n_steps=1)
    _, nl, sx = _inputs(c)
    with capi.Server(capi.PREC_FP64, capi.footprint((8, 8, 8)), ticks_per_round=4) as s:
        rid = s.submit(nl, sx, c.mesh.euler_deg, c.mesh.grain, c.mesh.phase, 1)
        s.poll()
        info = s.info(rid)
        assert info.status == capi.REQ_FAILED and info.error == 7


def test_time_slicing_suspends_and_resumes_bit_for_bit(voce_lib):
    """A budget for two requests, three requests and a quantum of 3 ticks:
    running requests are suspended to host memory to let the queue move, and
    every result still equals the request solved alone."""
    rng = np.random.Generator(np.random.PCG64(78))
    cases = []
    for i in range(3):
        c = synth.small_case(16, 8, 600 + i, n_steps=2, load=synth.random_traceless_load(rng))
        c.iter_max = 30
        cases.append((c, 2))
    alone = []
    for c, n in cases:
        nlp, _, _ = _inputs(c)
        with capi.Rve.from_files(nlp) as r:
            r.run(n)
            alone.append(([r.increment(k) for k in range(n)], r.field("sig_voigt")))
    budget = 2 * capi.footprint((16, 16, 16))
    with capi.Server(capi.PREC_FP64, budget, ticks_per_round=2, keep_fields=True) as s:
        s.set_quantum(3)
        ids = []
        for c, n in cases:
            _, nl, sx = _inputs(c)
            ids.append(s.submit(nl, sx, c.mesh.euler_deg, c.mesh.grain, c.mesh.phase, n))
        for _ in range(100000):
            run, que = s.poll()
            assert s.bytes_in_use <= budget
            if run == 0 and que == 0:
                break
        pre = 0
        for rid, (c, n), (incs, sig) in zip(ids, cases, alone):
            info = s.info(rid)
            assert info.status == capi.REQ_DONE and info.increments_done == n
            assert info.last.iters == incs[-1]["iters"] and list(info.last.sig_avg) == incs[-1]["sig_avg"]
            assert np.array_equal(s.result(rid, "sig_voigt", c.mesh.nvox), sig)
            pre += info.preemptions
        assert pre > 0


def test_active_limit_keeps_voxels_in_flight_under_it(voce_lib):
    """An active limit of 2 x 16^3 voxels: never more admitted than that (one
    request always runs), requests still finish first in first out by
    admission, and every result equals the request solved alone."""
    rng = np.random.Generator(np.random.PCG64(79))
    cases = []
    for i, n in enumerate([16, 8, 16, 12, 16]):
        c = synth.small_case(n, 6, 700 + i, n_steps=1, load=synth.random_traceless_load(rng))
        c.iter_max = 30
        cases.append(c)
    alone = []
    for c in cases:
        nlp, _, _ = _inputs(c)
        with capi.Rve.from_files(nlp) as r:
            r.run(1)
            alone.append(r.field("sig_voigt"))
    limit = 2 * 16 ** 3
    with capi.Server(capi.PREC_FP64, 64 << 30, ticks_per_round=3, keep_fields=True) as s:
        s.set_active_limit(limit)
        ids = []
        for c in cases:
            _, nl, sx = _inputs(c)
            ids.append(s.submit(nl, sx, c.mesh.euler_deg, c.mesh.grain, c.mesh.phase, 1))
        for _ in range(100000):
            run, que = s.poll()
            infos = [s.info(i) for i in ids]
            active = sum(int(np.prod(x.dims)) for x in infos if x.status == capi.REQ_RUNNING)
            assert active <= limit
            if run == 0 and que == 0:
                break
        admits = [s.info(i).t_admit for i in ids]
        assert admits == sorted(admits)
        for rid, c, sig in zip(ids, cases, alone):
            assert s.info(rid).status == capi.REQ_DONE
            assert np.array_equal(s.result(rid, "sig_voigt", c.mesh.nvox), sig)


def test_cancel_and_deadline_leave_the_others_bit_identical(voce_lib):
    """Four requests in one running batch: one is cancelled while it runs,
    one is given a deadline that expires mid-run, one is cancelled while
    still queued behind the active limit.  Each ended request frees its
    device memory at once; the survivors finish with the same bits as the
    same RVEs solved alone."""
    rng = np.random.Generator(np.random.PCG64(78))
    cases = []
    for i, (n, g, inc) in enumerate([(16, 10, 3), (12, 6, 3), (16, 12, 3), (8, 4, 2), (12, 5, 2)]):
        c = synth.small_case(n, g, 600 + i, n_steps=inc, load=synth.random_traceless_load(rng))
        c.iter_max = 40
        cases.append((c, inc))
    keep = [0, 3]
    alone = {}
    for k in keep:
        c, n = cases[k]
        nlp, _, _ = _inputs(c)
        with capi.Rve.from_files(nlp) as r:
            r.run(n)
            alone[k] = (r.increment(n - 1), r.field("sig_voigt"), r.field("edot_voigt"))
    with capi.Server(capi.PREC_FP64, 64 << 30, ticks_per_round=3, keep_fields=True) as s:
        # room for the first four in flight, the fifth waits in the queue
        s.set_active_limit(sum(c.mesh.nvox for c, _ in cases[:4]))
        ids = []
        for c, n in cases:
            _, nl, sx = _inputs(c)
            ids.append(s.submit(nl, sx, c.mesh.euler_deg, c.mesh.grain, c.mesh.phase, n))
        run, que = s.poll()
        assert (run, que) == (4, 1)
        used = s.bytes_in_use
        s.cancel(ids[1])                                   # running
        assert s.info(ids[1]).status == capi.REQ_CANCELLED
        assert s.bytes_in_use == used - capi.footprint(cases[1][0].mesh.dims)
        s.cancel(ids[4])                                   # queued
        s.set_deadline(ids[2], s.now() + 0.05)             # running, expires soon
        import time
        time.sleep(0.1)
        for _ in range(100000):
            run, que = s.poll()
            if run == 0 and que == 0:
                break
        i2 = s.info(ids[2])
        assert i2.status == capi.REQ_FAILED and i2.error == capi.ERR_DEADLINE
        assert i2.increments_done < cases[2][1]
        assert s.info(ids[4]).status == capi.REQ_CANCELLED and s.info(ids[4]).t_admit == 0.0
        assert s.bytes_in_use == 0
        for k in keep:
            c, n = cases[k]
            info = s.info(ids[k])
            inc, sig, edot = alone[k]
            assert info.status == capi.REQ_DONE and info.increments_done == n
            assert info.last.iters == inc["iters"] and list(info.last.sig_avg) == inc["sig_avg"]
            assert np.array_equal(s.result(ids[k], "sig_voigt", c.mesh.nvox), sig)
            assert np.array_equal(s.result(ids[k], "edot_voigt", c.mesh.nvox), edot)
