"""Batched RVEs (include/voce_batch.h): every RVE gives the same increment
records and fields alone and inside a batch of RVEs of other sizes, loads
and increment counts, bit for bit, in both precisions."""
import tempfile

import numpy as np
import pytest

from voce_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def _cases():
    rng = np.random.Generator(np.random.PCG64(2024))
    out = []
    for i, (n, g, inc) in enumerate([(8, 5, 3), (16, 20, 2), (12, 9, 4), (24, 30, 2), (16, 1, 3), (32, 40, 1)]):
        load = synth.random_traceless_load(rng) if i % 2 else synth.tension_z()
        c = synth.small_case(n, g, 300 + i, n_steps=inc, load=load)
        c.iter_max = 60
        out.append((c, inc))
    return out


def _make(case, prec):
    d = tempfile.mkdtemp(prefix="batch_")
    return capi.Rve.from_files(case.write(d), prec)


def _snapshot(r, n):
    return ([r.increment(k) for k in range(n)], r.field("sig_voigt"), r.field("edot_voigt"),
            r.field("crss"), r.field("tranmat"))


def _same(a, b):
    ia, sa, ea, ca, ta = a
    ib, sb, eb, cb, tb = b
    assert [x["iters"] for x in ia] == [x["iters"] for x in ib]
    for x, y in zip(ia, ib):
        assert x["sig_avg"] == y["sig_avg"] and x["s_vm"] == y["s_vm"] and x["evmp"] == y["evmp"]
    for u, v in ((sa, sb), (ea, eb), (ca, cb), (ta, tb)):
        assert np.array_equal(u, v)


@pytest.mark.parametrize("prec", [capi.PREC_FP64, capi.PREC_MIXED, capi.PREC_MIXED_NR32, capi.PREC_MIXED_IR])
def test_alone_equals_in_batch(prec, voce_lib):
    cases = _cases()
    alone = []
    for c, n in cases:
        with _make(c, prec) as r:
            r.run(n)
            alone.append(_snapshot(r, n))
    rves = [_make(c, prec) for c, _ in cases]
    with capi.Batch(prec) as b:
        for r, (c, n) in zip(rves, cases):
            b.add(r, n)
        left = b.run()
        assert left == 0
        assert b.ticks > 0
    for r, (c, n), ref in zip(rves, cases, alone):
        _same(_snapshot(r, n), ref)
        r.close()


def test_tick_budget_resume_and_rejoin(voce_lib):
    """Stopping on a tick budget mid-increment and resuming gives the same
    result; an RVE leaves the batch between increments and continues alone."""
    cases = _cases()[:3]
    ref = []
    for c, n in cases:
        with _make(c, capi.PREC_FP64) as r:
            r.run(n + 1)
            ref.append(_snapshot(r, n + 1))
    rves = [_make(c, capi.PREC_FP64) for c, _ in cases]
    b = capi.Batch(capi.PREC_FP64)
    for r, (c, n) in zip(rves, cases):
        b.add(r, n)
    steps = 0
    while b.run(max_ticks=7):
        steps += 1
    assert steps > 2
    for r in rves:
        b.remove(r)
    b.close()
    for r, (c, n), rf in zip(rves, cases, ref):
        r.run(1)                       # one more increment, alone
        _same(_snapshot(r, n + 1), rf)
        r.close()


def test_profiled_ticks_equal_graph_ticks(voce_lib):
    """Profiling drives the ticks from the host with timed launches: same
    kernels, bit-identical results, and every phase timed."""
    cases = _cases()[:4]
    snaps = []
    for prof in (False, True):
        rves = [_make(c, capi.PREC_MIXED_NR32) for c, _ in cases]
        with capi.Batch(capi.PREC_MIXED_NR32) as b:
            for r, (c, n) in zip(rves, cases):
                b.add(r, n)
            if prof:
                b.set_profiling(True)
            while b.run(max_ticks=9):
                pass
            kt = b.kernel_times()
        snaps.append([_snapshot(r, n) for r, (c, n) in zip(rves, cases)])
        for r in rves:
            r.close()
        if prof:
            for k in ("fft_z_fwd", "fft_x_green", "nr", "finalize_iter", "incr_end"):
                assert kt[k][1] > 0 and kt[k][0] > 0.0, k
        else:
            assert all(n == 0 for _, n in kt.values())
    for a, b_ in zip(*snaps):
        _same(a, b_)


def test_removed_mid_increment_continues_alone_or_elsewhere(voce_lib):
    """Taken out of a batch in the middle of an increment, an RVE finishes
    that increment where it stopped: alone, or (through a snapshot) in
    another batch -- the same results as never having left."""
    cases = _cases()[:2]
    ref = []
    for c, n in cases:
        with _make(c, capi.PREC_FP64) as r:
            r.run(2)
            ref.append(_snapshot(r, 2))
    rves = [_make(c, capi.PREC_FP64) for c, _ in cases]
    with capi.Batch(capi.PREC_FP64) as b:
        for r in rves:
            b.add(r, 2)
        b.run(max_ticks=7)                   # both are mid-increment now
        for r in rves:
            assert r.increments_done == 0
            b.remove(r)
    rves[0].run(2)                           # the partial increment + one more
    _same(_snapshot(rves[0], 2), ref[0])
    blob = rves[1].snapshot()
    rves[1].close()
    r1 = capi.Rve.restore(blob)
    with capi.Batch(capi.PREC_FP64) as b2:
        b2.add(r1, 2)
        assert b2.run() == 0
    _same(_snapshot(r1, 2), ref[1])
    rves[0].close()
    r1.close()


def test_launch_wait_with_members_added_in_flight(voce_lib):
    """voce_batch_launch / voce_batch_wait: RVEs created and added while the
    batch's ticks run join at the next launch and give the same bits as
    alone; so do the members that were running."""
    prec = capi.PREC_MIXED_IR
    cases = _cases()[:4]
    alone = []
    for c, n in cases:
        with _make(c, prec) as r:
            r.run(n)
            alone.append(_snapshot(r, n))
    first = [_make(c, prec) for c, _ in cases[:2]]
    with capi.Batch(prec) as b:
        for r, (c, n) in zip(first, cases[:2]):
            b.add(r, n)
        b.launch(3)
        later = [_make(c, prec) for c, _ in cases[2:]]     # created while the ticks run
        for r, (c, n) in zip(later, cases[2:]):
            b.add(r, n)
        b.wait()
        for _ in range(10000):
            b.launch(4)
            if b.wait() == 0:
                break
        assert b.wait() == 0
    for r, (c, n), ref in zip(first + later, cases, alone):
        _same(_snapshot(r, n), ref)
        r.close()
