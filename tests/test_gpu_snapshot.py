"""RVE snapshot / restore (include/voce_gpu.h): a restored handle continues
exactly as the original, bit for bit, in every precision form, from memory
and from a file, alone and inside a batch."""
import os
import tempfile

import numpy as np
import pytest

from voce_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def _case(seed, n=16, grains=12):
    rng = np.random.Generator(np.random.PCG64(seed))
    c = synth.small_case(n, grains, seed, n_steps=6, load=synth.random_traceless_load(rng))
    return c.write(tempfile.mkdtemp(prefix="snap_"))


def _state(r, ks):
    return ([r.increment(k) for k in ks], [r.iter_detail(k) for k in ks],
            r.field("sig_voigt"), r.field("edot_voigt"), r.field("crss"), r.field("tranmat"),
            r.field("disgrad"), r.field("gammatotal"))


def _same(a, b):
    ia, la, *fa = a
    ib, lb, *fb = b
    assert ia == ib
    # the per-iteration log (err.out's lines) of every increment
    assert len(la) == len(lb)
    for x, y in zip(la, lb):
        assert np.array_equal(x, y)
    for x, y in zip(fa, fb):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("prec", [capi.PREC_FP64, capi.PREC_MIXED, capi.PREC_MIXED_NR32, capi.PREC_MIXED_IR])
def test_restore_continues_bit_for_bit(prec, voce_lib):
    nl = _case(71)
    with capi.Rve.from_files(nl, prec) as r:
        r.run(2)
        blob = r.snapshot()
        r.run(2)
        want = _state(r, range(4))
    with capi.Rve.restore(blob) as r2:
        assert r2.increments_done == 2
        r2.run(2)
        _same(_state(r2, range(4)), want)


@pytest.mark.parametrize("prec", [capi.PREC_MIXED_IR, capi.PREC_FP64])
def test_restore_in_the_middle_of_an_increment(prec, voce_lib):
    """Taken out of a batch in the middle of an increment and restored from a
    snapshot, an RVE finishes the increment as if it had never stopped (the
    in-increment state: stress, displacement gradient, antisymmetric sum,
    macro state and iteration count)."""
    nl = _case(73)
    with capi.Rve.from_files(nl, prec) as r:
        r.run(2)
        want = _state(r, range(2))
        first = r.increment(0)["iters"]
    assert first > 12
    r = capi.Rve.from_files(nl, prec)
    with capi.Batch(prec) as b:
        b.add(r, 2)
        b.run(first // 2)                   # stops inside the first increment
        b.remove(r)
    assert r.increments_done == 0
    blob = r.snapshot()
    r.close()
    with capi.Rve.restore(blob) as r2:
        r2.run(2)                           # the increment in progress counts as the first
        _same(_state(r2, range(2)), want)


def test_save_load_file_and_join_batch(voce_lib):
    nl = _case(72, n=12, grains=8)
    nl2 = _case(73, n=8, grains=5)
    path = os.path.join(tempfile.mkdtemp(prefix="snapf_"), "rve.snap")
    with capi.Rve.from_files(nl) as r:
        r.run(1)
        r.save(path)
        r.run(3)
        want = _state(r, range(4))
    # the restored RVE finishes its increments inside a batch with another RVE
    r2 = capi.Rve.restore_file(path)
    other = capi.Rve.from_files(nl2)
    with capi.Batch(capi.PREC_FP64) as b:
        b.add(r2, 3)
        b.add(other, 2)
        assert b.run() == 0
    _same(_state(r2, range(4)), want)
    r2.close()
    other.close()


def test_snapshot_refused_inside_a_batch_and_damaged_blobs(voce_lib):
    nl = _case(74, n=8, grains=4)
    with capi.Rve.from_files(nl) as r, capi.Batch(capi.PREC_FP64) as b:
        b.add(r, 1)
        with pytest.raises(capi.VoceError) as ei:
            r.snapshot()
        assert ei.value.code == 9
        b.remove(r)
        blob = r.snapshot()
    with pytest.raises(capi.VoceError) as ei:
        capi.Rve.restore(blob[:-8])
    assert ei.value.code == 3


def test_restore_refuses_edited_descriptors_and_counters(voce_lib):
    """A snapshot whose descriptor or index-bearing state was changed is
    refused on the host (ERR_PARSE) before anything reaches the GPU: the
    precision, the work split, a grid edge, a phase id, the increment
    counter.  The intact snapshot then restores and continues bit for bit.
    The offsets follow this build's layout: a 64-byte header (macro-state
    size at 16, precision at 28, work split at 32, total at 56), the RVE
    descriptor from 64 (nx first), and the device state last (..., phase ids,
    the antisymmetric sum, the macro state)."""
    import struct
    n = 8
    nl = _case(75, n=n, grains=4)
    with capi.Rve.from_files(nl, capi.PREC_FP64) as r:
        r.run(1)
        blob = r.snapshot()
        r.run(1)
        want = _state(r, range(2))
    assert blob[:8] == b"VOCESNAP"
    macro_size, = struct.unpack_from("<I", blob, 16)
    total, = struct.unpack_from("<q", blob, 56)
    assert total == len(blob)
    assert struct.unpack_from("<iii", blob, 64) == (n, n, n)
    nv, nspec = n ** 3, (n // 2 + 1) * n * n
    # last: the log rows of the increment in progress, 12 doubles an iteration
    macro_at = total - 12 * 8 * capi.read_namelist(nl).IterMax - macro_size
    phase_at = macro_at - 3 * nspec * 16 - 4 * nv
    assert struct.unpack_from("<i", blob, phase_at)[0] in (1, 2)
    # istep follows 119 doubles and the ints iter, iter_total of the macro state
    istep_at = macro_at + 8 * 119 + 8
    assert struct.unpack_from("<i", blob, istep_at)[0] >= 1
    for at, value, what in ((28, 3, "precision"), (32, 1 << 30, "work split"),
                            (64, 2 * n, "grid"), (phase_at, 9, "phase id"),
                            (istep_at, 0, "counter")):
        bad = bytearray(blob)
        struct.pack_into("<i", bad, at, value)
        with pytest.raises(capi.VoceError) as ei:
            capi.Rve.restore(bytes(bad))
        assert ei.value.code == 3 and "damaged snapshot" in str(ei.value) and what in str(ei.value), str(ei.value)
    with capi.Rve.restore(blob) as r2:
        r2.run(1)
        _same(_state(r2, range(2)), want)


def test_batch_growing_the_record_ring_in_the_middle_of_an_increment(voce_lib):
    """An RVE taken out of a batch in the middle of an increment and added
    again for more increments than its record ring holds (the ring grows)
    keeps the log rows of the iterations it has run: the increment's record
    and err.out lines equal those of an uninterrupted run."""
    nl = _case(76, n=8, grains=4)
    with capi.Rve.from_files(nl) as r:
        r.run(1)
        want = _state(r, range(1))
        first = r.increment(0)["iters"]
    assert first > 12
    with capi.Rve.from_files(nl) as r:
        with capi.Batch(capi.PREC_FP64) as b:
            b.add(r, 1)
            b.run(first // 2)               # stops inside the first increment
            b.remove(r)
            assert r.increments_done == 0
            b.add(r, 40)                    # more than the 32 records the ring starts with
            for _ in range(first):
                if r.increments_done >= 1:
                    break
                b.run(8)
            assert r.increments_done >= 1
            b.remove(r)
        got = _state(r, range(1))
    # the fields have moved on into the next increment; the record and the log
    # of the first increment are compared
    assert got[0] == want[0]
    assert len(got[1]) == 1 and np.array_equal(got[1][0], want[1][0])
