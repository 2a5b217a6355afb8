"""FFT tiles (lines per block) never change results: the tuned tiles, the
fixed-budget ones and forced extreme ones give bit-identical increments,
in the FP64 and the single-precision-spectrum forms."""
import tempfile

import numpy as np
import pytest

from voce_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def _run(nl, prec, tiles=None):
    with capi.Rve.from_files(nl, prec) as r:
        if tiles is not None:
            r.set_tiles(tiles)
        used = r.tiles()
        r.run(2)
        return used, [r.increment(k) for k in range(2)], r.field("sig_voigt"), r.field("disgrad")


@pytest.mark.parametrize("prec", [capi.PREC_FP64, capi.PREC_MIXED_NR32])
def test_tiles_do_not_change_results(prec, voce_lib):
    rng = np.random.Generator(np.random.PCG64(81))
    case = synth.small_case(16, 10, 81, n_steps=2, load=synth.random_traceless_load(rng))
    nl = case.write(tempfile.mkdtemp(prefix="tiles_"))
    tuned = _run(nl, prec)
    smallest = _run(nl, prec, [1, 1, 1, 1, 1, 1])
    largest = _run(nl, prec, [4, 4, 2, 4, 4, 4])
    assert smallest[0] == [1, 1, 1, 1, 1, 1] and largest[0] == [4, 4, 2, 4, 4, 4]
    for other in (smallest, largest):
        assert other[1] == tuned[1]
        assert np.array_equal(other[2], tuned[2]) and np.array_equal(other[3], tuned[3])


def test_tuning_can_be_switched_off(voce_lib):
    case = synth.small_case(8, 4, 82, n_steps=1)
    nl = case.write(tempfile.mkdtemp(prefix="tiles_"))
    lib = capi.load()
    lib.voce_set_autotune(0)
    try:
        with capi.Rve.from_files(nl) as r:
            t = r.tiles()
    finally:
        lib.voce_set_autotune(1)
    assert all(x >= 1 for x in t)
    with capi.Rve.from_files(nl) as r:
        with pytest.raises(capi.VoceError):
            r.set_tiles([3, 1, 1, 1, 1, 1])      # 3 does not divide 8


def test_tile_cache_file_is_shared_between_processes(voce_lib):
    """VOCE_TILE_CACHE: the first process records its tuned tiles, a second
    one (with tuning timings that could differ, e.g. under a profiler) reads
    and uses them."""
    import os
    import subprocess
    import sys
    case = synth.small_case(12, 6, 83, n_steps=1)
    nl = case.write(tempfile.mkdtemp(prefix="tiles_"))
    cache = os.path.join(tempfile.mkdtemp(prefix="tilecache_"), "tiles.txt")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    prog = ("import sys; sys.path.insert(0, %r)\n"
            "from voce_gb300 import capi\n"
            "r = capi.Rve.from_files(%r)\n"
            "print(','.join(map(str, r.tiles())))\n" % (root, nl))
    env = dict(os.environ, VOCE_TILE_CACHE=cache)
    a = subprocess.run([sys.executable, "-c", prog], env=env, capture_output=True, text=True, check=True)
    lines = open(cache).read().split("\n")
    assert lines[0].startswith("12 12 12 0 ")
    # the second process finds the shape in the file: no new line, same tiles
    b = subprocess.run([sys.executable, "-c", prog], env=env, capture_output=True, text=True, check=True)
    assert a.stdout == b.stdout
    assert open(cache).read().count("\n") == 1


def _box_case(dims, seed):
    return synth.Case("box_%d_%d_%d" % tuple(dims), synth.voronoi_mesh_box(dims, 10, seed),
                      synth.CU_LIKE, synth.tension_z(), 0.2, 1)


def test_fft_schedules_agree_and_stay_with_the_rve(voce_lib):
    """Every radix schedule of a 24 x 32 x 48 grid (x: 4 candidates, y and z:
    2 each) gives the default's increment to rounding: the same iteration
    count, stress within 1e-12.  A forced schedule survives a snapshot and
    joins a batch unchanged (the batch member's increment is bit-identical to
    the lone run with that schedule)."""
    case = _box_case((24, 32, 48), 84)
    nl = case.write(tempfile.mkdtemp(prefix="sched_"))
    lib = capi.load()
    counts = [lib.voce_fft_schedule_count(n) for n in (24, 32, 48)]
    assert counts == [4, 2, 2]

    def run(axis=None, k=0):
        with capi.Rve.from_files(nl) as r:
            if axis is not None:
                r.set_fft_schedule(axis, k)
            sched = [r.fft_schedule(a) for a in range(3)]
            r.run(1)
            return sched, r.increment(0), r.field("sig_voigt")

    with capi.Rve.from_files(nl) as r:
        for a in range(3):
            r.set_fft_schedule(a, 0)
        r.run(1)
        base = r.increment(0), r.field("sig_voigt")
    seen = set()
    for axis, n in enumerate(counts):
        for k in range(n):
            sched, inc, sig = run(axis, k)
            seen.add(tuple(sched[axis]))
            assert inc["iters"] == base[0]["iters"]
            e = np.max(np.abs(sig - base[1])) / np.max(np.abs(base[1]))
            assert e < 1e-12, (axis, k, sched, e)
    assert len(seen) == sum(counts)
    # a forced schedule is part of the RVE: snapshot and batch keep it
    with capi.Rve.from_files(nl) as r:
        r.set_fft_schedule(0, 2)
        want = r.fft_schedule(0)
        assert want == [2, 4, 3]
        blob = r.snapshot()
        with capi.Rve.restore(blob) as q:
            assert q.fft_schedule(0) == want
        alone = run(0, 2)
        with capi.Batch() as b:
            b.add(r, 1)
            b.run()
        assert r.fft_schedule(0) == want
        assert r.increment(0) == alone[1]
        assert np.array_equal(r.field("sig_voigt"), alone[2])
    with capi.Rve.from_files(nl) as r:
        with pytest.raises(capi.VoceError):
            r.set_fft_schedule(1, 2)   # 32 has two candidates
