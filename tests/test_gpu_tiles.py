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
