"""voce_rve_get_field_noalloc (include/voce_gpu.h), the field download that
stages in the library's fixed device array instead of allocating: through the
C ABI it returns what voce_rve_get_field returns, call after call, and it
refuses fields larger than the array.  The file name makes pytest collect it
last, after the tests that allocate; it also passes alone in a new process,
where its first call does the per-device set-up."""
import os
import tempfile

import numpy as np
import pytest

from voce_gb300 import capi, synth

pytestmark = pytest.mark.gpu

# the bound the parity tests hold fields to (the staged values are expected to
# be the same doubles)
FIELD_TOL = 1e-9


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _case_dir(case):
    return case.write(tempfile.mkdtemp(prefix="noalloc_"))


def test_noalloc_matches_get_field_on_consecutive_calls():
    case = synth.small_case(16, 8, 41, n_steps=3)
    with capi.Rve.from_files(_case_dir(case), capi.PREC_FP64) as r:
        r.run(2)
        sig_a = r.field("sig_voigt")
        # call 1 and call 2 back to back, of different widths
        got1 = r.field_noalloc("sig_voigt")
        got2 = r.field_noalloc("svm")
        assert got1.shape == sig_a.shape and got2.shape == (r.nv, 1)
        assert _rel(got1, sig_a) <= FIELD_TOL
        assert _rel(got2, r.field("svm")) <= FIELD_TOL
        # one more increment: the array's earlier contents must not show
        r.run(1)
        sig_b = r.field("sig_voigt")
        assert _rel(sig_b, sig_a) > 1e-6
        for name in ("sig_voigt", "crss", "tranmat", "edot_voigt", "gamacum"):
            assert _rel(r.field_noalloc(name), r.field(name)) <= FIELD_TOL, name


def test_noalloc_mixed_precision_and_second_rve():
    # a second RVE of another size, and the mixed form, after the first
    case = synth.small_case(24, 12, 42, n_steps=1, load=synth.plane_strain_compression())
    with capi.Rve.from_files(_case_dir(case), capi.PREC_MIXED) as r:
        r.run(1)
        for name in ("edot_voigt", "evm"):
            a = r.field_noalloc(name)
            b = r.field_noalloc(name)
            ref = r.field(name)
            assert _rel(a, ref) <= FIELD_TOL and _rel(b, ref) <= FIELD_TOL, name


def test_noalloc_rejects_fields_beyond_the_array():
    case = synth.small_case(8, 2, 43, n_steps=1)
    nl_path = _case_dir(case)
    nl = capi.read_namelist(nl_path)
    dims = (64, 64, 128)
    nl.CellDim[0], nl.CellDim[1], nl.CellDim[2] = dims
    slip = capi.read_slip(os.path.join(os.path.dirname(nl_path), "mat.sx"))
    nv = int(np.prod(dims))
    rng = np.random.Generator(np.random.PCG64(7))
    eul = np.repeat(synth.so3_uniform_bunge(rng, 4), nv // 4, axis=0)
    grain = np.repeat(np.arange(1, 5, dtype=np.int32), nv // 4)
    phase = np.ones(nv, dtype=np.int32)
    with capi.Rve.create(nl, slip, eul, grain, phase, capi.PREC_FP64) as r:
        assert 12 * nv > capi.NOALLOC_MAX_DOUBLES >= nv
        with pytest.raises(capi.VoceError) as ei:
            r.field_noalloc("crss")
        assert ei.value.code == 6 and "no-allocation" in str(ei.value)
        # a 1-wide field of the same RVE fits, and the refusal left no trace
        assert _rel(r.field_noalloc("svm"), r.field("svm")) <= FIELD_TOL
