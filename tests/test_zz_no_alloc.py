"""voce_rve_get_field_noalloc (include/voce_gpu.h), the field download that
stages in the library's fixed device array instead of allocating.  Through
the C ABI it returns exactly what voce_rve_get_field returns (both run the
same field kernel, so the doubles are the same bits), call after call; it
takes no device memory (free device memory is unchanged across its calls on
an RVE that never allocated a download buffer); and it refuses fields larger
than the array.  The file name makes pytest collect it last, after the tests
that allocate; it also passes alone in a new process, where its first call
does the per-device set-up."""
import os
import tempfile

import numpy as np
import pytest

from voce_gb300 import capi, synth

pytestmark = pytest.mark.gpu


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
        assert np.array_equal(got1, sig_a)
        assert np.array_equal(got2, r.field("svm"))
        # one more increment: the array's earlier contents must not show
        r.run(1)
        sig_b = r.field("sig_voigt")
        assert not np.array_equal(sig_b, sig_a)
        for name in ("sig_voigt", "crss", "tranmat", "edot_voigt", "gamacum"):
            assert np.array_equal(r.field_noalloc(name), r.field(name)), name


def test_noalloc_takes_no_device_memory():
    """A 48^3 RVE that has never downloaded a field: voce_rve_get_field would
    allocate a 10.6 MB staging buffer on its first call; two no-allocation
    calls leave the free device memory as it was.  The allocating call that
    follows shows that the measurement sees such a buffer."""
    case = synth.small_case(48, 20, 44, n_steps=1)
    nl = _case_dir(case)
    with capi.Rve.from_files(nl, capi.PREC_FP64) as warm:
        warm.field_noalloc("svm")            # per-device set-up of the library's array
        with capi.Rve.from_files(nl, capi.PREC_FP64) as r:
            r.run(1)
            free0, _ = capi.device_memory()
            a = r.field_noalloc("sig_voigt")
            b = r.field_noalloc("edot_voigt")
            free1, _ = capi.device_memory()
            assert free1 == free0, (free0, free1)
            assert np.array_equal(a, r.field("sig_voigt"))   # allocates its buffer
            free2, _ = capi.device_memory()
            assert free2 < free1
            assert np.array_equal(b, r.field("edot_voigt"))


def test_noalloc_mixed_precision_and_second_rve():
    # a second RVE of another size, and the mixed form, after the first
    case = synth.small_case(24, 12, 42, n_steps=1, load=synth.plane_strain_compression())
    with capi.Rve.from_files(_case_dir(case), capi.PREC_MIXED) as r:
        r.run(1)
        for name in ("edot_voigt", "evm"):
            a = r.field_noalloc(name)
            b = r.field_noalloc(name)
            ref = r.field(name)
            assert np.array_equal(a, ref) and np.array_equal(b, ref), name


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
        assert np.array_equal(r.field_noalloc("svm"), r.field("svm"))
