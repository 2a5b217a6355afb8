"""The single-precision line FFT of the spectrum passes.

voce_diag_fft runs one block of the FFT the passes run (the same device
function, on the same shared-memory layout) on given lines.  Every transform
candidate of every length the single-precision forms plan -- the register
FFT where the length has one, the Stockham radix orders -- is checked against
numpy's FFT of the same float-rounded input, both directions.  The
reference hands its transforms to FFTW (evolution.c:350-394), so the bar is
the accuracy of a single-precision FFT, not bits: the RMS error over the
RMS of the result within 1.5e-7 log2(L) (FP32 rounding is 6e-8 per
operation, a radix-2 FFT has log2(L) levels)."""
import math
import tempfile

import numpy as np
import pytest

from voce_gb300 import capi, synth

pytestmark = pytest.mark.gpu

REG = {16: [4, 4], 24: [4, 6], 32: [4, 8], 48: [6, 8], 64: [8, 8], 96: [8, 12],
       128: [8, 16], 192: [12, 16], 256: [16, 16]}


def _lines(L, n, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    x = rng.standard_normal((n, L)) + 1j * rng.standard_normal((n, L))
    return x.astype(np.complex64).astype(np.complex128)   # what the device reads


def _rel_rms(a, b):
    return math.sqrt(np.mean(np.abs(a - b) ** 2) / np.mean(np.abs(b) ** 2))


@pytest.mark.parametrize("L", [12, 16, 18, 24, 32, 36, 48, 64, 96, 128, 192, 256, 384])
def test_every_candidate_matches_numpy(voce_lib, L):
    n = max(1, min(40, (200 * 1024) // (16 * L) - 1))
    x = _lines(L, n, L)
    fwd, inv = np.fft.fft(x, axis=1), np.fft.ifft(x, axis=1) * L
    cands = capi.load().voce_fft_schedule_count(L) + (1 if L in REG else 0)
    assert cands >= 1
    tol = 1.5e-7 * math.log2(L)
    for k in range(cands):
        for sign, want in ((-1, fwd), (1, inv)):
            got = capi.diag_fft(x, sign, k)
            e = _rel_rms(got, want)
            assert e < tol, (L, k, sign, e)


def test_fft_probe_rejects_bad_arguments(voce_lib):
    x = _lines(20, 2, 1)
    with pytest.raises(capi.VoceError):
        capi.diag_fft(x)            # 20 is not 2^a 3^b
    with pytest.raises(capi.VoceError):
        capi.diag_fft(_lines(16, 2, 1), -1, 9)
    with pytest.raises(capi.VoceError):
        capi.diag_fft(_lines(256, 60, 1))   # 2 x 256 x 61 complex floats > 200 KB


def test_single_precision_rves_plan_the_register_fft(voce_lib):
    """A 24 x 32 x 48 RVE of the mixed form: the register FFT is candidate 0
    of every axis, before the Stockham orders (x: 4, y and z: 2); every
    candidate solves the increment to the same iteration count and to the
    form's single-precision agreement; a forced candidate survives a
    snapshot.  The FP64 form keeps the Stockham orders only."""
    case = synth.Case("fft_24_32_48", synth.voronoi_mesh_box((24, 32, 48), 10, 84),
                      synth.CU_LIKE, synth.tension_z(), 0.2, 1)
    nl = case.write(tempfile.mkdtemp(prefix="regfft_"))
    with capi.Rve.from_files(nl, capi.PREC_FP64) as r:
        assert [r.fft_schedule_count(a) for a in range(3)] == [4, 2, 2]
        assert r.fft_schedule(0) == [4, 2, 3]

    def run(axis=None, k=0):
        with capi.Rve.from_files(nl, capi.PREC_MIXED) as r:
            for a in range(3):
                r.set_fft_schedule(a, 0)
            if axis is not None:
                r.set_fft_schedule(axis, k)
            sched = [r.fft_schedule(a) for a in range(3)]
            r.run(1)
            return sched, r.increment(0), r.field("sig_voigt")

    with capi.Rve.from_files(nl, capi.PREC_MIXED) as r:
        counts = [r.fft_schedule_count(a) for a in range(3)]
    assert counts == [5, 3, 3]
    base = run()
    assert base[0] == [REG[24], REG[32], REG[48]]
    for axis, n in enumerate(counts):
        for k in range(1, n):
            sched, inc, sig = run(axis, k)
            assert sched[axis] != REG[(24, 32, 48)[axis]]
            assert inc["iters"] == base[1]["iters"]
            e = np.max(np.abs(sig - base[2])) / np.max(np.abs(base[2]))
            assert e < 1e-5, (axis, k, sched, e)
    with capi.Rve.from_files(nl, capi.PREC_MIXED) as r:
        r.set_fft_schedule(1, 2)
        want = r.fft_schedule(1)
        with capi.Rve.restore(r.snapshot()) as q:
            assert q.fft_schedule(1) == want
            q.set_fft_schedule(2, 1)      # a restored RVE keeps its tiles and other axes
            assert q.fft_schedule(1) == want
            assert q.tiles() == r.tiles()
