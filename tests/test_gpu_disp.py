"""The displacement fluctuation (VOCE_FIELD_DISP_FLUCT, include/voce_gpu.h),
the corrected form of the reference's displacement_fluct (evolution.c:532-560),
and the new_position dumps written from it.

* Against the oracle (oracle_disp_fluct: the reference's loops with per-voxel
  accumulators and the 1/|xi|^2 weight, on the oracle's own accumulated
  `fluctuation`) on the same inputs, within the parity bound 1e-9 relative to
  the field's largest magnitude.  The oracle's fluctuation is pinned to the
  reference's own new_position output in test_oracle.py.
* Against the numpy form applied to the GPU's own DisGrad, to 1e-12: the
  transform chain alone (r2c, Hermitian half spectrum, Nyquist handling).
* The mixed forms (single-precision spectrum) against FP64 within 1e-4.

Shapes: 4x6x8 (radix 3, a Nyquist index on every even axis), 8^3 with a gas
phase, 12^3 under shear, 16^3 with one grain per voxel; creep resets DisGrad
every increment, so there the reference is the oracle's DisGrad form."""
import os
import tempfile

import numpy as np
import pytest

import make_golden
import make_outputs
import oracle
from voce_gb300 import capi

pytestmark = pytest.mark.gpu

PARITY_TOL = 1e-9
TRANSFORM_TOL = 1e-12
MIXED_TOL = 1e-4

CASES = {
    # name: (case constructor, increments, oracle input: accumulated fluctuation or DisGrad)
    "tex_4x6x8": (make_outputs.tex_case, 3, True),
    "vor8_gas": (make_golden.CASES["vor8_gas"][0], 4, True),
    "vor12_mix": (make_golden.CASES["vor12_mix"][0], 4, True),
    "cfg1_16": (make_golden.CASES["cfg1_16"][0], 3, True),
    "vor8_creep": (make_golden.CASES["vor8_creep"][0], 4, False),
}


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _inputs(case):
    return case.write(tempfile.mkdtemp(prefix="disp_"))


@pytest.mark.parametrize("name", sorted(CASES))
def test_disp_fluct_matches_the_oracle(name, voce_lib, oracle_lib):
    make, n, from_fluct = CASES[name]
    case = make()
    nl = _inputs(case)
    job = oracle.Job(nl)
    job.run(n)
    want = job.disp_fluct(from_fluct)
    job.close()
    with capi.Rve.from_files(nl) as r:
        r.run(n)
        got = r.field("disp_fluct")
        dg = r.field("disgrad")
        again = r.field("disp_fluct")
    assert got.shape == want.shape
    assert np.max(np.abs(want)) > 0.0
    e = _rel(got, want)
    assert e <= PARITY_TOL, (name, e)
    t = _rel(got, oracle.disp_fluct_np(dg, case.mesh.dims))
    assert t <= TRANSFORM_TOL, (name, t)
    # the field is computed from the state and leaves it unchanged
    assert np.array_equal(got, again)
    print(name, "oracle", e, "transform", t)


def test_disp_fluct_leaves_the_solve_unchanged(voce_lib):
    """Asking for the field between increments does not change what follows."""
    case = make_golden.CASES["vor12_mix"][0]()
    nl = _inputs(case)
    with capi.Rve.from_files(nl) as a, capi.Rve.from_files(nl) as b:
        a.run(2)
        b.run(2)
        b.field("disp_fluct")
        a.run(2)
        b.run(2)
        assert np.array_equal(a.field("sig"), b.field("sig"))
        assert np.array_equal(a.field("disp_fluct"), b.field("disp_fluct"))


@pytest.mark.parametrize("prec", [capi.PREC_MIXED, capi.PREC_MIXED_NR32])
def test_disp_fluct_mixed_forms(prec, voce_lib):
    case = make_golden.CASES["vor12_mix"][0]()
    nl = _inputs(case)
    with capi.Rve.from_files(nl) as r64, capi.Rve.from_files(nl, prec) as r32:
        r64.run(3)
        r32.run(3)
        e = _rel(r32.field("disp_fluct"), r64.field("disp_fluct"))
    assert e <= MIXED_TOL, e


def test_new_position_dumps_hold_the_displacement(voce_lib, oracle_lib):
    case = make_outputs.tex_case()
    d = tempfile.mkdtemp(prefix="newpos_")
    nl = case.write(d, print_control=make_outputs.PRINT_CONTROL, tex_flag=make_outputs.TEX_FLAG)
    job = oracle.Job(nl)
    job.run(3)
    want = job.disp_fluct(True)
    job.close()
    with capi.Rve.from_files(nl) as r:
        r.run(3)
        r.write_iout("new_position", os.path.join(d, "new_position"), 3)
    data = np.fromfile(os.path.join(d, "new_position_S0003.iout"), "<f8")
    assert data.size == 3 * case.mesh.nvox
    assert _rel(data.reshape(-1, 3), want) <= PARITY_TOL
