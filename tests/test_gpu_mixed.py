"""The mixed-precision forms against the reference's own macro curve and
fields (golden fixtures) and against the FP64 form on the GPU:
VOCE_PREC_MIXED (FP32 spectrum and Green operator, FP64 Newton, hardening,
norms and averages), VOCE_PREC_MIXED_IR (the same with the Newton correction
-- Jacobian and LDL^T solve -- in FP32, the residual, flow rule, stop test and
norms in FP64) and VOCE_PREC_MIXED_NR32 (FP32 Newton iterations ended by an
FP64-residual acceptance step).

Bounds: the macro stress / strain / strain-rate averages of every increment
within 1e-4 relative (the bound the mixed form is held to); per-voxel stress
and strain rate within 1e-3 relative, norm-wise; Green-iteration counts
within 10 % of the reference's."""
import tempfile

import numpy as np
import pytest

import golden_io as gio
import make_golden
from voce_gb300 import capi, synth

pytestmark = pytest.mark.gpu

MACRO_TOL = 1e-4
FIELD_TOL = 1e-3
CASES = ["vor8_tension", "vor8_psc", "vor8_gas", "vor8_creep", "vor8_noupd", "vor12_mix",
         "cfg1_16", "cfg2_64"]


def _write(case):
    return case.write(tempfile.mkdtemp(prefix="mixed_"))


FORMS = [capi.PREC_MIXED, capi.PREC_MIXED_IR, capi.PREC_MIXED_NR32]


@pytest.mark.parametrize("prec", FORMS)
@pytest.mark.parametrize("name", CASES)
def test_mixed_matches_reference_macro_curve(name, prec, voce_lib):
    if not gio.available(name):
        pytest.skip("fixture not generated")
    make, n, _ = make_golden.CASES[name]
    case = make()
    fx = gio.load(name)
    assert case.mesh.digest() == str(fx["digest"])
    seg = gio.segment(fx, case.update_flag)
    nv = case.mesh.nvox
    with capi.Rve.from_files(_write(case), prec) as r:
        r.run(n)
        worst = 0.0
        for k in range(n):
            inc = r.increment(k)
            ref = seg["incr"][k]
            n_ref = len(ref["its"])
            assert abs(inc["iters"] - n_ref) <= max(2, 0.1 * n_ref), (k, inc["iters"], n_ref)
            e = gio.rel(np.array(inc["sig_avg"]) * nv, ref["its"][-1]["sig"].ravel())
            worst = max(worst, e)
            assert e < MACRO_TOL, (k, e)
            assert gio.rel(np.array(inc["eps_avg"]) * nv, ref["eps"].ravel()) < MACRO_TOL
            assert gio.rel(np.array(inc["edot_avg"]) * nv, ref["edot"].ravel()) < MACRO_TOL
        sig = r.field("sig_voigt").T
        edot = r.field("edot_voigt").T
    if "sample_idx" in fx:
        idx = fx["sample_idx"]
        sig, edot = sig[idx], edot[idx]
    assert gio.rel(sig, fx["sig"]) < FIELD_TOL
    assert gio.rel(edot, fx["edot"]) < FIELD_TOL
    print(name, prec, "worst macro rel", worst)


@pytest.mark.parametrize("prec", FORMS)
def test_mixed_vs_fp64_random_load(prec, voce_lib):
    rng = np.random.Generator(np.random.PCG64(77))
    case = synth.small_case(24, 30, 77, n_steps=3, load=synth.random_traceless_load(rng))
    out = {}
    for p in (capi.PREC_FP64, prec):
        with capi.Rve.from_files(_write(case), p) as r:
            r.run(3)
            out[p] = ([r.increment(k) for k in range(3)], r.field("sig_voigt"),
                         r.field("edot_voigt"), r.field("crss"))
    (i64, s64, e64, c64), (i32, s32, e32, c32) = out[capi.PREC_FP64], out[prec]
    for a, b in zip(i32, i64):
        assert gio.rel(np.array(a["sig_avg"]), np.array(b["sig_avg"])) < MACRO_TOL
        assert abs(a["iters"] - b["iters"]) <= max(2, 0.1 * b["iters"])
    assert gio.rel(s32, s64) < FIELD_TOL
    assert gio.rel(e32, e64) < FIELD_TOL
    assert gio.rel(c32, c64) < FIELD_TOL


@pytest.mark.parametrize("name", ["vor8_psc", "vor12_mix", "cfg1_16"])
def test_mixed_chord_steps_against_exact_jacobian(name, voce_lib):
    """VOCE_PREC_MIXED with chord steps in its FP64 Newton (the default) and
    with the Jacobian refreshed every step: the Green-iteration counts agree
    within one, macro averages within 1e-7 and fields within 1e-6, far inside
    the form's bounds; both stay within them against the reference."""
    make, n, _ = make_golden.CASES[name]
    case = make()
    nl = _write(case)
    lib = capi.load()
    lib.voce_set_newton_chord(0)
    try:
        with capi.Rve.from_files(nl, capi.PREC_MIXED) as r:
            r.run(n)
            exact = ([r.increment(k) for k in range(n)], r.field("sig_voigt"), r.field("edot_voigt"))
    finally:
        lib.voce_set_newton_chord(1)
    with capi.Rve.from_files(nl, capi.PREC_MIXED) as r:
        r.run(n)
        chord = ([r.increment(k) for k in range(n)], r.field("sig_voigt"), r.field("edot_voigt"))
    fx = gio.load(name)
    seg = gio.segment(fx, case.update_flag)
    nv = case.mesh.nvox
    for k, (a, b) in enumerate(zip(chord[0], exact[0])):
        assert abs(a["iters"] - b["iters"]) <= 1
        assert gio.rel(a["sig_avg"], b["sig_avg"]) < 1e-7
        ref = seg["incr"][k]
        assert gio.rel(np.array(a["sig_avg"]) * nv, ref["its"][-1]["sig"].ravel()) < MACRO_TOL
    assert gio.rel(chord[1], exact[1]) < 1e-6
    assert gio.rel(chord[2], exact[2]) < 1e-6


@pytest.mark.parametrize("pred", [0, 1])
@pytest.mark.parametrize("name", ["vor8_psc", "vor12_mix", "cfg1_16"])
def test_float_jacobian_converges_to_the_fp64_residual_root(name, pred, voce_lib):
    """VOCE_PREC_MIXED_IR (with and without its FP32-pipe start) against
    VOCE_PREC_MIXED with the exact FP64 Jacobian (chord steps off): both drive
    the same FP64 residual to its root under the same stop test, so they
    differ only by where each stops (updates below 1e-7 relative): macro
    averages within 1e-7, stress fields within 1e-6, Green-iteration counts
    within one.  The strain rate is evaluated at the stress before the last
    Newton update (evolution.c:67), which lies up to the stop tolerance from
    the root; through the n = 20 power law that moves it by up to ~2e-6, so
    strain-rate fields are held to 1e-5."""
    make, n, _ = make_golden.CASES[name]
    case = make()
    nl = _write(case)
    lib = capi.load()
    lib.voce_set_newton_chord(0)
    try:
        with capi.Rve.from_files(nl, capi.PREC_MIXED) as r:
            r.run(n)
            exact = ([r.increment(k) for k in range(n)], r.field("sig_voigt"), r.field("edot_voigt"))
    finally:
        lib.voce_set_newton_chord(1)
    lib.voce_set_ir_predictor(pred)
    try:
        with capi.Rve.from_files(nl, capi.PREC_MIXED_IR) as r:
            r.run(n)
            ir = ([r.increment(k) for k in range(n)], r.field("sig_voigt"), r.field("edot_voigt"))
    finally:
        lib.voce_set_ir_predictor(1)
    for a, b in zip(ir[0], exact[0]):
        assert abs(a["iters"] - b["iters"]) <= 1
        assert gio.rel(a["sig_avg"], b["sig_avg"]) < 1e-7
    assert gio.rel(ir[1], exact[1]) < 1e-6
    assert gio.rel(ir[2], exact[2]) < 1e-5
