"""GPU parity: libvoce_gpu.so, called through its C ABI, against the
reference's own outputs (golden fixtures) and against the oracle on inputs
the fixtures do not cover.  Tolerance: 1e-9 relative, norm-wise (max |a-b| /
max |b| over a field or a curve), the bound the plain FP64 path is held to;
Green-iteration counts must match exactly."""
import os
import tempfile

import numpy as np
import pytest

import golden_io as gio
import make_golden
from voce_gb300 import capi, synth

pytestmark = pytest.mark.gpu

TOL = 1e-9
SMALL = ["vor8_tension", "vor8_psc", "vor8_gas", "vor8_creep", "vor8_noupd", "vor12_mix",
         "cfg1_16"]


def _write(case):
    d = tempfile.mkdtemp(prefix="gpu_")
    return case.write(d)


def _check_against_fixture(name, r, case, n):
    fx = gio.load(name)
    seg = gio.segment(fx, case.update_flag)
    nv = case.mesh.nvox
    for k in range(n):
        inc = r.increment(k)
        ref = seg["incr"][k]
        assert inc["iters"] == len(ref["its"]), (k, inc["iters"], len(ref["its"]))
        det = r.iter_detail(k)
        sums_e = np.array([it["sum_e"] for it in ref["its"]])
        sums_s = np.array([it["sum_s"] for it in ref["its"]])
        assert gio.rel(det[:, 4], sums_e) < TOL
        assert gio.rel(det[:, 5], sums_s) < TOL
        sig_ref = np.array([it["sig"] for it in ref["its"]])
        sig_gpu = np.array([gio.b6_to_tensor(row[6:12]) for row in det])
        assert gio.rel(sig_gpu, sig_ref) < TOL
        assert gio.rel(np.array(inc["eps_avg"]) * nv, ref["eps"].ravel()) < TOL
        assert gio.rel(np.array(inc["edot_avg"]) * nv, ref["edot"].ravel()) < TOL
        if ref["rot"] is not None:
            assert gio.rel([inc["rot_slip_avg"], inc["rot_loc_avg"]], ref["rot"]) < TOL
    sig = r.field("sig_voigt").T
    edot = r.field("edot_voigt").T
    if "sample_idx" in fx:
        idx = fx["sample_idx"]
        assert gio.rel(sig[idx], fx["sig"]) < TOL
        assert gio.rel(edot[idx], fx["edot"]) < TOL
        for f, st in ((sig, fx["sig_stats"]), (edot, fx["edot_stats"])):
            assert gio.rel(np.abs(f).max(0), st[2]) < TOL
            assert gio.rel((f ** 2).sum(0), st[1]) < 1e-8
    else:
        assert gio.rel(sig, fx["sig"]) < TOL
        assert gio.rel(edot, fx["edot"]) < TOL


@pytest.mark.parametrize("name", SMALL)
def test_gpu_matches_reference_fixture(name, voce_lib):
    make, n, _ = make_golden.CASES[name]
    case = make()
    fx = gio.load(name)
    assert case.mesh.digest() == str(fx["digest"])
    with capi.Rve.from_files(_write(case)) as r:
        r.run(n)
        _check_against_fixture(name, r, case, n)


def test_gpu_matches_reference_64cubed(voce_lib):
    """Config 2 (64^3, 125 Voronoi grains, tension): the reference's first
    increments, sampled voxels and whole-field statistics."""
    if not gio.available("cfg2_64"):
        pytest.skip("fixture not generated")
    make, n, _ = make_golden.CASES["cfg2_64"]
    case = make()
    assert case.mesh.digest() == str(gio.load("cfg2_64")["digest"])
    with capi.Rve.from_files(_write(case)) as r:
        r.run(n)
        _check_against_fixture("cfg2_64", r, case, n)


def _vs_oracle(case, n, threads=16):
    import oracle as orc
    nl = _write(case)
    with capi.Rve.from_files(nl) as r:
        r.run(n)
        g = [r.increment(k) for k in range(n)]
        gf = {k: r.field(k) for k in ("sig", "edot", "eps", "disgrad", "tranmat", "crss", "gamacum")}
    o = orc.Job(nl, threads=threads)
    o.run(n)
    oi = [o.increment(k) for k in range(n)]
    for a, b in zip(g, oi):
        assert a["iters"] == b["iters"]
        assert gio.rel(a["sig_avg"], b["sig_avg"]) < TOL
        assert abs(a["s_vm"] - b["s_vm"]) < TOL * abs(b["s_vm"])
        assert abs(a["evmp"] - b["evmp"]) < TOL * abs(b["evmp"])
    for k, f in gf.items():
        assert gio.rel(f, o.field(k)) < TOL, k
    o.close()


def test_gpu_vs_oracle_anisotropic_grid(voce_lib):
    """Unequal edges (16 x 12 x 8), so x, y and z transforms all differ."""
    m = synth.voronoi_mesh(8, 5, 61)
    nx, ny, nz = 16, 12, 8
    rng = np.random.Generator(np.random.PCG64(61))
    seeds = rng.random((7, 3))
    g = [(np.arange(k) + 0.5) / k for k in (nx, ny, nz)]
    pts = np.stack(np.meshgrid(*g, indexing="ij"), -1).reshape(-1, 3)
    d = pts[:, None, :] - seeds[None]
    d -= np.round(d)
    lab = np.argmin((d * d).sum(-1), 1)
    eul = synth.so3_uniform_bunge(rng, 7)
    mesh = synth.Mesh((nx, ny, nz), eul[lab], (lab + 1).astype(np.int32),
                      np.ones(nx * ny * nz, np.int32))
    case = synth.Case("aniso", mesh, synth.CU_LIKE, synth.tension_z(), 0.2, 3)
    _vs_oracle(case, 3)
    del m


def test_gpu_vs_oracle_radix3_grid(voce_lib):
    """A 24^3 grid (radix-3 transforms), shorter iteration cap."""
    case = synth.small_case(24, 12, 71, n_steps=2)
    case.iter_max = 30
    _vs_oracle(case, 2)


def test_gpu_homogeneous_crystal_has_no_fluctuation(voce_lib):
    """Size-independent property at 128^3: one orientation everywhere gives
    a uniform stress field equal to that of a 2^3 grid of the same crystal."""
    out = []
    for n in (2, 128):
        nv = n ** 3
        eul = np.tile([[30.0, 40.0, 50.0]], (nv, 1))
        mesh = synth.Mesh((n, n, n), eul, np.ones(nv, np.int32), np.ones(nv, np.int32))
        case = synth.Case("homog%d" % n, mesh, synth.CU_LIKE, synth.tension_z(), 0.2, 2)
        case.iter_max = 20
        with capi.Rve.from_files(_write(case)) as r:
            r.run(2)
            s = r.field("sig_voigt")
            out.append((s, [r.increment(k) for k in range(2)]))
    s2, i2 = out[0]
    s128, i128 = out[1]
    assert np.abs(s128 - s128[:, :1]).max() < 1e-9 * np.abs(s128).max()
    assert gio.rel(s128[:, 0], s2[:, 0]) < 1e-9
    assert [x["iters"] for x in i128] == [x["iters"] for x in i2]


def test_gpu_rejects_bad_input(voce_lib):
    case = synth.small_case(8, 4, 81, n_steps=1)
    case.load = synth.Load((0, 0, 1, 1, 1, 1), (0, 0, 1e-3, 0, 0, 0), (1, 1, 1, 0, 0, 0))
    with pytest.raises(capi.VoceError) as e:
        capi.Rve.from_files(_write(case))
    assert e.value.code == 4            # Stress_BC_Flag and VelGrad_BC_Flag both set
    m = synth.voronoi_mesh(10, 3, 1)    # 10 = 2 * 5: no radix-5 transform here
    with pytest.raises(capi.VoceError) as e:
        capi.Rve.from_files(_write(synth.Case("r5", m, synth.CU_LIKE, synth.tension_z(), 0.2, 1)))
    assert e.value.code == 6


def test_fp64_form_ignores_the_chord_switch(voce_lib):
    """The FP64 form always refreshes the Jacobian (the reference's Newton
    path): switching chord steps off changes none of its bits."""
    make, n, _ = make_golden.CASES["vor12_mix"]
    nl = _write(make())
    lib = capi.load()
    lib.voce_set_newton_chord(0)
    try:
        with capi.Rve.from_files(nl) as r:
            r.run(2)
            a = ([r.increment(k) for k in range(2)], r.field("sig_voigt"), r.field("edot_voigt"))
    finally:
        lib.voce_set_newton_chord(1)
    with capi.Rve.from_files(nl) as r:
        r.run(2)
        b = ([r.increment(k) for k in range(2)], r.field("sig_voigt"), r.field("edot_voigt"))
    assert a[0] == b[0]
    assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])
