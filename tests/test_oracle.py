"""The oracle (C restatement, oracle/evp_oracle.c) against the reference's own
outputs: the golden fixtures were made by running the unmodified reference
sources (tests/golden/make_golden.py).  CPU only."""
import os
import tempfile

import numpy as np
import pytest

import golden_io as gio
import make_golden
import oracle as orc
from voce_gb300 import synth

SMALL = ["vor8_tension", "vor8_psc", "vor8_gas", "vor8_creep", "vor8_noupd", "vor12_mix",
         "cfg1_16"]


def _run(case, n, threads=4, trace=True):
    d = tempfile.mkdtemp(prefix="orc_")
    nl = case.write(d)
    tp = os.path.join(d, "trace.txt") if trace else None
    j = orc.Job(nl, threads=threads, trace=tp)
    j.run(n)
    vals = np.array([float(l.split()[2]) for l in open(tp)]) if trace else None
    return j, vals


@pytest.mark.parametrize("name", SMALL)
def test_oracle_reproduces_reference(name, oracle_lib):
    """Every reduced value (error sums, stress averages, strain averages,
    rotation averages) and the final stress / strain-rate fields of the
    reference, to 1e-12 relative (bit-identical on x86-64 with gcc)."""
    if not gio.available(name):
        pytest.skip("fixture missing")
    fx = gio.load(name)
    make, n, _ = make_golden.CASES[name]
    case = make()
    assert case.mesh.digest() == str(fx["digest"]), "synthetic input generator changed"
    j, vals = _run(case, n)
    assert len(vals) == len(fx["trace"])
    assert [j.increment(k)["iters"] for k in range(n)] == [int(x) for x in fx["iters"]]
    scale = np.maximum(np.abs(fx["trace"]), 1e-300)
    # error sums and averages are compared value by value
    assert np.max(np.abs(vals - fx["trace"]) / scale) < 1e-12
    sig = j.field("sig")[:, [0, 4, 8, 5, 2, 1]]
    edot = j.field("edot")[:, [0, 4, 8, 5, 2, 1]]
    assert gio.rel(sig, fx["sig"]) < 1e-12
    assert gio.rel(edot, fx["edot"]) < 1e-12


def test_oracle_threads_do_not_change_results(oracle_lib):
    case = synth.small_case(8, 5, 3, n_steps=2)
    _, a = _run(case, 2, threads=1)
    _, b = _run(case, 2, threads=7)
    assert np.array_equal(a, b)


def test_trace_segmentation_matches_iteration_counts():
    for name in SMALL:
        if not gio.available(name):
            continue
        case = make_golden.CASES[name][0]()
        seg = gio.segment(gio.load(name), case.update_flag)
        assert len(seg["incr"]) == make_golden.CASES[name][1]


def test_fft_core_matches_numpy(oracle_lib):
    import ctypes
    lib = ctypes.CDLL(orc.PORT_LIB)
    lib.fftc_3d.argtypes = [ctypes.c_int] * 4 + [ctypes.c_void_p, ctypes.c_int]
    rng = np.random.default_rng(0)
    for dims in [(16, 16, 16), (8, 12, 6), (48, 4, 10), (7, 5, 3), (2, 2, 2)]:
        a = rng.standard_normal(dims) + 1j * rng.standard_normal(dims)
        b = np.ascontiguousarray(a.copy())
        lib.fftc_3d(*dims, -1, b.ctypes.data, 2)
        assert gio.rel(b, np.fft.fftn(a)) < 1e-14
        c = np.ascontiguousarray(a.copy())
        lib.fftc_3d(*dims, 1, c.ctypes.data, 1)
        assert gio.rel(c, np.fft.ifftn(a) * a.size) < 1e-14


def test_oracle_lu_inverse_known_answer(oracle_lib):
    """The LU inverse on the 6x6 the reference's commented-out self-check
    uses (init.c:467-479)."""
    s0 = np.zeros((6, 6))
    s0[0, 1] = 1.0
    s0[1, 0], s0[1, 2] = 2.0, 2.0
    s0[2, 1], s0[2, 3] = 3.0, 1.0
    s0[3, 2], s0[3, 4] = 1.0, 2.0
    s0[4, 3], s0[4, 5] = 3.0, 1.0
    s0[5, 4] = 2.0
    a = np.ascontiguousarray(s0.copy())
    assert oracle_lib.oracle_lu_inv66(a.ctypes.data) == 0
    assert np.allclose(a @ s0, np.eye(6), atol=1e-13)
    z = np.zeros((6, 6))
    z[3, :] = 1e-7          # a near-zero row: the reference exits with 35
    z += np.eye(6) * (np.arange(6) != 3)
    assert oracle_lib.oracle_lu_inv66(z.ctypes.data) == 35


def test_synthetic_meshes_are_reproducible():
    a = synth.voronoi_mesh(16, 20, 5)
    b = synth.voronoi_mesh(16, 20, 5)
    assert a.digest() == b.digest()
    assert len(np.unique(a.grain)) <= 20
    # SO(3)-uniform: cos(Phi) uniform on [-1, 1]
    e = synth.so3_uniform_bunge(np.random.Generator(np.random.PCG64(0)), 20000)
    c = np.cos(np.radians(e[:, 1]))
    assert abs(c.mean()) < 0.02 and abs((c ** 2).mean() - 1 / 3) < 0.02


def test_oracle_fluctuation_pinned_to_the_reference_new_position(oracle_lib):
    """The reference's new_position dump (evolution.c:532-560, io.c:806-858)
    is, because of its stale index, the inverse transform of the forward
    transform of fluctuation[i][2]: -fluctuation[i][2] per voxel.  The
    oracle's accumulated fluctuation reproduces the reference's own file, and
    so does DisGrad minus its average (the fluctuation reaches DisGrad with
    uniform terms only)."""
    import make_outputs
    import outputs_io
    fx = outputs_io.load()
    case = make_outputs.tex_case()
    d = tempfile.mkdtemp(prefix="orc_np_")
    nl = case.write(d, print_control=make_outputs.PRINT_CONTROL, tex_flag=make_outputs.TEX_FLAG)
    j = orc.Job(nl)
    j.run(3)
    ref = np.frombuffer(fx["files"]["new_position_S0003.iout"], "<f8").reshape(-1, 3)
    dg = j.field("disgrad").reshape(-1, 3, 3)
    fl = dg - dg.mean(axis=0)
    assert gio.rel(-fl[:, :, 2], ref) < 1e-12
    # the corrected field from the accumulated fluctuation and from DisGrad
    a = j.disp_fluct(True)
    b = j.disp_fluct(False)
    assert gio.rel(a, b) < 1e-12
    assert gio.rel(b, orc.disp_fluct_np(j.field("disgrad"), case.mesh.dims)) < 1e-12


def test_disp_fluct_known_answer():
    """The corrected transform inverts the gradient: for a band-limited
    periodic u (no Nyquist content), the displacement of F = grad u is u minus
    its mean, on a grid with radix-2, -3 and -5 axes."""
    nx, ny, nz = 8, 6, 10
    x, y, z = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    kx, ky, kz = 2 * np.pi / nx, 2 * np.pi / ny, 2 * np.pi / nz
    a1 = 2 * ky * y + kz * z
    u = np.stack([np.sin(kx * x) + 0.3 * np.cos(a1), 0.5 * np.cos(kx * x + ky * y),
                  0.2 * np.sin(3 * kz * z) + 0.1 * np.sin(kx * x)], -1)
    F = np.zeros((nx, ny, nz, 3, 3))
    F[..., 0, 0] = kx * np.cos(kx * x)
    F[..., 0, 1] = -0.3 * 2 * ky * np.sin(a1)
    F[..., 0, 2] = -0.3 * kz * np.sin(a1)
    F[..., 1, 0] = -0.5 * kx * np.sin(kx * x + ky * y)
    F[..., 1, 1] = -0.5 * ky * np.sin(kx * x + ky * y)
    F[..., 2, 0] = 0.1 * kx * np.cos(kx * x)
    F[..., 2, 2] = 0.6 * kz * np.cos(3 * kz * z)
    got = orc.disp_fluct_np(F.reshape(-1, 9), (nx, ny, nz))
    want = (u - u.mean(axis=(0, 1, 2))).reshape(-1, 3)
    assert np.max(np.abs(got - want)) < 1e-12
