"""The C ABI's host side (no GPU needed): the library loads, exports every
function include/voce_gpu.h declares, and its readers follow the reference's
formats and quirks (io.c:54-122, init.c:51-186, init.c:393-442)."""
import os
import re
import tempfile

import numpy as np
import pytest

from voce_gb300 import capi, synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = "".join(open(os.path.join(ROOT, "include", f)).read()
                  for f in sorted(os.listdir(os.path.join(ROOT, "include"))) if f.endswith(".h"))
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(voce_[a-z_0-9]+)\s*\(", src)))


def test_exports_every_declared_symbol(voce_lib):
    names = declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(voce_lib, n), n
    assert {p[0] for p in capi.PROTOTYPES} == set(names)
    assert voce_lib.voce_abi_version() == 1


def _case_dir(case):
    d = tempfile.mkdtemp(prefix="capi_")
    return d, case.write(d)


def test_namelist_reader_matches_reference_semantics(voce_lib):
    case = synth.small_case(8, 4, 1, n_steps=3)
    d, nl_path = _case_dir(case)
    nl = capi.read_namelist(nl_path)
    assert list(nl.CellDim) == [8, 8, 8]
    assert nl.N_phases == 2 and list(nl.Type_phases) == [0, 1]
    assert nl.TimeStep == 0.2 and nl.N_steps == 3 and nl.IterMax == 200
    assert list(nl.VelGrad_BC_Flag) == [0, 0, 1, 1, 1, 1]
    assert list(nl.VelGrad_BC) == [-0.0005, -0.0005, 0.001, 0.0, 0.0, 0.0]
    assert nl.Slip_PhaseI == b"mat.sx" and nl.initial_ms == b"mesh.txt"
    # the key is "Hirth" in the file, "hirth" in the reader: stays 0
    assert list(nl.hirth) == [0.0, 0.0] and list(nl.self) == [1.0, 0.0]
    # repeated key keeps the first values; unknown keys are ignored;
    # a line without a first token ends the read
    with open(nl_path, "a") as f:
        f.write("TimeStep 0.5\nNotAKey 3 4\n   \nN_steps 99\n")
    nl2 = capi.read_namelist(nl_path)
    assert nl2.TimeStep == 0.2 and nl2.N_steps == 3


def test_slip_and_mesh_readers(voce_lib):
    case = synth.small_case(8, 4, 2, n_steps=1)
    d, nl_path = _case_dir(case)
    sx = capi.read_slip(os.path.join(d, "mat.sx"))
    assert sx.nsys == 12 and sx.nrs == 20.0 and sx.gamd0 == 1e-3
    assert (sx.tau0f, sx.tau0b, sx.tau1, sx.thet0, sx.thet1) == (12.0, 12.0, 6.0, 200.0, 3.0)
    assert list(sx.bn[0]) == [1.0, 1.0, -1.0] and list(sx.bb[0]) == [0.0, 1.0, 1.0]
    eul, gr, ph = capi.read_mesh(os.path.join(d, "mesh.txt"), (8, 8, 8))
    assert np.array_equal(eul, case.mesh.euler_deg)
    assert np.array_equal(gr, case.mesh.grain) and np.array_equal(ph, case.mesh.phase)


def test_reader_errors(voce_lib):
    with pytest.raises(capi.VoceError) as e:
        capi.read_namelist("/nonexistent/input")
    assert e.value.code == 2
    case = synth.small_case(4, 2, 3, n_steps=1)
    d, _ = _case_dir(case)
    lines = open(os.path.join(d, "mesh.txt")).read().splitlines()
    lines[5], lines[6] = lines[6], lines[5]       # index order broken (init.c:420-423)
    open(os.path.join(d, "mesh.txt"), "w").write("\n".join(lines) + "\n")
    with pytest.raises(capi.VoceError) as e:
        capi.read_mesh(os.path.join(d, "mesh.txt"), (4, 4, 4))
    assert e.value.code == 3
    # an index far out of range (17 digits, whose linear index exceeds 64
    # bits on a 1 x 10 x 10 grid) is an index mismatch, with no overflow in
    # the index arithmetic (the sanitizer run checks that)
    rows = ["0.0 0.0 0.0 1 %d %d 1 1" % (j + 1, k + 1) for j in range(10) for k in range(10)]
    rows[7] = "0.0 0.0 0.0 99999999999999999 99999999999999999 -99999999999999999 1 1"
    open(os.path.join(d, "mesh.txt"), "w").write("\n".join(rows) + "\n")
    with pytest.raises(capi.VoceError) as e:
        capi.read_mesh(os.path.join(d, "mesh.txt"), (1, 10, 10))
    assert e.value.code == 3 and "index" in str(e.value) and "voxel 7" in str(e.value)


def test_readers_on_edited_files(voce_lib):
    """The namelist, .sx and mesh readers, and creation's host checks, on 300
    randomly edited input files (characters replaced, inserted, deleted or
    copied from elsewhere in the file; seeded): each call returns a result or
    a status code.  Under the sanitizer run this is a small fuzz test of the
    host parsers."""
    import random
    rng = random.Random(11)
    case = synth.small_case(4, 2, 3, n_steps=1)
    d, nlp = _case_dir(case)
    names = {"nl": os.path.basename(nlp), "sx": "mat.sx", "mesh": "mesh.txt"}
    text = {k: open(os.path.join(d, f)).read() for k, f in names.items()}
    alphabet = "0123456789.-+eEnaifx \t\n,#"

    def edit(t):
        t = list(t)
        for _ in range(rng.randint(1, 8)):
            i, op = rng.randrange(max(1, len(t))), rng.random()
            if op < 0.4 and t:
                t[i] = rng.choice(alphabet)
            elif op < 0.6:
                t.insert(i, rng.choice(alphabet) * rng.randint(1, 120))
            elif op < 0.8 and t:
                del t[i:i + rng.randint(1, 40)]
            else:
                j = rng.randrange(max(1, len(t)))
                t[i:i] = t[j:j + rng.randint(1, 60)]
        return "".join(t)

    try:
        capi.device_memory()
        host_only = False       # a GPU is present: creation would run on it; skip that part
    except capi.VoceError:
        host_only = True
    outcomes = {"ok": 0, "refused": 0}
    for _ in range(300):
        which = rng.choice(sorted(names))
        for k, f in names.items():
            open(os.path.join(d, f), "w").write(edit(text[k]) if k == which else text[k])
        try:
            nl = capi.read_namelist(os.path.join(d, names["nl"]))
            sx = capi.read_slip(os.path.join(d, names["sx"]))
            dims = tuple(nl.CellDim)
            if all(0 < x <= 64 for x in dims):
                eul, gr, ph = capi.read_mesh(os.path.join(d, names["mesh"]), dims)
                if host_only:
                    with pytest.raises(capi.VoceError):     # refused on the host, or at the GPU
                        capi.Rve.create(nl, sx, eul, gr, ph)
            outcomes["ok"] += 1
        except capi.VoceError:
            outcomes["refused"] += 1
    assert outcomes["ok"] > 50 and outcomes["refused"] > 50, outcomes


def test_create_refuses_bad_inputs_before_the_gpu(voce_lib):
    """Host-side fault injection (no GPU touched): a NaN Euler angle in the
    mesh buffer, a singular crystal stiffness (C11 = C12, init.c:120-135 would
    hit the LU's TINY pivot and exit(35), kinematics.c:306-309) and a phase id
    outside the namelist's phases come back as status codes."""
    import dataclasses
    case = synth.small_case(4, 2, 5, n_steps=1)
    d, nlp = _case_dir(case)
    nl = capi.read_namelist(nlp)
    sx = capi.read_slip(os.path.join(d, "mat.sx"))
    eul = case.mesh.euler_deg.copy()
    eul[7, 1] = np.nan
    with pytest.raises(capi.VoceError) as e:
        capi.Rve.create(nl, sx, eul, case.mesh.grain, case.mesh.phase)
    assert e.value.code == 1 and "non-finite" in str(e.value)
    # mesh arrays shorter than the grid never reach the library, which reads
    # them through plain pointers
    with pytest.raises(ValueError):
        capi.Rve.create(nl, sx, case.mesh.euler_deg[:-1], case.mesh.grain, case.mesh.phase)
    with pytest.raises(ValueError):
        capi.Rve.create(nl, sx, case.mesh.euler_deg, case.mesh.grain[:5], case.mesh.phase)
    with capi.Server(capi.PREC_FP64, 1 << 30) as srv, pytest.raises(ValueError):
        srv.submit(nl, sx, case.mesh.euler_deg, case.mesh.grain, case.mesh.phase[1:], 1)
    with pytest.raises(ValueError):
        capi.mesh_voronoi((4, 4, 4), np.zeros((3, 3)), np.zeros((2, 3)))
    # an x edge of 1152 points: an FP64 line does not fit a block's shared
    # memory in the FFT passes (refused before the GPU; FP32 lines fit)
    dims = (1152, 4, 4)
    big = capi.read_namelist(nlp)
    big.CellDim[0], big.CellDim[1], big.CellDim[2] = dims
    nv = int(np.prod(dims))
    with pytest.raises(capi.VoceError) as e:
        capi.Rve.create(big, sx, np.zeros((nv, 3)), np.ones(nv, np.int32), np.ones(nv, np.int32))
    assert e.value.code == 6 and "too long" in str(e.value), str(e.value)
    ph = case.mesh.phase.copy()
    ph[3] = 3
    with pytest.raises(capi.VoceError) as e:
        capi.Rve.create(nl, sx, case.mesh.euler_deg, case.mesh.grain, ph)
    assert e.value.code == 3
    bad = dataclasses.replace(case, mat=dataclasses.replace(case.mat, c12=case.mat.c11))
    d2, nlp2 = _case_dir(bad)
    with pytest.raises(capi.VoceError) as e:
        capi.Rve.create(capi.read_namelist(nlp2), capi.read_slip(os.path.join(d2, "mat.sx")),
                        bad.mesh.euler_deg, bad.mesh.grain, bad.mesh.phase)
    assert e.value.code == 5


def test_footprint_scales_with_grid(voce_lib):
    a = capi.footprint((64, 64, 64))
    b = capi.footprint((128, 128, 128))
    assert 7.9 < b / a < 8.1
    nv = 64 ** 3
    nspec = 33 * 64 * 64
    # the mixed forms hold the spectrum in FP32; the single-precision Newton
    # form also keeps float copies of the Schmid vectors, 1/crss and S_g + S0
    # (the FP64 form also stores n and omega of every frequency: 9 doubles)
    assert capi.footprint((64, 64, 64), capi.PREC_MIXED) == a - 9 * 8 * nspec - 9 * 8 * nspec
    assert capi.footprint((64, 64, 64), capi.PREC_MIXED_NR32) == a + 840 * nv - 2 * 9 * 8 * nspec
    assert capi.footprint((64, 64, 64), capi.PREC_MIXED_IR) == a + (840 + 168) * nv - 2 * 9 * 8 * nspec
    assert capi.footprint((256, 256, 256)) < 40e9


def test_restore_rejects_damaged_snapshots(voce_lib):
    """Header checks run before any device work (no GPU needed)."""
    import ctypes as C
    h = C.c_void_p()
    for blob, code in ((b"", 3), (b"x" * 64, 3), (b"VOCESNAP" + bytes(56), 6)):
        assert voce_lib.voce_rve_restore(blob, len(blob), C.byref(h)) == code


def test_mesh_reader_parses_like_strtod_on_every_format(voce_lib):
    """The parallel mesh reader (more than 1 MiB: several chunks) gives the
    doubles the C library's conversion gives (Python's float() is correctly
    rounded, as glibc's strtod is), for every number format a mesh file may
    hold: fixed with up to 22 fraction digits, more than 15 significant
    digits, exponents, signs, negative zero; blanks, tabs, CRLF and blank
    lines between records."""
    rng = np.random.Generator(np.random.PCG64(5))
    dims = (40, 40, 40)
    nv = 40 ** 3
    fmts = ["%.6f", "%.17g", "%.3e", "%+.9f", "%.22f", "%.0f", "%.20g"]
    lines, want = [], np.zeros((nv, 3))
    v = 0
    for i in range(40):
        for j in range(40):
            for k in range(40):
                toks = []
                for q in range(3):
                    x = float(rng.uniform(-400, 400)) * (10.0 ** int(rng.integers(-3, 4)))
                    if v % 997 == 0 and q == 0:
                        x = -0.0
                    t = fmts[(v + q) % len(fmts)] % x
                    toks.append(t)
                    want[v, q] = float(t)
                sep = "\t" if v % 3 == 0 else " "
                end = "\r\n" if v % 5 == 0 else "\n"
                lines.append(sep.join(toks) + " %d %d +%d %d %d" % (i + 1, j + 1, k + 1, v % 7 + 1, 1) + end)
                if v % 4999 == 0:
                    lines.append("   \n")
                v += 1
    d = tempfile.mkdtemp(prefix="meshfmt_")
    path = os.path.join(d, "mesh.txt")
    with open(path, "w", newline="") as f:
        f.write("".join(lines))
    assert os.path.getsize(path) > (1 << 20)
    eul, grain, phase = capi.read_mesh(path, dims)
    got = np.asarray(eul).reshape(nv, 3)
    assert got.tobytes() == want.tobytes()
    assert np.array_equal(grain, np.arange(nv) % 7 + 1) and (phase == 1).all()
    # a record out of place is still caught in a later chunk
    bad = list(lines)
    idx = len(bad) * 3 // 4
    bad[idx] = bad[idx].replace("\t", " ").split(" ")
    bad[idx][3] = "999"
    bad[idx] = " ".join(bad[idx])
    with open(path, "w", newline="") as f:
        f.write("".join(bad))
    with pytest.raises(capi.VoceError) as ei:
        capi.read_mesh(path, dims)
    assert ei.value.code == 3


def test_fft_schedule_candidates(voce_lib):
    """Radix schedules per axis length (host only): the stage orders of the
    radix-4/2/3 passes, duplicates dropped; lengths other than 2^a 3^b have
    none."""
    lib = capi.load()
    want = {2: 1, 4: 1, 6: 2, 8: 2, 12: 2, 16: 1, 24: 4, 32: 2, 48: 2, 64: 1, 96: 4, 128: 2,
            256: 1, 384: 4, 5: 0, 10: 0, 1: 0}
    for n, c in want.items():
        assert lib.voce_fft_schedule_count(n) == c, n


def test_server_cancel_and_deadline_on_the_host(voce_lib):
    """Queue handling of voce_serve.h without a GPU: a server that has
    admitted nothing needs no device.  A queued request is cancelled (status
    CANCELLED, error ERR_CANCELLED, t_done set); one whose deadline has
    passed ends at the start of the next poll with ERR_DEADLINE, before any
    admission; ended requests cannot be cancelled or given a deadline again.
    A budget smaller than every footprint keeps the remaining request from
    being admitted, so that no GPU work is tried."""
    from voce_gb300 import synth
    c = synth.small_case(8, 3, 5, n_steps=1)
    d = tempfile.mkdtemp(prefix="srv_host_")
    nlp = c.write(d)
    nl = capi.read_namelist(nlp)
    sx = capi.read_slip(os.path.join(d, "mat.sx"))
    tiny = capi.footprint((8, 8, 8)) // 2
    with capi.Server(capi.PREC_MIXED_IR, tiny, ticks_per_round=2) as s:
        args = (nl, sx, c.mesh.euler_deg, c.mesh.grain, c.mesh.phase, 1)
        a, b, late = s.submit(*args), s.submit(*args), s.submit(*args)
        s.cancel(b)
        ib = s.info(b)
        assert ib.status == capi.REQ_CANCELLED and ib.error == capi.ERR_CANCELLED
        assert ib.t_done >= ib.t_submit
        s.set_deadline(late, 1e-9)                     # already past
        assert s.info(late).t_deadline > 0
        with pytest.raises(capi.VoceError) as e:
            s.cancel(b)
        assert e.value.code == 9
        run, que = s.poll()
        il = s.info(late)
        assert il.status == capi.REQ_FAILED and il.error == capi.ERR_DEADLINE
        # a's footprint exceeds the budget: it fails with ERR_NOMEM, no device work
        ia = s.info(a)
        assert ia.status == capi.REQ_FAILED and ia.error == 7
        assert (run, que) == (0, 0) and s.bytes_in_use == 0
        for rid in (a, late):
            with pytest.raises(capi.VoceError):
                s.set_deadline(rid, s.now() + 5.0)
        with pytest.raises(capi.VoceError) as e:
            s.cancel(12345)
        assert e.value.code == 1
