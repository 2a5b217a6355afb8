"""Reading the reference's output-file fixture (tests/golden/make_outputs.py)
and comparing a directory of output files against it."""
from __future__ import annotations

import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "outputs_tex_4x6x8.npz")
# written by both, with values that differ on purpose: the reference's
# displacement_fluct (evolution.c:532-560) sums over voxels into one value per
# component and leaves the transform of the last gradient component in place,
# while this library writes the corrected displacement fluctuation; names and
# record sizes are compared, values are checked against the oracle instead
VALUES_DIFFER = ("new_position",)
# bound on every value of a dump relative to the largest magnitude in it, as
# for the fields in the parity tests
VALUE_TOL = 1e-9
# printed values (%e: 7 significant digits) may differ in the last digit
TEXT_REL = 1.5e-6


def load():
    z = np.load(FIXTURE)
    names = [str(n) for n in z["names"]]
    off = z["offsets"]
    blob = z["blob"].tobytes()
    files = {n: blob[off[i]:off[i + 1]] for i, n in enumerate(names)}
    return dict(digest=str(z["digest"]), vm_out=z["vm_out"].tobytes().decode(),
                err_out=z["err_out"].tobytes().decode(), files=files)


def record_kind(name: str) -> str:
    if name.startswith("tex"):
        return "tex"
    if name.startswith(("slip", "taux", "crss")):
        return "sys"
    return "f8"


def split_records(name: str, data: bytes):
    """(doubles, ints, pad bytes) of one dump."""
    k = record_kind(name)
    if k == "f8":
        return np.frombuffer(data, "<f8"), np.zeros(0, np.int32), b""
    if k == "sys":
        r = np.frombuffer(data, np.uint8).reshape(-1, 104)
        return (r[:, 8:].copy().view("<f8").ravel(), r[:, :4].copy().view("<i4").ravel(),
                r[:, 4:8].tobytes())
    r = np.frombuffer(data, np.uint8).reshape(-1, 48)
    return r[:, :24].copy().view("<f8").ravel(), r[:, 24:].copy().view("<i4").ravel(), b""


def rel(a: np.ndarray, b: np.ndarray) -> float:
    if a.size == 0:
        return 0.0
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def compare_text(ours: str, ref: str) -> int:
    """Lines must agree token by token; numeric tokens within the printed
    precision.  Returns the number of lines that differ in their text."""
    lo, lr = ours.splitlines(), ref.splitlines()
    assert len(lo) == len(lr), (len(lo), len(lr))
    differ = 0
    for a, b in zip(lo, lr):
        if a == b:
            continue
        differ += 1
        ta, tb = a.split(), b.split()
        assert len(ta) == len(tb), (a, b)
        for x, y in zip(ta, tb):
            if x == y:
                continue
            fx, fy = float(x), float(y)
            assert abs(fx - fy) <= TEXT_REL * max(abs(fy), 1e-300), (a, b)
    return differ


def compare_dir(d: str, fx) -> dict:
    """Check the .iout files, vm.out and err.out in d against the fixture;
    returns a small report."""
    ours = sorted(f for f in os.listdir(d) if f.endswith(".iout"))
    want = sorted(fx["files"])
    assert ours == want, (set(ours) ^ set(want))
    worst = 0.0
    for n in want:
        a = open(os.path.join(d, n), "rb").read()
        b = fx["files"][n]
        assert len(a) == len(b), n
        if n.startswith(VALUES_DIFFER):
            continue
        fa, ia, pa = split_records(n, a)
        fb, ib, pb = split_records(n, b)
        assert np.array_equal(ia, ib), n
        assert pa == pb, n
        e = rel(fa, fb)
        assert e <= VALUE_TOL, (n, e)
        worst = max(worst, e)
    dv = compare_text(open(os.path.join(d, "vm.out")).read(), fx["vm_out"])
    de = compare_text(open(os.path.join(d, "err.out")).read(), fx["err_out"])
    return dict(files=len(want), worst_rel=worst, vm_lines_differ=dv, err_lines_differ=de)
