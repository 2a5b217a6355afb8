"""Reading the golden fixtures made from the reference (tests/golden/*.npz).

The reference's reductions come in a fixed order (evolution.c, init.c,
constitutive.c call sites of MPI_Allreduce):
  setup          nph1, then the 36 C066 sums           (init.c:446,452)
  per iteration  Err_e sum, Err_s sum                  (evolution.c:406-409)
                 9 x (sigma sum, sigma-phase-1 sum)     (evolution.c:191-194)
  per increment  9 x (eps sum, edot sum)               (evolution.c:483-486)
                 rot-slip and rot-local averages when
                 Update_Flag and istep > 1             (constitutive.c:237-240)
"""
from __future__ import annotations

import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def available(name: str) -> bool:
    return os.path.exists(os.path.join(GOLDEN, name + ".npz"))


def load(name: str) -> dict:
    z = np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)
    return {k: z[k] for k in z.files}


def segment(fx: dict, update_flag: int) -> dict:
    t = fx["trace"]
    iters = [int(x) for x in fx["iters"]]
    out = {"nph1": t[0], "c066_sum": t[1:37], "incr": []}
    pos = 37
    for k, n in enumerate(iters):
        its = []
        for _ in range(n):
            blk = t[pos:pos + 20]
            its.append({"sum_e": blk[0], "sum_s": blk[1],
                        "sig": blk[2:20:2].reshape(3, 3), "sig1": blk[3:20:2].reshape(3, 3)})
            pos += 20
        blk = t[pos:pos + 18]
        inc = {"its": its, "eps": blk[0:18:2].reshape(3, 3), "edot": blk[1:18:2].reshape(3, 3),
               "rot": None}
        pos += 18
        if update_flag and k >= 1:
            inc["rot"] = t[pos:pos + 2]
            pos += 2
        out["incr"].append(inc)
    if pos != len(t):
        raise ValueError("trace length %d does not match the iteration counts (%d)" % (len(t), pos))
    return out


# Lebensohn-Tome basis (reference kinematics.c:346-364)
_R2, _R3, _R6 = 0.70710678118654744, 0.57735026918962584, 0.40824829046386304
BASIS = np.zeros((6, 3, 3))
BASIS[0, 0, 0], BASIS[0, 1, 1] = -_R2, _R2
BASIS[1, 0, 0], BASIS[1, 1, 1], BASIS[1, 2, 2] = -_R6, -_R6, 2 * _R6
BASIS[2, 1, 2] = BASIS[2, 2, 1] = _R2
BASIS[3, 0, 2] = BASIS[3, 2, 0] = _R2
BASIS[4, 0, 1] = BASIS[4, 1, 0] = _R2
BASIS[5, 0, 0] = BASIS[5, 1, 1] = BASIS[5, 2, 2] = _R3


def b6_to_tensor(b6) -> np.ndarray:
    return np.einsum("i,ijk->jk", np.asarray(b6, float), BASIS)


def rel(a, b) -> float:
    """max |a - b| / max |b| (norm-wise relative error of a field or curve)."""
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))
