"""Generate the full-length stress-strain curve fixtures of configs 1 and 2.

  cfg1_curve.npz  config 1: 16^3, 4096 one-voxel grains, tension z, all 50
                  increments of 2e-4, run by oracle/_ref/evp_ref -- the
                  unmodified reference sources compiled with the single-rank
                  MPI / FFTW-2 shims (oracle/Makefile).
  cfg2_curve.npz  config 2: 64^3, 125 periodic Voronoi grains, tension z, all
                  100 increments of 2e-4, run by the oracle's C restatement
                  (oracle/_build/liboracle.so, 8 threads).  Its reduction trace
                  and fields are bit-identical to evp_ref's on every fixture
                  case (tests/test_oracle.py); evp_ref itself would take about
                  6 hours on one core for this case.

Each file holds, besides the mesh digest (the tests regenerate the inputs from
the same seeds and check it first):

  iters       Green-operator iterations of every increment
  it_sums     per iteration, the reduced error sums (Err_e and Err_s before
              normalisation, evolution.c:406-409), rows in iteration order
  incr_sums   per increment 38 values: the 9 stress sums and the 9 phase-1
              stress sums of its last iteration (evolution.c:191-194), the 9
              strain and 9 strain-rate sums of its end (evolution.c:483-486)
              and the two rotation averages (constitutive.c:237-240; 0 when
              the increment does not reorient)
  sample_idx  1024 voxels (fixed seed); sig, edot there after the last
              increment, Voigt order 11,22,33,23,13,12 (the order of the
              sig_*/edot_* dumps, io.c:321-397)
  sig_stats, edot_stats   whole-field sum, sum of squares and max |.| per
              component

    python tests/golden/make_curves.py [cfg1_curve] [cfg2_curve]
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
from voce_gb300 import synth  # noqa: E402

import golden_io  # noqa: E402
import make_golden  # noqa: E402

VOIGT = [0, 4, 8, 5, 2, 1]   # 11,22,33,23,13,12 of a row-major 3x3


def _condense(trace, iters, update_flag):
    seg = golden_io.segment({"trace": np.asarray(trace), "iters": np.asarray(iters)}, update_flag)
    it_sums, incr_sums = [], []
    for inc in seg["incr"]:
        for it in inc["its"]:
            it_sums.append([it["sum_e"], it["sum_s"]])
        last = inc["its"][-1]
        rot = inc["rot"] if inc["rot"] is not None else np.zeros(2)
        incr_sums.append(np.concatenate([last["sig"].ravel(), last["sig1"].ravel(),
                                         inc["eps"].ravel(), inc["edot"].ravel(), rot]))
    return np.array(it_sums), np.array(incr_sums)


def _fields_out(sig, edot):
    nv = sig.shape[0]
    rng = np.random.Generator(np.random.PCG64(1234))
    idx = np.sort(rng.choice(nv, size=min(1024, nv), replace=False))
    return dict(sample_idx=idx, sig=sig[idx], edot=edot[idx],
                sig_stats=np.array([sig.sum(0), (sig ** 2).sum(0), np.abs(sig).max(0)]),
                edot_stats=np.array([edot.sum(0), (edot ** 2).sum(0), np.abs(edot).max(0)]))


def cfg1_curve(out_dir=HERE):
    case = synth.config1(50)
    n = case.n_steps
    d = tempfile.mkdtemp(prefix="curve_cfg1_")
    case.write(d, print_control=(1, n))
    env = dict(os.environ, VOCE_REF_TRACE=os.path.join(d, "trace.txt"))
    subprocess.run([make_golden.REF_BIN, "input", "timing.json"], cwd=d, env=env, check=True,
                   stdout=subprocess.DEVNULL)
    vals = [float(l.split()[2]) for l in open(os.path.join(d, "trace.txt"))]
    iters = make_golden.parse_iters(os.path.join(d, "err.out"), n)[:n]
    nv = case.mesh.nvox
    sig = make_golden.read_iout(d, "sig", n, nv)
    edot = make_golden.read_iout(d, "edot", n, nv)
    it_sums, incr_sums = _condense(vals, iters, case.update_flag)
    out = dict(digest=case.mesh.digest(), iters=np.array(iters, np.int32), it_sums=it_sums,
               incr_sums=incr_sums, n_steps=n, nv=nv, source="reference (oracle/_ref/evp_ref)")
    out.update(_fields_out(sig, edot))
    np.savez_compressed(os.path.join(out_dir, "cfg1_curve.npz"), **out)
    print("cfg1_curve iters", iters)


def cfg2_curve(out_dir=HERE, threads=8):
    import oracle as orc
    case = synth.config2(100)
    n = case.n_steps
    d = tempfile.mkdtemp(prefix="curve_cfg2_")
    nl = case.write(d)
    trace = os.path.join(d, "trace.txt")
    job = orc.Job(nl, threads=threads, trace=trace)
    job.run(n)
    iters = [job.increment(k)["iters"] for k in range(n)]
    sig = job.field("sig")[:, VOIGT]
    edot = job.field("edot")[:, VOIGT]
    job.close()
    vals = []
    for line in open(trace):
        t = line.split()
        vals.append(float(t[2]))
    it_sums, incr_sums = _condense(vals, iters, case.update_flag)
    out = dict(digest=case.mesh.digest(), iters=np.array(iters, np.int32), it_sums=it_sums,
               incr_sums=incr_sums, n_steps=n, nv=case.mesh.nvox,
               source="oracle C restatement (oracle/_build/liboracle.so), %d threads" % threads)
    out.update(_fields_out(sig, edot))
    np.savez_compressed(os.path.join(out_dir, "cfg2_curve.npz"), **out)
    print("cfg2_curve iters", iters)


if __name__ == "__main__":
    names = sys.argv[1:] or ["cfg1_curve", "cfg2_curve"]
    for name in names:
        {"cfg1_curve": cfg1_curve, "cfg2_curve": cfg2_curve}[name]()
