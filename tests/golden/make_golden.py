"""Generate the golden fixtures in this directory from the REFERENCE itself.

Runs oracle/_ref/evp_ref -- the unmodified reference sources compiled with
the single-rank MPI / FFTW-2 shims (oracle/Makefile) -- on synthetic inputs
written by voce_gb300.synth, and stores per case (``<case>.npz``):

  digest    hash of the generated mesh (the tests regenerate the inputs from
            the same seeds and check this first)
  iters     Green-operator iterations of every increment (from err.out)
  trace     every value the reference reduces with MPI_Allreduce, in call
            order, at full precision (the MPI shim's trace): the C066 sums,
            per iteration the error sums and the 9 x (sigma, sigma_phase1)
            sums, per increment the 9 x (eps, edot) sums and the two
            rotation averages
  sig, edot stress and plastic strain rate after the last increment, Voigt
            order 11,22,33,23,13,12 (the sig_*/edot_* .iout dumps,
            io.c:321-397), either for every voxel or for a fixed sample of
            voxels (sample_idx) plus whole-field statistics

Needs the reference sources (only present where the fixtures are made):
    python tests/golden/make_golden.py [case ...] [--from-run case=dir]
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from voce_gb300 import synth  # noqa: E402

REF_BIN = os.path.join(ROOT, "oracle", "_ref", "evp_ref")


def _gas_case() -> synth.Case:
    c = synth.small_case(8, 6, 21, n_steps=4)
    ph = c.mesh.phase.copy()
    ph[c.mesh.grain == 2] = 2            # one grain is a pore (gas phase)
    c.mesh = synth.Mesh(c.mesh.dims, c.mesh.euler_deg, c.mesh.grain, ph)
    c.name = "vor8_gas"
    return c


def _creep_case() -> synth.Case:
    c = synth.small_case(8, 6, 31, n_steps=4,
                         load=synth.Load((0,) * 6, (0.0,) * 6, (1,) * 6,
                                         (0.0, 0.0, 22.0, 0.0, 0.0, 0.0)))
    c.name = "vor8_creep"
    return c


def _noupd_case() -> synth.Case:
    c = synth.small_case(8, 6, 41, n_steps=4)
    c.update_flag = 0
    c.hard_flag = 0
    c.name = "vor8_noupd"
    return c


def _shear_case() -> synth.Case:
    rng = np.random.Generator(np.random.PCG64(51))
    c = synth.small_case(12, 9, 51, n_steps=4, load=synth.random_traceless_load(rng))
    c.name = "vor12_mix"
    return c


CASES = {
    # name: (constructor, increments, store full fields)
    "cfg1_16": (lambda: synth.config1(3), 3, True),
    "vor8_tension": (lambda: synth.small_case(8, 6, 11, n_steps=4), 4, True),
    "vor8_psc": (lambda: synth.small_case(8, 6, 12, n_steps=4,
                                          load=synth.plane_strain_compression()), 4, True),
    "vor8_gas": (_gas_case, 4, True),
    "vor8_creep": (_creep_case, 4, True),
    "vor8_noupd": (_noupd_case, 4, True),
    "vor12_mix": (_shear_case, 4, True),
    "cfg2_64": (lambda: synth.config2(3), 3, False),
}


def parse_iters(err_out: str, n_steps: int) -> list:
    iters, cur = [], None
    for line in open(err_out):
        t = line.split()
        if not t:
            continue
        if t[0] == "STEP":
            if cur is not None:
                iters.append(cur)
            cur = 0
        elif t[0].isdigit():
            cur = int(t[0]) if cur is not None else int(t[0])
    if cur is not None:
        iters.append(cur)
    if n_steps == 1 and not iters:
        iters = [cur or 0]
    return iters


def read_iout(d: str, stem: str, step: int, nv: int) -> np.ndarray:
    out = np.empty((nv, 6))
    for i in range(6):
        out[:, i] = np.fromfile(os.path.join(d, "%s_%d_S%04d.iout" % (stem, i + 1, step)),
                                dtype=np.float64, count=nv)
    return out


def run_case(name: str, run_dir: str | None = None) -> None:
    make, n, full = CASES[name]
    case = make()
    tmp = None
    if run_dir is None:
        tmp = tempfile.mkdtemp(prefix="golden_" + name + "_")
        run_dir = tmp
        nl = case.write(run_dir, print_control=(1, n))
        env = dict(os.environ, VOCE_REF_TRACE=os.path.join(run_dir, "trace.txt"))
        subprocess.run([REF_BIN, "input", "timing.json"], cwd=run_dir, env=env, check=True,
                       stdout=subprocess.DEVNULL)
    nv = case.mesh.nvox
    vals = [float(l.split()[2]) for l in open(os.path.join(run_dir, "trace.txt"))]
    iters = parse_iters(os.path.join(run_dir, "err.out"), n)[:n]
    sig = read_iout(run_dir, "sig", n, nv)
    edot = read_iout(run_dir, "edot", n, nv)
    out = dict(digest=case.mesh.digest(), iters=np.array(iters, dtype=np.int32),
               trace=np.array(vals), n_steps=n, nv=nv)
    if full:
        out.update(sig=sig, edot=edot)
    else:
        rng = np.random.Generator(np.random.PCG64(1234))
        idx = np.sort(rng.choice(nv, size=1024, replace=False))
        out.update(sample_idx=idx, sig=sig[idx], edot=edot[idx],
                   sig_stats=np.array([sig.sum(0), (sig ** 2).sum(0), np.abs(sig).max(0)]),
                   edot_stats=np.array([edot.sum(0), (edot ** 2).sum(0), np.abs(edot).max(0)]))
    t = os.path.join(run_dir, "timing.json")
    if os.path.exists(t):
        out["ref_timing"] = json.dumps(json.load(open(t)))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, "iters", iters, "trace", len(vals))


def main(argv):
    from_run = {}
    names = []
    for a in argv:
        if a.startswith("--from-run"):
            continue
        if "=" in a:
            k, v = a.split("=", 1)
            from_run[k] = v
        else:
            names.append(a)
    if not os.path.exists(REF_BIN):
        raise SystemExit("build the reference oracle first: make -C oracle ref")
    for name in names or list(CASES):
        run_case(name, from_run.get(name))


if __name__ == "__main__":
    main(sys.argv[1:])
