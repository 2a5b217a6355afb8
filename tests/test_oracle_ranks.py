"""The reference build on several ranks (test infrastructure): the
unmodified reference sources run as P forked ranks over the shim's shared
memory (oracle/shim: slab-decomposed FFT, rank-ordered MPI_Allreduce,
MPI-IO at each rank's offsets), as the reference's MPI build runs on P cores.
The results must be those of one rank up to the order of the reductions:
identical Green-iteration counts, the same fields to 1e-12 and every reduced
value of the trace to 1e-8 relative.  Needs the reference build
(oracle/_ref, made where the reference sources are present)."""
import os
import subprocess
import sys
import tempfile

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden as mg  # noqa: E402
from voce_gb300 import synth  # noqa: E402


def _run(case, n, ranks):
    d = tempfile.mkdtemp(prefix="ranks_")
    case.write(d, print_control=(1, n))
    env = dict(os.environ, VOCE_REF_TRACE=os.path.join(d, "trace.txt"), VOCE_REF_RANKS=str(ranks))
    r = subprocess.run([mg.REF_BIN, "input"], cwd=d, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    trace = np.array([float(l.split()[2]) for l in open(os.path.join(d, "trace.txt"))])
    iters = mg.parse_iters(os.path.join(d, "err.out"), n)
    nv = case.mesh.nvox
    return trace, iters, mg.read_iout(d, "sig", n, nv), mg.read_iout(d, "edot", n, nv), \
        open(os.path.join(d, "vm.out")).read().count("\n")


@pytest.mark.skipif(not os.path.exists(mg.REF_BIN), reason="reference build not made")
def test_reference_on_several_ranks_matches_one_rank():
    rng = np.random.Generator(np.random.PCG64(9))
    case = synth.small_case(8, 6, 61, n_steps=3, load=synth.random_traceless_load(rng))
    n = 3
    one = _run(case, n, 1)
    for ranks in (2, 4, 8):
        tr, iters, sig, edot, vm_lines = _run(case, n, ranks)
        assert iters == one[1], (ranks, iters, one[1])
        assert vm_lines == one[4]
        assert tr.shape == one[0].shape
        rel = np.abs(tr - one[0]) / np.maximum(np.abs(one[0]), 1e-300)
        assert rel.max() < 1e-8, (ranks, rel.max())
        for a, b in ((sig, one[2]), (edot, one[3])):
            assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max()
