"""The FP64 form gives the same bits in every process.  Two fresh Python
processes, with no tile-cache file between them, each set up and solve the
same RVE (a 24 x 32 x 48 grid, whose axes have 4, 2 and 2 radix-schedule
candidates) and save the stress and strain-rate fields, the iteration counts
and the radix schedules; everything must be equal, bit for bit.  Tile tuning
(results never depend on the tile) runs in both; the radix schedule, which
changes roundings, stays at the default in the FP64 form."""
import os
import subprocess
import sys
import tempfile

import numpy as np
import pytest

from voce_gb300 import synth

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROG = """
import sys
sys.path.insert(0, %(root)r)
import numpy as np
from voce_gb300 import capi
with capi.Rve.from_files(%(nl)r, capi.PREC_FP64) as r:
    sched = [r.fft_schedule(a) for a in range(3)]
    r.run(2)
    inc = [r.increment(k) for k in range(2)]
    np.savez(%(out)r, sig=r.field("sig_voigt"), edot=r.field("edot_voigt"),
             disgrad=r.field("disgrad"), iters=[x["iters"] for x in inc],
             s_vm=[x["s_vm"] for x in inc], nr=[x["nr_iters_total"] for x in inc],
             sched=np.array([len(s) for s in sched] + sum(sched, [])))
"""


def _solve_in_fresh_process(nl, out):
    env = {k: v for k, v in os.environ.items() if k != "VOCE_TILE_CACHE"}
    subprocess.run([sys.executable, "-c", PROG % {"root": ROOT, "nl": nl, "out": out}],
                   env=env, check=True, timeout=600)
    z = np.load(out)
    return {k: z[k] for k in z.files}


def test_fp64_bits_do_not_depend_on_the_process(voce_lib):
    case = synth.Case("det_24_32_48", synth.voronoi_mesh_box((24, 32, 48), 12, 91),
                      synth.CU_LIKE, synth.tension_z(), 0.2, 2)
    d = tempfile.mkdtemp(prefix="determinism_")
    nl = case.write(d)
    a = _solve_in_fresh_process(nl, os.path.join(d, "a.npz"))
    b = _solve_in_fresh_process(nl, os.path.join(d, "b.npz"))
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    # default schedules: 4s-2-3s on every axis (24 = 4.2.3, 32 = 4.4.2, 48 = 4.4.3)
    assert list(a["sched"]) == [3, 3, 3, 4, 2, 3, 4, 4, 2, 4, 4, 3]
