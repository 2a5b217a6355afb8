"""Output files against the reference's own (tests/golden/outputs_*.npz): the
.iout dumps, vm.out and err.out written through the handle API
(include/voce_io.h) and by the reference's entry points SetupJob / Evolution /
DestroyJob of libvoce_legacy.so driven from a program that defines the
reference's globals.  Names, sizes, integer columns and padding must be
identical; doubles within the parity bound; printed numbers within their last
digit."""
import os
import shutil
import subprocess
import tempfile

import pytest

from voce_gb300 import build, capi

import make_outputs
import outputs_io
from test_legacy_host import build_host

pytestmark = pytest.mark.gpu

N_STEPS = 3


def _inputs() -> str:
    case = make_outputs.tex_case()
    d = tempfile.mkdtemp(prefix="outputs_")
    case.write(d, print_control=make_outputs.PRINT_CONTROL, tex_flag=make_outputs.TEX_FLAG)
    return d


def test_handle_api_writes_the_reference_outputs():
    fx = outputs_io.load()
    d = _inputs()
    with capi.Rve.from_files(os.path.join(d, "input")) as r:
        r.run(N_STEPS)
        out = os.path.join(d, "out")
        os.makedirs(out)
        for istep in range(1, N_STEPS + 1):
            r.write_step_iout(istep, out)   # only increment 3 is selected
        r.write_final_iout(out)
        r.write_logs(out, N_STEPS)
    rep = outputs_io.compare_dir(out, fx)
    assert rep["files"] == 69
    print(rep)


def test_legacy_entry_points_run_the_reference_job():
    fx = outputs_io.load()
    if not os.path.exists(capi.LEGACY_LIB_PATH):
        build.build_legacy()
    d = _inputs()
    exe = build_host(d)
    run = subprocess.run([exe, "input"], cwd=d, capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stderr
    rep = outputs_io.compare_dir(d, fx)
    print(rep)
    # the globals Evolution leaves behind match the handle API's state
    g = [ln for ln in run.stdout.splitlines() if ln.startswith("GLOBALS")][0].split()[1:]
    nv = int(g[0])
    with capi.Rve.from_files(os.path.join(d, "input")) as r:
        r.run(N_STEPS)
        rec = r.increment(N_STEPS - 1)
        sig = r.field("sig")
        dg = r.field("disgrad")
    assert nv == r.nv
    assert float(g[1]) == rec["s_vm"]
    assert float(g[2]) == rec["sig_avg"][8]
    assert float(g[3]) == sig[0, 8] and float(g[4]) == sig[nv - 1, 1]
    assert float(g[5]) == dg[nv // 2, 5]


def test_legacy_entry_points_without_tex_outputs():
    """PrintControl 0: only vm.out / err.out, no dumps."""
    case = make_outputs.tex_case()
    d = tempfile.mkdtemp(prefix="outputs_plain_")
    case.write(d, print_control=(0, 1), tex_flag=0)
    exe = build_host(d)
    run = subprocess.run([exe, "input"], cwd=d, capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stderr
    assert not [f for f in os.listdir(d) if f.endswith(".iout")]
    fx = outputs_io.load()
    outputs_io.compare_text(open(os.path.join(d, "vm.out")).read(), fx["vm_out"])
    outputs_io.compare_text(open(os.path.join(d, "err.out")).read(), fx["err_out"])
    shutil.rmtree(d, ignore_errors=True)
