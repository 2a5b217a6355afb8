"""The library's host code under AddressSanitizer and
UndefinedBehaviorSanitizer (no GPU needed): a copy of libvoce_gpu.so built
with both sanitizers in its host code runs the host-side tests of
tests/test_capi_host.py -- the namelist, .sx and mesh readers on valid and
malformed inputs (the chunked decimal parser included, and 300 randomly
edited input files through the readers and creation's host checks), the
footprint, the
rejection of damaged snapshots and the server's queue, cancellation and
deadline handling -- in a child process with the sanitizer runtimes
preloaded.  Any invalid memory access or undefined behaviour stops that
process with a report, and the test fails (leak checking is off: the Python
interpreter that hosts the library keeps memory until exit by design)."""
import os
import shutil
import subprocess
import sys
import tempfile

import pytest

from voce_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import sys
sys.path.insert(0, %(root)r)
sys.path.insert(0, %(tests)r)
from voce_gb300 import capi
lib = capi.load(%(lib)r)
import test_capi_host as t
names = [n for n in dir(t) if n.startswith("test_")]
for n in names:
    f = getattr(t, n)
    if f.__code__.co_argcount:
        f(lib)
    else:
        f()
print("ran", len(names), "host tests under the sanitizers")
"""


def _runtime(name):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        return None
    p = subprocess.run([cc, "-print-file-name=" + name], capture_output=True, text=True).stdout.strip()
    return p if p and os.path.isabs(p) and os.path.exists(p) else None


def test_host_code_under_asan_and_ubsan():
    asan, ubsan = _runtime("libasan.so"), _runtime("libubsan.so")
    if not (asan and ubsan):
        pytest.skip("no sanitizer runtimes")
    try:
        build._nvcc()
    except RuntimeError:
        pytest.skip("no nvcc")
    with tempfile.TemporaryDirectory() as d:
        lib = build.build_sanitized(d)
        if shutil.which("nm"):
            syms = subprocess.run(["nm", "-D", lib], capture_output=True, text=True).stdout
            assert "__asan_" in syms and "__ubsan_" in syms   # the host code is instrumented
        env = dict(os.environ,
                   LD_PRELOAD=asan + ":" + ubsan,
                   ASAN_OPTIONS="detect_leaks=0:verify_asan_link_order=0:halt_on_error=1",
                   UBSAN_OPTIONS="halt_on_error=1:print_stacktrace=1")
        code = CHILD % {"root": ROOT, "tests": os.path.join(ROOT, "tests"), "lib": lib}
        r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                           timeout=900)
        report = r.stdout[-3000:] + r.stderr[-6000:]
        assert r.returncode == 0, report
        assert "AddressSanitizer" not in r.stderr and "runtime error:" not in r.stderr, report
        assert "host tests under the sanitizers" in r.stdout, report
