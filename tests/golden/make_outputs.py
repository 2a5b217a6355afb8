"""Generate the output-file fixture in this directory from the REFERENCE.

Runs oracle/_ref/evp_ref (the unmodified reference sources with the
single-rank MPI / FFTW-2 shims, oracle/Makefile) on a small anisotropic case
with every output switched on -- PrintControl 1 3, Tex_Flag 1 -- and stores
in ``outputs_<case>.npz``:

  digest        hash of the generated mesh (tests regenerate the inputs)
  vm_out        the bytes of vm.out
  err_out       the bytes of err.out
  names         every .iout file the run wrote
  blob, offsets their bytes, concatenated (file i is blob[offsets[i]:offsets[i+1]])

The rho_rss / rho_crss / work_p values are computed from the third increment
on (evolution.c:505-529); the case prints at increment 3, so every stored
value is defined.  Needs the reference sources:
    python tests/golden/make_outputs.py
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
from voce_gb300 import synth  # noqa: E402

REF_BIN = os.path.join(ROOT, "oracle", "_ref", "evp_ref")


def tex_case() -> synth.Case:
    """4 x 6 x 8 voxels, 5 grains, tension z, 3 increments, all outputs."""
    return synth.Case("tex_4x6x8", synth.voronoi_mesh_box((4, 6, 8), 5, 61), synth.CU_LIKE,
                      synth.tension_z(), 0.2, 3)


CASES = {"tex_4x6x8": tex_case}
PRINT_CONTROL = (1, 3)
TEX_FLAG = 1


def run_case(name: str) -> None:
    case = CASES[name]()
    d = tempfile.mkdtemp(prefix="outputs_" + name + "_")
    case.write(d, print_control=PRINT_CONTROL, tex_flag=TEX_FLAG)
    subprocess.run([REF_BIN, "input"], cwd=d, check=True, stdout=subprocess.DEVNULL)
    names = sorted(f for f in os.listdir(d) if f.endswith(".iout"))
    blobs = [open(os.path.join(d, f), "rb").read() for f in names]
    offsets = np.cumsum([0] + [len(b) for b in blobs]).astype(np.int64)
    np.savez_compressed(os.path.join(HERE, "outputs_%s.npz" % name),
                        digest=case.mesh.digest(),
                        vm_out=np.frombuffer(open(os.path.join(d, "vm.out"), "rb").read(), np.uint8),
                        err_out=np.frombuffer(open(os.path.join(d, "err.out"), "rb").read(), np.uint8),
                        names=np.array(names), offsets=offsets,
                        blob=np.frombuffer(b"".join(blobs), np.uint8))
    print(name, len(names), "files", offsets[-1], "bytes")


if __name__ == "__main__":
    for n in sys.argv[1:] or list(CASES):
        run_case(n)
