"""An RVE holds the device memory voce_rve_footprint (include/voce_gpu.h)
counts, which is what the server admits requests by: the per-voxel state,
the spectrum arrays and, in the FP64 form, the stored Green-operator
frequencies.  Set-up's staging arrays (the Euler angles, the tuner's saved
stress) are gone once creation returns; what remains beyond the footprint is
a few small tables and the allocator's rounding of each array."""
import os
import tempfile

import numpy as np
import pytest

from voce_gb300 import capi, synth

pytestmark = pytest.mark.gpu

DIMS = (96, 96, 96)


def _inputs():
    case = synth.small_case(8, 2, 51, n_steps=1)
    nl_path = case.write(tempfile.mkdtemp(prefix="footprint_"))
    nl = capi.read_namelist(nl_path)
    nl.CellDim[0], nl.CellDim[1], nl.CellDim[2] = DIMS
    slip = capi.read_slip(os.path.join(os.path.dirname(nl_path), "mat.sx"))
    nv = int(np.prod(DIMS))
    rng = np.random.Generator(np.random.PCG64(51))
    eul = np.repeat(synth.so3_uniform_bunge(rng, 8), nv // 8, axis=0)
    grain = np.repeat(np.arange(1, 9, dtype=np.int32), nv // 8)
    phase = np.ones(nv, dtype=np.int32)
    return nl, slip, eul, grain, phase


@pytest.mark.parametrize("prec", [capi.PREC_FP64, capi.PREC_MIXED_IR])
def test_rve_holds_its_footprint(prec):
    nl, slip, eul, grain, phase = _inputs()
    # the first RVE of the shape loads the modules and times the FFT tiles
    with capi.Rve.create(nl, slip, eul, grain, phase, prec):
        pass
    free0, _ = capi.device_memory()
    with capi.Rve.create(nl, slip, eul, grain, phase, prec):
        free1, _ = capi.device_memory()
    fp = capi.footprint(DIMS, prec)
    held = free0 - free1
    # at most 40 arrays, each rounded up by the allocator (by 2 MiB at
    # most), and tables of a few MB
    assert fp <= held <= fp + (96 << 20), (held, fp)
