"""The legacy drop-in (include/voce_legacy.h) and the output fixture, without a
GPU: libvoce_legacy.so exports the reference's entry points under C and C++
linkage; the reference's own main program and output code link against it
in place of its solver objects; the test host links; the reference's output
bytes have the layouts the writers of include/voce_io.h produce."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from voce_gb300 import build, capi

import make_outputs
import outputs_io

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# the names the reference's objects bind (C linkage; C++ linkage as its
# mpicxx build mangles them, evp.h:333-380 and kinematics.c prototypes)
LEGACY_SYMBOLS = ["SetupJob", "Evolution", "DestroyJob", "chg_basis", "EulerToTransMatrix",
                  "_Z8SetupJobv", "_Z9Evolutionv", "_Z10DestroyJobv",
                  "_Z9chg_basisPdPA3_dPA6_dPA3_A3_S0_i", "_Z18EulerToTransMatrixPdS_S_PA3_di"]


@pytest.fixture(scope="module")
def legacy_lib(voce_lib):
    if not os.path.exists(capi.LEGACY_LIB_PATH):
        build.build_legacy()
    return capi.LEGACY_LIB_PATH


def test_legacy_library_exports_reference_entry_points(legacy_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", legacy_lib], capture_output=True,
                         text=True, check=True).stdout
    defined = {line.split()[-1] for line in out.splitlines() if line.strip()}
    for s in LEGACY_SYMBOLS:
        assert s in defined, s
    # its only undefined data symbols are the reference program's globals
    und = subprocess.run(["nm", "-D", "-u", legacy_lib], capture_output=True, text=True,
                         check=True).stdout.split()
    for g in ("CellDim", "TimeStep", "fp_vm", "fp_err", "Sig", "SigAvg", "B", "rank"):
        assert g in und, g


def build_host(out_dir: str) -> str:
    exe = os.path.join(out_dir, "host_main")
    lib = os.path.dirname(capi.LIB_PATH)
    subprocess.run(["gcc", "-O2", "-Wall", "-Werror", os.path.join(ROOT, "tests", "legacy", "host_main.c"),
                    "-I" + os.path.join(ROOT, "include"), "-L" + lib, "-lvoce_legacy", "-lvoce_gpu",
                    "-Wl,-rpath," + lib, "-o", exe], check=True)
    return exe


def test_test_host_links(legacy_lib):
    d = tempfile.mkdtemp(prefix="legacy_host_")
    assert os.path.exists(build_host(d))


def test_reference_program_links_against_legacy_library(legacy_lib):
    import oracle
    src = oracle.reference_src()
    if not src:
        pytest.skip("reference sources not present")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "legacy-link",
                    "REF=" + src], check=True)
    for exe in ("evp_gpu_cxx", "evp_gpu_c"):
        assert os.path.exists(os.path.join(ROOT, "oracle", "_ref", exe))


def test_output_fixture_layouts():
    """The reference's own bytes: record sizes, padding, and the integer
    columns (grain ids, 1-based x,y,z with z fastest, phase) the writers
    reproduce."""
    fx = outputs_io.load()
    case = make_outputs.tex_case()
    assert fx["digest"] == case.mesh.digest()
    nx, ny, nz = case.mesh.dims
    nv = nx * ny * nz
    for n, data in fx["files"].items():
        kind = outputs_io.record_kind(n)
        if n.startswith("new_position"):
            assert len(data) == 24 * nv
            continue
        size = {"f8": 8, "sys": 104, "tex": 48}[kind]
        assert len(data) == size * nv, n
        f, ints, pad = outputs_io.split_records(n, data)
        if kind == "sys":
            assert np.array_equal(ints, case.mesh.grain), n
            assert pad == bytes(4 * nv), n
        if kind == "tex":
            ints = ints.reshape(nv, 6)
            x, y, z = np.meshgrid(np.arange(1, nx + 1), np.arange(1, ny + 1), np.arange(1, nz + 1),
                                  indexing="ij")
            assert np.array_equal(ints[:, 0], x.ravel()) and np.array_equal(ints[:, 2], z.ravel())
            assert np.array_equal(ints[:, 1], y.ravel())
            assert np.array_equal(ints[:, 3], case.mesh.grain)
            assert np.array_equal(ints[:, 4], case.mesh.phase) and not ints[:, 5].any()
    # the step and final names the reference used
    assert "els_1_S000003.iout" in fx["files"] and "work_p_S000003.iout" in fx["files"]
    assert "sig_final_1_S0000.iout" in fx["files"] and "work_e_final_S000000.iout" in fx["files"]
    assert fx["vm_out"].startswith("EVM\tEVMP\tDVM\tDVMP\tSVM\tSVMSVM_1\tIteration_tot\n")
    assert fx["err_out"].startswith("IT\tERRE\tERRS\tSVM\nSTEP = 1\n")
