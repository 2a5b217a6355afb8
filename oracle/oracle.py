"""Python access to the oracle (TEST INFRASTRUCTURE ONLY).

Loads ``oracle/_build/liboracle.so`` (the C restatement, built by
``build_port()`` with gcc on any machine) and, where it was built from the
reference sources, ``oracle/_ref/libevp_ref.so`` / ``oracle/_ref/evp_ref``.
Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
bench.py use this module, as the checker or the timed CPU baseline.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "liboracle.so")
PORT_BIN = os.path.join(HERE, "_build", "evp_oracle")
REF_BIN = os.path.join(HERE, "_ref", "evp_ref")
REF_LIB = os.path.join(HERE, "_ref", "libevp_ref.so")
# where the reference sources lie: given by the caller, by the environment
# variable VOCE_REFERENCE_SRC, or else a directory "reference" beside the
# repository's own directory
REFERENCE_ENV = "VOCE_REFERENCE_SRC"


def reference_src() -> str:
    """The reference source directory, or "" when there is none."""
    src = os.environ.get(REFERENCE_ENV, "")
    if not src:
        src = os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
    return os.path.abspath(src) if os.path.isfile(os.path.join(src, "evolution.c")) else ""

FIELDS = {"sig": (0, 9), "eps": (1, 9), "edot": (2, 9), "disgrad": (3, 9),
          "tranmat": (4, 9), "crss": (5, 12), "gamdot": (6, 12), "gamacum": (7, 1),
          "svm": (8, 1), "evm": (9, 1), "schmid": (10, 60), "cgr": (11, 36)}


def build_port() -> str:
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return PORT_LIB


def build_ref(src: str | None = None) -> bool:
    """Compile the reference sources in directory ``src`` (default:
    reference_src()) with the shims; False when there are none."""
    src = src or reference_src()
    if not src or not os.path.isdir(src):
        return False
    subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + os.path.abspath(src)], check=True)
    return True


class OracleIncr(C.Structure):
    _fields_ = [("istep", C.c_int), ("iters", C.c_int), ("iter_total", C.c_int),
                ("e_vm", C.c_double), ("evmp", C.c_double), ("d_vm", C.c_double),
                ("dvmp", C.c_double), ("s_vm", C.c_double), ("s_vm1", C.c_double),
                ("sig_avg", C.c_double * 9), ("sig_avg1", C.c_double * 9),
                ("eps_avg", C.c_double * 9), ("edot_avg", C.c_double * 9),
                ("disgrad_avg", C.c_double * 9), ("err_e", C.c_double),
                ("err_s", C.c_double)]

    def as_dict(self):
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if hasattr(v, "__len__") else v
        return out


_LIB = None


def lib() -> C.CDLL:
    global _LIB
    if _LIB is None:
        if not os.path.exists(PORT_LIB):
            build_port()
        L = C.CDLL(PORT_LIB)
        L.oracle_create.restype = C.c_void_p
        L.oracle_create.argtypes = [C.c_char_p, C.c_int, C.c_char_p, C.c_char_p]
        L.oracle_destroy.argtypes = [C.c_void_p]
        L.oracle_run.argtypes = [C.c_void_p, C.c_int]
        L.oracle_get_field.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.oracle_get_increment.argtypes = [C.c_void_p, C.c_int, C.POINTER(OracleIncr)]
        L.oracle_get_iter_log.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_nvox.restype = C.c_long
        L.oracle_nvox.argtypes = [C.c_void_p]
        L.oracle_get_reference_medium.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_lu_inv66.argtypes = [C.c_void_p]
        L.oracle_disp_fluct.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        _LIB = L
    return _LIB


class Job:
    """One oracle run of a namelist (reads the same files as the reference)."""

    def __init__(self, namelist: str, threads: int = 1, trace: str | None = None):
        err = C.create_string_buffer(256)
        self._h = lib().oracle_create(namelist.encode(), threads,
                                      trace.encode() if trace else None, err)
        if not self._h:
            raise RuntimeError("oracle: " + err.value.decode())
        self.nv = lib().oracle_nvox(self._h)

    def run(self, n: int) -> None:
        lib().oracle_run(self._h, n)

    def increment(self, k: int) -> dict:
        r = OracleIncr()
        if lib().oracle_get_increment(self._h, k, C.byref(r)) != 0:
            raise IndexError(k)
        return r.as_dict()

    def iter_log(self, k: int):
        n = self.increment(k)["iters"]
        a = np.zeros((3, n))
        lib().oracle_get_iter_log(self._h, k, a[0].ctypes.data, a[1].ctypes.data,
                                  a[2].ctypes.data)
        return a

    def field(self, name: str) -> np.ndarray:
        fid, w = FIELDS[name]
        out = np.zeros((self.nv, w))
        lib().oracle_get_field(self._h, fid, out.ctypes.data)
        return out

    def disp_fluct(self, from_fluct: bool = True) -> np.ndarray:
        """The corrected displacement fluctuation (evolution.c:532-560), from
        the accumulated fluctuation or from DisGrad; (nv, 3)."""
        out = np.zeros((self.nv, 3))
        if lib().oracle_disp_fluct(self._h, 1 if from_fluct else 0, out.ctypes.data) != 0:
            raise MemoryError("oracle_disp_fluct")
        return out

    def reference_medium(self):
        c = np.zeros(36)
        s = np.zeros(36)
        w = C.c_double()
        lib().oracle_get_reference_medium(self._h, c.ctypes.data, s.ctypes.data, C.byref(w))
        return c.reshape(6, 6), s.reshape(6, 6), w.value

    def close(self):
        if self._h:
            lib().oracle_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


TWO_PI_REF = 6.28318530718   # evp.h:58


def ref_freq(n: int) -> np.ndarray:
    """The reference's frequencies of one axis (init.c:660-667): 2 pi
    (i/n - round(i/n)), C's round (halves away from zero, so the Nyquist
    index of an even n gets -pi)."""
    t = np.arange(n) * (1.0 / n)
    r = np.floor(np.abs(t) + 0.5) * np.sign(t)
    return (t - r) * TWO_PI_REF


def disp_fluct_np(grad: np.ndarray, dims) -> np.ndarray:
    """numpy form of oracle_disp_fluct: grad (nv, 9) row-major 3x3 per voxel,
    voxels x slowest; returns (nv, 3) = -Re(IFFT(sum_j i FFT(grad_ij) q_j))/N
    with q = xi/|xi|^2, q(0) = 0."""
    nx, ny, nz = dims
    g = grad.reshape(nx, ny, nz, 3, 3)
    xi = np.meshgrid(ref_freq(nx), ref_freq(ny), ref_freq(nz), indexing="ij")
    s = xi[0] ** 2 + xi[1] ** 2 + xi[2] ** 2
    s[0, 0, 0] = 1.0
    q = [x / s for x in xi]
    for x in q:
        x[0, 0, 0] = 0.0
    out = np.zeros((nx, ny, nz, 3))
    for i in range(3):
        acc = np.zeros((nx, ny, nz), complex)
        for j in range(3):
            acc += 1j * np.fft.fftn(g[..., i, j]) * q[j]
        out[..., i] = -np.fft.ifftn(acc).real
    return out.reshape(-1, 3)
