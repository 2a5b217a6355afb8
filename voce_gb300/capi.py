"""ctypes binding of libvoce_gpu.so (include/voce_gpu.h).

This is the Python mirror of the library's C ABI: the same entry points,
argument meanings and status codes.  It loads the in-tree library built by
``voce_gb300.build`` and fails loudly when it is missing -- there is no
fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libvoce_gpu.so")
LEGACY_LIB_PATH = os.path.join(HERE, "lib", "libvoce_legacy.so")

VOCE_OK = 0
STATUS = {0: "OK", 1: "ERR_ARG", 2: "ERR_IO", 3: "ERR_PARSE", 4: "ERR_BC",
          5: "ERR_SINGULAR", 6: "ERR_UNSUPPORTED", 7: "ERR_NOMEM", 8: "ERR_CUDA",
          9: "ERR_STATE", 10: "ERR_CANCELLED", 11: "ERR_DEADLINE"}
PREC_FP64, PREC_MIXED, PREC_MIXED_NR32, PREC_MIXED_IR = 0, 1, 2, 3
NOALLOC_MAX_DOUBLES = 4194304   # VOCE_NOALLOC_MAX_DOUBLES
# .iout dump kinds (include/voce_io.h)
IOUT = {"eps": 0, "sig": 1, "els": 2, "edot": 3, "slip": 4, "taux": 5, "crss": 6, "tex": 7,
        "svm": 8, "evm": 9, "rho_rss": 10, "rho_crss": 11, "work_p": 12, "work_e": 13,
        "new_position": 14}
FIELD = {"sig": 0, "eps": 1, "edot": 2, "disgrad": 3, "tranmat": 4, "crss": 5,
         "gamdot": 6, "gamacum": 7, "svm": 8, "evm": 9, "gammatotal": 10,
         "taux": 11, "rho_rss": 12, "rho_crss": 13, "work_p": 14, "disp_fluct": 15,
         "sig_voigt": 20, "edot_voigt": 21}
FIELD_WIDTH = {0: 9, 1: 9, 2: 9, 3: 9, 4: 9, 5: 12, 6: 12, 7: 1, 8: 1, 9: 1,
               10: 12, 11: 12, 12: 1, 13: 1, 14: 1, 15: 3, 20: 6, 21: 6}


class VoceNamelist(C.Structure):
    _fields_ = [
        ("CellDim", C.c_int * 3), ("N_phases", C.c_int), ("Type_phases", C.c_int * 2),
        ("TimeStep", C.c_double), ("N_steps", C.c_int),
        ("Update_Flag", C.c_int), ("Hard_Flag", C.c_int), ("Tex_Flag", C.c_int),
        ("IterMax", C.c_int), ("PrintControl", C.c_int * 2), ("Err", C.c_double),
        ("VelGrad_BC_Flag", C.c_int * 6), ("VelGrad_BC", C.c_double * 6),
        ("Stress_BC_Flag", C.c_int * 6), ("Stress_BC", C.c_double * 6),
        ("ElastConst_PhaseI", C.c_double * 4), ("ElastConst_PhaseII", C.c_double * 4),
        ("Slip_PhaseI", C.c_char * 100), ("Slip_PhaseII", C.c_char * 100),
        ("initial_ms", C.c_char * 100),
        ("self", C.c_double * 2), ("coplane", C.c_double * 2), ("cross", C.c_double * 2),
        ("glissile", C.c_double * 2), ("hirth", C.c_double * 2), ("lomer", C.c_double * 2),
    ]


class VoceSlip(C.Structure):
    _fields_ = [
        ("nsys", C.c_int), ("nrs", C.c_double), ("gamd0", C.c_double),
        ("tau0f", C.c_double), ("tau0b", C.c_double), ("tau1", C.c_double),
        ("thet0", C.c_double), ("thet1", C.c_double),
        ("bn", (C.c_double * 3) * 12), ("bb", (C.c_double * 3) * 12),
    ]


class VoceMesh(C.Structure):
    _fields_ = [("dims", C.c_int * 3), ("euler_deg", C.POINTER(C.c_double)),
                ("grain", C.POINTER(C.c_int)), ("phase", C.POINTER(C.c_int))]


class VoceIncrement(C.Structure):
    _fields_ = [
        ("istep", C.c_int), ("iters", C.c_int), ("iter_total", C.c_int), ("nr_max", C.c_int),
        ("e_vm", C.c_double), ("evmp", C.c_double), ("d_vm", C.c_double), ("dvmp", C.c_double),
        ("s_vm", C.c_double), ("s_vm1", C.c_double),
        ("sig_avg", C.c_double * 9), ("sig_avg1", C.c_double * 9),
        ("eps_avg", C.c_double * 9), ("edot_avg", C.c_double * 9),
        ("disgrad_avg", C.c_double * 9), ("err_e", C.c_double), ("err_s", C.c_double),
        ("rot_slip_avg", C.c_double), ("rot_loc_avg", C.c_double),
        ("nr_iters_total", C.c_double),
    ]

    def as_dict(self) -> dict:
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if hasattr(v, "__len__") else v
        return out


# every function declared in include/voce_gpu.h: (name, restype, argtypes)
PROTOTYPES = [
    ("voce_abi_version", C.c_int, []),
    ("voce_last_error", C.c_char_p, []),
    ("voce_namelist_read", C.c_int, [C.c_char_p, C.POINTER(VoceNamelist)]),
    ("voce_slip_read", C.c_int, [C.c_char_p, C.POINTER(VoceSlip)]),
    ("voce_mesh_read", C.c_int, [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                 C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("voce_rve_create", C.c_int, [C.POINTER(VoceNamelist), C.POINTER(C.POINTER(VoceSlip)),
                                  C.POINTER(VoceMesh), C.c_int, C.POINTER(C.c_void_p)]),
    ("voce_rve_create_from_files", C.c_int, [C.c_char_p, C.c_int, C.POINTER(C.c_void_p)]),
    ("voce_rve_run", C.c_int, [C.c_void_p, C.c_int]),
    ("voce_rve_increments_done", C.c_int, [C.c_void_p]),
    ("voce_rve_get_increment", C.c_int, [C.c_void_p, C.c_int, C.POINTER(VoceIncrement)]),
    ("voce_rve_get_iter_log", C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double),
                                        C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int]),
    ("voce_rve_get_iter_detail", C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.c_int]),
    ("voce_rve_get_field", C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double)]),
    ("voce_rve_get_field_noalloc", C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double)]),
    ("voce_rve_write_iout", C.c_int, [C.c_void_p, C.c_int, C.c_char_p, C.c_int]),
    ("voce_rve_write_step_iout", C.c_int, [C.c_void_p, C.c_int, C.c_char_p]),
    ("voce_rve_write_final_iout", C.c_int, [C.c_void_p, C.c_char_p]),
    ("voce_write_log_headers", C.c_int, [C.c_void_p, C.c_void_p]),
    ("voce_rve_write_log", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
    ("voce_rve_get_ids", C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("voce_rve_get_namelist", C.c_int, [C.c_void_p, C.POINTER(VoceNamelist)]),
    ("voce_rve_destroy", C.c_int, [C.c_void_p]),
    ("voce_rve_footprint", C.c_longlong, [C.POINTER(C.c_int), C.c_int]),
    # voce_gpu_diag.h
    ("voce_rve_run_timed", C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double)]),
    ("voce_rve_set_graph", C.c_int, [C.c_void_p, C.c_int]),
    ("voce_rve_set_profiling", C.c_int, [C.c_void_p, C.c_int]),
    ("voce_rve_get_kernel_time", C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double),
                                           C.POINTER(C.c_longlong)]),
    ("voce_rve_reset_kernel_times", C.c_int, [C.c_void_p]),
    ("voce_rve_kernel_launches", C.c_longlong, [C.c_void_p]),
    ("voce_rve_flush_l2", C.c_int, [C.c_void_p, C.c_longlong]),
    ("voce_host_alloc", C.c_void_p, [C.c_longlong]),
    ("voce_host_free", None, [C.c_void_p]),
    ("voce_measure_fp64_tflops", C.c_double, []),
    ("voce_device_memory", C.c_int, [C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
    ("voce_diag_rcp", C.c_int, [C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int]),
    ("voce_diag_sqrt", C.c_int, [C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int]),
    ("voce_diag_fft", C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
    # voce_batch.h
    ("voce_batch_create", C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    ("voce_batch_add", C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    ("voce_batch_remove", C.c_int, [C.c_void_p, C.c_void_p]),
    ("voce_batch_size", C.c_int, [C.c_void_p]),
    ("voce_batch_run", C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int)]),
    ("voce_batch_launch", C.c_int, [C.c_void_p, C.c_int]),
    ("voce_batch_wait", C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    ("voce_batch_ticks", C.c_longlong, [C.c_void_p]),
    ("voce_batch_destroy", C.c_int, [C.c_void_p]),
    # voce_serve.h
    ("voce_server_create", C.c_int, [C.c_int, C.c_longlong, C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
    ("voce_server_submit", C.c_int, [C.c_void_p, C.POINTER(VoceNamelist), C.POINTER(C.POINTER(VoceSlip)),
                                     C.POINTER(VoceMesh), C.c_int, C.POINTER(C.c_longlong)]),
    ("voce_server_poll", C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("voce_server_now", C.c_double, [C.c_void_p]),
    ("voce_server_info", C.c_int, [C.c_void_p, C.c_longlong, C.c_void_p]),
    ("voce_server_result", C.c_int, [C.c_void_p, C.c_longlong, C.c_int, C.POINTER(C.c_double)]),
    ("voce_server_bytes_in_use", C.c_longlong, [C.c_void_p]),
    ("voce_server_destroy", C.c_int, [C.c_void_p]),
    ("voce_batch_set_profiling", C.c_int, [C.c_void_p, C.c_int]),
    ("voce_batch_get_kernel_time", C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double),
                                            C.POINTER(C.c_longlong)]),
    ("voce_batch_reset_kernel_times", C.c_int, [C.c_void_p]),
    ("voce_rve_snapshot_size", C.c_longlong, [C.c_void_p]),
    ("voce_rve_snapshot", C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong]),
    ("voce_rve_restore", C.c_int, [C.c_void_p, C.c_longlong, C.POINTER(C.c_void_p)]),
    ("voce_rve_save", C.c_int, [C.c_void_p, C.c_char_p]),
    ("voce_rve_load", C.c_int, [C.c_char_p, C.POINTER(C.c_void_p)]),
    ("voce_mesh_voronoi", C.c_int, [C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_double),
                                    C.POINTER(C.c_double), C.POINTER(C.c_double),
                                    C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("voce_set_autotune", C.c_int, [C.c_int]),
    ("voce_rve_get_tiles", C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    ("voce_rve_set_tiles", C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    ("voce_fft_schedule_count", C.c_int, [C.c_int]),
    ("voce_rve_fft_schedule_count", C.c_int, [C.c_void_p, C.c_int]),
    ("voce_set_newton_chord", C.c_int, [C.c_int]),
    ("voce_set_ir_predictor", C.c_int, [C.c_int]),
    ("voce_rve_get_fft_schedule", C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.c_int]),
    ("voce_rve_set_fft_schedule", C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    ("voce_server_set_quantum", C.c_int, [C.c_void_p, C.c_int]),
    ("voce_server_set_active_limit", C.c_int, [C.c_void_p, C.c_longlong]),
    ("voce_server_cancel", C.c_int, [C.c_void_p, C.c_longlong]),
    ("voce_server_set_deadline", C.c_int, [C.c_void_p, C.c_longlong, C.c_double]),
]
KERNELS = ["fft_z_fwd", "fft_y_fwd", "fft_x_green", "fft_y_inv", "fft_z_inv", "nr",
           "finalize_iter", "prelude", "incr_fft", "incr_end", "finalize_incr"]

_LIB: Optional[C.CDLL] = None


class VoceError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("%s (%d): %s" % (STATUS.get(code, "?"), code, msg))
        self.code = code


def load(path: str = LIB_PATH) -> C.CDLL:
    """Load libvoce_gpu.so.  Raises if the library has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(path):
        raise RuntimeError("libvoce_gpu.so is not built (%s); run "
                           "`python -m voce_gb300.build`" % path)
    lib = C.CDLL(path)
    for name, res, args in PROTOTYPES:
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _LIB = lib
    return lib


def _check(rc: int) -> None:
    if rc != VOCE_OK:
        raise VoceError(rc, load().voce_last_error().decode(errors="replace"))


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _iptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _mesh_arrays(dims: Sequence[int], euler_deg, grain, phase):
    """The mesh arrays as the C ABI reads them (contiguous float64 Euler
    angles of shape (nv, 3), int32 grain and phase ids of nv each), checked
    against the grid: the library reads 3 nv + 2 nv values through plain
    pointers and cannot check their lengths itself."""
    nv = int(np.prod(dims))
    eul = np.ascontiguousarray(euler_deg, dtype=np.float64)
    gr = np.ascontiguousarray(grain, dtype=np.int32)
    ph = np.ascontiguousarray(phase, dtype=np.int32)
    if eul.size != 3 * nv or gr.size != nv or ph.size != nv:
        raise ValueError("mesh arrays of %d Euler angles, %d grain ids and %d phase ids for a "
                         "%s grid (%d voxels)" % (eul.size, gr.size, ph.size, tuple(dims), nv))
    mesh = VoceMesh()
    mesh.dims = (C.c_int * 3)(*dims)
    mesh.euler_deg = _dptr(eul)
    mesh.grain = _iptr(gr)
    mesh.phase = _iptr(ph)
    return mesh, (eul, gr, ph)


def _slip_pair(slip: "VoceSlip", solid_phase: int):
    if solid_phase not in (0, 1):
        raise ValueError("solid_phase %r: 0 or 1" % (solid_phase,))
    sp = (C.POINTER(VoceSlip) * 2)()
    sp[solid_phase] = C.pointer(slip)
    return sp


def read_namelist(path: str) -> VoceNamelist:
    nl = VoceNamelist()
    _check(load().voce_namelist_read(path.encode(), C.byref(nl)))
    return nl


def read_slip(path: str) -> VoceSlip:
    s = VoceSlip()
    _check(load().voce_slip_read(path.encode(), C.byref(s)))
    return s


def mesh_voronoi(dims: Sequence[int], seeds: np.ndarray, grain_euler_deg: np.ndarray):
    """voce_mesh_voronoi: (euler (nv, 3), grain, phase) of the periodic Voronoi
    tessellation of the grid by `seeds` (n, 3), computed on the GPU."""
    nv = int(np.prod(dims))
    s = np.ascontiguousarray(seeds, dtype=np.float64).reshape(-1, 3)
    ge = np.ascontiguousarray(grain_euler_deg, dtype=np.float64)
    if ge.size != s.size:
        raise ValueError("%d seeds and %d grain orientations" % (len(s), ge.size // 3))
    eul = np.zeros((nv, 3))
    grain = np.zeros(nv, dtype=np.int32)
    phase = np.zeros(nv, dtype=np.int32)
    d = (C.c_int * 3)(*dims)
    _check(load().voce_mesh_voronoi(d, len(s), _dptr(s), _dptr(ge), _dptr(eul), _iptr(grain), _iptr(phase)))
    return eul, grain, phase


def read_mesh(path: str, dims: Sequence[int]):
    nv = int(np.prod(dims))
    eul = np.zeros((nv, 3))
    grain = np.zeros(nv, dtype=np.int32)
    phase = np.zeros(nv, dtype=np.int32)
    d = (C.c_int * 3)(*dims)
    _check(load().voce_mesh_read(path.encode(), d, _dptr(eul), _iptr(grain), _iptr(phase)))
    return eul, grain, phase


def footprint(dims: Sequence[int], precision: int = PREC_FP64) -> int:
    return int(load().voce_rve_footprint((C.c_int * 3)(*dims), precision))


def device_memory():
    """(free, total) bytes of the current device."""
    f, t = C.c_longlong(), C.c_longlong()
    _check(load().voce_device_memory(C.byref(f), C.byref(t)))
    return int(f.value), int(t.value)


def diag_sqrt(x: np.ndarray) -> np.ndarray:
    """The mixed_ir norms' device square root (voce_diag_sqrt) of every value of x."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    _check(load().voce_diag_sqrt(_dptr(x), _dptr(out), x.size))
    return out


def diag_rcp(x: np.ndarray) -> np.ndarray:
    """The library's device reciprocal (voce_diag_rcp) of every value of x."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    _check(load().voce_diag_rcp(_dptr(x), _dptr(out), x.size))
    return out


def diag_fft(x: np.ndarray, sign: int = -1, schedule: int = 0) -> np.ndarray:
    """The single-precision line FFT of the spectrum passes (voce_diag_fft)
    of every row of the complex array x [nlines, L], unnormalised."""
    x = np.ascontiguousarray(x, dtype=np.complex128)
    out = np.empty_like(x)
    _check(load().voce_diag_fft(x.shape[1], x.shape[0], sign, schedule, x.ctypes.data, out.ctypes.data))
    return out


class Rve:
    """One RVE resident on the GPU (the handle of include/voce_gpu.h)."""

    def __init__(self, handle: C.c_void_p, dims):
        self._h = handle
        self.dims = tuple(dims)
        self.nv = int(np.prod(self.dims))

    @classmethod
    def from_files(cls, namelist_path: str, precision: int = PREC_FP64) -> "Rve":
        lib = load()
        h = C.c_void_p()
        _check(lib.voce_rve_create_from_files(namelist_path.encode(), precision, C.byref(h)))
        nl = read_namelist(namelist_path)
        return cls(h, tuple(nl.CellDim))

    @classmethod
    def create(cls, nl: VoceNamelist, slip: VoceSlip, euler_deg: np.ndarray,
               grain: np.ndarray, phase: np.ndarray, precision: int = PREC_FP64,
               solid_phase: int = 0) -> "Rve":
        lib = load()
        mesh, keep = _mesh_arrays(tuple(nl.CellDim), euler_deg, grain, phase)
        sp = _slip_pair(slip, solid_phase)
        h = C.c_void_p()
        _check(lib.voce_rve_create(C.byref(nl), sp, C.byref(mesh), precision, C.byref(h)))
        return cls(h, tuple(nl.CellDim))

    def run(self, n: int) -> None:
        _check(load().voce_rve_run(self._h, n))

    @property
    def increments_done(self) -> int:
        return load().voce_rve_increments_done(self._h)

    def increment(self, k: int) -> dict:
        r = VoceIncrement()
        _check(load().voce_rve_get_increment(self._h, k, C.byref(r)))
        return r.as_dict()

    def iter_log(self, k: int, max_iters: int = 100000):
        ee = np.zeros(max_iters)
        es = np.zeros(max_iters)
        sv = np.zeros(max_iters)
        n = load().voce_rve_get_iter_log(self._h, k, _dptr(ee), _dptr(es), _dptr(sv), max_iters)
        if n < 0:
            _check(-n)
        return ee[:n], es[:n], sv[:n]

    def run_timed(self, n: int) -> float:
        """Run n increments; returns device milliseconds between CUDA events
        recorded on the RVE's stream before and after."""
        ms = C.c_double()
        _check(load().voce_rve_run_timed(self._h, n, C.byref(ms)))
        return ms.value

    def set_graph(self, on: bool) -> None:
        _check(load().voce_rve_set_graph(self._h, int(on)))

    def set_profiling(self, on: bool) -> None:
        _check(load().voce_rve_set_profiling(self._h, int(on)))

    def kernel_times(self) -> dict:
        out = {}
        for k, name in enumerate(KERNELS):
            ms = C.c_double()
            n = C.c_longlong()
            _check(load().voce_rve_get_kernel_time(self._h, k, C.byref(ms), C.byref(n)))
            out[name] = (ms.value, n.value)
        return out

    def reset_kernel_times(self) -> None:
        _check(load().voce_rve_reset_kernel_times(self._h))

    @property
    def kernel_launches(self) -> int:
        return int(load().voce_rve_kernel_launches(self._h))

    def flush_l2(self, nbytes: int = 512 << 20) -> None:
        _check(load().voce_rve_flush_l2(self._h, nbytes))

    def iter_detail(self, k: int, max_iters: int = 100000) -> np.ndarray:
        """Rows of 12 per iteration: err_e, err_s, s_vm, newton_sum,
        sum_conv_e, sum_conv_s, sum of the stress 6-vector (6)."""
        rows = np.zeros((max_iters, 12))
        n = load().voce_rve_get_iter_detail(self._h, k, _dptr(rows), max_iters)
        if n < 0:
            _check(-n)
        return rows[:n]

    def field(self, name: str) -> np.ndarray:
        fid = FIELD[name]
        w = FIELD_WIDTH[fid]
        out = np.zeros(self.nv * w)
        _check(load().voce_rve_get_field(self._h, fid, _dptr(out)))
        if fid in (20, 21):
            return out.reshape(w, self.nv)
        return out.reshape(self.nv, w)

    def field_noalloc(self, name: str) -> np.ndarray:
        """field() through voce_rve_get_field_noalloc: staged in the library's
        fixed device array, no device allocation; VoceError ERR_UNSUPPORTED
        when the field has more than NOALLOC_MAX_DOUBLES values."""
        fid = FIELD[name]
        w = FIELD_WIDTH[fid]
        out = np.zeros(self.nv * w)
        _check(load().voce_rve_get_field_noalloc(self._h, fid, _dptr(out)))
        if fid in (20, 21):
            return out.reshape(w, self.nv)
        return out.reshape(self.nv, w)

    def ids(self):
        """Grain and phase id of every voxel."""
        g = np.zeros(self.nv, dtype=np.int32)
        p = np.zeros(self.nv, dtype=np.int32)
        _check(load().voce_rve_get_ids(self._h, _iptr(g), _iptr(p)))
        return g, p

    def namelist(self) -> "VoceNamelist":
        nl = VoceNamelist()
        _check(load().voce_rve_get_namelist(self._h, C.byref(nl)))
        return nl

    def write_iout(self, kind: str, name: str, step: int) -> None:
        _check(load().voce_rve_write_iout(self._h, IOUT[kind], name.encode(), step))

    def write_step_iout(self, istep: int, directory: str = "") -> None:
        _check(load().voce_rve_write_step_iout(self._h, istep, directory.encode()))

    def write_final_iout(self, directory: str = "") -> None:
        _check(load().voce_rve_write_final_iout(self._h, directory.encode()))

    def write_logs(self, directory: str, n_steps: int) -> None:
        """vm.out and err.out of every finished increment, as the reference
        writes them for a run of n_steps increments."""
        libc = C.CDLL(None)
        libc.fopen.restype = C.c_void_p
        libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
        libc.fclose.argtypes = [C.c_void_p]
        vm = libc.fopen(os.path.join(directory, "vm.out").encode(), b"w+")
        err = libc.fopen(os.path.join(directory, "err.out").encode(), b"w+")
        if not vm or not err:
            raise OSError("cannot open vm.out / err.out in " + directory)
        try:
            _check(load().voce_write_log_headers(vm, err))
            for k in range(self.increments_done):
                _check(load().voce_rve_write_log(self._h, k, n_steps, vm, err))
        finally:
            libc.fclose(vm)
            libc.fclose(err)

    def tiles(self) -> list:
        """FFT tiles (lines per block): z forward, y, x/Green, z inverse, and
        the two antisymmetric back-transform tiles."""
        t = (C.c_int * 6)()
        _check(load().voce_rve_get_tiles(self._h, t))
        return list(t)

    def set_tiles(self, tiles) -> None:
        _check(load().voce_rve_set_tiles(self._h, (C.c_int * 6)(*tiles)))

    def fft_schedule_count(self, axis: int) -> int:
        """Transform candidates of axis (0 x, 1 y, 2 z) of this RVE."""
        n = load().voce_rve_fft_schedule_count(self._h, axis)
        if n < 0:
            _check(-n)
        return n

    def fft_schedule(self, axis: int) -> list:
        """Radices of axis (0 x, 1 y, 2 z) in stage order (the register FFT:
        its two lengths N1, N2)."""
        buf = (C.c_int * 16)()
        n = load().voce_rve_get_fft_schedule(self._h, axis, buf, 16)
        if n < 0:
            _check(-n)
        return list(buf[:n])

    def set_fft_schedule(self, axis: int, k: int) -> None:
        _check(load().voce_rve_set_fft_schedule(self._h, axis, k))

    def snapshot(self) -> bytes:
        """The RVE's whole state as bytes (voce_rve_snapshot)."""
        n = load().voce_rve_snapshot_size(self._h)
        if n < 0:
            _check(-n)
        buf = C.create_string_buffer(n)
        _check(load().voce_rve_snapshot(self._h, buf, n))
        return buf.raw

    @classmethod
    def restore(cls, blob: bytes) -> "Rve":
        h = C.c_void_p()
        _check(load().voce_rve_restore(blob, len(blob), C.byref(h)))
        r = cls(h, (0, 0, 0))
        r.dims = tuple(r.namelist().CellDim)
        r.nv = int(np.prod(r.dims))
        return r

    def save(self, path: str) -> None:
        _check(load().voce_rve_save(self._h, path.encode()))

    @classmethod
    def restore_file(cls, path: str) -> "Rve":
        """A handle from a file written by save (voce_rve_load)."""
        h = C.c_void_p()
        _check(load().voce_rve_load(path.encode(), C.byref(h)))
        r = cls(h, (0, 0, 0))
        r.dims = tuple(r.namelist().CellDim)
        r.nv = int(np.prod(r.dims))
        return r

    def close(self) -> None:
        if self._h:
            load().voce_rve_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many RVEs advanced together (include/voce_batch.h)."""

    def __init__(self, precision: int = PREC_FP64):
        h = C.c_void_p()
        _check(load().voce_batch_create(precision, C.byref(h)))
        self._h = h
        self.members = []

    def add(self, rve: Rve, n_increments: int) -> None:
        _check(load().voce_batch_add(self._h, rve._h, n_increments))
        self.members.append(rve)

    def remove(self, rve: Rve) -> None:
        _check(load().voce_batch_remove(self._h, rve._h))
        self.members.remove(rve)

    def run(self, max_ticks: int = 1 << 30) -> int:
        left = C.c_int()
        _check(load().voce_batch_run(self._h, max_ticks, C.byref(left)))
        return left.value

    def launch(self, max_ticks: int = 1 << 30) -> None:
        """Enqueue up to max_ticks ticks and return (voce_batch_launch)."""
        _check(load().voce_batch_launch(self._h, max_ticks))

    def wait(self) -> int:
        """Wait for launched ticks; RVEs with increments left (voce_batch_wait)."""
        left = C.c_int()
        _check(load().voce_batch_wait(self._h, C.byref(left)))
        return left.value

    @property
    def ticks(self) -> int:
        return int(load().voce_batch_ticks(self._h))

    def set_profiling(self, on: bool) -> None:
        """Host-driven ticks with every launch timed (same results)."""
        _check(load().voce_batch_set_profiling(self._h, int(on)))

    def kernel_times(self) -> dict:
        """{kernel name: (milliseconds, launches)} since the last reset."""
        out = {}
        for k, name in enumerate(KERNELS):
            ms = C.c_double()
            n = C.c_longlong()
            _check(load().voce_batch_get_kernel_time(self._h, k, C.byref(ms), C.byref(n)))
            out[name] = (ms.value, n.value)
        return out

    def reset_kernel_times(self) -> None:
        _check(load().voce_batch_reset_kernel_times(self._h))

    def close(self) -> None:
        if self._h:
            load().voce_batch_destroy(self._h)
            self._h = None
            self.members = []

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class RequestInfo(C.Structure):
    _fields_ = [("id", C.c_longlong), ("status", C.c_int), ("error", C.c_int),
                ("increments_done", C.c_int), ("increments_wanted", C.c_int),
                ("dims", C.c_int * 3), ("t_submit", C.c_double), ("t_admit", C.c_double),
                ("t_done", C.c_double), ("voxel_iterations", C.c_longlong),
                ("last", VoceIncrement), ("preemptions", C.c_int), ("t_deadline", C.c_double)]


REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED, REQ_CANCELLED = 0, 1, 2, 3, 4
ERR_CANCELLED, ERR_DEADLINE = 10, 11


class Server:
    """Continuous-batching request server (include/voce_serve.h)."""

    def __init__(self, precision: int = PREC_FP64, hbm_budget: int = 64 << 30,
                 ticks_per_round: int = 8, keep_fields: bool = False):
        h = C.c_void_p()
        _check(load().voce_server_create(precision, hbm_budget, ticks_per_round,
                                         int(keep_fields), C.byref(h)))
        self._h = h

    def submit(self, nl: VoceNamelist, slip: VoceSlip, euler_deg, grain, phase,
               n_increments: int, solid_phase: int = 0) -> int:
        mesh, keep = _mesh_arrays(tuple(nl.CellDim), euler_deg, grain, phase)
        sp = _slip_pair(slip, solid_phase)
        rid = C.c_longlong()
        _check(load().voce_server_submit(self._h, C.byref(nl), sp, C.byref(mesh), n_increments,
                                         C.byref(rid)))
        return rid.value

    def set_quantum(self, ticks: int) -> None:
        _check(load().voce_server_set_quantum(self._h, ticks))

    def set_active_limit(self, voxels: int) -> None:
        """Admit only while the admitted requests hold at most this many
        voxels (0: no limit)."""
        _check(load().voce_server_set_active_limit(self._h, int(voxels)))

    def cancel(self, rid: int) -> None:
        """End a queued or running request; its device memory is freed."""
        _check(load().voce_server_cancel(self._h, rid))

    def set_deadline(self, rid: int, t: float) -> None:
        """Server time (now()'s clock) by which the request must be done;
        0 clears it."""
        _check(load().voce_server_set_deadline(self._h, rid, float(t)))

    def poll(self):
        run = C.c_int()
        que = C.c_int()
        _check(load().voce_server_poll(self._h, C.byref(run), C.byref(que)))
        return run.value, que.value

    def now(self) -> float:
        return load().voce_server_now(self._h)

    def info(self, rid: int) -> RequestInfo:
        out = RequestInfo()
        _check(load().voce_server_info(self._h, rid, C.byref(out)))
        return out

    def result(self, rid: int, which: str, nv: int) -> np.ndarray:
        out = np.zeros(6 * nv)
        _check(load().voce_server_result(self._h, rid, FIELD[which], _dptr(out)))
        return out.reshape(6, nv)

    @property
    def bytes_in_use(self) -> int:
        return int(load().voce_server_bytes_in_use(self._h))

    def close(self) -> None:
        if self._h:
            load().voce_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
