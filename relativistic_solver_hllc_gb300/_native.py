"""ctypes binding of librts_scatter.so (include/rts_scatter.h).

The product path is the native library; this module only marshals numpy
arrays into the C ABI.  It never computes anything itself: if the library is
missing or was built for another machine, loading fails loudly.
"""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import numpy as np

from .build import INCLUDE, LIB_PATH

OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_CUDA = 2
ERR_OUT_OF_MEMORY = 3
ERR_BAD_STATE = 4
ERR_TIMEOUT = 5
ERR_OVER_BUDGET = 6
ERR_UNSUPPORTED = 7
ERR_DEVICE_WAIT = 8

STATUS_NAMES = {
    OK: "RTS_OK",
    ERR_INVALID_ARGUMENT: "RTS_ERR_INVALID_ARGUMENT",
    ERR_CUDA: "RTS_ERR_CUDA",
    ERR_OUT_OF_MEMORY: "RTS_ERR_OUT_OF_MEMORY",
    ERR_BAD_STATE: "RTS_ERR_BAD_STATE",
    ERR_TIMEOUT: "RTS_ERR_TIMEOUT",
    ERR_OVER_BUDGET: "RTS_ERR_OVER_BUDGET",
    ERR_UNSUPPORTED: "RTS_ERR_UNSUPPORTED",
    ERR_DEVICE_WAIT: "RTS_ERR_DEVICE_WAIT",
}

STREAM_SCATTERING_1 = 0
STREAM_SCATTERING_2 = 1
STREAM_PARAMS = 2

PHASE_THOMSON = 0
PHASE_HG = 1
PHASE_CUSTOM = 2

PREC_FP64 = 0
PREC_BF16X3 = 1
PREC_FP16X3 = 2
PREC_TF32X3 = 3

PRECISIONS = {"fp64": PREC_FP64, "bf16x3": PREC_BF16X3, "fp16x3": PREC_FP16X3, "tf32x3": PREC_TF32X3}


class RtsError(RuntimeError):
    def __init__(self, status: int, where: str, message: str = ""):
        self.status = status
        name = STATUS_NAMES.get(status, str(status))
        super().__init__(f"{where}: {name}" + (f": {message}" if message else ""))


TUNE_FLUSH = 1  # RTS_TUNE_FLUSH
TUNE_BIAS = 2   # RTS_TUNE_BIAS
TUNE_SERVE_POLICY = 3  # RTS_TUNE_SERVE_POLICY
TUNE_SERVE_BUDGET = 4  # RTS_TUNE_SERVE_BUDGET
TUNE_SERVE_SLACK = 5  # RTS_TUNE_SERVE_SLACK
TUNE_SWEEP_CACHE = 6  # RTS_TUNE_SWEEP_CACHE

_dp = C.POINTER(C.c_double)
_i64 = C.c_int64
_vp = C.c_void_p

# name -> (restype, argtypes)
_SIGNATURES = {
    "rts_abi_version": (C.c_int, []),
    "rts_ctx_create": (C.c_int, [C.c_int, C.POINTER(_vp)]),
    "rts_ctx_destroy": (C.c_int, [_vp]),
    "rts_last_error": (C.c_char_p, [_vp]),
    "rts_set_hbm_budget": (C.c_int, [_vp, _i64]),
    "rts_hbm_used": (C.c_int, [_vp, C.POINTER(_i64)]),
    "rts_init": (C.c_int, [_vp, _dp, _dp, _i64, C.c_double, _i64, _i64, _i64]),
    "rts_host_illum": (C.c_int, [_vp, C.POINTER(_dp)]),
    "rts_host_scattering": (C.c_int, [_vp, C.POINTER(_dp)]),
    "rts_set_phase": (C.c_int, [_vp, C.c_int, C.c_double]),
    "rts_set_weights": (C.c_int, [_vp, _dp]),
    "rts_send_illum_async": (C.c_int, [_vp, _i64, _i64, _i64, _dp]),
    "rts_copy_illum": (C.c_int, [_vp, _i64, _dp]),
    "rts_set_precision": (C.c_int, [_vp, C.c_int]),
    "rts_get_precision": (C.c_int, [_vp, C.POINTER(C.c_int)]),
    "rts_scattering_async": (C.c_int, [_vp, _i64, _i64, C.c_int, _dp]),
    "rts_scattering": (C.c_int, [_vp, _dp, _dp]),
    "rts_read_scattering": (C.c_int, [_vp, _i64, _i64, C.c_int, _dp]),
    "rts_scattering_update": (C.c_int, [_vp, C.c_int, _dp, _dp, C.c_double, _dp]),
    "rts_send_scattering": (C.c_int, [_vp, _i64, _i64, C.c_int, _dp]),
    "rts_device_arrays": (C.c_int, [_vp, C.POINTER(_dp), C.POINTER(_dp)]),
    "rts_moments": (C.c_int, [_vp, C.c_int, _dp, _dp]),
    "rts_set_geometry": (C.c_int, [_vp, _dp, _dp, _dp]),
    "rts_illum_params": (C.c_int, [_vp, C.c_int, _dp, _dp, _dp, _dp, _dp]),
    "rts_write_solution": (C.c_int, [_vp, C.c_char_p]),
    "rts_source_update": (C.c_int, [_vp, _dp, C.c_double, _i64, _i64, C.c_int, _dp]),
    "rts_sync_stream": (C.c_int, [_vp, C.c_int, _i64]),
    "rts_wait": (C.c_int, [_vp, _i64]),
    "rts_solve_setup": (C.c_int, [_vp, C.c_int, _dp, C.c_double]),
    "rts_solve_step": (C.c_int, [_vp, C.c_int, _dp]),
    "rts_solve_step_async": (C.c_int, [_vp, C.c_int]),
    "rts_solve_residual": (C.c_int, [_vp, _dp]),
    "rts_solve_residual_history": (C.c_int, [_vp, _dp, _i64]),
    "rts_read_illum": (C.c_int, [_vp, _i64, _dp]),
    "rts_solve_read": (C.c_int, [_vp, _dp]),
    "rts_solve_read_ibar": (C.c_int, [_vp, _dp]),
    "rts_synth_illum": (C.c_int, [_vp, C.c_uint64, C.c_double, C.c_double, C.c_int]),
    "rts_synth_directions": (C.c_int, [_i64, _dp, _dp, _dp]),
    "rts_synth_uniform": (C.c_int, [C.c_uint64, C.c_uint64, C.c_double, C.c_double, _i64, _i64, _dp]),
    "rts_read_direction_file": (C.c_int, [C.c_char_p, _i64, C.POINTER(_i64), _dp, _dp, _dp]),
    "rts_write_direction_file": (C.c_int, [C.c_char_p, _i64, _dp, _dp, C.c_double]),
    "rts_read_simple_bin": (C.c_int, [C.c_char_p, _i64, _i64, _vp, C.POINTER(_i64)]),
    "rts_write_simple_bin": (C.c_int, [C.c_char_p, _i64, _i64, _vp]),
    "rts_partition": (C.c_int, [C.c_int, _i64, C.POINTER(_i64), C.POINTER(_i64)]),
    "rts_set_tuning": (C.c_int, [_vp, C.c_int, C.c_int]),
    "rts_flush_period": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_int)]),
    "rts_autotune": (C.c_int, [_vp, _i64, C.c_int, C.c_int, _i64, C.POINTER(C.c_int), _dp, C.POINTER(C.c_int), _dp,
                               C.c_int, C.POINTER(C.c_int)]),
    "rts_autotune_schedule": (C.c_int, [_vp, _i64, C.c_int, _i64, _vp, _vp, C.c_int, C.POINTER(C.c_int)]),
    "rts_autotune_save": (C.c_int, [_vp, C.c_char_p]),
    "rts_autotune_load": (C.c_int, [_vp, C.c_char_p]),
    "rts_stream_handle": (C.c_int, [_vp, C.c_int, C.POINTER(_vp)]),
    "rts_launch_count": (C.c_int, [_vp, C.POINTER(_i64)]),
    "rts_measure_fp64_peak": (C.c_int, [_vp, C.c_double, _dp]),
    "rts_measure_link": (C.c_int, [_vp, _i64, C.c_int, _dp, _dp, _dp]),
    "rts_kernel_timing": (C.c_int, [_vp, C.c_int, _dp, C.POINTER(_i64)]),
    "rts_mesh_cube": (C.c_int, [C.c_int, C.c_int, C.c_int, _dp, _vp, _dp]),
    "rts_sweep_set_mesh": (C.c_int, [_vp, _dp, _vp, _dp]),
    "rts_sweep_build": (C.c_int, [_vp, C.POINTER(_i64), C.POINTER(_i64)]),
    "rts_sweep_import_direction": (C.c_int, [_vp, _i64, _vp, _vp, _vp, _i64]),
    "rts_sweep_export_direction": (C.c_int, [_vp, _i64, _vp, _vp, _vp, _i64, C.POINTER(_i64)]),
    "rts_sweep_set_medium": (C.c_int, [_vp, _vp, _dp, _dp, _dp, _dp]),
    "rts_sweep_medium_gas": (C.c_int, [_i64, _dp, _dp, _dp, _dp, _dp, _vp]),
    "rts_sweep": (C.c_int, [_vp, C.c_int, _dp]),
    "rts_sweep_exp_check": (C.c_int, [_vp, _i64, _dp]),
    "rts_illum_solve": (C.c_int, [_vp, C.c_int, C.c_int, C.c_double, C.POINTER(_i64), _dp]),
}

BOUND_FREE, BOUND_LOCK, BOUND_OUTSOURCE, BOUND_INNER = -1, -2, -3, -4
MEDIUM_SCATTERING = 0
MEDIUM_ABSORPTION = 1


class Medium(C.Structure):
    """rts_medium: GetCurIllum's medium (see include/rts_scatter.h)."""
    _fields_ = [("mode", C.c_int), ("reserved", C.c_int), ("s_scale", C.c_double), ("i_scale", C.c_double),
                ("ball", C.c_double * 3), ("radius", C.c_double), ("ball_alpha", C.c_double),
                ("ball_beta", C.c_double), ("ball_q", C.c_double)]


def medium(mode=MEDIUM_SCATTERING, s_scale=1.0, i_scale=1.0, ball=(0.0, 0.0, 0.0), radius=0.0,
           ball_coef=(0.0, 0.0, 0.0)) -> Medium:
    m = Medium()
    m.mode, m.s_scale, m.i_scale = mode, s_scale, i_scale
    m.ball[:] = list(ball)
    m.radius = radius
    m.ball_alpha, m.ball_beta, m.ball_q = ball_coef
    return m


def medium_gas(density, pressure):
    """Class 11 of GetCurIllum: (Medium, alpha, beta, Q) from the gas density
    and pressure per cell (code units); host only."""
    d = np.ascontiguousarray(density, dtype=np.float64)
    p = np.ascontiguousarray(pressure, dtype=np.float64)
    n = d.size
    a, b, q = np.empty(n), np.empty(n), np.empty(n)
    md = Medium()
    _status(load_library().rts_sweep_medium_gas(n, _ptr(d), _ptr(p), _ptr(a), _ptr(b), _ptr(q), C.byref(md)),
            "rts_sweep_medium_gas")
    return md, a, b, q


# byte layout of the reference's cell_local records (LocX0<k>.bin)
LOCX0_DTYPE = np.dtype({"names": ["s", "x0", "in_face_id"], "formats": [np.float64, (np.float64, 2), np.uint8],
                        "offsets": [0, 8, 24], "itemsize": 32})


def synth_directions(M: int):
    """Spherical Fibonacci directions (xyz [M][3], area [M], full_area)."""
    lib = load_library()
    xyz = np.empty(3 * M)
    area = np.empty(M)
    fa = C.c_double()
    rc = lib.rts_synth_directions(int(M), _ptr(xyz), _ptr(area), C.byref(fa))
    if rc != OK:
        raise RtsError(rc, "rts_synth_directions")
    return xyz.reshape(M, 3), area, fa.value


def _status(rc: int, where: str):
    if rc != OK:
        raise RtsError(rc, where)


def read_direction_file(path):
    """(xyz [M][3], area [M], full_area) from a direction-set text file."""
    lib = load_library()
    M = _i64()
    _status(lib.rts_read_direction_file(str(path).encode(), 0, C.byref(M), None, None, None), "rts_read_direction_file")
    xyz = np.empty(3 * M.value)
    area = np.empty(M.value)
    fa = C.c_double()
    _status(lib.rts_read_direction_file(str(path).encode(), M.value, C.byref(M), _ptr(xyz), _ptr(area), C.byref(fa)),
            "rts_read_direction_file")
    return xyz.reshape(-1, 3), area, fa.value


def write_direction_file(path, xyz, area, full_area: float):
    xyz = _f64(xyz)
    area = _f64(area)
    _status(load_library().rts_write_direction_file(str(path).encode(), area.size, _ptr(xyz), _ptr(area),
                                                    float(full_area)), "rts_write_direction_file")


def read_simple_bin(path, dtype=np.float64) -> np.ndarray:
    lib = load_library()
    dt = np.dtype(dtype)
    n = _i64()
    _status(lib.rts_read_simple_bin(str(path).encode(), dt.itemsize, 0, None, C.byref(n)), "rts_read_simple_bin")
    out = np.empty(n.value, dtype=dt)
    _status(lib.rts_read_simple_bin(str(path).encode(), dt.itemsize, n.value, out.ctypes.data_as(_vp), C.byref(n)),
            "rts_read_simple_bin")
    return out


def write_simple_bin(path, data: np.ndarray):
    a = np.ascontiguousarray(data)
    _status(load_library().rts_write_simple_bin(str(path).encode(), a.dtype.itemsize, a.size, a.ctypes.data_as(_vp)),
            "rts_write_simple_bin")


def mesh_cube(n: int, bound_rule: int = 1, tilt: bool = True):
    """Synthetic tetrahedral mesh of the unit cube (host only): vert [N][4][3],
    pairs [N][4] int32, normals [N][4][3]."""
    N = 6 * n * n * n
    vert = np.empty((N, 4, 3))
    pairs = np.empty((N, 4), dtype=np.int32)
    normals = np.empty((N, 4, 3))
    _status(load_library().rts_mesh_cube(int(n), int(bound_rule), int(tilt), _ptr(vert), pairs.ctypes.data,
                                         _ptr(normals)), "rts_mesh_cube")
    return vert, pairs, normals


def partition(np_: int, n: int):
    s = (C.c_int64 * np_)()
    d = (C.c_int64 * np_)()
    _status(load_library().rts_partition(int(np_), int(n), s, d), "rts_partition")
    return list(s), list(d)


def synth_uniform(seed: int, stream: int, lo: float, hi: float, n: int, i0: int = 0) -> np.ndarray:
    lib = load_library()
    out = np.empty(n)
    rc = lib.rts_synth_uniform(C.c_uint64(seed), C.c_uint64(stream), float(lo), float(hi), int(i0), int(n), _ptr(out))
    if rc != OK:
        raise RtsError(rc, "rts_synth_uniform")
    return out

class TuneChoice(C.Structure):
    """rts_tune_choice"""
    _fields_ = [("M", C.c_int64), ("precision", C.c_int), ("flush", C.c_int), ("bn", C.c_int), ("order", C.c_int),
                ("bucket", C.c_int), ("ms", C.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class ProblemDesc(C.Structure):
    """rts_problem_desc"""
    _fields_ = [("N", C.c_int64), ("M", C.c_int64), ("groups", C.c_int64), ("phase", C.c_int), ("g", C.c_double),
                ("precision", C.c_int), ("flush", C.c_int), ("bn", C.c_int)]


_SIGNATURES.update({
    "rts_problem_footprint": (C.c_int, [C.POINTER(ProblemDesc), C.POINTER(_i64)]),
    "rts_batch_create": (C.c_int, [_vp, C.POINTER(_vp)]),
    "rts_batch_destroy": (C.c_int, [_vp]),
    "rts_batch_add": (C.c_int, [_vp, C.POINTER(ProblemDesc), C.POINTER(C.c_float), C.POINTER(C.c_float), _dp,
                                C.POINTER(_i64)]),
    "rts_batch_remove": (C.c_int, [_vp, _i64]),
    "rts_batch_size": (C.c_int, [_vp, C.POINTER(_i64), C.POINTER(_i64)]),
    "rts_batch_step": (C.c_int, [_vp, C.c_int]),
    "rts_batch_capture": (C.c_int, [_vp, C.c_int, C.c_int]),
    "rts_batch_replay": (C.c_int, [_vp]),
    "rts_batch_sync": (C.c_int, [_vp, _i64]),
    "rts_batch_read": (C.c_int, [_vp, _i64, C.POINTER(C.c_float), _dp]),
    "rts_batch_add_synthetic": (C.c_int, [_vp, C.POINTER(ProblemDesc), C.c_uint64, C.c_double, C.c_double,
                                          C.c_double, C.c_double, _dp, C.POINTER(_i64)]),
    "rts_synth_host_f32": (C.c_int, [_vp, C.c_uint64, C.c_uint64, C.c_int, C.c_double, C.c_double, _i64, _i64,
                                     C.POINTER(C.c_float)]),
})

_lib = None


def header_symbols() -> list[str]:
    """Every function the public headers declare (for the export check)."""
    names = []
    for h in sorted(Path(INCLUDE).glob("*.h")):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        names += re.findall(r"\b(rts_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def load_library(path: str | Path | None = None):
    """Load librts_scatter.so (built in-tree by build.build_library)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build it with relativistic_solver_hllc_gb300.build.build_library() "
            "(there is no CPU fallback)"
        )
    lib = C.CDLL(str(p))
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def _ptr(a: np.ndarray | None):
    if a is None:
        return None
    return a.ctypes.data_as(_dp)


def _f64(a, shape=None) -> np.ndarray:
    arr = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None and arr.size != int(np.prod(shape)):
        raise ValueError(f"expected {int(np.prod(shape))} values, got {arr.size}")
    return arr


class Context:
    """One device context of the scattering library (one host thread at a time)."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = _vp()
        rc = self.lib.rts_ctx_create(int(device), C.byref(h))
        if rc != OK:
            raise RtsError(rc, "rts_ctx_create", f"device {device}")
        self.h = h
        self._keep = []  # host arrays referenced by queued async copies
        self.N = self.M = 0
        self.start = self.end = 0

    # -- plumbing -------------------------------------------------------
    def _check(self, rc: int, where: str):
        if rc != OK:
            msg = self.lib.rts_last_error(self.h)
            raise RtsError(rc, where, msg.decode() if msg else "")

    def close(self):
        if getattr(self, "h", None):
            self.lib.rts_ctx_destroy(self.h)
            self.h = None
            self._keep.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def last_error(self) -> str:
        return self.lib.rts_last_error(self.h).decode()

    def set_hbm_budget(self, nbytes: int):
        self._check(self.lib.rts_set_hbm_budget(self.h, int(nbytes)), "rts_set_hbm_budget")

    def hbm_used(self) -> int:
        v = _i64()
        self._check(self.lib.rts_hbm_used(self.h, C.byref(v)), "rts_hbm_used")
        return v.value

    # -- grid -----------------------------------------------------------
    def init(self, xyz, area, full_area: float, N: int, start: int = 0, end: int | None = None):
        xyz = _f64(xyz)
        area = _f64(area)
        M = area.size
        if xyz.size != 3 * M:
            raise ValueError("xyz must hold 3 values per direction")
        end = M if end is None else end
        self._check(
            self.lib.rts_init(self.h, _ptr(xyz), _ptr(area), M, float(full_area), int(N), int(start), int(end)),
            "rts_init",
        )
        self.N, self.M, self.start, self.end = int(N), int(M), int(start), int(end)

    def host_illum(self) -> np.ndarray:
        p = _dp()
        self._check(self.lib.rts_host_illum(self.h, C.byref(p)), "rts_host_illum")
        return np.ctypeslib.as_array(p, shape=(self.M * self.N * 4,))

    def host_scattering(self) -> np.ndarray:
        p = _dp()
        self._check(self.lib.rts_host_scattering(self.h, C.byref(p)), "rts_host_scattering")
        return np.ctypeslib.as_array(p, shape=((self.end - self.start) * self.N,))

    def set_phase(self, phase: int, g: float = 0.0):
        self._check(self.lib.rts_set_phase(self.h, int(phase), float(g)), "rts_set_phase")

    def set_weights(self, W):
        W = _f64(W, (self.M, self.end - self.start))
        self._check(self.lib.rts_set_weights(self.h, _ptr(W)), "rts_set_weights")

    # -- transfers --------------------------------------------------------
    def send_illum_async(self, size: int, shift_dev: int, shift_host: int, illum_host: np.ndarray):
        if illum_host.dtype != np.float64 or not illum_host.flags.c_contiguous:
            raise ValueError("illum_host must be a C-contiguous float64 array")
        if shift_host + size > illum_host.size:
            raise ValueError("host range outside the array")
        self._keep.append(illum_host)
        self._check(
            self.lib.rts_send_illum_async(self.h, int(size), int(shift_dev), int(shift_host), _ptr(illum_host)),
            "rts_send_illum_async",
        )

    def copy_illum(self, illum_host, size: int | None = None):
        a = _f64(illum_host)
        size = a.size if size is None else size
        self._check(self.lib.rts_copy_illum(self.h, int(size), _ptr(a)), "rts_copy_illum")

    # -- integrals --------------------------------------------------------
    def set_precision(self, precision):
        """Arithmetic of scattering_async / scattering ("fp64", "fp16x3", "bf16x3", "tf32x3")."""
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        self._check(self.lib.rts_set_precision(self.h, prec), "rts_set_precision")

    def get_precision(self) -> int:
        v = C.c_int()
        self._check(self.lib.rts_get_precision(self.h, C.byref(v)), "rts_get_precision")
        return v.value

    def scattering_async(self, start: int, end: int, stream: int, out: np.ndarray | None = None):
        if out is not None:
            if out.dtype != np.float64 or not out.flags.c_contiguous:
                raise ValueError("out must be a C-contiguous float64 array")
            if out.size < end * self.N:
                raise ValueError("out too small for the requested rows")
            self._keep.append(out)
        self._check(
            self.lib.rts_scattering_async(self.h, int(start), int(end), int(stream), _ptr(out)),
            "rts_scattering_async",
        )

    def scattering(self, illum=None) -> np.ndarray:
        out = np.empty((self.end - self.start) * self.N, dtype=np.float64)
        src = None if illum is None else _f64(illum, (self.M * self.N * 4,))
        self._check(self.lib.rts_scattering(self.h, _ptr(src), _ptr(out)), "rts_scattering")
        return out.reshape(self.end - self.start, self.N)

    def moments(self, stream: int = STREAM_PARAMS):
        e = np.empty(self.N, dtype=np.float64)
        f = np.empty(self.N * 3, dtype=np.float64)
        self._check(self.lib.rts_moments(self.h, int(stream), _ptr(e), _ptr(f)), "rts_moments")
        return e, f.reshape(self.N, 3)

    def set_geometry(self, normals, face_areas, volume):
        """Outward face normals [N][4][3], face areas [N][4], volumes [N]."""
        n = _f64(normals, (self.N, 4, 3))
        s = _f64(face_areas, (self.N, 4))
        v = _f64(volume, (self.N,))
        self._check(self.lib.rts_set_geometry(self.h, _ptr(n), _ptr(s), _ptr(v)), "rts_set_geometry")

    def illum_params(self, stream: int = STREAM_PARAMS, divergence: bool = True):
        """energy [N], flux [N][3], impuls [N][3][3], divstream [N], divimpuls [N][3]
        (the last two None unless divergence)."""
        N = self.N
        e, f, im = np.empty(N), np.empty(3 * N), np.empty(9 * N)
        ds = np.empty(N) if divergence else None
        di = np.empty(3 * N) if divergence else None
        self._check(self.lib.rts_illum_params(self.h, int(stream), _ptr(e), _ptr(f), _ptr(im), _ptr(ds), _ptr(di)),
                    "rts_illum_params")
        return (e, f.reshape(N, 3), im.reshape(N, 3, 3), ds, None if di is None else di.reshape(N, 3))

    def write_solution(self, directory):
        """Illum.bin, energy.bin, stream.bin, impuls.bin (and divstream.bin,
        divimpuls.bin with the geometry) in the reference's file layout."""
        self._check(self.lib.rts_write_solution(self.h, str(directory).encode()), "rts_write_solution")

    def source_update(self, B, lam: float, start: int, end: int, stream: int = STREAM_SCATTERING_1,
                      residual: bool = True):
        B = _f64(B, (self.N,))
        r = C.c_double(0.0)
        self._check(
            self.lib.rts_source_update(self.h, _ptr(B), float(lam), int(start), int(end), int(stream),
                                       C.byref(r) if residual else None),
            "rts_source_update",
        )
        return r.value if residual else None

    def scattering_update(self, precision, illum_host: np.ndarray, B: np.ndarray | None, lam: float,
                          out: np.ndarray) -> np.ndarray:
        """One evaluation with host buffers (H2D Illum and B, integral + update, D2H S)."""
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        for a in (illum_host, out) + ((B,) if B is not None else ()):
            if a.dtype != np.float64 or not a.flags.c_contiguous:
                raise ValueError("host buffers must be C-contiguous float64 arrays")
        if illum_host.size != self.M * self.N * 4 or out.size != (self.end - self.start) * self.N:
            raise ValueError("host buffer sizes do not match the grid")
        self._check(self.lib.rts_scattering_update(self.h, prec, _ptr(illum_host), _ptr(B), float(lam), _ptr(out)),
                    "rts_scattering_update")
        return out

    def read_scattering(self, start: int, end: int, stream: int, out: np.ndarray | None = None):
        if out is not None:
            if out.dtype != np.float64 or not out.flags.c_contiguous or out.size < end * self.N:
                raise ValueError("out must be a C-contiguous float64 array covering the rows")
            self._keep.append(out)
        self._check(self.lib.rts_read_scattering(self.h, int(start), int(end), int(stream), _ptr(out)),
                    "rts_read_scattering")

    def send_scattering(self, S, start: int = 0, end: int | None = None, stream: int = STREAM_SCATTERING_1):
        """Rows [start, end) of S ([local][N] FP64, host) into the device scattering array (synchronous)."""
        end = (self.end - self.start) if end is None else end
        a = _f64(S, ((self.end - self.start) * self.N,))
        self._check(self.lib.rts_send_scattering(self.h, int(start), int(end), int(stream), _ptr(a)),
                    "rts_send_scattering")
        self.sync_stream(stream)

    def device_arrays(self):
        a, b = _dp(), _dp()
        self._check(self.lib.rts_device_arrays(self.h, C.byref(a), C.byref(b)), "rts_device_arrays")
        return C.cast(a, C.c_void_p).value, C.cast(b, C.c_void_p).value

    # -- synchronisation --------------------------------------------------
    def sync_stream(self, stream: int, timeout_us: int = -1):
        rc = self.lib.rts_sync_stream(self.h, int(stream), int(timeout_us))
        if rc == OK:
            self._keep.clear()
        self._check(rc, "rts_sync_stream")

    def wait(self, timeout_us: int = -1):
        rc = self.lib.rts_wait(self.h, int(timeout_us))
        if rc == OK:
            self._keep.clear()
        self._check(rc, "rts_wait")

    # -- resident source iteration ---------------------------------------
    def solve_setup(self, precision, B, lam: float):
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        B = _f64(B, (self.N,))
        self._check(self.lib.rts_solve_setup(self.h, prec, _ptr(B), float(lam)), "rts_solve_setup")

    def solve_step(self, relax: bool = False) -> float:
        r = C.c_double(0.0)
        self._check(self.lib.rts_solve_step(self.h, int(bool(relax)), C.byref(r)), "rts_solve_step")
        return r.value

    def solve_step_async(self, relax: bool = False):
        self._check(self.lib.rts_solve_step_async(self.h, int(bool(relax))), "rts_solve_step_async")

    def solve_residual(self) -> float:
        r = C.c_double(0.0)
        self._check(self.lib.rts_solve_residual(self.h, C.byref(r)), "rts_solve_residual")
        return r.value

    def solve_residual_history(self, n: int) -> np.ndarray:
        out = np.empty(n)
        self._check(self.lib.rts_solve_residual_history(self.h, _ptr(out), int(n)), "rts_solve_residual_history")
        return out

    def read_illum(self, out: np.ndarray, size: int | None = None) -> np.ndarray:
        if out.dtype != np.float64 or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous float64 array")
        size = out.size if size is None else size
        self._check(self.lib.rts_read_illum(self.h, int(size), _ptr(out)), "rts_read_illum")
        return out

    def solve_read(self) -> np.ndarray:
        out = np.empty(self.M * self.N, dtype=np.float64)
        self._check(self.lib.rts_solve_read(self.h, _ptr(out)), "rts_solve_read")
        return out.reshape(self.M, self.N)

    def solve_read_ibar(self) -> np.ndarray:
        out = np.empty(self.M * self.N, dtype=np.float64)
        self._check(self.lib.rts_solve_read_ibar(self.h, _ptr(out)), "rts_solve_read_ibar")
        return out.reshape(self.M, self.N)

    def set_tuning(self, key: int, value: int):
        self._check(self.lib.rts_set_tuning(self.h, int(key), int(value)), "rts_set_tuning")

    def flush_period(self, precision="fp16x3") -> int:
        """K-slices per FP32 drain that the tensor-core calls at `precision` use (RTS_TUNE_FLUSH or automatic)."""
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        v = C.c_int()
        self._check(self.lib.rts_flush_period(self.h, prec, C.byref(v)), "rts_flush_period")
        return v.value

    def autotune(self, M: int, precision="fp16x3", flush: int = 0, cells: int = 0):
        """Best tile width for M directions; returns (bn, ms, {bn: ms})."""
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        best, tried = C.c_int(), C.c_int()
        best_ms = C.c_double()
        bns = (C.c_int * 16)()
        mss = (C.c_double * 16)()
        self._check(self.lib.rts_autotune(self.h, int(M), prec, int(flush), int(cells), C.byref(best), C.byref(best_ms),
                                          bns, mss, 16, C.byref(tried)), "rts_autotune")
        return best.value, best_ms.value, {bns[i]: mss[i] for i in range(min(tried.value, 16))}

    def autotune_schedule(self, M: int, precision="fp16x3", cells: int = 0):
        """Fastest (drain period, tile width, tile order) for M directions;
        returns (best, tried), each schedule a dict."""
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        cap = 64
        best = TuneChoice()
        tried = (TuneChoice * cap)()
        n = C.c_int()
        self._check(self.lib.rts_autotune_schedule(self.h, int(M), prec, int(cells), C.byref(best), tried, cap,
                                                   C.byref(n)), "rts_autotune_schedule")
        return best.as_dict(), [tried[i].as_dict() for i in range(min(n.value, cap))]

    def autotune_save(self, path):
        self._check(self.lib.rts_autotune_save(self.h, str(path).encode()), "rts_autotune_save")

    def autotune_load(self, path):
        self._check(self.lib.rts_autotune_load(self.h, str(path).encode()), "rts_autotune_load")

    def stream_handle(self, stream: int) -> int:
        v = _vp()
        self._check(self.lib.rts_stream_handle(self.h, int(stream), C.byref(v)), "rts_stream_handle")
        return int(v.value or 0)

    def measure_fp64_peak(self, seconds: float = 2.0) -> float:
        """FP64 FMA throughput of the device, TFLOP/s."""
        v = C.c_double()
        self._check(self.lib.rts_measure_fp64_peak(self.h, float(seconds), C.byref(v)), "rts_measure_fp64_peak")
        return v.value

    def measure_link(self, nbytes: int = 1 << 30, reps: int = 5) -> dict:
        """Pinned host <-> device copy rates, GB/s."""
        a, b, c = C.c_double(), C.c_double(), C.c_double()
        self._check(self.lib.rts_measure_link(self.h, int(nbytes), int(reps), C.byref(a), C.byref(b), C.byref(c)),
                    "rts_measure_link")
        return {"h2d_gbs": a.value, "d2h_gbs": b.value, "bidirectional_gbs": c.value, "bytes": int(nbytes)}

    def launch_count(self) -> int:
        v = _i64()
        self._check(self.lib.rts_launch_count(self.h, C.byref(v)), "rts_launch_count")
        return v.value

    def kernel_timing(self, enable: bool):
        """enable=True clears and starts event timing of the dominant kernel;
        enable=False stops it and returns (total_ms, launches)."""
        ms = C.c_double()
        n = _i64()
        self._check(self.lib.rts_kernel_timing(self.h, int(bool(enable)), C.byref(ms), C.byref(n)),
                    "rts_kernel_timing")
        return ms.value, n.value

    def synth_host_f32(self, seed: int, stream: int, lognormal: bool, a: float, b: float, n: int, i0: int = 0,
                       out: np.ndarray | None = None) -> np.ndarray:
        """n counter-hash values (indices i0..i0+n of `stream`) generated on the
        device into a host FP32 array: lognormal(a, b) or uniform(a, b)."""
        if out is None:
            out = np.empty(int(n), dtype=np.float32)
        if out.dtype != np.float32 or not out.flags.c_contiguous or out.size < n:
            raise ValueError("out must be a contiguous float32 array of at least n values")
        self._check(self.lib.rts_synth_host_f32(self.h, C.c_uint64(seed), C.c_uint64(stream), int(bool(lognormal)),
                                                float(a), float(b), int(i0), int(n),
                                                out.ctypes.data_as(C.POINTER(C.c_float))), "rts_synth_host_f32")
        return out

    # -- transport sweep ------------------------------------------------
    def sweep_set_mesh(self, vert, pairs, normals):
        v = _f64(vert, (self.N, 4, 3))
        p = np.ascontiguousarray(pairs, dtype=np.int32)
        nrm = _f64(normals, (self.N, 4, 3))
        if p.size != 4 * self.N:
            raise ValueError("pairs must hold N*4 entries")
        self._check(self.lib.rts_sweep_set_mesh(self.h, _ptr(v), p.ctypes.data, _ptr(nrm)), "rts_sweep_set_mesh")

    def sweep_build(self):
        """Per-direction structures on the device: (node records, largest step count)."""
        rec, lev = _i64(), _i64()
        self._check(self.lib.rts_sweep_build(self.h, C.byref(rec), C.byref(lev)), "rts_sweep_build")
        return rec.value, lev.value

    def sweep_import_direction(self, d: int, order, states, locx0):
        o = np.ascontiguousarray(order, dtype=np.int32)
        st = np.ascontiguousarray(states, dtype=np.int32)
        rec = np.asarray(locx0)
        if rec.dtype.names:  # structured: lay the fields out as cell_local
            rec = rec.astype(LOCX0_DTYPE)
        rec = np.ascontiguousarray(rec)
        if rec.dtype.itemsize != 32:
            raise ValueError("LocX0 records are 32 bytes")
        self._check(self.lib.rts_sweep_import_direction(self.h, int(d), o.ctypes.data, st.ctypes.data,
                                                        rec.ctypes.data if rec.size else None, rec.shape[0]),
                    "rts_sweep_import_direction")

    def sweep_export_direction(self, d: int):
        """(order [N], states [N], LocX0 records [n] of LOCX0_DTYPE) of local direction d."""
        n = _i64()
        self._check(self.lib.rts_sweep_export_direction(self.h, int(d), None, None, None, 0, C.byref(n)),
                    "rts_sweep_export_direction")
        order = np.empty(self.N, dtype=np.int32)
        states = np.empty(self.N, dtype=np.int32)
        rec = np.zeros(n.value, dtype=LOCX0_DTYPE)
        self._check(self.lib.rts_sweep_export_direction(self.h, int(d), order.ctypes.data, states.ctypes.data,
                                                        rec.ctypes.data, n.value, C.byref(n)),
                    "rts_sweep_export_direction")
        return order, states, rec

    def sweep_set_medium(self, md: Medium, alpha, beta, Q, bc=None):
        a, b, q = (_f64(x, (self.N,)) for x in (alpha, beta, Q))
        bcv = None if bc is None else _f64(bc, (4,))
        self._check(self.lib.rts_sweep_set_medium(self.h, C.byref(md), _ptr(a), _ptr(b), _ptr(q), _ptr(bcv)),
                    "rts_sweep_set_medium")

    def sweep(self, stream: int = STREAM_SCATTERING_1, read_norm: bool = True):
        out = C.c_double(0.0)
        self._check(self.lib.rts_sweep(self.h, int(stream), C.byref(out) if read_norm else None), "rts_sweep")
        return out.value if read_norm else None

    def sweep_exp_check(self, n: int = 1 << 20) -> float:
        out = C.c_double()
        self._check(self.lib.rts_sweep_exp_check(self.h, int(n), C.byref(out)), "rts_sweep_exp_check")
        return out.value

    def illum_solve(self, precision="fp64", max_iter: int = 1, accuracy: float = 1e-5):
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        norms = np.zeros(max_iter)
        it = _i64()
        self._check(self.lib.rts_illum_solve(self.h, prec, int(max_iter), float(accuracy), C.byref(it), _ptr(norms)),
                    "rts_illum_solve")
        return norms[: it.value].copy()

    def synth_illum(self, seed: int, mu: float, sigma: float, independent_faces: bool = False):
        self._check(
            self.lib.rts_synth_illum(self.h, C.c_uint64(seed), float(mu), float(sigma), int(bool(independent_faces))),
            "rts_synth_illum",
        )


def problem_desc(N, M, groups=1, phase=PHASE_THOMSON, g=0.0, precision="fp16x3", flush=0, bn=0) -> ProblemDesc:
    prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
    return ProblemDesc(int(N), int(M), int(groups), int(phase), float(g), prec, int(flush), int(bn))


def problem_footprint(desc: ProblemDesc) -> int:
    v = _i64()
    _status(load_library().rts_problem_footprint(C.byref(desc), C.byref(v)), "rts_problem_footprint")
    return v.value


class Batch:
    """Resident scattering problems advanced together (one grouped launch per step)."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        self.lib = ctx.lib
        h = _vp()
        ctx._check(self.lib.rts_batch_create(ctx.h, C.byref(h)), "rts_batch_create")
        self.h = h
        self.shapes = {}

    def close(self):
        if getattr(self, "h", None):
            self.lib.rts_batch_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def add(self, desc: ProblemDesc, ibar, B, lam) -> int:
        """ibar [groups][M][N] FP32, B [groups][N] FP32, lam [groups]."""
        ibar = np.ascontiguousarray(ibar, dtype=np.float32)
        B = np.ascontiguousarray(B, dtype=np.float32)
        lam = np.ascontiguousarray(np.atleast_1d(lam), dtype=np.float64)
        G, M, N = desc.groups, desc.M, desc.N
        if ibar.size != G * M * N or B.size != G * N or lam.size != G:
            raise ValueError("input sizes do not match the descriptor")
        pid = _i64()
        fp = C.POINTER(C.c_float)
        self.ctx._check(self.lib.rts_batch_add(self.h, C.byref(desc), ibar.ctypes.data_as(fp), B.ctypes.data_as(fp),
                                               _ptr(lam), C.byref(pid)), "rts_batch_add")
        self.shapes[pid.value] = (G, M, N)
        return pid.value

    def add_synthetic(self, desc: ProblemDesc, seed: int, mu: float, sigma: float, b_lo: float, b_hi: float,
                      lam) -> int:
        """A problem whose Ibar (lognormal(mu, sigma)) and B (uniform(b_lo, b_hi))
        are generated on the device from the counter hash."""
        lam = np.ascontiguousarray(np.atleast_1d(lam), dtype=np.float64)
        if lam.size != desc.groups:
            raise ValueError("lambda needs one value per group")
        pid = _i64()
        self.ctx._check(self.lib.rts_batch_add_synthetic(self.h, C.byref(desc), C.c_uint64(seed), float(mu),
                                                         float(sigma), float(b_lo), float(b_hi), _ptr(lam),
                                                         C.byref(pid)), "rts_batch_add_synthetic")
        self.shapes[pid.value] = (desc.groups, desc.M, desc.N)
        return pid.value

    def remove(self, pid: int):
        self.ctx._check(self.lib.rts_batch_remove(self.h, int(pid)), "rts_batch_remove")
        self.shapes.pop(pid, None)

    def size(self):
        p, t = _i64(), _i64()
        self.ctx._check(self.lib.rts_batch_size(self.h, C.byref(p), C.byref(t)), "rts_batch_size")
        return p.value, t.value

    def step(self, relax: bool = False):
        self.ctx._check(self.lib.rts_batch_step(self.h, int(bool(relax))), "rts_batch_step")

    def capture(self, steps: int, relax: bool = False):
        self.ctx._check(self.lib.rts_batch_capture(self.h, int(steps), int(bool(relax))), "rts_batch_capture")

    def replay(self):
        self.ctx._check(self.lib.rts_batch_replay(self.h), "rts_batch_replay")

    def sync(self, timeout_us: int = -1):
        self.ctx._check(self.lib.rts_batch_sync(self.h, int(timeout_us)), "rts_batch_sync")

    def read(self, pid: int):
        G, M, N = self.shapes[pid]
        S = np.empty(G * M * N, dtype=np.float32)
        r = C.c_double()
        self.ctx._check(self.lib.rts_batch_read(self.h, int(pid), S.ctypes.data_as(C.POINTER(C.c_float)), C.byref(r)),
                        "rts_batch_read")
        return S.reshape(G, M, N), r.value


class Request(C.Structure):
    """rts_request"""
    _fields_ = [("arrival_s", C.c_double), ("desc", ProblemDesc), ("iterations", C.c_int),
                ("ibar", C.POINTER(C.c_float)), ("B", C.POINTER(C.c_float)), ("lambda_", _dp),
                ("S_out", C.POINTER(C.c_float))]


class ServeStats(C.Structure):
    """rts_serve_stats"""
    _fields_ = [("completed", C.c_int64), ("rejected", C.c_int64), ("max_active", C.c_int64), ("steps", C.c_int64),
                ("peak_bytes", C.c_int64), ("makespan_s", C.c_double), ("throughput", C.c_double),
                ("p50_ms", C.c_double), ("p99_ms", C.c_double), ("mean_ms", C.c_double), ("max_ms", C.c_double),
                ("admit_s", C.c_double), ("step_s", C.c_double), ("retire_s", C.c_double)]


_SIGNATURES.update({
    "rts_serve_run": (C.c_int, [_vp, C.POINTER(Request), _i64, _i64, _i64, _dp, C.POINTER(ServeStats)]),
    "rts_host_alloc": (C.c_int, [_i64, C.POINTER(_vp)]),
    "rts_host_free": (C.c_int, [_vp]),
})


def serve(ctx: Context, requests, hbm_cap: int, step_timeout_us: int = 10_000_000):
    """Run a list of Request structures (sorted by arrival) through the
    continuous-batching loop; returns (stats, latencies_ms)."""
    n = len(requests)
    arr = (Request * n)(*requests)
    lat = np.empty(max(n, 1))
    st = ServeStats()
    ctx._check(ctx.lib.rts_serve_run(ctx.h, arr, n, int(hbm_cap), int(step_timeout_us), _ptr(lat), C.byref(st)),
               "rts_serve_run")
    return st, lat[:n]


class PinnedBuffer:
    """Pinned host memory from the library (rts_host_alloc)."""

    def __init__(self, nbytes: int):
        self.lib = load_library()
        p = _vp()
        _status(self.lib.rts_host_alloc(int(nbytes), C.byref(p)), "rts_host_alloc")
        self.ptr = p.value
        self.nbytes = int(nbytes)

    def array(self, dtype, count, offset_bytes: int = 0):
        buf = (C.c_char * self.nbytes).from_address(self.ptr)
        return np.frombuffer(buf, dtype=dtype, count=count, offset=offset_bytes)

    def close(self):
        if self.ptr:
            self.lib.rts_host_free(C.c_void_p(self.ptr))
            self.ptr = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
