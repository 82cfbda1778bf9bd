"""CPU oracle of the scattering path -- TEST INFRASTRUCTURE ONLY.

Python binding of oracle/scatter_oracle.c (the C restatement of the
reference's CPU scattering integral, moments and direction partition) and of
oracle/_ref/libref_scatter.so (the reference's own functions, compiled from the
reference source text where that tree exists).  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg import this package;
the product library never does.

Parity pin: tests/golden/ holds outputs of the reference's own functions
(generated by tests/golden/make_golden.py through libref_scatter.so); the
restatement is checked against them in tests/test_oracle.py.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
BUILD_DIR = ORACLE_DIR / "_build"
LIB_PATH = BUILD_DIR / "liborc.so"
REF_DIR = ORACLE_DIR / "_ref"
REF_LIB = REF_DIR / "libref_scatter.so"
# The reference tree: RTS_REFERENCE_ROOT, else the directory "reference" beside
# this repository's root (the development layout).  Absent on the GPU hosts.
REFERENCE_ROOT = Path(os.environ.get("RTS_REFERENCE_ROOT") or (ORACLE_DIR.parent.parent / "reference"))

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_i64 = C.c_int64
_i64p = C.POINTER(C.c_int64)
_u64 = C.c_uint64


def build(force: bool = False) -> Path:
    """Compile the C restatements (gcc -O3 -fopenmp) into oracle/_build/liborc.so."""
    srcs = [ORACLE_DIR / "scatter_oracle.c", ORACLE_DIR / "sweep_oracle.c"]
    BUILD_DIR.mkdir(exist_ok=True)
    if not force and LIB_PATH.exists() and all(LIB_PATH.stat().st_mtime >= s.stat().st_mtime for s in srcs):
        return LIB_PATH
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        raise RuntimeError("no C compiler found for the oracle")
    tmp = LIB_PATH.with_suffix(".so.tmp")
    cmd = [cc, "-O3", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-std=c11", *map(str, srcs), "-o", str(tmp),
           "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def build_ref() -> Path | None:
    """Compile the reference's own functions (only where the reference tree exists)."""
    if not (REFERENCE_ROOT / "solver_hllc_illum_cuda").is_dir():
        return None
    script = ORACLE_DIR / "build_ref.sh"
    res = subprocess.run(["sh", str(script)], capture_output=True, text=True,
                         env={**os.environ, "RTS_REFERENCE_ROOT": str(REFERENCE_ROOT)})
    if res.returncode != 0:
        raise RuntimeError(f"reference build failed:\n{res.stdout}\n{res.stderr}")
    return REF_LIB


_SIG = {
    "orc_uniform": (C.c_double, [_u64, _u64, _u64]),
    "orc_normal": (C.c_double, [_u64, _u64, _u64]),
    "orc_fill_illum": (None, [_u64, C.c_double, C.c_double, _i64, _i64, _i64, C.c_int, _dp]),
    "orc_fill_uniform": (None, [_u64, _u64, C.c_double, C.c_double, _i64, _i64, _dp]),
    "orc_fill_normal": (None, [_u64, _u64, _i64, _dp]),
    "orc_fill_illum_cells": (None, [_u64, C.c_double, C.c_double, _i64, _i64, _i64, _i64, C.c_int, _dp]),
    "orc_fibonacci_directions": (None, [_i64, _dp, _dp, _dp]),
    "orc_weights_thomson": (None, [_i64, _dp, _dp, C.c_double, _i64, _i64, _dp]),
    "orc_weights_hg": (None, [_i64, _dp, _dp, C.c_double, _i64, _i64, _dp]),
    "orc_gets": (C.c_double, [_dp, _i64, _i64, _dp, _dp, C.c_double, _dp, _i64]),
    "orc_calculate_int_cpu": (None, [_i64, _i64, _dp, _dp, C.c_double, _dp, _i64, _i64, _dp, C.c_int]),
    "orc_calculate_int_cells": (None, [_i64, _i64, _dp, _dp, C.c_double, _dp, _i64, _i64, _i64p, _i64, _dp, C.c_int]),
    "orc_scatter_matrix": (None, [_dp, _i64, _i64, _dp, _i64, _dp, C.c_int]),
    "orc_face_mean": (None, [_dp, _i64, _i64, _dp]),
    "orc_energy": (None, [_dp, _i64, _i64, _dp, C.c_double, _dp]),
    "orc_stream": (None, [_dp, _i64, _i64, _dp, _dp, C.c_double, _dp]),
    "orc_illum_params": (None, [_dp, _i64, _i64, _dp, _dp, C.c_double, _dp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "orc_source_update": (None, [_i64, _i64, _dp, _dp, C.c_double]),
    "orc_max_abs_diff": (C.c_double, [_dp, _dp, _i64]),
    "orc_iterate": (None, [_dp, _i64, _dp, _i64, _dp, C.c_double, C.c_int, C.c_int, _dp, _dp]),
    "orc_get_send": (None, [C.c_int, C.c_int, _ip]),
    "orc_get_disp": (None, [C.c_int, C.c_int, _ip]),
    "orc_max_threads": (C.c_int, []),
    # transport sweep (sweep_oracle.c)
    "orc_cube_cells": (_i64, [C.c_int]),
    "orc_cube_mesh": (C.c_int, [C.c_int, C.c_int, C.c_int, _dp, C.c_void_p, _dp]),
    "orc_face_normals": (None, [_i64, _dp, _dp]),
    "orc_sweep_nodes": (None, [_i64, _dp, _dp]),
    "orc_face_states": (None, [_i64, _dp, _dp, C.c_void_p]),
    "orc_sweep_graph": (_i64, [_i64, C.c_void_p, C.c_void_p, C.c_void_p, _i64p]),
    "orc_sweep_x0": (_i64, [_i64, _dp, _dp, _dp, C.c_void_p, C.c_void_p, _dp, _dp, C.c_void_p]),
    "orc_sweep_dir": (C.c_double, [_i64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, _dp, C.c_void_p, _dp,
                                   C.c_void_p, _dp, _dp, _dp, _dp, _dp, _dp]),
    "orc_medium_gas": (None, [_i64, _dp, _dp, _dp, _dp, _dp, C.c_void_p]),
    "orc_sweep_all": (C.c_double, [_i64, _i64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, _i64p, _dp,
                                   C.c_void_p, _dp, C.c_void_p, _dp, _dp, _dp, _dp, _dp, C.c_int]),
}

_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB_PATH))
        for n, (r, a) in _SIG.items():
            f = getattr(L, n)
            f.restype = r
            f.argtypes = a
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(_dp)


# ---------------------------------------------------------------- inputs
def fibonacci_directions(M: int):
    xyz = np.empty(3 * M)
    area = np.empty(M)
    fa = C.c_double()
    lib().orc_fibonacci_directions(M, _p(xyz), _p(area), C.byref(fa))
    return xyz.reshape(M, 3), area, fa.value


def illum(seed: int, mu: float, sigma: float, N: int, M: int, j0: int = 0, j1: int | None = None,
          independent_faces: bool = False) -> np.ndarray:
    j1 = M if j1 is None else j1
    out = np.empty((j1 - j0) * N * 4)
    lib().orc_fill_illum(seed, mu, sigma, N, j0, j1, int(independent_faces), _p(out))
    return out


def illum_cells_into(out: np.ndarray, seed: int, mu: float, sigma: float, N: int, M: int, c0: int, c1: int,
                     independent_faces: bool = False) -> None:
    """Fill cells [c0, c1) of a full [M][N][4] array (others untouched)."""
    assert out.dtype == np.float64 and out.size >= M * N * 4
    lib().orc_fill_illum_cells(seed, mu, sigma, N, M, c0, c1, int(independent_faces), _p(out))


def uniform(seed: int, stream: int, lo: float, hi: float, n: int, i0: int = 0) -> np.ndarray:
    out = np.empty(n)
    lib().orc_fill_uniform(seed, stream, lo, hi, i0, n, _p(out))
    return out


def weights_thomson(xyz, area, full_area, k0: int = 0, Mout: int | None = None) -> np.ndarray:
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    area = np.ascontiguousarray(area, dtype=np.float64)
    M = area.size
    Mout = M - k0 if Mout is None else Mout
    W = np.empty(M * Mout)
    lib().orc_weights_thomson(M, _p(xyz), _p(area), full_area, k0, Mout, _p(W))
    return W.reshape(M, Mout)


def weights_hg(xyz, area, g: float, k0: int = 0, Mout: int | None = None) -> np.ndarray:
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    area = np.ascontiguousarray(area, dtype=np.float64)
    M = area.size
    Mout = M - k0 if Mout is None else Mout
    W = np.empty(M * Mout)
    lib().orc_weights_hg(M, _p(xyz), _p(area), g, k0, Mout, _p(W))
    return W.reshape(M, Mout)


# ---------------------------------------------------------------- integrals
def calculate_int_cpu(N, xyz, area, full_area, illum_arr, disp_loc=0, size_loc=None, nthreads=0):
    """Restated CalculateIntCPU: scattering [size_loc][N] (FP64)."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    area = np.ascontiguousarray(area, dtype=np.float64)
    illum_arr = np.ascontiguousarray(illum_arr, dtype=np.float64)
    M = area.size
    size_loc = M - disp_loc if size_loc is None else size_loc
    out = np.empty(size_loc * N)
    lib().orc_calculate_int_cpu(N, M, _p(xyz), _p(area), full_area, _p(illum_arr), disp_loc, size_loc,
                                _p(out), nthreads)
    return out.reshape(size_loc, N)


def calculate_int_cells(N, xyz, area, full_area, illum_arr, cells, disp_loc=0, size_loc=None, nthreads=0):
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    area = np.ascontiguousarray(area, dtype=np.float64)
    cells = np.ascontiguousarray(cells, dtype=np.int64)
    M = area.size
    size_loc = M - disp_loc if size_loc is None else size_loc
    out = np.empty(size_loc * cells.size)
    lib().orc_calculate_int_cells(N, M, _p(xyz), _p(area), full_area, _p(illum_arr), disp_loc, size_loc,
                                  cells.ctypes.data_as(_i64p), cells.size, _p(out), nthreads)
    return out.reshape(size_loc, cells.size)


def scatter_matrix(W, Ibar, nthreads=0) -> np.ndarray:
    W = np.ascontiguousarray(W, dtype=np.float64)
    Ibar = np.ascontiguousarray(Ibar, dtype=np.float64)
    Min, Mout = W.shape
    N = Ibar.size // Min
    out = np.empty(Mout * N)
    lib().orc_scatter_matrix(_p(W), Min, Mout, _p(Ibar), N, _p(out), nthreads)
    return out.reshape(Mout, N)


def face_mean(illum_arr, N, M) -> np.ndarray:
    illum_arr = np.ascontiguousarray(illum_arr, dtype=np.float64)
    out = np.empty(M * N)
    lib().orc_face_mean(_p(illum_arr), N, M, _p(out))
    return out.reshape(M, N)


def energy(illum_arr, N, area, full_area) -> np.ndarray:
    illum_arr = np.ascontiguousarray(illum_arr, dtype=np.float64)
    area = np.ascontiguousarray(area, dtype=np.float64)
    out = np.empty(N)
    lib().orc_energy(_p(illum_arr), N, area.size, _p(area), full_area, _p(out))
    return out


def stream(illum_arr, N, xyz, area, full_area) -> np.ndarray:
    illum_arr = np.ascontiguousarray(illum_arr, dtype=np.float64)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    area = np.ascontiguousarray(area, dtype=np.float64)
    out = np.empty(3 * N)
    lib().orc_stream(_p(illum_arr), N, area.size, _p(xyz), _p(area), full_area, _p(out))
    return out.reshape(N, 3)


def illum_params(illum_arr, N, xyz, area, full_area, normals, face_areas, volume):
    """flux [N][3], impuls [N][9], divstream [N], divimpuls [N][3]."""
    illum_arr = np.ascontiguousarray(illum_arr, dtype=np.float64)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    area = np.ascontiguousarray(area, dtype=np.float64)
    normals = np.ascontiguousarray(normals, dtype=np.float64)
    face_areas = np.ascontiguousarray(face_areas, dtype=np.float64)
    volume = np.ascontiguousarray(volume, dtype=np.float64)
    fl, im, ds, di = np.empty(3 * N), np.empty(9 * N), np.empty(N), np.empty(3 * N)
    lib().orc_illum_params(_p(illum_arr), N, area.size, _p(xyz), _p(area), full_area, _p(normals), _p(face_areas),
                           _p(volume), _p(fl), _p(im), _p(ds), _p(di))
    return fl.reshape(N, 3), im.reshape(N, 9), ds, di.reshape(N, 3)


def cell_geometry(seed: int, N: int):
    """Seeded synthetic tetrahedron geometry: unit outward normals [N][4][3],
    face areas [N][4] in (0.5, 1.5), volumes [N] in (0.2, 1.2)."""
    n = np.empty(N * 12)
    lib().orc_fill_normal(seed, 11, N * 12, _p(n))
    n = n.reshape(N, 4, 3)
    n /= np.linalg.norm(n, axis=2, keepdims=True)
    fa = uniform(seed, 12, 0.5, 1.5, 4 * N).reshape(N, 4)
    vol = uniform(seed, 13, 0.2, 1.2, N)
    return n, fa, vol


def source_update(S, B, lam) -> np.ndarray:
    S = np.array(S, dtype=np.float64, copy=True, order="C")
    B = np.ascontiguousarray(B, dtype=np.float64)
    Mout, N = S.shape
    lib().orc_source_update(N, Mout, _p(S), _p(B), lam)
    return S


def iterate(W, Ibar_cells, B_cells, lam, iters, relax=True):
    """FP64 source iteration on a subset of cells; Ibar_cells [M][ncell]."""
    W = np.ascontiguousarray(W, dtype=np.float64)
    I = np.array(Ibar_cells, dtype=np.float64, copy=True, order="C")
    B = np.ascontiguousarray(B_cells, dtype=np.float64)
    M, ncell = I.shape
    S = np.empty(M * ncell)
    res = np.empty(iters)
    lib().orc_iterate(_p(W), M, _p(I), ncell, _p(B), lam, iters, int(relax), _p(S), _p(res))
    return S.reshape(M, ncell), res, I


def get_send_disp(np_: int, n: int):
    s = (C.c_int * np_)()
    d = (C.c_int * np_)()
    lib().orc_get_send(np_, n, s)
    lib().orc_get_disp(np_, n, d)
    return list(s), list(d)


def max_threads() -> int:
    return lib().orc_max_threads()


# ---------------------------------------------------------------- transport sweep
BOUND_FREE, BOUND_LOCK, BOUND_OUTSOURCE, BOUND_INNER = -1, -2, -3, -4
DEFAULT_BC = (0.0, 0.0, 1.0, 0.0)  # intensity of boundary codes -1..-4 (BoundaryConditions)


class Medium(C.Structure):
    """GetCurIllum's medium: mode 0 scattering form, 1 absorption form."""
    _fields_ = [("mode", C.c_int), ("reserved", C.c_int), ("s_scale", C.c_double), ("i_scale", C.c_double),
                ("ball", C.c_double * 3), ("radius", C.c_double), ("ball_alpha", C.c_double),
                ("ball_beta", C.c_double), ("ball_q", C.c_double)]


def medium(mode=0, s_scale=1.0, i_scale=1.0, ball=(0.0, 0.0, 0.0), radius=0.0, ball_coef=(0.0, 0.0, 0.0)) -> Medium:
    m = Medium()
    m.mode, m.s_scale, m.i_scale = mode, s_scale, i_scale
    m.ball[:] = list(ball)
    m.radius = radius
    m.ball_alpha, m.ball_beta, m.ball_q = ball_coef
    return m


def medium_gas(density, pressure):
    """Class 11 of GetCurIllum: (Medium, alpha, beta, Q) from the gas state."""
    d = np.ascontiguousarray(density, dtype=np.float64)
    p = np.ascontiguousarray(pressure, dtype=np.float64)
    n = d.size
    a, b, q = np.empty(n), np.empty(n), np.empty(n)
    md = Medium()
    lib().orc_medium_gas(n, _p(d), _p(p), _p(a), _p(b), _p(q), C.byref(md))
    return md, a, b, q


def cube_mesh(n: int, bound_rule: int = 1, tilt: bool = True):
    """Unit cube, n^3 hexahedra x 6 tetrahedra: (vert [N][4][3], pairs [N][4], normals [N][4][3])."""
    N = lib().orc_cube_cells(n)
    vert = np.empty((N, 4, 3))
    pairs = np.empty((N, 4), dtype=np.int32)
    normals = np.empty((N, 4, 3))
    if lib().orc_cube_mesh(n, bound_rule, int(tilt), _p(vert), pairs.ctypes.data, _p(normals)) != 0:
        raise ValueError(f"cube mesh n={n} out of range")
    return vert, pairs, normals


def face_normals(vert) -> np.ndarray:
    vert = np.ascontiguousarray(vert, dtype=np.float64)
    out = np.empty_like(vert)
    lib().orc_face_normals(vert.shape[0], _p(vert), _p(out))
    return out


def sweep_nodes(vert) -> np.ndarray:
    vert = np.ascontiguousarray(vert, dtype=np.float64)
    nodes = np.empty((vert.shape[0], 4, 3, 3))
    lib().orc_sweep_nodes(vert.shape[0], _p(vert), _p(nodes))
    return nodes


def face_states(normals, direction) -> np.ndarray:
    normals = np.ascontiguousarray(normals, dtype=np.float64)
    d = np.ascontiguousarray(direction, dtype=np.float64)
    st = np.empty(normals.shape[0], dtype=np.int32)
    lib().orc_face_states(normals.shape[0], _p(normals), _p(d), st.ctypes.data)
    return st


def sweep_graph(pairs, states):
    """build_graph's order for one direction: (order [N], level offsets [L+1])."""
    pairs = np.ascontiguousarray(pairs, dtype=np.int32)
    states = np.ascontiguousarray(states, dtype=np.int32)
    N = states.shape[0]
    order = np.empty(N, dtype=np.int32)
    off = np.empty(N + 1, dtype=np.int64)
    L = lib().orc_sweep_graph(N, pairs.ctypes.data, states.ctypes.data, order.ctypes.data,
                              off.ctypes.data_as(_i64p))
    if L < 0:
        raise RuntimeError("sweep graph has a dependency cycle")
    return order, off[: L + 1].copy()


def sweep_x0(vert, normals, nodes, order, states, direction):
    """LocX0 records of one direction in sweep order: (s [n], in-face [n])."""
    vert = np.ascontiguousarray(vert, dtype=np.float64)
    normals = np.ascontiguousarray(normals, dtype=np.float64)
    nodes = np.ascontiguousarray(nodes, dtype=np.float64)
    N = vert.shape[0]
    d = np.ascontiguousarray(direction, dtype=np.float64)
    s = np.empty(9 * N)
    face = np.empty(9 * N, dtype=np.int8)
    n = lib().orc_sweep_x0(N, _p(vert), _p(normals), _p(nodes), np.ascontiguousarray(order, np.int32).ctypes.data,
                           np.ascontiguousarray(states, np.int32).ctypes.data, _p(d), _p(s), face.ctypes.data)
    if n < 0:
        raise RuntimeError(f"no in-face found for record {-n - 1}")
    return s[:n].copy(), face[:n].copy()


class SweepStructures:
    """Per-direction structures of a mesh (make_illum_struct + build_graph)."""

    def __init__(self, vert, pairs, normals, xyz):
        self.vert = np.ascontiguousarray(vert, dtype=np.float64)
        self.pairs = np.ascontiguousarray(pairs, dtype=np.int32)
        self.normals = np.ascontiguousarray(normals, dtype=np.float64)
        self.nodes = sweep_nodes(self.vert)
        xyz = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)
        self.N, self.D = self.vert.shape[0], xyz.shape[0]
        self.order = np.empty((self.D, self.N), dtype=np.int32)
        self.states = np.empty((self.D, self.N), dtype=np.int32)
        self.levels = []
        s_parts, f_parts, off = [], [], [0]
        for d in range(self.D):
            self.states[d] = face_states(self.normals, xyz[d])
            self.order[d], lv = sweep_graph(self.pairs, self.states[d])
            self.levels.append(lv)
            s, f = sweep_x0(self.vert, self.normals, self.nodes, self.order[d], self.states[d], xyz[d])
            s_parts.append(s)
            f_parts.append(f)
            off.append(off[-1] + s.shape[0])
        self.rec_off = np.array(off, dtype=np.int64)
        self.s = np.concatenate(s_parts)
        self.face = np.concatenate(f_parts)


def sweep(st: SweepStructures, S, alpha, beta, Q, illum, md: Medium | None = None, bc=DEFAULT_BC,
          use_nodes: bool | None = None, nthreads: int = 0) -> float:
    """Sweep every direction of `st` in place on illum [D][N][4] (FP64);
    S [D][N].  Returns ReCalcIllum's max norm."""
    md = md if md is not None else medium()
    S = np.ascontiguousarray(S, dtype=np.float64)
    a, b, q = (np.ascontiguousarray(x, dtype=np.float64) for x in (alpha, beta, Q))
    bcv = np.ascontiguousarray(bc, dtype=np.float64)
    assert illum.dtype == np.float64 and illum.flags.c_contiguous and illum.size == st.D * st.N * 4
    use_nodes = md.radius > 0 if use_nodes is None else use_nodes
    nodes = st.nodes.ctypes.data if use_nodes else None
    return lib().orc_sweep_all(st.N, st.D, st.pairs.ctypes.data, nodes, st.order.ctypes.data, st.states.ctypes.data,
                               st.rec_off.ctypes.data_as(_i64p), _p(st.s), st.face.ctypes.data, _p(S),
                               C.byref(md), _p(a), _p(b), _p(q), _p(bcv), _p(illum), nthreads)


# ---------------------------------------------------------------- reference
_ref = None


def ref_lib():
    """The reference's own functions (None where the reference tree is absent)."""
    global _ref
    if _ref is None:
        if not REF_LIB.exists():
            if build_ref() is None:
                return None
        L = C.CDLL(str(REF_LIB))
        L.ref_calculate_int_cpu.restype = C.c_int
        L.ref_calculate_int_cpu.argtypes = [C.c_int, C.c_int, _dp, _dp, C.c_double, _dp, C.c_int, C.c_int, _dp]
        L.ref_energy_cell.restype = C.c_double
        L.ref_energy_cell.argtypes = [C.c_int, _dp, _dp, C.c_double, _dp]
        L.ref_stream_cell.restype = None
        L.ref_stream_cell.argtypes = [C.c_int, _dp, _dp, C.c_double, _dp, _dp]
        L.ref_get_send_disp.restype = None
        L.ref_get_send_disp.argtypes = [C.c_int, C.c_int, _ip, _ip]
        _ref = L
    return _ref
