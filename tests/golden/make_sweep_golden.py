"""Generate the golden vectors of the transport sweep from the reference's own
functions.

Runs only where the reference tree exists (the development container): it
builds oracle/_ref/libref_sweep.so from the reference source text
(oracle/build_ref.sh) -- build_graph's ordering, make_illum_struct's nodes and
characteristic records, and the sweep loop of MPI_CalculateIllumAsync with
GetCurIllum, BoundaryConditions and ReCalcIllum -- runs it on the tilted cube
mesh (oracle.cube_mesh, boundary rule 1) with spherical-Fibonacci directions
and seeded inputs, and stores what it returns as .npz files here.

    python tests/golden/make_sweep_golden.py
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

import oracle  # noqa: E402

VP = C.c_void_p
# reference classes of GetCurIllum pinned here (class 11 reads the gas state)
CLASSES = (0, 1, 2, 3, 10, 11)


def ref_lib():
    oracle.build_ref()
    L = C.CDLL(str(oracle.REF_DIR / "libref_sweep.so"))
    L.ref_sweep_structs.restype = C.c_longlong
    L.ref_sweep_dirs.restype = C.c_double
    L.ref_sweep_nodes.restype = C.c_int
    return L


def p(a):
    return a.ctypes.data_as(VP)


def structures(L, vert, pairs, normals, xyz):
    N = vert.shape[0]
    orders, states, recs_s, recs_f, off, steps = [], [], [], [], [0], []
    for d in range(xyz.shape[0]):
        g = np.empty(N, np.int32)
        st = np.empty(N, np.int32)
        sv = np.empty(9 * N)
        fv = np.empty(9 * N, np.uint8)
        ns = C.c_int()
        r = L.ref_sweep_structs(N, p(vert), p(pairs), p(normals), p(np.ascontiguousarray(xyz[d])), p(g), p(st),
                                p(sv), p(fv), C.byref(ns))
        assert r > 0, (d, r)
        orders.append(g)
        states.append(st)
        recs_s.append(sv[:r])
        recs_f.append(fv[:r])
        off.append(off[-1] + r)
        steps.append(ns.value)
    return (np.stack(orders), np.stack(states), np.concatenate(recs_s), np.concatenate(recs_f),
            np.array(off, dtype=np.int64), np.array(steps, dtype=np.int32))


def main():
    L = ref_lib()
    # structures on a 3^3 cube, 12 directions
    n, M = 3, 12
    vert, pairs, normals = oracle.cube_mesh(n, 1, True)
    xyz, _, _ = oracle.fibonacci_directions(M)
    N = vert.shape[0]
    nodes = np.empty((N, 4, 3, 3))
    assert L.ref_sweep_nodes(N, p(vert), p(nodes)) == 0
    order, states, s, face, off, steps = structures(L, vert, pairs, normals, xyz)
    np.savez_compressed(HERE / "sweep_structs_n3_m12.npz", n=n, M=M, bound_rule=1, tilt=1, nodes=nodes, order=order,
                        states=states, s=s, face=face, rec_off=off, steps=steps)
    # one sweep of every reference class on a 2^3 cube, 16 directions
    n, M, seed = 2, 16, 7
    vert, pairs, normals = oracle.cube_mesh(n, 1, True)
    xyz, _, _ = oracle.fibonacci_directions(M)
    N = vert.shape[0]
    nodes = np.empty((N, 4, 3, 3))
    assert L.ref_sweep_nodes(N, p(vert), p(nodes)) == 0
    order, states, s, face, off, steps = structures(L, vert, pairs, normals, xyz)
    rng = np.random.default_rng(seed)
    S = rng.uniform(0.0, 2.0, (M, N))
    il0 = rng.uniform(0.1, 1.0, (M, N, 4))
    gas = np.random.default_rng(seed + 1)
    density = gas.uniform(0.5, 2.0, N)
    pressure = 10.0 ** gas.uniform(-8.0, -5.0, N)  # T below and at the 5000 K cap
    out, norms = {}, {}
    for cls in CLASSES:
        il = il0.copy()
        norms[cls] = L.ref_sweep_dirs(N, M, p(pairs), p(order), p(states), p(off), p(s), p(face), p(nodes), p(S),
                                      cls, p(density), p(pressure), p(il))
        out[cls] = il
    np.savez_compressed(HERE / "sweep_classes_n2_m16.npz", n=n, M=M, bound_rule=1, tilt=1, seed=seed,
                        S_pin=S.ravel()[:8], il0_pin=il0.ravel()[:8], density=density, pressure=pressure,
                        classes=np.array(CLASSES),
                        **{f"illum_{c}": out[c] for c in CLASSES}, norms=np.array([norms[c] for c in CLASSES]))
    print("wrote sweep_structs_n3_m12.npz, sweep_classes_n2_m16.npz")


if __name__ == "__main__":
    main()
