"""Generate the golden vectors of the scattering path from the reference's own
functions.

Runs only where the reference tree exists (the development container): it
builds oracle/_ref/libref_scatter.so from the reference source text
(oracle/build_ref.sh), feeds it seeded synthetic inputs from the oracle's
generators and stores the outputs here as small .npz files.  Inputs are not
stored in full; each file keeps the generator parameters plus a handful of
input samples ("pins") so a drift of the generator is caught too.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

import oracle  # noqa: E402

I32 = np.int32


def _p(a):
    return a.ctypes.data_as(oracle._dp)


def ref_scatter(ref, N, xyz, area, full_area, illum, disp, size):
    out = np.zeros(size * N)
    illum = np.ascontiguousarray(illum)
    rc = ref.ref_calculate_int_cpu(N, area.size, _p(np.ascontiguousarray(xyz).ravel()), _p(area), full_area,
                                   _p(illum), disp, size, _p(out))
    assert rc == 0
    return out.reshape(size, N)


def ref_moments(ref, N, xyz, area, full_area, illum):
    M = area.size
    I = illum.reshape(M, N, 4)
    e = np.empty(N)
    s = np.empty((N, 3))
    xyzf = np.ascontiguousarray(xyz).ravel()
    for c in range(N):
        cell = np.ascontiguousarray(I[:, c, :]).ravel()
        e[c] = ref.ref_energy_cell(M, _p(xyzf), _p(area), full_area, _p(cell))
        o = np.empty(3)
        ref.ref_stream_cell(M, _p(xyzf), _p(area), full_area, _p(cell), _p(o))
        s[c] = o
    return e, s


CASES = [
    # name, N, M, seed, sigma, independent_faces, disp, size
    ("tiny_n7_m3", 7, 3, 11, 1.0, True, 0, 3),
    ("n64_m17", 64, 17, 5, 1.5, True, 0, 17),
    ("n33_m16_part", 33, 16, 7, 1.0, True, 5, 7),
    ("n130_m1", 130, 1, 9, 1.0, False, 0, 1),
    ("n5_m2", 5, 2, 13, 0.5, True, 0, 2),
    ("n257_m40", 257, 40, 21, 1.0, False, 0, 40),
]


def main():
    ref = oracle.ref_lib()
    if ref is None:
        raise SystemExit("reference tree not present: golden vectors cannot be regenerated here")
    for name, N, M, seed, sigma, indep, disp, size in CASES:
        xyz, area, fa = oracle.fibonacci_directions(M)
        il = oracle.illum(seed, 0.0, sigma, N, M, independent_faces=indep)
        S = ref_scatter(ref, N, xyz, area, fa, il, disp, size)
        e, s = ref_moments(ref, N, xyz, area, fa, il)
        pin_idx = np.linspace(0, il.size - 1, 16).astype(np.int64)
        np.savez_compressed(
            HERE / f"{name}.npz",
            N=N, M=M, seed=seed, mu=0.0, sigma=sigma, independent_faces=int(indep), disp=disp, size=size,
            S=S, energy=e, stream=s, pin_idx=pin_idx, pin_val=il[pin_idx], xyz=xyz, area=area, full_area=fa,
        )
        print(f"{name}: S{S.shape} sum={S.sum():.17g}")

    # configuration 1 (12^3 x 6 = 10,368 cells, 200 Fibonacci directions,
    # Thomson, lognormal(0,1) seed 0): sampled outputs plus per-direction sums
    N, M, seed = 10368, 200, 0
    xyz, area, fa = oracle.fibonacci_directions(M)
    il = oracle.illum(seed, 0.0, 1.0, N, M)
    S = ref_scatter(ref, N, xyz, area, fa, il, 0, M)
    cells = np.unique(np.linspace(0, N - 1, 48).astype(np.int64))
    pin_idx = np.linspace(0, il.size - 1, 64).astype(np.int64)
    np.savez_compressed(
        HERE / "config1_sample.npz",
        N=N, M=M, seed=seed, mu=0.0, sigma=1.0, independent_faces=0, disp=0, size=M,
        cells=cells, S_cells=S[:, cells], row_sums=S.sum(axis=1), total=S.sum(),
        pin_idx=pin_idx, pin_val=il[pin_idx], xyz=xyz, area=area, full_area=fa,
    )
    print(f"config1_sample: total={S.sum():.17g}")

    # flux, impulse tensor and their divergences (MakeStream / MakeDivImpuls)
    # on seeded synthetic geometry, two direction sets
    for name, N, M, seed in [("div_n40_m24", 40, 24, 31), ("div_n7_m5", 7, 5, 37)]:
        xyz, area, fa = oracle.fibonacci_directions(M)
        il = oracle.illum(seed, 0.0, 1.0, N, M, independent_faces=True)
        nrm, fS, vol = oracle.cell_geometry(seed, N)
        out = [np.empty(3 * N), np.empty(9 * N), np.empty(N), np.empty(3 * N)]
        f = ref.ref_illum_params
        f.restype = None
        f.argtypes = [oracle.C.c_int, oracle.C.c_int] + [oracle._dp] * 2 + [oracle.C.c_double] + [oracle._dp] * 8
        f(N, M, _p(np.ascontiguousarray(xyz).ravel()), _p(area), fa, _p(il), _p(nrm.ravel()), _p(fS.ravel()),
          _p(vol), *[_p(o) for o in out])
        pin_idx = np.linspace(0, il.size - 1, 16).astype(np.int64)
        np.savez_compressed(
            HERE / f"{name}.npz", N=N, M=M, seed=seed, mu=0.0, sigma=1.0, independent_faces=1,
            flux=out[0].reshape(N, 3), impuls=out[1].reshape(N, 9), divstream=out[2], divimpuls=out[3].reshape(N, 3),
            normals=nrm, face_areas=fS, volume=vol, pin_idx=pin_idx, pin_val=il[pin_idx],
        )
        print(f"{name}: divstream sum={out[2].sum():.17g}")

    # direction partition GetSend / GetDisp
    rows = []
    for np_, n in [(1, 7), (2, 7), (3, 10), (4, 3), (5, 1000), (7, 590), (16, 1202), (6, 6)]:
        s = (oracle.C.c_int * np_)()
        d = (oracle.C.c_int * np_)()
        ref.ref_get_send_disp(np_, n, s, d)
        rows.append((np_, n, list(s), list(d)))
    flat_s = np.array([v for r in rows for v in r[2]], dtype=I32)
    flat_d = np.array([v for r in rows for v in r[3]], dtype=I32)
    np.savez_compressed(
        HERE / "partition.npz",
        np_=np.array([r[0] for r in rows], dtype=I32), n=np.array([r[1] for r in rows], dtype=I32),
        send=flat_s, disp=flat_d,
    )
    print("partition:", rows)


if __name__ == "__main__":
    main()
