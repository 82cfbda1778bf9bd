"""The transport sweep pinned to the reference's own code.

tests/golden/make_sweep_golden.py ran the reference's build_graph ordering,
make_illum_struct nodes and characteristic records, and the sweep loop of
MPI_CalculateIllumAsync (with GetCurIllum for classes 0, 1, 2, 3, 10, 11,
BoundaryConditions and ReCalcIllum), compiled from the reference source text,
on small tilted cube meshes.  The oracle must reproduce those outputs bit for
bit (same operation order, no fused multiply-adds); the device sweep, run on
the reference's own structures (imported in its file layouts), within 1e-12
relative (FP64 contract: the device's exp and fused multiply-adds differ from
the host's by an ulp)."""
import numpy as np
import pytest

import oracle
from conftest import GOLDEN

# the constants of GetCurIllum's classes (solve_module/illum/Illum_async.cpp:259-470)
CLASS_MEDIUM = {
    0: ((2.0, 1.0, 0.0), dict(ball=(0.5, 0.0, 0.0), radius=0.05, ball_coef=(0.5, 0.5, 0.0))),
    1: ((1.0, 0.5, 1.0), {}),
    2: ((1.0, 0.0, 1.0), dict(mode=1, s_scale=388189 * 1e5)),
    3: ((0.0, 0.0, 0.0), {}),
    10: ((0.5, 100.0, 0.0), {}),
}


def case_inputs(g):
    n, M = int(g["n"]), int(g["M"])
    vert, pairs, normals = oracle.cube_mesh(n, int(g["bound_rule"]), bool(g["tilt"]))
    xyz, area, fa = oracle.fibonacci_directions(M)
    return vert, pairs, normals, xyz, area, fa


def test_structures_equal_the_reference():
    g = np.load(GOLDEN / "sweep_structs_n3_m12.npz")
    vert, pairs, normals, xyz, _, _ = case_inputs(g)
    assert np.array_equal(oracle.sweep_nodes(vert), g["nodes"])
    st = oracle.SweepStructures(vert, pairs, normals, xyz)
    assert np.array_equal(st.order, g["order"])
    assert np.array_equal(st.states, g["states"])
    assert np.array_equal(st.rec_off, g["rec_off"])
    assert np.array_equal(st.s, g["s"])
    assert np.array_equal(st.face.astype(np.uint8), g["face"])
    assert [len(lv) - 1 for lv in st.levels] == g["steps"].tolist()


def sweep_inputs(g, N, M):
    rng = np.random.default_rng(int(g["seed"]))
    S = rng.uniform(0.0, 2.0, (M, N))
    il0 = rng.uniform(0.1, 1.0, (M, N, 4))
    assert np.array_equal(S.ravel()[:8], g["S_pin"]) and np.array_equal(il0.ravel()[:8], g["il0_pin"])
    return S, il0


def oracle_medium(g, cls, N):
    if cls == 11:
        return oracle.medium_gas(g["density"], g["pressure"])
    (a, b, q), kw = CLASS_MEDIUM[cls]
    return oracle.medium(**kw), np.full(N, a), np.full(N, b), np.full(N, q)


@pytest.mark.parametrize("cls", [0, 1, 2, 3, 10, 11])
def test_oracle_sweep_equals_the_reference(cls):
    g = np.load(GOLDEN / "sweep_classes_n2_m16.npz")
    vert, pairs, normals, xyz, _, _ = case_inputs(g)
    st = oracle.SweepStructures(vert, pairs, normals, xyz)
    N, M = st.N, st.D
    S, il = sweep_inputs(g, N, M)
    md, a, b, q = oracle_medium(g, cls, N)
    norm = oracle.sweep(st, S, a, b, q, il, md=md, use_nodes=True)
    assert np.array_equal(il, g[f"illum_{cls}"])
    ref_norm = g["norms"][list(g["classes"]).index(cls)]
    assert norm == ref_norm or (np.isnan(norm) and np.isnan(ref_norm))


def test_gas_medium_equals_the_oracle(native_lib):
    from relativistic_solver_hllc_gb300 import medium_gas

    g = np.load(GOLDEN / "sweep_classes_n2_m16.npz")
    md, a, b, q = medium_gas(g["density"], g["pressure"])
    md2, a2, b2, q2 = oracle.medium_gas(g["density"], g["pressure"])
    assert np.array_equal(a, a2) and np.array_equal(b, b2) and np.array_equal(q, q2)
    assert (md.mode, md.s_scale, md.i_scale) == (md2.mode, md2.s_scale, md2.i_scale)


@pytest.mark.gpu
@pytest.mark.parametrize("cls", [0, 1, 2, 3, 10, 11])
def test_device_sweep_on_reference_structures(ctx, cls):
    from relativistic_solver_hllc_gb300 import LOCX0_DTYPE, medium, medium_gas

    g = np.load(GOLDEN / "sweep_classes_n2_m16.npz")
    vert, pairs, normals, xyz, area, fa = case_inputs(g)
    N, M = vert.shape[0], int(g["M"])
    ctx.init(xyz, area, fa, N)
    ctx.sweep_set_mesh(vert, pairs, normals)
    # the reference's own structures, in its file layouts
    st = oracle.SweepStructures(vert, pairs, normals, xyz)
    for d in range(M):
        a0, a1 = st.rec_off[d], st.rec_off[d + 1]
        rec = np.zeros(a1 - a0, dtype=LOCX0_DTYPE)
        rec["s"] = st.s[a0:a1]
        rec["in_face_id"] = st.face[a0:a1]
        ctx.sweep_import_direction(d, st.order[d], st.states[d], rec)
    S, il0 = sweep_inputs(g, N, M)
    if cls == 11:
        md, a, b, q = medium_gas(g["density"], g["pressure"])
    else:
        (a, b, q), kw = CLASS_MEDIUM[cls]
        md, a, b, q = medium(**kw), np.full(N, a), np.full(N, b), np.full(N, q)
    ctx.sweep_set_medium(md, a, b, q)
    ctx.send_scattering(S)
    ctx.copy_illum(il0.ravel())
    ctx.sweep()
    got = np.empty(M * N * 4)
    ctx.read_illum(got)
    ref = g[f"illum_{cls}"].ravel()
    den = np.maximum(np.abs(ref), 1e-300)
    assert np.max(np.abs(got - ref) / den) <= 1e-12
