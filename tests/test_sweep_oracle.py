"""The oracle of the transport sweep on the CPU: the synthetic mesh, the
per-direction structures (make_illum_struct + build_graph restated), known
answers of the sweep, and the product's host-only mesh generator against the
oracle's.  The pin against the reference's own sweep code is in
test_sweep_golden.py."""
import numpy as np
import pytest

import oracle
from relativistic_solver_hllc_gb300 import mesh_cube


def tet_volume(v):
    return abs(np.linalg.det(np.stack([v[1] - v[0], v[2] - v[0], v[3] - v[0]]))) / 6


@pytest.mark.parametrize("n,tilt", [(2, False), (3, True)])
def test_cube_mesh_is_a_conforming_tiling(n, tilt):
    vert, pairs, normals = oracle.cube_mesh(n, 1, tilt)
    N = 6 * n ** 3
    assert vert.shape == (N, 4, 3)
    assert abs(sum(tet_volume(v) for v in vert) - 1.0) < 1e-12
    inner = pairs >= 0
    # neighbours point back, and the shared face has the opposite normal
    ids = np.flatnonzero(inner.ravel())
    back = pairs.ravel()[pairs.ravel()[ids]]
    assert np.array_equal(back, ids)
    nn = normals.reshape(-1, 3)
    assert np.allclose(nn[ids], -nn[pairs.ravel()[ids]], atol=1e-12)
    assert np.allclose(np.linalg.norm(nn, axis=1), 1.0, atol=1e-14)
    # every boundary face lies on the cube's surface: 2 triangles per side square
    assert (~inner).sum() == 6 * 2 * n * n
    assert (pairs == oracle.BOUND_OUTSOURCE).sum() == 2 * n * n


@pytest.mark.parametrize("n,rule,tilt", [(2, 0, False), (3, 1, True), (4, 1, True)])
def test_product_mesh_equals_oracle_mesh(native_lib, n, rule, tilt):
    a = mesh_cube(n, rule, tilt)
    b = oracle.cube_mesh(n, rule, tilt)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_outward_normals():
    vert, pairs, normals = oracle.cube_mesh(2, 0, True)
    centroid = vert.mean(axis=1)
    FV = [[0, 1, 3], [1, 2, 3], [2, 0, 3], [0, 2, 1]]
    for c in range(0, vert.shape[0], 7):
        for f in range(4):
            fc = vert[c, FV[f]].mean(axis=0)
            assert np.dot(normals[c, f], fc - centroid[c]) > 0


def test_nodes_lie_inside_their_faces():
    vert, _, _ = oracle.cube_mesh(2, 0, True)
    nodes = oracle.sweep_nodes(vert)
    FV = [[0, 1, 3], [1, 2, 3], [2, 0, 3], [0, 2, 1]]
    for c in range(vert.shape[0]):
        for f in range(4):
            A, B, C = vert[c, FV[f]]
            for m in range(3):
                lam = np.linalg.lstsq(np.stack([B - A, C - A]).T, nodes[c, f, m] - A, rcond=None)[0]
                bary = np.array([1 - lam.sum(), *lam])
                assert np.all(bary > 0.1)
                assert np.allclose(A + lam[0] * (B - A) + lam[1] * (C - A), nodes[c, f, m], atol=1e-14)


def test_graph_is_a_dependency_order():
    vert, pairs, normals = oracle.cube_mesh(4, 1, True)
    xyz, _, _ = oracle.fibonacci_directions(20)
    N = vert.shape[0]
    for d in range(20):
        st = oracle.face_states(normals, xyz[d])
        order, off = oracle.sweep_graph(pairs, st)
        assert sorted(order.tolist()) == list(range(N))
        step = np.empty(N, dtype=np.int64)
        for L in range(len(off) - 1):
            seg = order[off[L]:off[L + 1]]
            assert np.all(np.diff(seg) > 0)  # ascending ids within a step
            step[seg] = L
        for c in range(N):
            ups = [pairs[c, f] // 4 for f in range(4) if (st[c] >> f) & 1 and pairs[c, f] >= 0]
            # one step after the latest upstream cell
            assert step[c] == (1 + max(step[u] for u in ups) if ups else 0)


def test_characteristics_hit_their_in_faces():
    vert, pairs, normals = oracle.cube_mesh(3, 1, True)
    xyz, _, _ = oracle.fibonacci_directions(10)
    nodes = oracle.sweep_nodes(vert)
    FV = [[0, 1, 3], [1, 2, 3], [2, 0, 3], [0, 2, 1]]
    for d in range(10):
        st = oracle.face_states(normals, xyz[d])
        order, _ = oracle.sweep_graph(pairs, st)
        s, face = oracle.sweep_x0(vert, normals, nodes, order, st, xyz[d])
        k = 0
        for c in order:
            for f in range(4):
                if (st[c] >> f) & 1:
                    continue
                for m in range(3):
                    g = face[k]
                    assert (st[c] >> g) & 1
                    x0 = nodes[c, f, m] - s[k] * xyz[d]  # back along the direction
                    A = vert[c, FV[g][0]]
                    assert abs(np.dot(normals[c, g], x0 - A)) < 1e-13
                    assert s[k] > 0
                    k += 1
        assert k == s.shape[0]


def structures(n=3, M=16):
    vert, pairs, normals = oracle.cube_mesh(n, 1, True)
    xyz, area, fa = oracle.fibonacci_directions(M)
    return oracle.SweepStructures(vert, pairs, normals, xyz), xyz, area, fa


def test_equilibrium_is_reproduced():
    """alpha = Q, beta = 0 and every boundary at 1: I = 1 everywhere."""
    st, *_ = structures()
    N, D = st.N, st.D
    il = np.zeros((D, N, 4))
    one = np.ones(N)
    oracle.sweep(st, np.zeros((D, N)), 2.0 * one, 0 * one, 2.0 * one, il, bc=(1.0, 1.0, 1.0, 1.0))
    assert np.max(np.abs(il - 1.0)) < 1e-14


def test_vacuum_transports_the_boundary_unchanged():
    st, *_ = structures()
    N, D = st.N, st.D
    il = np.zeros((D, N, 4))
    z = np.zeros(N)
    nrm = oracle.sweep(st, np.zeros((D, N)), z, z, z, il, bc=(0.75, 0.75, 0.75, 0.75))
    assert np.all(il == 0.75)
    assert nrm == 1.0  # from zero: |0 - 0.75| / 0.75


def test_second_sweep_with_same_source_has_zero_norm():
    st, *_ = structures()
    N, D = st.N, st.D
    rng = np.random.default_rng(1)
    a, b, q = rng.uniform(0.5, 2, N), rng.uniform(0, 1, N), rng.uniform(0, 1, N)
    S = rng.uniform(0, 1, (D, N))
    il = rng.uniform(0, 1, (D, N, 4))
    first = oracle.sweep(st, S, a, b, q, il)
    assert first > 0
    again = oracle.sweep(st, S, a, b, q, il)
    assert again == 0.0


def test_absorption_form_limits():
    """Class 2: far from the boundary the intensity settles at Q / alpha."""
    st, *_ = structures(4, 8)
    N, D = st.N, st.D
    one = np.ones(N)
    il = np.zeros((D, N, 4))
    oracle.sweep(st, np.zeros((D, N)), one, 0 * one, 3.0 * one, il, md=oracle.medium(1, s_scale=1e4),
                 bc=(0.0, 0.0, 0.0, 0.0))
    inner = il[il > 0]  # all but the boundary in-faces
    assert inner.size > 0.8 * il.size
    assert np.max(np.abs(inner - 3.0)) < 1e-12
