"""The device transport sweep against the oracle's restatement of the
reference's sweep (Illum_async.cpp:726-783 with GetCurIllum, ReCalcIllum,
BoundaryConditions) and of make_illum_struct / build_graph, through the C ABI.

Tolerances: the per-direction structures match exactly (cell order, step
boundaries, face states, in-faces) and the node distances to 1e-13 relative
(FP64 geometry, fused multiply-adds on the device); Illum after FP64 sweeps
and source iterations to 1e-12 relative (FP64 contract; the device exp
differs from the host's by an ulp); iterations with the FP16x3 tensor-core
scattering to 1e-6 relative (the split-precision contract)."""
import numpy as np
import pytest

import oracle
from relativistic_solver_hllc_gb300 import (
    BOUND_OUTSOURCE,
    LOCX0_DTYPE,
    MEDIUM_ABSORPTION,
    RtsError,
    _native,
    medium,
    mesh_cube,
)

pytestmark = pytest.mark.gpu
TOL = 1e-12


def rel_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    den = np.maximum(np.abs(b), 1e-300)
    mask = (np.abs(a) > 0) | (np.abs(b) > 0)
    return float(np.max(np.abs(a - b)[mask] / den[mask])) if mask.any() else 0.0


def setup(ctx, n, M, tilt=True, rule=1):
    vert, pairs, normals = mesh_cube(n, rule, tilt)
    xyz, area, fa = oracle.fibonacci_directions(M)
    N = vert.shape[0]
    ctx.init(xyz, area, fa, N)
    ctx.sweep_set_mesh(vert, pairs, normals)
    return vert, pairs, normals, xyz, area, fa, N


def coefficients(N, seed, kind):
    rng = np.random.default_rng(seed)
    if kind == "class1":
        return np.full(N, 1.0), np.full(N, 0.5), np.full(N, 1.0)
    if kind == "class10":
        return np.full(N, 0.5), np.full(N, 100.0), np.zeros(N)
    if kind == "thin":  # k s below 1e-3: the reference's own expression
        return np.full(N, 2e-3), np.full(N, 1e-3), rng.uniform(0.0, 1.0, N)
    return rng.uniform(0.5, 3.0, N), rng.uniform(0.0, 2.0, N), rng.uniform(0.0, 1.5, N)


def same_norm(a, b, tol=TOL):
    if np.isinf(a) or np.isinf(b):
        return a == b
    return abs(a - b) <= tol * max(1.0, abs(b))


def test_structures_match_oracle(ctx):
    vert, pairs, normals, xyz, area, fa, N = setup(ctx, 4, 24)
    rec, lev = ctx.sweep_build()
    st = oracle.SweepStructures(vert, pairs, normals, xyz)
    assert rec == st.s.shape[0]
    assert lev == max(len(x) - 1 for x in st.levels)
    for d in range(24):
        order, states, recs = ctx.sweep_export_direction(d)
        assert np.array_equal(order, st.order[d])
        assert np.array_equal(states, st.states[d])
        a, b = st.rec_off[d], st.rec_off[d + 1]
        assert np.array_equal(recs["in_face_id"], st.face[a:b].astype(np.uint8))
        assert rel_err(recs["s"], st.s[a:b]) <= 1e-13


@pytest.mark.parametrize("kind,mode", [("class1", 0), ("class10", 0), ("random", 0), ("random", 1), ("ball", 0),
                                       ("thin", 0)])
def test_sweep_matches_oracle(ctx, kind, mode):
    vert, pairs, normals, xyz, area, fa, N = setup(ctx, 4, 40)
    ctx.sweep_build()
    st = oracle.SweepStructures(vert, pairs, normals, xyz)
    a, b, q = coefficients(N, 5, "random" if kind == "ball" else kind)
    if kind == "ball":
        md = medium(0, ball=(0.5, 0.4, 0.5), radius=0.3, ball_coef=(0.5, 0.5, 2.0))
    else:
        md = medium(mode, s_scale=3.0 if mode == MEDIUM_ABSORPTION else 1.0)
    bc = (0.0, 0.25, 1.0, 0.5)
    ctx.sweep_set_medium(md, a, b, q, bc)
    il0 = np.random.default_rng(9).uniform(0.1, 1.0, (40, N, 4))
    # the sweep's source term is the device scattering array: fill it with the
    # FP64 integral of il0 (which also leaves il0 as the device Illum) and
    # hand the oracle the same numbers
    S = ctx.scattering(il0.ravel()).reshape(40, N)
    ref = il0.copy()
    n_ref = oracle.sweep(st, S, a, b, q, ref, md=oracle.medium(md.mode, md.s_scale, md.i_scale, tuple(md.ball),
                                                                md.radius, (md.ball_alpha, md.ball_beta, md.ball_q)),
                         bc=bc)
    n_dev = ctx.sweep()
    got = np.empty(40 * N * 4)
    ctx.read_illum(got)
    assert rel_err(got, ref.ravel()) <= TOL, rel_err(got, ref.ravel())
    assert same_norm(n_dev, n_ref), (n_dev, n_ref)


def oracle_solve(st, xyz, area, fa, il, S, a, b, q, md, bc, iters, accuracy, W=None):
    """Sweeps and scattering integrals alternated as in the reference's
    CalculateIllum loop; W (M x M) replaces the Thomson integral when given."""
    N, D = st.N, st.D
    norms = []
    for it in range(iters):
        norms.append(oracle.sweep(st, S, a, b, q, il, md=md, bc=bc))
        if iters > 1 and W is None:
            S = oracle.calculate_int_cpu(N, xyz, area, fa, il.ravel()).reshape(D, N)
        elif iters > 1:
            S = oracle.scatter_matrix(W, oracle.face_mean(il.ravel(), N, D))
        if not norms[-1] > accuracy:
            break
    return np.array(norms), S


@pytest.mark.parametrize("precision,tol", [("fp64", TOL), ("fp16x3", 1e-6)])
def test_illum_solve_matches_oracle(ctx, precision, tol):
    M = 30
    vert, pairs, normals, xyz, area, fa, N = setup(ctx, 4, M)
    ctx.sweep_build()
    st = oracle.SweepStructures(vert, pairs, normals, xyz)
    a, b, q = coefficients(N, 2, "class1")
    bc = (0.0, 0.0, 1.0, 0.0)
    ctx.sweep_set_medium(medium(), a, b, q, bc)
    il = np.zeros((M, N, 4))
    ctx.copy_illum(il.ravel())
    norms = ctx.illum_solve(precision, max_iter=6, accuracy=1e-300)
    ref_norms, _ = oracle_solve(st, xyz, area, fa, il, np.zeros((M, N)), a, b, q, oracle.medium(), bc, 6, 1e-300)
    got = np.empty(M * N * 4)
    ctx.read_illum(got)
    assert len(norms) == len(ref_norms) == 6
    assert rel_err(got, il.ravel()) <= tol, rel_err(got, il.ravel())
    assert rel_err(norms[1:], ref_norms[1:]) <= 1e-9 if precision == "fp64" else True


@pytest.mark.parametrize("precision,tol", [("fp64", TOL), ("fp16x3", 1e-6)])
def test_illum_solve_hg_phase(ctx, precision, tol):
    """The source iteration with the Henyey-Greenstein phase function (g = 0.6)
    between sweeps: the device's weights against the oracle's HG matrix."""
    M, g = 24, 0.6
    vert, pairs, normals, xyz, area, fa, N = setup(ctx, 3, M)
    ctx.set_phase(_native.PHASE_HG, g)
    ctx.sweep_build()
    st = oracle.SweepStructures(vert, pairs, normals, xyz)
    a, b, q = coefficients(N, 5, "random")
    bc = (0.0, 0.0, 1.0, 0.0)
    ctx.sweep_set_medium(medium(), a, b, q, bc)
    il = np.zeros((M, N, 4))
    ctx.copy_illum(il.ravel())
    norms = ctx.illum_solve(precision, max_iter=5, accuracy=1e-300)
    W = oracle.weights_hg(xyz, area, g)
    ref_norms, _ = oracle_solve(st, xyz, area, fa, il, np.zeros((M, N)), a, b, q, oracle.medium(), bc, 5, 1e-300,
                                W=W)
    got = np.empty(M * N * 4)
    ctx.read_illum(got)
    assert len(norms) == len(ref_norms) == 5
    assert rel_err(got, il.ravel()) <= tol, rel_err(got, il.ravel())


def test_illum_solve_and_the_calls_share_the_staging(ctx):
    """The device source iteration at a tensor precision prepares its rows
    in the staging of the asynchronous integral calls (FP64 face sums and
    per-cell maxima).  With the iteration between them, the calls still give
    the values they give alone: the pair of calls on the Illum the iteration
    left equals the host-buffer call on that Illum bit for bit (another
    preparation, the same rows), and the pair on the first Illum again
    repeats its first result."""
    M = 30
    S1, S2 = _native.STREAM_SCATTERING_1, _native.STREAM_SCATTERING_2
    vert, pairs, normals, xyz, area, fa, N = setup(ctx, 4, M)
    ctx.sweep_build()
    a, b, q = coefficients(N, 2, "class1")
    ctx.sweep_set_medium(medium(), a, b, q, (0.0, 0.0, 1.0, 0.0))
    il0 = np.random.default_rng(5).uniform(0.1, 1.0, M * N * 4)

    def pair():
        out1, out2 = np.zeros(M * N), np.zeros(M * N)
        ctx.scattering_async(0, M // 3, S1, out1)
        ctx.scattering_async(0, M, S2, out2)
        ctx.wait()
        assert np.array_equal(out1[: (M // 3) * N], out2[: (M // 3) * N])
        return out2

    ctx.set_precision("fp16x3")
    try:
        ctx.copy_illum(il0)
        first = pair()
        ctx.illum_solve("fp16x3", max_iter=3, accuracy=1e-300)
        il1 = np.empty(M * N * 4)
        ctx.read_illum(il1)
        after = pair()
        host_call = ctx.scattering(il1)
        ctx.copy_illum(il0)
        again = pair()
    finally:
        ctx.set_precision("fp64")
    assert np.array_equal(after, host_call.ravel())
    assert np.array_equal(again, first)
    assert rel_err(after.reshape(M, N), oracle.calculate_int_cpu(N, xyz, area, fa, il1)) <= 1e-6
    assert rel_err(first.reshape(M, N), oracle.calculate_int_cpu(N, xyz, area, fa, il0)) <= 1e-6


def test_no_room_for_the_staging(ctx):
    """Under an HBM budget with room for everything the tensor-precision
    source iteration and the integral calls hold except the staging of the
    staged preparation, both prepare their rows directly from the faces: the
    same norms, Illum and integrals bit for bit."""
    M = 30
    S1, S2 = _native.STREAM_SCATTERING_1, _native.STREAM_SCATTERING_2
    il0 = None

    def run(room=None):
        nonlocal il0
        vert, pairs, normals, xyz, area, fa, N = setup(ctx, 4, M)
        ctx.sweep_build()
        a, b, q = coefficients(N, 2, "class1")
        ctx.sweep_set_medium(medium(), a, b, q, (0.0, 0.0, 1.0, 0.0))
        if il0 is None:
            il0 = np.random.default_rng(6).uniform(0.1, 1.0, M * N * 4)
        ctx.copy_illum(np.zeros(M * N * 4))  # the first norm compares against it
        used0 = ctx.hbm_used()
        if room is not None:
            ctx.set_hbm_budget(used0 + room)
        norms = ctx.illum_solve("fp16x3", max_iter=3, accuracy=1e-300)
        il = np.empty(M * N * 4)
        ctx.read_illum(il)
        ctx.set_precision("fp16x3")
        try:
            ctx.copy_illum(il0)
            out1, out2 = np.zeros(M * N), np.zeros(M * N)
            ctx.scattering_async(0, M // 3, S1, out1)
            ctx.scattering_async(0, M, S2, out2)
            ctx.wait()
        finally:
            ctx.set_precision("fp64")
        return N, ctx.hbm_used() - used0, list(norms), il, out2

    try:
        N, held, n1, il1, out1 = run()
        staging = M * N * 8 + N * 8
        _, held2, n2, il2, out2 = run(held - staging // 2)
    finally:
        ctx.set_hbm_budget(1 << 62)
    assert held2 <= held - staging  # the staging was not allocated
    assert n1 == n2
    assert np.array_equal(il1, il2)
    assert np.array_equal(out1, out2)


def test_stored_attenuation_factors_give_the_same_sweep(ctx):
    """The sweep that stores the nodes' attenuation factors, the sweeps that
    read them and the sweeps that evaluate them (RTS_TUNE_SWEEP_CACHE 0) give
    the same Illum and norm bit for bit; a new medium replaces the factors."""
    M = 14
    vert, pairs, normals, xyz, area, fa, N = setup(ctx, 3, M)
    ctx.sweep_build()
    il0 = np.random.default_rng(21).uniform(0.1, 1.0, M * N * 4)
    ctx.scattering(il0)  # the source term of the sweeps
    media = [(medium(), *coefficients(N, 6, "random")),
             (medium(), *coefficients(N, 7, "thin")),  # nodes on the reference's expression
             (medium(ball=(0.5, 0.5, 0.5), radius=0.3, ball_coef=(3.0, 0.5, 0.2)), *coefficients(N, 8, "random")),
             (medium(MEDIUM_ABSORPTION, s_scale=2.0, i_scale=0.5), *coefficients(N, 9, "random"))]
    results = []
    for md, a, b, q in media:
        ctx.set_tuning(_native.TUNE_SWEEP_CACHE, 1)
        ctx.sweep_set_medium(md, a, b, q)
        runs = []
        for cache in (1, 1, 1, 0):  # stores, reads, reads, evaluates
            if cache == 0:
                ctx.set_tuning(_native.TUNE_SWEEP_CACHE, 0)
            ctx.copy_illum(il0)
            n = ctx.sweep()
            got = np.empty(M * N * 4)
            ctx.read_illum(got)
            runs.append((n, got))
        for n, got in runs[1:]:
            assert np.array_equal(got, runs[0][1]) and n == runs[0][0]
        assert all(not np.array_equal(runs[0][1], r) for r in results)
        results.append(runs[0][1])
    # factors stored under one medium are not read under the next
    ctx.set_tuning(_native.TUNE_SWEEP_CACHE, 1)
    md, a, b, q = media[0]
    ctx.sweep_set_medium(md, a, b, q)
    ctx.copy_illum(il0)
    ctx.sweep()
    ctx.sweep_set_medium(*media[1])
    ctx.copy_illum(il0)
    ctx.sweep()
    got = np.empty(M * N * 4)
    ctx.read_illum(got)
    assert np.array_equal(got, results[1])


def test_illum_solve_stops_at_accuracy(ctx):
    M = 16
    vert, pairs, normals, xyz, area, fa, N = setup(ctx, 3, M)
    ctx.sweep_build()
    a, b, q = coefficients(N, 2, "class1")
    ctx.sweep_set_medium(medium(), a, b, q)
    ctx.copy_illum(np.zeros(M * N * 4))
    norms = ctx.illum_solve("fp64", max_iter=200, accuracy=1e-8)
    assert norms[-1] <= 1e-8 and len(norms) < 200
    assert np.all(norms[:-1] > 1e-8)


def test_import_equals_build(ctx):
    """The reference's file layouts (graph, state_face, LocX0) exported from
    the built structures and imported again give the same sweep."""
    M = 12
    vert, pairs, normals, xyz, area, fa, N = setup(ctx, 3, M)
    ctx.sweep_build()
    a, b, q = coefficients(N, 4, "random")
    ctx.sweep_set_medium(medium(), a, b, q)
    il0 = np.random.default_rng(3).uniform(0.1, 1.0, M * N * 4)
    ctx.copy_illum(il0)
    ctx.sweep()
    built = np.empty(M * N * 4)
    ctx.read_illum(built)
    files = [ctx.sweep_export_direction(d) for d in range(M)]
    # reverse each step's cells: still a valid dependency order
    for d, (order, states, recs) in enumerate(files):
        st = oracle.SweepStructures(vert, pairs, normals, xyz[d:d + 1])
        rev = np.concatenate([order[st.levels[0][i]:st.levels[0][i + 1]][::-1] for i in range(len(st.levels[0]) - 1)])
        # records follow the file's cell order
        pos = {int(c): i for i, c in enumerate(order)}
        nrec = 3 * (4 - np.array([bin(int(s)).count("1") for s in states]))
        start = np.concatenate([[0], np.cumsum(nrec[order])])
        recs2 = np.concatenate([recs[start[pos[int(c)]]:start[pos[int(c)] + 1]] for c in rev])
        ctx.sweep_import_direction(d, rev, states, recs2)
    ctx.copy_illum(il0)
    ctx.sweep()
    imported = np.empty(M * N * 4)
    ctx.read_illum(imported)
    assert np.array_equal(built, imported)


def test_degenerate_direction_is_reported(ctx):
    # the axis-aligned cube: the first Fibonacci direction (y = 0) runs along
    # the y faces, where no in-face contains the back-traced node
    setup(ctx, 3, 8, tilt=False)
    with pytest.raises(RtsError) as e:
        ctx.sweep_build()
    assert e.value.status == _native.ERR_UNSUPPORTED


def test_sweep_needs_structures_and_medium(ctx):
    vert, pairs, normals, xyz, area, fa, N = setup(ctx, 2, 4)
    with pytest.raises(RtsError) as e:
        ctx.sweep()
    assert e.value.status == _native.ERR_BAD_STATE
    ctx.sweep_build()
    with pytest.raises(RtsError) as e:
        ctx.sweep()
    assert e.value.status == _native.ERR_BAD_STATE
    bad = pairs.copy()
    bad[0, 0] = 4 * N + 7
    with pytest.raises(RtsError) as e:
        ctx.sweep_set_mesh(vert, bad, normals)
    assert e.value.status == _native.ERR_INVALID_ARGUMENT


def test_boundary_codes_of_the_cube(ctx):
    vert, pairs, normals = mesh_cube(3, 1, True)
    assert (pairs == BOUND_OUTSOURCE).sum() == 2 * 9
    assert LOCX0_DTYPE.itemsize == 32


def test_sweep_exponential_within_two_ulp_of_cuda(ctx):
    """The sweep's table-driven exp against CUDA's exp over [-700, 0]: each is
    within about an ulp of the exact value, so they differ by at most 2."""
    assert ctx.sweep_exp_check(1 << 22) <= 2.0


def warp(x, eps):
    """A smooth deformation of the cube (a function of position, so the
    cells sharing a vertex move it together): irregular tetrahedra."""
    s = np.sin(2 * np.pi * x)
    return x + eps * np.stack([s[..., 1] * s[..., 2], s[..., 2] * s[..., 0], s[..., 0] * s[..., 1]], -1)


def test_sweep_on_a_warped_mesh(ctx):
    vert, pairs, _ = mesh_cube(4, 1, True)
    vert = warp(vert, 0.05)
    normals = oracle.face_normals(vert)
    M = 48
    xyz, area, fa = oracle.fibonacci_directions(M)
    N = vert.shape[0]
    ctx.init(xyz, area, fa, N)
    ctx.sweep_set_mesh(vert, pairs, normals)
    ctx.sweep_build()
    st = oracle.SweepStructures(vert, pairs, normals, xyz)
    for d in (0, 17, 47):
        order, states, recs = ctx.sweep_export_direction(d)
        assert np.array_equal(order, st.order[d]) and np.array_equal(states, st.states[d])
        a0, a1 = st.rec_off[d], st.rec_off[d + 1]
        assert np.array_equal(recs["in_face_id"], st.face[a0:a1].astype(np.uint8))
    a, b, q = coefficients(N, 8, "random")
    ctx.sweep_set_medium(medium(), a, b, q, (0.2, 0.0, 1.0, 0.0))
    il0 = np.random.default_rng(12).uniform(0.1, 1.0, (M, N, 4))
    S = ctx.scattering(il0.ravel()).reshape(M, N)
    ref = il0.copy()
    n_ref = oracle.sweep(st, S, a, b, q, ref, bc=(0.2, 0.0, 1.0, 0.0))
    n_dev = ctx.sweep()
    got = np.empty(M * N * 4)
    ctx.read_illum(got)
    assert rel_err(got, ref.ravel()) <= TOL
    assert same_norm(n_dev, n_ref)


def test_direction_shards_equal_the_whole(native_lib):
    """The reference shards the sweep by direction over its ranks
    (Illum_async.cpp:726-784 on each rank's local directions).  Two contexts
    owning directions [0, 10) and [10, 24) -- each sweeping its own rows of
    Illum with the scattering of its own out-directions -- reproduce the
    single-context sweep bit for bit, and the larger of their norms is its
    norm.  (The contexts run one after the other on the one GPU.)"""
    from relativistic_solver_hllc_gb300 import Context

    M = 24
    vert, pairs, normals = mesh_cube(3, 1, True)
    xyz, area, fa = oracle.fibonacci_directions(M)
    N = vert.shape[0]
    a, b, q = coefficients(N, 6, "random")
    il0 = np.random.default_rng(21).uniform(0.1, 1.0, M * N * 4)

    def run(start, end):
        with Context(0) as c:
            c.init(xyz, area, fa, N, start, end)
            c.sweep_set_mesh(vert, pairs, normals)
            c.sweep_build()
            c.sweep_set_medium(medium(), a, b, q)
            c.scattering(il0)  # S of the local out-directions from il0; leaves il0 on the device
            norm = c.sweep()
            out = np.empty(M * N * 4)
            c.read_illum(out)
        return out.reshape(M, N * 4)[start:end], norm

    whole, n_whole = run(0, M)
    lo, n_lo = run(0, 10)
    hi, n_hi = run(10, M)
    assert np.array_equal(np.concatenate([lo, hi]), whole)
    assert max(n_lo, n_hi) == n_whole


def test_import_rejects_inconsistent_files(ctx):
    """rts_sweep_import_direction checks the reference's files against the
    mesh: the record count the face states imply, an order that lists
    upstream cells first, and records naming in-faces only."""
    M = 4
    vert, pairs, normals, xyz, area, fa, N = setup(ctx, 2, M)
    ctx.sweep_build()
    order, states, recs = ctx.sweep_export_direction(1)
    with pytest.raises(RtsError) as e:
        ctx.sweep_import_direction(1, order, states, recs[:-3])
    assert e.value.status == _native.ERR_INVALID_ARGUMENT
    with pytest.raises(RtsError) as e:
        ctx.sweep_import_direction(1, order[::-1].copy(), states, recs)
    assert e.value.status == _native.ERR_INVALID_ARGUMENT
    bad = recs.copy()
    c0 = int(order[0])
    out_face = next(f for f in range(4) if not (int(states[c0]) >> f) & 1)
    bad["in_face_id"][0] = out_face
    with pytest.raises(RtsError) as e:
        ctx.sweep_import_direction(1, order, states, bad)
    assert e.value.status == _native.ERR_INVALID_ARGUMENT
    # the consistent files are accepted and sweep as built
    ctx.sweep_import_direction(1, order, states, recs)
