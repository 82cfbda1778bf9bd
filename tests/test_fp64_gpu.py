"""Parity of the FP64 CUDA path with the oracle and the reference's golden
vectors, through the C ABI.  Tolerance: 1e-12 relative (the FP64 contract of
the scattering integral); moments 1e-12 relative to the energy scale."""
import numpy as np
import pytest

import oracle
from conftest import GOLDEN
from relativistic_solver_hllc_gb300 import (
    PHASE_HG,
    STREAM_PARAMS,
    STREAM_SCATTERING_1,
    STREAM_SCATTERING_2,
    Context,
    RtsError,
    _native,
)

pytestmark = pytest.mark.gpu
TOL = 1e-12
CASES = ["tiny_n7_m3", "n64_m17", "n33_m16_part", "n130_m1", "n5_m2", "n257_m40"]


def rel_err(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


def golden(name):
    g = np.load(GOLDEN / f"{name}.npz")
    N, M = int(g["N"]), int(g["M"])
    il = oracle.illum(int(g["seed"]), float(g["mu"]), float(g["sigma"]), N, M,
                      independent_faces=bool(g["independent_faces"]))
    return g, N, M, il


@pytest.mark.parametrize("name", CASES)
def test_scattering_sync_matches_golden(ctx, name):
    g, N, M, il = golden(name)
    xyz, area, fa = oracle.fibonacci_directions(M)
    d, s = int(g["disp"]), int(g["size"])
    ctx.init(xyz, area, fa, N, d, d + s)
    S = ctx.scattering(il)
    assert S.shape == g["S"].shape
    assert rel_err(S, g["S"]) <= TOL


@pytest.mark.parametrize("name", CASES)
def test_moments_match_golden(ctx, name):
    g, N, M, il = golden(name)
    xyz, area, fa = oracle.fibonacci_directions(M)
    ctx.init(xyz, area, fa, N)
    ctx.copy_illum(il)
    e, f = ctx.moments(STREAM_PARAMS)
    assert rel_err(e, g["energy"]) <= TOL
    assert float(np.max(np.abs(f - g["stream"]) / np.abs(g["energy"])[:, None])) <= TOL


def test_async_streams_like_the_source_iteration(ctx):
    """Per-direction H2D on stream 0, then the two scattering launches of
    Illum_async.cpp:1019-1020 on streams 1 and 2 into one host array."""
    N, M = 1000, 37
    xyz, area, fa = oracle.fibonacci_directions(M)
    il = oracle.illum(4, 0.0, 1.2, N, M, independent_faces=True)
    ctx.init(xyz, area, fa, N)
    for j in range(M):
        ctx.send_illum_async(4 * N, 4 * N * j, 4 * N * j, il)
    out = np.zeros(M * N)
    size_1 = M // 3
    ctx.scattering_async(0, size_1, STREAM_SCATTERING_1, out)
    ctx.scattering_async(size_1, M, STREAM_SCATTERING_2, out)
    ctx.wait()
    ref = oracle.calculate_int_cpu(N, xyz, area, fa, il)
    assert rel_err(out.reshape(M, N), ref) <= TOL
    # the library-owned pinned array is the default destination
    ctx.scattering_async(0, M, STREAM_SCATTERING_1)
    ctx.sync_stream(STREAM_SCATTERING_1)
    assert rel_err(ctx.host_scattering().reshape(M, N), ref) <= TOL


@pytest.mark.parametrize("prec", ["fp64", "fp16x3"])
def test_call_on_stream_2_waits_for_input_writes(ctx, prec):
    """A call on scattering stream 2 sees every Illum write queued on stream 1
    before it -- copies queued after a stream-1 call, and the Illum the FP64
    source iteration relaxed -- while the pair of calls of the source
    iteration overlaps (rows both cover agree bit for bit)."""
    N, M = 20_000, 37
    tol = TOL if prec == "fp64" else 1e-5
    xyz, area, fa = oracle.fibonacci_directions(M)
    il_a = oracle.illum(4, 0.0, 1.2, N, M, independent_faces=True)
    il_b = oracle.illum(5, 0.0, 0.8, N, M, independent_faces=True)
    ctx.init(xyz, area, fa, N)
    ctx.set_precision(prec)
    try:
        out1, out2 = np.zeros(M * N), np.zeros(M * N)
        for j in range(M):
            ctx.send_illum_async(4 * N, 4 * N * j, 4 * N * j, il_a)
        ctx.scattering_async(0, M // 3, STREAM_SCATTERING_1, out1)
        ctx.scattering_async(0, M, STREAM_SCATTERING_2, out2)
        ctx.wait()
        ref_a = oracle.calculate_int_cpu(N, xyz, area, fa, il_a)
        assert rel_err(out2.reshape(M, N), ref_a) <= tol
        assert np.array_equal(out1[: (M // 3) * N], out2[: (M // 3) * N])
        # new Illum queued on stream 1 after a stream-1 call, read on stream 2
        ctx.scattering_async(0, M, STREAM_SCATTERING_1, out1)
        for j in range(M):
            ctx.send_illum_async(4 * N, 4 * N * j, 4 * N * j, il_b)
        ctx.scattering_async(0, M, STREAM_SCATTERING_2, out2)
        ctx.wait()
        assert rel_err(out1.reshape(M, N), ref_a) <= tol
        ref_b = oracle.calculate_int_cpu(N, xyz, area, fa, il_b)
        assert rel_err(out2.reshape(M, N), ref_b) <= tol
    finally:
        ctx.set_precision("fp64")
    # the FP64 iteration relaxes the device Illum on stream 1
    ctx.solve_setup("fp64", oracle.uniform(2, 2, 0.1, 1.0, N), 0.9)
    ctx.solve_step_async(True)
    ctx.scattering_async(0, M, STREAM_SCATTERING_2, out2)
    ctx.wait()
    relaxed = ctx.read_illum(np.empty(M * N * 4))
    ref_r = oracle.calculate_int_cpu(N, xyz, area, fa, relaxed)
    assert rel_err(out2.reshape(M, N), ref_r) <= TOL


def test_shard_of_out_directions(ctx):
    """InitDevice(start, end) shards out-directions like d_GetS_MPI_Stream."""
    N, M = 300, 50
    xyz, area, fa = oracle.fibonacci_directions(M)
    il = oracle.illum(8, 0.0, 1.0, N, M)
    for start, end in [(0, 50), (10, 27), (49, 50)]:
        ctx.init(xyz, area, fa, N, start, end)
        ctx.copy_illum(il)
        out = np.zeros((end - start) * N)
        ctx.scattering_async(0, end - start, STREAM_SCATTERING_2, out)
        ctx.wait()
        ref = oracle.calculate_int_cpu(N, xyz, area, fa, il, start, end - start)
        assert rel_err(out.reshape(end - start, N), ref) <= TOL


def test_config1_full(ctx):
    """Configuration 1: 10,368 cells x 200 directions, Thomson, lognormal(0,1)."""
    g = np.load(GOLDEN / "config1_sample.npz")
    N, M = int(g["N"]), int(g["M"])
    xyz, area, fa = oracle.fibonacci_directions(M)
    il = oracle.illum(0, 0.0, 1.0, N, M)
    ctx.init(xyz, area, fa, N)
    S = ctx.scattering(il)
    assert rel_err(S[:, g["cells"]], g["S_cells"]) <= TOL
    assert rel_err(S.sum(axis=1), g["row_sums"]) <= TOL
    ref = oracle.calculate_int_cpu(N, xyz, area, fa, il)
    assert rel_err(S, ref) <= TOL


def test_source_update_and_residual(ctx):
    N, M, lam = 517, 29, 0.5
    xyz, area, fa = oracle.fibonacci_directions(M)
    il = oracle.illum(2, 0.0, 1.0, N, M)
    B = oracle.uniform(2, 2, 0.1, 1.0, N)
    ctx.init(xyz, area, fa, N)
    S0 = ctx.scattering(il)
    r = ctx.source_update(B, lam, 0, M)
    out = np.zeros(M * N)
    ctx.read_scattering(0, M, STREAM_SCATTERING_1, out)
    ctx.wait()
    ref_int = oracle.calculate_int_cpu(N, xyz, area, fa, il)
    ref = oracle.source_update(ref_int, B, lam)
    assert rel_err(S0, ref_int) <= TOL
    assert rel_err(out.reshape(M, N), ref) <= TOL
    assert abs(r - np.max(np.abs(ref - ref_int))) <= TOL * np.max(np.abs(ref))


@pytest.mark.parametrize("relax", [False, True])
def test_fp64_source_iteration(ctx, relax):
    N, M, lam, iters = 700, 24, 0.9, 4
    xyz, area, fa = oracle.fibonacci_directions(M)
    il = oracle.illum(1, 0.0, 1.5, N, M)
    B = oracle.uniform(1, 2, 0.1, 1.0, N)
    ctx.init(xyz, area, fa, N)
    ctx.copy_illum(il)
    ctx.solve_setup("fp64", B, lam)
    res = [ctx.solve_step(relax) for _ in range(iters)]
    S = ctx.solve_read()
    W = oracle.weights_thomson(xyz, area, fa)
    S_ref, r_ref, _ = oracle.iterate(W, oracle.face_mean(il, N, M), B, lam, iters, relax)
    assert rel_err(S, S_ref) <= TOL
    assert rel_err(np.array(res), r_ref) <= 1e-10


def test_hg_phase_matches_matrix_oracle(ctx):
    N, M, g = 400, 60, 0.7
    xyz, area, fa = oracle.fibonacci_directions(M)
    il = oracle.illum(5, 0.0, 1.0, N, M)
    ctx.init(xyz, area, fa, N)
    ctx.set_phase(PHASE_HG, g)
    S = ctx.scattering(il)
    W = oracle.weights_hg(xyz, area, g)
    ref = oracle.scatter_matrix(W, oracle.face_mean(il, N, M))
    assert rel_err(S, ref) <= TOL
    # custom weights reproduce the same result
    ctx.set_weights(W)
    assert rel_err(ctx.scattering(il), ref) <= TOL


def test_synthetic_generator_matches_cpu(ctx):
    N, M = 333, 11
    xyz, area, fa = oracle.fibonacci_directions(M)
    ctx.init(xyz, area, fa, N)
    for indep in (False, True):
        ctx.synth_illum(42, 0.0, 1.5, indep)
        cpu = oracle.illum(42, 0.0, 1.5, N, M, independent_faces=indep)
        ctx.solve_setup("fp64", np.ones(N), 0.0)
        ib = ctx.solve_read_ibar()
        # device exp/log/cos against glibc: a few ulp at most
        assert rel_err(ib, oracle.face_mean(cpu, N, M)) <= 1e-13


def test_errors_are_status_codes(ctx):
    N, M = 64, 8
    xyz, area, fa = oracle.fibonacci_directions(M)
    with pytest.raises(RtsError) as e:
        ctx.scattering_async(0, 1, STREAM_SCATTERING_1)
    assert e.value.status == _native.ERR_BAD_STATE
    with pytest.raises(RtsError) as e:
        ctx.init(xyz, area, fa, N, 3, 2)
    assert e.value.status == _native.ERR_INVALID_ARGUMENT
    ctx.init(xyz, area, fa, N)
    il = np.zeros(M * N * 4)
    with pytest.raises(RtsError) as e:
        ctx.send_illum_async(8, M * N * 4 - 4, 0, il)
    assert e.value.status == _native.ERR_INVALID_ARGUMENT
    with pytest.raises(RtsError) as e:
        ctx.scattering_async(0, M + 1, STREAM_SCATTERING_1)
    assert e.value.status == _native.ERR_INVALID_ARGUMENT
    with pytest.raises(RtsError) as e:
        ctx.scattering_async(0, M, 7)
    assert e.value.status == _native.ERR_INVALID_ARGUMENT
    with pytest.raises(RtsError) as e:
        ctx.solve_step()
    assert e.value.status == _native.ERR_BAD_STATE
    assert "rts_solve_step" in ctx.last_error


def test_hbm_budget_rejects_oversized_grid(ctx):
    M = 100
    xyz, area, fa = oracle.fibonacci_directions(M)
    used = ctx.hbm_used()
    ctx.set_hbm_budget(used + (64 << 20))
    with pytest.raises(RtsError) as e:
        ctx.init(xyz, area, fa, 1_000_000)  # 3.2 GB of Illum
    assert e.value.status == _native.ERR_OVER_BUDGET
    assert ctx.hbm_used() == used
    ctx.init(xyz, area, fa, 1000)  # fits
    assert ctx.hbm_used() > used


def test_sync_deadline_returns_timeout(ctx):
    """A host wait with a deadline reports RTS_ERR_TIMEOUT while the work runs,
    and the context stays usable afterwards."""
    N, M = 200_000, 400
    xyz, area, fa = oracle.fibonacci_directions(M)
    ctx.init(xyz, area, fa, N)
    ctx.synth_illum(1, 0.0, 1.0)
    for _ in range(3):
        ctx.scattering_async(0, M, STREAM_SCATTERING_2)
    with pytest.raises(RtsError) as e:
        ctx.sync_stream(STREAM_SCATTERING_2, timeout_us=1)
    assert e.value.status == _native.ERR_TIMEOUT
    ctx.sync_stream(STREAM_SCATTERING_2, timeout_us=-1)
    ctx.wait(timeout_us=60_000_000)
