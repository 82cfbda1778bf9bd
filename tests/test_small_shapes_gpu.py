"""The smallest shapes on every path, against the oracle.

One cell and one direction; fewer than 16 out-directions, so that a tile
is 16 columns wide and three of the epilogue's four column slices are empty;
16 directions, where the conservation correction's extra output column
(index M) opens an 8-column block and a column slice of its own; cell counts
just below and above one 128-row tile.  The FP64 kernel (1e-12), the
tensor-core iteration (single evaluation and relaxed steps), the pair of
asynchronous calls and the host-buffer call at a tensor precision, and
batched problems down to the minimum tile width of 16 (the width leaves
every output's arithmetic unchanged, so the results are bit-identical to
the automatic width).

Tolerances (max relative error against the oracle): FP64 1e-12; fp16x3 and
tf32x3 1e-6; bf16x3 2e-5; relaxed steps as the single evaluation (4x for
bf16x3, whose 16-bit split errors compound through the relaxation).
"""
import numpy as np
import pytest

import oracle
from relativistic_solver_hllc_gb300 import STREAM_SCATTERING_1, STREAM_SCATTERING_2
from relativistic_solver_hllc_gb300._native import PHASE_THOMSON, Batch, problem_desc

pytestmark = pytest.mark.gpu
TOL = {"fp16x3": 1e-6, "bf16x3": 2e-5, "tf32x3": 1e-6}
RELAX_TOL = {"fp16x3": 1e-6, "bf16x3": 8e-5, "tf32x3": 1e-6}
SHAPES = [(1, 1), (1, 16), (5, 3), (127, 15), (129, 16), (130, 33)]


def rel_err(a, b):
    return float(np.max(np.abs(a - b) / np.abs(b)))


def problem(N, M, seed):
    xyz, area, fa = oracle.fibonacci_directions(M)
    il = oracle.illum(seed, 0.0, 1.5, N, M, independent_faces=True)
    B = oracle.uniform(seed, 2, 0.1, 1.0, N)
    return xyz, area, fa, il, B


# the FP64 kernel's tiles of 64 out-directions and its last, narrower tile:
# 16 (M = 1, 3, 15, 16, 200), 32 (90), 48 (33), 64 wide (127: 63 used)
FP64_SHAPES = SHAPES + [(700, 90), (300, 127), (257, 200)]


@pytest.mark.parametrize("N,M", FP64_SHAPES)
def test_fp64_small_shapes(ctx, N, M):
    xyz, area, fa, il, _ = problem(N, M, 3)
    ctx.init(xyz, area, fa, N)
    S = ctx.scattering(il).reshape(M, N)
    assert rel_err(S, oracle.calculate_int_cpu(N, xyz, area, fa, il)) <= 1e-12


@pytest.mark.parametrize("prec", ["fp16x3", "bf16x3", "tf32x3"])
@pytest.mark.parametrize("N,M", SHAPES)
def test_tensor_iteration_small_shapes(ctx, prec, N, M):
    lam, iters = 0.9, 3
    xyz, area, fa, il, B = problem(N, M, 4)
    ctx.init(xyz, area, fa, N)
    ctx.copy_illum(il)
    ctx.solve_setup(prec, B, lam)
    ctx.solve_step(False)
    ref = oracle.source_update(oracle.calculate_int_cpu(N, xyz, area, fa, il), B, lam)
    assert rel_err(ctx.solve_read(), ref) <= TOL[prec]
    # relaxed steps with the conservation correction, from the same input
    ctx.copy_illum(il)
    ctx.solve_setup(prec, B, lam)
    for _ in range(iters):
        ctx.solve_step(True)
    W = oracle.weights_thomson(xyz, area, fa)
    S_ref, _, _ = oracle.iterate(W, oracle.face_mean(il, N, M), B, lam, iters, True)
    assert rel_err(ctx.solve_read(), S_ref) <= RELAX_TOL[prec]


@pytest.mark.parametrize("prec", ["fp16x3", "tf32x3"])
@pytest.mark.parametrize("N,M", SHAPES)
def test_calls_at_tensor_precision_small_shapes(ctx, prec, N, M):
    """The reference's pair of asynchronous calls ([0, M/3) rounded up on
    scattering stream 1, [0, M) on stream 2) and the host-buffer call."""
    xyz, area, fa, il, _ = problem(N, M, 5)
    ref = oracle.calculate_int_cpu(N, xyz, area, fa, il)
    ctx.init(xyz, area, fa, N)
    ctx.set_precision(prec)
    try:
        S_sync = ctx.scattering(il).reshape(M, N)
        ctx.copy_illum(il)
        m1 = max(1, M // 3)
        out1, out2 = np.zeros(M * N), np.zeros(M * N)
        ctx.scattering_async(0, m1, STREAM_SCATTERING_1, out1)
        ctx.scattering_async(0, M, STREAM_SCATTERING_2, out2)
        ctx.wait()
    finally:
        ctx.set_precision("fp64")
    out1, out2 = out1.reshape(M, N), out2.reshape(M, N)
    assert rel_err(out2, ref) <= TOL[prec]
    assert rel_err(S_sync, ref) <= TOL[prec]
    assert np.array_equal(out1[:m1], out2[:m1])


@pytest.mark.parametrize("N,M", [(1, 1), (5, 3), (127, 15), (300, 40)])
def test_batch_minimum_tile_width(ctx, N, M):
    """Batched problems at the automatic width and at 16 columns per tile:
    identical results, within 4e-6 of the oracle after two relaxed steps of
    FP32 inputs (the batch relaxation tests' tolerance)."""
    rng = np.random.default_rng(N * 1000 + M)
    ibar = rng.lognormal(0.0, 1.0, size=(1, M, N)).astype(np.float32)
    B = rng.uniform(0.1, 1.0, size=(1, N)).astype(np.float32)
    lam = np.array([0.6])
    xyz, area, fa = oracle.fibonacci_directions(M)
    W = oracle.weights_thomson(xyz, area, fa)
    S_ref, _, _ = oracle.iterate(W, ibar[0].astype(np.float64), B[0].astype(np.float64), lam[0], 2, True)
    out = {}
    for bn in (0, 16):
        b = Batch(ctx)
        try:
            pid = b.add(problem_desc(N, M, 1, PHASE_THOMSON, 0.0, bn=bn), ibar, B, lam)
            b.step(True)
            b.step(True)
            out[bn] = b.read(pid)[0]
        finally:
            b.close()
    assert np.array_equal(out[0], out[16])
    assert rel_err(out[16].reshape(M, N), S_ref) <= 4 * TOL["fp16x3"]
