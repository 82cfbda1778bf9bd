"""Parity of the split-precision tensor-core path (tcgen05) with the FP64
oracle, through the C ABI.

Tolerances (max relative error against FP64, written per precision):
  fp16x3: 1e-6  (scaled FP16 hi/lo split, three products, FP32 accumulate)
  bf16x3: 2e-5  (BF16 hi/lo split: 2^-17 per operand, reported, not the headline)
  tf32x3: 1e-6  (TF32 hi/lo split, kind::tf32 products, FP32 accumulate; no scaling)
"""
import numpy as np
import pytest

import oracle
from relativistic_solver_hllc_gb300 import PHASE_HG, TUNE_BIAS

pytestmark = pytest.mark.gpu
TOL = {"fp16x3": 1e-6, "bf16x3": 2e-5, "tf32x3": 1e-6}
# the split of Ibar alone: FP16 and TF32 hi+lo keep 22 bits, BF16 hi+lo 16 bits
SPLIT_TOL = {"fp16x3": 4e-7, "bf16x3": 1.6e-5, "tf32x3": 4e-7}


def rel_err(a, b):
    return float(np.max(np.abs(a - b) / np.abs(b)))


def problem(N, M, seed=1, sigma=1.5, indep=False):
    xyz, area, fa = oracle.fibonacci_directions(M)
    il = oracle.illum(seed, 0.0, sigma, N, M, independent_faces=indep)
    B = oracle.uniform(seed, 2, 0.1, 1.0, N)
    return xyz, area, fa, il, B


@pytest.mark.parametrize("prec", ["fp16x3", "bf16x3", "tf32x3"])
@pytest.mark.parametrize("N,M", [(1000, 64), (333, 17), (700, 200), (260, 300), (128, 1000)])
def test_single_evaluation(ctx, prec, N, M):
    xyz, area, fa, il, B = problem(N, M, indep=True)
    lam = 0.9
    ctx.init(xyz, area, fa, N)
    ctx.copy_illum(il)
    ctx.solve_setup(prec, B, lam)
    r = ctx.solve_step(False)
    S = ctx.solve_read()
    ref = oracle.source_update(oracle.calculate_int_cpu(N, xyz, area, fa, il), B, lam)
    assert rel_err(S, ref) <= TOL[prec]
    # first step: residual is max|S - 0|
    assert abs(r - np.max(np.abs(ref))) <= TOL[prec] * np.max(np.abs(ref))


@pytest.mark.parametrize("prec", ["fp16x3", "bf16x3", "tf32x3"])
def test_split_of_ibar(ctx, prec):
    N, M = 500, 96
    xyz, area, fa, il, B = problem(N, M, indep=True)
    ctx.init(xyz, area, fa, N)
    ctx.copy_illum(il)
    ctx.solve_setup(prec, B, 0.5)
    ib = ctx.solve_read_ibar()
    assert rel_err(ib, oracle.face_mean(il, N, M)) <= SPLIT_TOL[prec]


@pytest.mark.parametrize("prec", ["fp16x3", "bf16x3", "tf32x3"])
def test_source_iteration_with_relaxation(ctx, prec):
    N, M, lam, iters = 900, 120, 0.9, 6
    xyz, area, fa, il, B = problem(N, M)
    ctx.init(xyz, area, fa, N)
    ctx.copy_illum(il)
    ctx.solve_setup(prec, B, lam)
    res = [ctx.solve_step(True) for _ in range(iters)]
    S = ctx.solve_read()
    W = oracle.weights_thomson(xyz, area, fa)
    S_ref, r_ref, I_ref = oracle.iterate(W, oracle.face_mean(il, N, M), B, lam, iters, True)
    # errors of successive steps compound through a contraction of norm <= 0.95
    assert rel_err(S, S_ref) <= (4 if prec == "bf16x3" else 1) * TOL[prec]
    assert rel_err(np.array(res[1:]), r_ref[1:]) <= 1e-2
    assert rel_err(ctx.solve_read_ibar(), I_ref) <= 4 * TOL[prec]
    hist = ctx.solve_residual_history(iters)
    assert np.allclose(hist, res, rtol=0, atol=0)


@pytest.mark.parametrize("prec", ["fp16x3", "tf32x3"])
@pytest.mark.parametrize("M,hg", [(384, False), (1024, False), (146, True)])
def test_conservation_correction_of_relaxed_steps(ctx, prec, M, hg):
    """tcgen05.mma rounds every FP32 accumulate toward zero, so uncorrected
    sums come out low and the loss compounds through a relaxed iteration.
    The default correction (RTS_TUNE_BIAS 0) scales each cell's integrals by
    the ratio of the conserved sum_j v_j I_j (v = W 1 in FP64) to the sum of
    its integrals in the previous step; RTS_TUNE_BIAS -1 switches it off.
    The sum of v_j S_j comes from one extra output column: at M = 1024 it
    takes a tile of its own, at M = 146 it shares the last 8-column block
    with real out-directions (and Henyey-Greenstein g = 0.8 spreads v most)."""
    N, lam, iters = 2048, 0.9, 12
    xyz, area, fa, il, B = problem(N, M, seed=4, sigma=1.5)
    W = oracle.weights_hg(xyz, area, 0.8) if hg else oracle.weights_thomson(xyz, area, fa)
    S_ref, _, _ = oracle.iterate(W, oracle.face_mean(il, N, M), B, lam, iters, True)
    ctx.init(xyz, area, fa, N)
    if hg:
        ctx.set_phase(PHASE_HG, 0.8)
    stats = {}
    try:
        for mode in (-1, 0):
            ctx.set_tuning(TUNE_BIAS, mode)
            ctx.copy_illum(il)
            ctx.solve_setup(prec, B, lam)
            for _ in range(iters):
                ctx.solve_step_async(True)
            ctx.wait()
            d = (ctx.solve_read() - S_ref) / S_ref
            stats[mode] = (float(d.mean()), float(np.abs(d).max()))
    finally:
        ctx.set_tuning(TUNE_BIAS, 0)
    off, on = stats[-1], stats[0]
    assert off[0] < -1e-7  # truncation loses
    assert abs(on[0]) < 0.25 * abs(off[0]), stats
    assert on[1] <= TOL[prec]
    with pytest.raises(Exception):
        ctx.set_tuning(TUNE_BIAS, -2)


def test_correction_follows_a_change_of_w(ctx):
    """An iteration set up again after a change of phase kernel (same sizes:
    the problem is reused) recomputes the correction's statistics of W with
    the split W rows."""
    N, M, lam, iters = 2048, 302, 0.9, 12
    xyz, area, fa, il, B = problem(N, M, seed=6, sigma=1.5)
    ctx.init(xyz, area, fa, N)
    ctx.copy_illum(il)
    ctx.solve_setup("fp16x3", B, lam)
    ctx.solve_step(True)
    ctx.set_phase(PHASE_HG, 0.6)

    def run():
        ctx.copy_illum(il)
        ctx.solve_setup("fp16x3", B, lam)
        for _ in range(iters):
            ctx.solve_step_async(True)
        ctx.wait()
        return ctx.solve_read()

    S_reused = run()
    ctx.init(xyz, area, fa, N)  # a fresh problem, set up with the new kernel from the start
    ctx.set_phase(PHASE_HG, 0.6)
    S_fresh = run()
    assert np.array_equal(S_reused, S_fresh)
    W = oracle.weights_hg(xyz, area, 0.6)
    S_ref, _, _ = oracle.iterate(W, oracle.face_mean(il, N, M), B, lam, iters, True)
    assert float(np.max(np.abs(S_reused - S_ref) / S_ref)) <= TOL["fp16x3"]


@pytest.mark.parametrize("prec", ["fp16x3", "bf16x3", "tf32x3"])
def test_host_buffer_entry_point(ctx, prec):
    """rts_scattering_update: H2D Illum + B, tensor-core integral + update, D2H S."""
    N, M, lam = 777, 150, 0.7
    xyz, area, fa, il, B = problem(N, M, seed=3, indep=True)
    ctx.init(xyz, area, fa, N)
    out = np.zeros(M * N)
    ctx.scattering_update(prec, il, B, lam, out)
    ref = oracle.source_update(oracle.calculate_int_cpu(N, xyz, area, fa, il), B, lam)
    assert rel_err(out.reshape(M, N), ref) <= TOL[prec]
    # lambda = 1: the bare integral (CalculateIntScattering at this precision)
    ctx.scattering_update(prec, il, None, 1.0, out)
    assert rel_err(out.reshape(M, N), oracle.calculate_int_cpu(N, xyz, area, fa, il)) <= TOL[prec]


def test_host_buffer_call_pipelined_over_cell_ranges(ctx):
    """The tensor-precision host call runs over up to 8 cell ranges (ragged
    tail here); the result, the device copy of Illum and a change of W between
    calls (Thomson -> HG: the split W is refreshed) must all come out right."""
    N, M, lam = 128 * 8 * 3 + 77, 64, 0.8
    xyz, area, fa, il, B = problem(N, M, seed=8, indep=True)
    ctx.init(xyz, area, fa, N)
    pinned = ctx.host_illum()
    pinned[:] = il.reshape(-1)
    out = np.zeros(M * N)
    ctx.scattering_update("fp16x3", pinned, B, lam, out)
    ref = oracle.source_update(oracle.calculate_int_cpu(N, xyz, area, fa, il), B, lam)
    assert rel_err(out.reshape(M, N), ref) <= TOL["fp16x3"]
    back = np.zeros_like(pinned)
    ctx.read_illum(back)
    assert np.array_equal(back, pinned)
    ctx.set_phase(PHASE_HG, 0.5)
    ctx.scattering_update("fp16x3", il, B, lam, out)  # pageable host buffers this time
    ref64 = np.zeros(M * N)
    ctx.scattering_update("fp64", il, B, lam, ref64)
    assert rel_err(out, ref64) <= TOL["fp16x3"]


def test_shard_of_out_directions_tensor(ctx):
    N, M = 400, 80
    xyz, area, fa, il, B = problem(N, M, seed=4)
    start, end = 13, 61
    ctx.init(xyz, area, fa, N, start, end)
    out = np.zeros((end - start) * N)
    ctx.scattering_update("fp16x3", il, None, 1.0, out)
    ref = oracle.calculate_int_cpu(N, xyz, area, fa, il, start, end - start)
    assert rel_err(out.reshape(end - start, N), ref) <= TOL["fp16x3"]


def test_hg_phase_tensor(ctx):
    N, M, g, lam = 600, 146, 0.8, 0.6
    xyz, area, fa, il, B = problem(N, M, seed=6)
    ctx.init(xyz, area, fa, N)
    ctx.set_phase(PHASE_HG, g)
    ctx.copy_illum(il)
    ctx.solve_setup("fp16x3", B, lam)
    ctx.solve_step(False)
    S = ctx.solve_read()
    W = oracle.weights_hg(xyz, area, g)
    ref = oracle.source_update(oracle.scatter_matrix(W, oracle.face_mean(il, N, M)), B, lam)
    assert rel_err(S, ref) <= TOL["fp16x3"]


def test_isotropic_intensity_is_exact_under_hg(ctx):
    """Known answer: I = c with row-normalised HG weights gives S = c."""
    N, M, c = 256, 302, 3.25
    xyz, area, fa = oracle.fibonacci_directions(M)
    ctx.init(xyz, area, fa, N)
    ctx.set_phase(PHASE_HG, 0.5)
    ctx.copy_illum(np.full(M * N * 4, c))
    ctx.solve_setup("fp16x3", np.ones(N), 1.0)
    ctx.solve_step(False)
    S = ctx.solve_read()
    assert np.max(np.abs(S / c - 1.0)) <= 1e-6
