"""Accuracy of the relaxed tensor-core source iteration on 65,536 cells,
with the library's correction of the truncating accumulate, at the drain
periods the library uses.

Every case runs a relaxed source iteration (S = (1 - lambda) B + lambda W^T
Ibar, Ibar <- 0.5 Ibar + 0.5 S) at fp16x3 or tf32x3 and compares the final S
of every cell with the FP64 path on the same device inputs, and the S of a
block of cells with the oracle's FP64 iteration (the restated reference
integral).  The cases vary what the accuracy could depend on: the spread of
the intensities (lognormal sigma 0.5 to 2), the direction count (146 to
1202), the phase kernel (Thomson, Henyey-Greenstein g = 0.8), the albedo and
the number of relaxed steps (20, and 40 as the longest serving requests).

* test_default_setting: every case at the library's default drain period
  (automatic: for FP16 two K-slices per drain only for smooth kernels, for
  TF32 always two);
* test_two_slices_per_drain_on_smooth_kernels: the benchmark's setting --
  two K-slices per drain forced -- on the Thomson cases, the ones the
  automatic choice gives it to.

Tolerance: max relative error <= 1e-6 after the last step (the accuracy gate
of the tensor path), for the max over all cells and for the oracle block.
"""
import numpy as np
import pytest

import oracle
from relativistic_solver_hllc_gb300 import PHASE_HG, PHASE_THOMSON, TUNE_FLUSH

pytestmark = pytest.mark.gpu
TOL = 1e-6
N = 65_536
SEED = 5

# (sigma, M, phase, g, lambda, steps)
CASES = [
    (0.5, 1000, PHASE_THOMSON, 0.0, 0.9, 20),
    (1.0, 1000, PHASE_THOMSON, 0.0, 0.9, 20),
    (1.5, 1000, PHASE_THOMSON, 0.0, 0.9, 20),
    (2.0, 1000, PHASE_THOMSON, 0.0, 0.9, 20),
    (1.5, 146, PHASE_THOMSON, 0.0, 0.9, 20),
    (1.5, 590, PHASE_THOMSON, 0.0, 0.9, 20),
    (1.5, 1202, PHASE_THOMSON, 0.0, 0.9, 20),
    (1.0, 590, PHASE_HG, 0.8, 0.9, 20),
    (1.0, 1202, PHASE_HG, 0.8, 0.9, 20),
    (1.5, 146, PHASE_HG, 0.8, 0.9, 20),
    (1.0, 1000, PHASE_THOMSON, 0.0, 0.95, 40),
    (1.0, 302, PHASE_HG, 0.8, 0.9, 40),
]
SMOOTH = [c for c in CASES if c[2] == PHASE_THOMSON and c[1] >= 302]


def _case_id(c):
    s, M, ph, g, lam, it = c
    return f"s{s}-M{M}-{'hg' if ph == PHASE_HG else 'th'}{g}-l{lam}-{it}steps"


def _run(ctx, prec, B, lam, steps):
    ctx.solve_setup(prec, B, lam)
    for _ in range(steps):
        ctx.solve_step_async(True)
    ctx.wait()
    return ctx.solve_read()


def _check(ctx, prec, case, flush):
    sigma, M, phase, g, lam, steps = case
    xyz, area, fa = oracle.fibonacci_directions(M)
    B = oracle.uniform(SEED, 2, 0.1, 1.0, N)
    ctx.init(xyz, area, fa, N)
    if phase == PHASE_HG:
        ctx.set_phase(PHASE_HG, g)
    ctx.set_tuning(TUNE_FLUSH, flush)
    try:
        used = ctx.flush_period(prec)
        ctx.synth_illum(SEED, 0.0, sigma)
        S_t = _run(ctx, prec, B, lam, steps)
        ctx.synth_illum(SEED, 0.0, sigma)
        S_64 = _run(ctx, "fp64", B, lam, steps)
    finally:
        ctx.set_tuning(TUNE_FLUSH, 0)
    rel = np.abs(S_t - S_64) / np.abs(S_64)
    assert float(rel.max()) <= TOL, (used, float(rel.max()), float(rel.mean()))

    # a block of 48 cells against the oracle's FP64 iteration of the same inputs
    c0, c1 = N // 3, N // 3 + 48
    il = np.empty(M * N * 4)  # only the block's pages are written
    oracle.illum_cells_into(il, SEED, 0.0, sigma, N, M, c0, c1)
    blk = il.reshape(M, N, 4)[:, c0:c1, :]
    ibar = (((blk[..., 0] + blk[..., 1]) + blk[..., 2]) + blk[..., 3]) / 4
    W = oracle.weights_hg(xyz, area, g) if phase == PHASE_HG else oracle.weights_thomson(xyz, area, fa)
    S_ref, _, _ = oracle.iterate(W, ibar, B[c0:c1], lam, steps, True)
    assert float(np.max(np.abs(S_t[:, c0:c1] - S_ref) / S_ref)) <= TOL
    # the FP64 path itself follows the oracle (its own gate is 1e-12 on one
    # evaluation; the iteration compounds a few ulps)
    assert float(np.max(np.abs(S_64[:, c0:c1] - S_ref) / S_ref)) <= 1e-11
    return used


@pytest.mark.parametrize("prec", ["fp16x3", "tf32x3"])
@pytest.mark.parametrize("case", CASES, ids=_case_id)
def test_default_setting(ctx, prec, case):
    used = _check(ctx, prec, case, 0)
    # the automatic drain period: FP16 drains two K-slices (64 in-directions)
    # only for the smooth kernels; TF32 always two (32 in-directions)
    assert used == (2 if (case in SMOOTH or prec == "tf32x3") else 1)


@pytest.mark.parametrize("prec", ["fp16x3", "tf32x3"])
@pytest.mark.parametrize("case", SMOOTH, ids=_case_id)
def test_two_slices_per_drain_on_smooth_kernels(ctx, prec, case):
    assert _check(ctx, prec, case, 2) == 2
