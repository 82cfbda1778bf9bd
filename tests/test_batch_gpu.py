"""Batched problems on the grouped tcgen05 kernel (one launch per step):
parity of every problem with the FP64 oracle, multigroup albedo, graph
replay, removal, and that each result is the same alone and in the mix.
Tolerance: 1e-6 max relative for FP16x3 (the split-precision contract)."""
import numpy as np
import pytest

import oracle
from relativistic_solver_hllc_gb300 import PHASE_HG, PHASE_THOMSON, _native
from relativistic_solver_hllc_gb300._native import Batch, problem_desc

pytestmark = pytest.mark.gpu
TOL = 1e-6


def rel_err(a, b):
    return float(np.max(np.abs(a - b) / np.abs(b)))


def make_inputs(seed, N, M, G):
    rng = np.random.default_rng(seed)
    ibar = rng.lognormal(0.0, 1.0, size=(G, M, N)).astype(np.float32)
    B = rng.uniform(0.1, 1.0, size=(G, N)).astype(np.float32)
    lam = 0.3 + 0.08 * np.arange(G)
    return ibar, B, lam


def weights(M, phase, g):
    xyz, area, fa = oracle.fibonacci_directions(M)
    return oracle.weights_thomson(xyz, area, fa) if phase == PHASE_THOMSON else oracle.weights_hg(xyz, area, g)


def reference(W, ibar, B, lam, iters=1, relax=False):
    G = ibar.shape[0]
    out, res = [], []
    for g in range(G):
        S, r, _ = oracle.iterate(W, ibar[g].astype(np.float64), B[g].astype(np.float64), lam[g], iters, relax)
        out.append(S)
        res.append(r)
    return np.stack(out), np.array(res)


PROBLEMS = [
    # N, M, groups, phase, g
    (700, 17, 1, PHASE_THOMSON, 0.0),
    (1500, 146, 2, PHASE_HG, 0.6),
    (333, 302, 1, PHASE_HG, 0.8),
    (2000, 64, 3, PHASE_THOMSON, 0.0),
]


@pytest.fixture()
def batch(ctx):
    b = Batch(ctx)
    yield b
    b.close()


def test_batch_single_step_matches_oracle(batch):
    ids = []
    for i, (N, M, G, ph, g) in enumerate(PROBLEMS):
        ibar, B, lam = make_inputs(i, N, M, G)
        ids.append((batch.add(problem_desc(N, M, G, ph, g), ibar, B, lam), (ibar, B, lam, M, ph, g)))
    n, tiles = batch.size()
    assert n == len(PROBLEMS) and tiles > 0
    batch.step(False)
    for pid, (ibar, B, lam, M, ph, g) in ids:
        S, r = batch.read(pid)
        ref, rres = reference(weights(M, ph, g), ibar, B, lam)
        assert rel_err(S, ref) <= TOL, (M, rel_err(S, ref))
        assert abs(r - rres[:, 0].max()) <= TOL * rres[:, 0].max()


def test_batch_relaxation_steps(batch):
    N, M, G, ph, g = 900, 120, 2, PHASE_HG, 0.5
    ibar, B, lam = make_inputs(7, N, M, G)
    pid = batch.add(problem_desc(N, M, G, ph, g), ibar, B, lam)
    res = []
    for _ in range(4):
        batch.step(True)
        res.append(batch.read(pid)[1])
    S, _ = batch.read(pid)
    ref, rres = reference(weights(M, ph, g), ibar, B, lam, iters=4, relax=True)
    assert rel_err(S, ref) <= 4 * TOL
    assert rel_err(np.array(res), rres.max(axis=0)) <= 1e-2


def test_batch_mixed_precisions_one_launch(batch):
    """FP16x3, BF16x3 and TF32x3 problems in one grouped launch: the TF32
    ones use kind::tf32 MMAs over 16-direction K-slices, the others kind::f16
    over 32-direction slices; every problem is checked against FP64 after
    relaxed steps."""
    specs = [(900, 146, 1, PHASE_HG, 0.5, "tf32x3"), (700, 302, 2, PHASE_THOMSON, 0.0, "fp16x3"),
             (500, 146, 1, PHASE_HG, 0.7, "bf16x3"), (1100, 590, 1, PHASE_THOMSON, 0.0, "tf32x3"),
             (260, 17, 1, PHASE_HG, 0.3, "tf32x3")]
    tol = {"fp16x3": 4 * TOL, "tf32x3": 4 * TOL, "bf16x3": 8e-5}
    ids = []
    for i, (N, M, G, ph, g, prec) in enumerate(specs):
        ibar, B, lam = make_inputs(40 + i, N, M, G)
        ids.append((batch.add(problem_desc(N, M, G, ph, g, precision=prec), ibar, B, lam), ibar, B, lam, M, ph, g, prec))
    for _ in range(3):
        batch.step(True)
    for pid, ibar, B, lam, M, ph, g, prec in ids:
        S, _ = batch.read(pid)
        ref, _ = reference(weights(M, ph, g), ibar, B, lam, iters=3, relax=True)
        assert rel_err(S, ref) <= tol[prec], (prec, M, rel_err(S, ref))


def test_graph_replay_equals_eager_steps(ctx):
    N, M = 1100, 146
    ibar, B, lam = make_inputs(3, N, M, 1)
    with Batch(ctx) as eager, Batch(ctx) as graph:
        a = eager.add(problem_desc(N, M, 1, PHASE_HG, 0.4), ibar, B, lam)
        b = graph.add(problem_desc(N, M, 1, PHASE_HG, 0.4), ibar, B, lam)
        for _ in range(4):
            eager.step(True)
        graph.capture(2, True)
        graph.replay()
        graph.replay()
        graph.sync(timeout_us=10_000_000)
        Se, re_ = eager.read(a)
        Sg, rg = graph.read(b)
        assert np.array_equal(Se, Sg) and re_ == rg


def test_result_alone_equals_result_in_the_mix(ctx):
    """Continuous batching must not change any problem's numbers."""
    N, M = 800, 302
    ibar, B, lam = make_inputs(11, N, M, 1)
    desc = problem_desc(N, M, 1, PHASE_HG, 0.7)
    with Batch(ctx) as alone:
        pid = alone.add(desc, ibar, B, lam)
        alone.step(True)
        alone.step(True)
        S_alone, r_alone = alone.read(pid)
    with Batch(ctx) as mix:
        others = []
        for i, (n2, m2, g2, ph2, gg2) in enumerate(PROBLEMS):
            x, y, z = make_inputs(100 + i, n2, m2, g2)
            others.append(mix.add(problem_desc(n2, m2, g2, ph2, gg2), x, y, z))
        pid = mix.add(desc, ibar, B, lam)
        mix.step(True)
        mix.remove(others[1])  # membership changes between steps
        mix.step(True)
        S_mix, r_mix = mix.read(pid)
    assert np.array_equal(S_alone, S_mix) and r_alone == r_mix


def test_batch_rejects_bad_descriptors(batch):
    ibar, B, lam = make_inputs(0, 10, 8, 1)
    with pytest.raises(_native.RtsError) as e:
        batch.add(problem_desc(10, 8, 1, precision="fp64"), ibar, B, lam)
    assert e.value.status == _native.ERR_INVALID_ARGUMENT
    with pytest.raises(_native.RtsError):
        batch.add(problem_desc(10, 8, 1, PHASE_HG, 1.5), ibar, B, lam)
    with pytest.raises(_native.RtsError):
        batch.add(problem_desc(10, 8, 1, bn=40), ibar, B, lam)
    with pytest.raises(_native.RtsError):
        batch.remove(12345)


def test_footprint_counts_resident_bytes(ctx):
    desc = problem_desc(50_000, 590, 2)
    fp = _native.problem_footprint(desc)
    used0 = ctx.hbm_used()
    with Batch(ctx) as b:
        ibar, B, lam = make_inputs(1, 50_000, 590, 2)
        b.add(desc, ibar, B, lam)
        held = ctx.hbm_used() - used0
    # the problem's own buffers plus the batch's staging / table scratch
    assert fp <= held <= fp + 2 * 590 * 590 * 8 + 2 * 50_000 * 2 * 590 * 4 + (1 << 20)
