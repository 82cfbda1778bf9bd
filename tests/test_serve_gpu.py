"""Continuous-batching serving loop: every request completes with the same
numbers as when solved alone, requests arriving while others run share the
device (more than one resident), the HBM cap is honoured and oversized
requests are rejected."""
import ctypes as C

import numpy as np
import pytest

from relativistic_solver_hllc_gb300 import PHASE_HG, _native
from relativistic_solver_hllc_gb300._native import Batch, Request, problem_desc, serve

pytestmark = pytest.mark.gpu


def make_requests(shapes, arrivals, iters, seed=0):
    rng = np.random.default_rng(seed)
    keep, reqs = [], []
    for (N, M, g), t, it in zip(shapes, arrivals, iters):
        ibar = rng.lognormal(0.0, 1.0, size=(M, N)).astype(np.float32)
        B = rng.uniform(0.1, 1.0, size=N).astype(np.float32)
        lam = np.array([0.6])
        out = np.zeros((M, N), dtype=np.float32)
        keep.append((ibar, B, lam, out, problem_desc(N, M, 1, PHASE_HG, g)))
        fp = C.POINTER(C.c_float)
        reqs.append(Request(t, keep[-1][4], it, ibar.ctypes.data_as(fp), B.ctypes.data_as(fp),
                            lam.ctypes.data_as(_native._dp), out.ctypes.data_as(fp)))
    return reqs, keep


@pytest.mark.parametrize("policy,budget", [(1, 0), (1, 24), (2, 24), (0, 0)])
def test_serving_results_equal_isolated_solves(ctx, policy, budget):
    """Every policy (least remaining work first, with the default budget and
    with one so small that most steps advance a subset; all resident) gives
    each request exactly its isolated result."""
    shapes = [(3000, 110, 0.2), (5000, 302, 0.5), (2000, 590, 0.7), (4000, 146, 0.0), (2500, 302, 0.8)]
    arrivals = [0.0, 0.0, 0.002, 0.004, 0.006]
    iters = [5, 8, 6, 7, 5]
    reqs, keep = make_requests(shapes, arrivals, iters)
    ctx.set_tuning(_native.TUNE_SERVE_POLICY, policy)
    ctx.set_tuning(_native.TUNE_SERVE_BUDGET, budget)
    stats, lat = serve(ctx, reqs, hbm_cap=ctx.hbm_used() + (8 << 30))
    assert stats.completed == len(reqs) and stats.rejected == 0
    assert stats.max_active >= 2  # requests overlapped on the device
    assert np.all(lat > 0) and stats.p99_ms >= stats.p50_ms > 0
    # each result equals the same solve run alone
    for (ibar, B, lam, out, desc), it in zip(keep, iters):
        with Batch(ctx) as b:
            pid = b.add(desc, ibar.reshape(1, *ibar.shape), B.reshape(1, -1), lam)
            for _ in range(it):
                b.step(True)
            S, _ = b.read(pid)
        assert np.array_equal(S[0], out)


def test_serving_respects_the_hbm_cap(ctx):
    shapes = [(20000, 302, 0.5)] * 4 + [(4_000_000, 1202, 0.5)]
    arrivals = [0.0, 0.0, 0.0, 0.0, 0.0]
    iters = [3, 3, 3, 3, 3]
    reqs, keep = make_requests(shapes[:4], arrivals[:4], iters[:4], seed=1)
    big = problem_desc(4_000_000, 1202, 1, PHASE_HG, 0.5)
    dummy = np.zeros(4, dtype=np.float32)
    lam = np.array([0.5])
    fp = C.POINTER(C.c_float)
    reqs.append(Request(0.0, big, 3, dummy.ctypes.data_as(fp), dummy.ctypes.data_as(fp),
                        lam.ctypes.data_as(_native._dp), None))
    one = _native.problem_footprint(problem_desc(20000, 302, 1, PHASE_HG, 0.5))
    cap = ctx.hbm_used() + 2 * one + 302 * 302 * 8 + 20000 * 302 * 4 + (4 << 20)
    stats, lat = serve(ctx, reqs, hbm_cap=cap)
    assert stats.completed == 4 and stats.rejected == 1 and lat[4] == -1.0
    assert stats.max_active <= 2  # the cap admits two at a time
    assert stats.peak_bytes <= cap
