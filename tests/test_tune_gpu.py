"""Autotuner of the tensor-core kernel's schedule (drain period, tile width,
tile order): it picks the fastest of the schedules it timed, results do not
depend on the width or the order (each output is summed over the same K-slices
in the same order) and agree across drain periods within the path's
accuracy, and the table survives a save / load into another context."""
import numpy as np
import pytest

import oracle
from relativistic_solver_hllc_gb300 import PHASE_HG, Context
from relativistic_solver_hllc_gb300._native import Batch, problem_desc

pytestmark = pytest.mark.gpu


def run(ctx, M, bn, steps=3):
    with Batch(ctx) as b:
        pid = b.add_synthetic(problem_desc(5000, M, 1, PHASE_HG, 0.5, bn=bn), 3, 0.0, 1.0, 0.1, 1.0, [0.7])
        for _ in range(steps):
            b.step(True)
        S, _ = b.read(pid)
        _, tiles = b.size()
    return S, tiles


def test_autotune_and_width_independence(ctx, tmp_path):
    M = 300
    bn, ms, tried = ctx.autotune(M, "fp16x3", 0, cells=20000)
    assert len(tried) >= 2 and bn in tried and ms == min(tried.values())
    ref, _ = run(ctx, M, 0)
    for w in sorted(tried):
        S, tiles = run(ctx, M, w)
        assert np.array_equal(S, ref), w
        assert tiles == ((5000 + 127) // 128) * ((M + w - 1) // w)
    # problems created with bn = 0 now use the tuned width
    _, tiles = run(ctx, M, 0, steps=1)
    assert tiles == ((5000 + 127) // 128) * ((M + bn - 1) // bn)
    path = tmp_path / "tune.txt"
    ctx.autotune_save(path)
    assert str(bn) in path.read_text()
    other = Context(0)
    try:
        other.autotune_load(path)
        _, tiles = run(other, M, 0, steps=1)
        assert tiles == ((5000 + 127) // 128) * ((M + bn - 1) // bn)
        bad = tmp_path / "bad.txt"
        bad.write_text("300 2 1 17 1.0\n")  # width not a multiple of 16
        with pytest.raises(Exception):
            other.autotune_load(bad)
    finally:
        other.close()


def _run_desc(ctx, M, steps=3, flush=0, bn=0):
    with Batch(ctx) as b:
        pid = b.add_synthetic(problem_desc(20000, M, 1, 0, 0.0, flush=flush, bn=bn), 3, 0.0, 1.0, 0.1, 1.0, [0.7])
        for _ in range(steps):
            b.step(True)
        S, _ = b.read(pid)
        _, tiles = b.size()
    return S, tiles


def test_schedule_tuner(ctx, tmp_path):
    """Drain period, width and order: every allowed combination is timed, the
    fastest is kept per period, new problems take the faster period and its
    schedule, and the table round-trips."""
    M = 1000  # Thomson at M = 1000 allows one and two K-slices per drain
    best, tried = ctx.autotune_schedule(M, "fp16x3", cells=20000)
    assert {t["flush"] for t in tried} == {1, 2}
    assert {t["order"] for t in tried} == {0, 1}
    assert best["ms"] == min(t["ms"] for t in tried)
    fastest = {f: min((t for t in tried if t["flush"] == f), key=lambda t: t["ms"]) for f in (1, 2)}
    pick = min(fastest.values(), key=lambda t: t["ms"])
    xyz, area, fa = oracle.fibonacci_directions(M)
    ctx.init(xyz, area, fa, 20000)
    assert ctx.flush_period("fp16x3") == pick["flush"]
    _, tiles = _run_desc(ctx, M, steps=1)
    assert tiles == ((20000 + 127) // 128) * ((M + pick["bn"] - 1) // pick["bn"])
    path = tmp_path / "sched.txt"
    ctx.autotune_save(path)
    other = Context(0)
    try:
        other.autotune_load(path)
        other.init(xyz, area, fa, 20000)
        assert other.flush_period("fp16x3") == pick["flush"]
    finally:
        other.close()


def test_tile_order_and_period(ctx, tmp_path):
    """The two tile orders give bit-identical steps; the two drain periods
    agree within the accuracy of the path."""
    M, bn = 600, 160  # 4 column tiles, 157 row tiles
    out = {}
    for order in (0, 1):
        for flush in (1, 2):
            t = tmp_path / f"t{order}{flush}.txt"
            t.write_text(f"{M} 2 {flush} -1 {bn} {order} 1.0\n")
            c = Context(0)
            try:
                c.autotune_load(t)
                out[order, flush], tiles = _run_desc(c, M, flush=flush)
                assert tiles == 157 * 4
            finally:
                c.close()
    for flush in (1, 2):
        assert np.array_equal(out[0, flush], out[1, flush])
    rel = np.abs(out[0, 1] - out[0, 2]) / np.abs(out[0, 1])
    assert float(rel.max()) <= 2e-6
