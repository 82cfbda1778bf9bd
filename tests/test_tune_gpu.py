"""Autotuner of the tensor-core kernel's tile width: it picks the fastest of
the widths it timed, results do not depend on the width (each output is summed
over the same K-slices in the same order), and the table survives a save /
load into another context."""
import numpy as np
import pytest

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
