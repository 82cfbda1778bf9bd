"""The operand preparation of the asynchronous integral calls at a tensor
precision (one pass over the face-layout Illum into FP64 face sums and
per-cell maxima, then the scaled conversion to FP32 on the integer pipe and
the split; the rows shared by the stream slots) gives the rows of the direct
preparation bit for bit: rts_scattering_async and rts_scattering (whose
host-buffer pipeline prepares each cell range directly from the FP64 faces)
return identical S.

The Illum holds, besides lognormal values, face sums that sit exactly on an
FP32 rounding tie after the division by 4 (ties to even, both parities),
zeros, values whose quarter is subnormal in FP32 (the conversion's fallback),
negative values and a wide spread of magnitudes within cells."""
import numpy as np
import pytest

import oracle
from relativistic_solver_hllc_gb300 import STREAM_SCATTERING_1, STREAM_SCATTERING_2

pytestmark = pytest.mark.gpu


def _edge_illum(N, M, seed):
    rng = np.random.default_rng(seed)
    il = oracle.illum(seed, 0.0, 2.0, N, M, independent_faces=True).reshape(M, N, 4)
    cells = rng.permutation(N)
    # exact ties: a float32 value plus half its ulp, times 4, on face 0 with
    # the other faces 0 (the sum is exact)
    f = rng.lognormal(0.0, 1.0, size=(M, 64)).astype(np.float32)
    ulp = np.spacing(f).astype(np.float64)
    tie = (f.astype(np.float64) + ulp / 2) * 4
    c = cells[:64]
    il[:, c, :] = 0.0
    il[:, c, 0] = tie
    # zeros, FP32-subnormal quarters (the conversion's fallback; in FP16 mode
    # the clamped row scale), negatives, spread within a cell
    il[:, cells[64:80], :] = 0.0
    il[:, cells[80:96], :] = rng.uniform(1e-45, 1e-39, size=(M, 16, 4))
    il[:, cells[96:112], :] *= -1.0
    il[::3, cells[112:128], :] *= 1e12
    il[1::3, cells[112:128], :] *= 1e-12
    return il.reshape(-1)


@pytest.mark.parametrize("prec", ["fp16x3", "tf32x3", "bf16x3"])
@pytest.mark.parametrize("M", [37, 146])
def test_staged_rows_match_direct_rows(ctx, prec, M):
    N = 3001
    xyz, area, fa = oracle.fibonacci_directions(M)
    il = _edge_illum(N, M, 17)
    ctx.init(xyz, area, fa, N)
    ctx.set_precision(prec)
    try:
        S_sync = ctx.scattering(il)
        ctx.copy_illum(il)
        out1, out2 = np.zeros(M * N), np.zeros(M * N)
        ctx.scattering_async(0, M // 3, STREAM_SCATTERING_1, out1)  # prepares the rows
        ctx.scattering_async(0, M, STREAM_SCATTERING_2, out2)       # reuses them
        ctx.wait()
        ctx.scattering_async(M // 3, M, STREAM_SCATTERING_1, out1)  # prepares again
        ctx.wait()
    finally:
        ctx.set_precision("fp64")
    S_sync = S_sync.reshape(M, N)
    assert np.array_equal(out2.reshape(M, N), S_sync, equal_nan=True)
    assert np.array_equal(out1.reshape(M, N), S_sync, equal_nan=True)
    # and the lognormal cells are the integral (the edge cells hold values a
    # split format cannot carry to 1e-5: zeros, FP32 subnormals, 1e+-12 spreads)
    ref = oracle.calculate_int_cpu(N, xyz, area, fa, il)
    normal = np.ones(N, bool)
    normal[np.random.default_rng(17).permutation(N)[:128]] = False
    rel = np.abs(S_sync[:, normal] - ref[:, normal]) / np.abs(ref[:, normal])
    assert float(rel.max()) <= (1e-4 if prec == "bf16x3" else 1e-5)


@pytest.mark.parametrize("prec", ["fp16x3", "tf32x3"])
def test_face_sums_while_the_illum_arrives(ctx, prec):
    """Whole directions copied in order from direction 0 (the reference's
    per-direction CudaSendIllumAsync) are summed as they arrive; the pair of
    calls then only scales and splits.  The result is the whole preparation's
    bit for bit, and copies in another order, in pieces that are not whole
    directions, or followed by another write fall back to it."""
    N, M = 4099, 75
    xyz, area, fa = oracle.fibonacci_directions(M)
    il = oracle.illum(31, 0.0, 1.5, N, M, independent_faces=True)
    ctx.init(xyz, area, fa, N)
    ctx.set_precision(prec)

    def pair():
        out1, out2 = np.zeros(M * N), np.zeros(M * N)
        ctx.scattering_async(0, M // 3, STREAM_SCATTERING_1, out1)
        ctx.scattering_async(0, M, STREAM_SCATTERING_2, out2)
        ctx.wait()
        assert np.array_equal(out1[: (M // 3) * N], out2[: (M // 3) * N])
        return out2

    try:
        ctx.copy_illum(il)
        whole = pair()
        runs = {}
        for j in range(M):  # in order, one direction per copy
            ctx.send_illum_async(4 * N, 4 * N * j, 4 * N * j, il)
        runs["in order"] = pair()
        for j0 in range(0, M, 4):  # in order, several directions per copy
            n = min(4, M - j0)
            ctx.send_illum_async(4 * N * n, 4 * N * j0, 4 * N * j0, il)
        runs["in order, 4 per copy"] = pair()
        for j in reversed(range(M)):
            ctx.send_illum_async(4 * N, 4 * N * j, 4 * N * j, il)
        runs["reversed"] = pair()
        for j in range(2 * M):  # half directions
            ctx.send_illum_async(2 * N, 2 * N * j, 2 * N * j, il)
        runs["halves"] = pair()
        for j in range(M):
            ctx.send_illum_async(4 * N, 4 * N * j, 4 * N * j, il)
        ctx.copy_illum(il)  # another write after the copies
        runs["then a copy"] = pair()
    finally:
        ctx.set_precision("fp64")
    for name, S in runs.items():
        assert np.array_equal(S, whole), name


@pytest.mark.parametrize("prec", ["fp16x3", "tf32x3"])
def test_shard_of_out_directions_at_tensor_precision(ctx, prec):
    """InitDevice(start, end) shards the out-directions (d_GetS_MPI): the pair
    of calls over the local range at a tensor precision, after whole-direction
    copies in order, against the oracle's integral of the same shard."""
    N, M = 2000, 90
    xyz, area, fa = oracle.fibonacci_directions(M)
    il = oracle.illum(33, 0.0, 1.2, N, M, independent_faces=True)
    for start, end in [(0, 90), (17, 61), (89, 90)]:
        loc = end - start
        ctx.init(xyz, area, fa, N, start, end)
        ctx.set_precision(prec)
        try:
            for j in range(M):
                ctx.send_illum_async(4 * N, 4 * N * j, 4 * N * j, il)
            out1, out2 = np.zeros(loc * N), np.zeros(loc * N)
            ctx.scattering_async(0, loc // 3, STREAM_SCATTERING_1, out1)
            ctx.scattering_async(0, loc, STREAM_SCATTERING_2, out2)
            ctx.wait()
        finally:
            ctx.set_precision("fp64")
        ref = oracle.calculate_int_cpu(N, xyz, area, fa, il, start, loc)
        assert float(np.max(np.abs(out2.reshape(loc, N) - ref) / np.abs(ref))) <= 1e-5, (start, end)
        assert np.array_equal(out1[: (loc // 3) * N], out2[: (loc // 3) * N])
