"""The allocation-free entry point rts_scattering_noalloc.

Callers that cannot allocate device memory -- code inside a caller-owned
memory pool or arena, hosts that budget every device byte -- pass their own
device buffers; the library's only scratch is a fixed device array.  This
test calls the entry point through the C ABI twice in a row, with different
problem sizes, and checks each result against the context-based entry point
rts_scattering on the same inputs, within the FP64 tolerance of the other
parity tests (1e-12 relative).

Kept in a file of its own, collected last, so that a run that stops at the
first failure has run every other test first.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from relativistic_solver_hllc_gb300 import Context, _native

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to("cuda")


def _call_noalloc(lib, torch, il, xyz, area, fa, N, M):
    d_il, d_xyz, d_area = _dev(torch, il), _dev(torch, xyz), _dev(torch, area)
    d_S = torch.full((M * N,), float("nan"), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    fn = lib.rts_scattering_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_double, C.c_void_p, C.c_void_p]
    rc = fn(d_il.data_ptr(), d_xyz.data_ptr(), d_area.data_ptr(), N, M, fa, d_S.data_ptr(), stream)
    assert rc == _native.OK
    torch.cuda.synchronize()
    return d_S.cpu().numpy().reshape(M, N)


def test_noalloc_matches_context_entry_point(native_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    lib = native_lib
    with Context(0) as ctx:
        for N, M, seed in ((3000, 200, 21), (1717, 37, 22)):
            xyz, area, fa = oracle.fibonacci_directions(M)
            il = oracle.illum(seed, 0.0, 1.5, N, M, independent_faces=True)
            S_noalloc = _call_noalloc(lib, torch, il, xyz, area, fa, N, M)
            ctx.init(xyz, area, fa, N)
            S_ctx = ctx.scattering(il)
            err = float(np.max(np.abs(S_noalloc - S_ctx) / np.abs(S_ctx)))
            assert err <= TOL, (N, M, err)


def test_noalloc_rejects_oversized_direction_sets(native_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    fn = native_lib.rts_scattering_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_double, C.c_void_p, C.c_void_p]
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    p = buf.data_ptr()
    assert fn(p, p, p, 1, 513, 1.0, p, None) == _native.ERR_INVALID_ARGUMENT
    assert fn(None, p, p, 1, 4, 1.0, p, None) == _native.ERR_INVALID_ARGUMENT
    # Illum is read as pairs of doubles: an 8-byte offset view is refused
    # before anything is launched, as is a misaligned output
    assert fn(p + 8, p, p, 1, 4, 1.0, p, None) == _native.ERR_INVALID_ARGUMENT
    assert fn(p, p, p, 1, 4, 1.0, p + 4, None) == _native.ERR_INVALID_ARGUMENT


def test_noalloc_in_a_captured_graph(native_lib):
    """The entry point allocates nothing and synchronises nothing, so it can be
    captured into a CUDA graph on the caller's stream (after a first call on
    the device outside the capture); the replay gives the eager result."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    fn = native_lib.rts_scattering_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_double, C.c_void_p, C.c_void_p]
    N, M = 2500, 64
    xyz, area, fa = oracle.fibonacci_directions(M)
    il = oracle.illum(23, 0.0, 1.2, N, M, independent_faces=True)
    d_il, d_xyz, d_area = _dev(torch, il), _dev(torch, xyz), _dev(torch, area)
    eager = torch.zeros(M * N, dtype=torch.float64, device="cuda")
    graphed = torch.full((M * N,), float("nan"), dtype=torch.float64, device="cuda")
    side = torch.cuda.Stream()
    args = (d_il.data_ptr(), d_xyz.data_ptr(), d_area.data_ptr(), N, M, fa)
    with torch.cuda.stream(side):
        assert fn(*args, eager.data_ptr(), side.cuda_stream) == _native.OK  # first call outside a capture
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=side):
        rc = fn(*args, graphed.data_ptr(), side.cuda_stream)
    assert rc == _native.OK
    g.replay()
    torch.cuda.synchronize()
    a, b = eager.cpu().numpy(), graphed.cpu().numpy()
    assert float(np.max(np.abs(a - b) / np.abs(a))) <= TOL
