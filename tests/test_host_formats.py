"""Host-side pieces of the path that need no GPU: the direction-set text
file, count-prefixed binary arrays and the out-direction partition."""
import numpy as np

import oracle
from conftest import GOLDEN
from relativistic_solver_hllc_gb300 import _native


def test_partition_matches_reference(native_lib):
    g = np.load(GOLDEN / "partition.npz")
    off = 0
    for np_, n in zip(g["np_"], g["n"]):
        s, d = _native.partition(int(np_), int(n))
        assert s == list(g["send"][off:off + np_])
        assert d == list(g["disp"][off:off + np_])
        off += np_
    # wider sweep against the oracle's restatement
    for np_ in range(1, 20):
        for n in (0, 1, 5, 146, 302, 590, 1000, 1202):
            assert _native.partition(np_, n) == oracle.get_send_disp(np_, n)


def test_direction_file_round_trip(native_lib, tmp_path):
    xyz, area, fa = _native.synth_directions(146)
    p = tmp_path / "surface_146_dir.txt"
    _native.write_direction_file(p, xyz, area, fa)
    xyz2, area2, fa2 = _native.read_direction_file(p)
    assert np.array_equal(xyz, xyz2) and np.array_equal(area, area2) and fa == fa2
    # the text layout of the reference's reader: M, then "area x y z", then full_area
    lines = p.read_text().split("\n")
    assert int(lines[0]) == 146 and len(lines[1].split()) == 4
    assert float(lines[147]) == fa


def test_direction_file_errors(native_lib, tmp_path):
    lib = native_lib
    M = _native.C.c_int64()
    assert lib.rts_read_direction_file(str(tmp_path / "missing.txt").encode(), 0, _native.C.byref(M),
                                       None, None, None) == _native.ERR_INVALID_ARGUMENT
    bad = tmp_path / "bad.txt"
    bad.write_text("3\n1 0 0 1\n1 0 1\n")
    xyz = np.empty(9)
    area = np.empty(3)
    fa = _native.C.c_double()
    assert lib.rts_read_direction_file(str(bad).encode(), 3, _native.C.byref(M), _native._ptr(xyz),
                                       _native._ptr(area), _native.C.byref(fa)) == _native.ERR_INVALID_ARGUMENT


def test_synth_directions_match_oracle(native_lib):
    for M in (1, 2, 17, 200, 1000):
        a = _native.synth_directions(M)
        b = oracle.fibonacci_directions(M)
        assert np.allclose(a[0], b[0], rtol=0, atol=1e-15) and np.array_equal(a[1], b[1]) and a[2] == b[2]
    assert np.array_equal(_native.synth_uniform(3, 2, 0.1, 1.0, 1000), oracle.uniform(3, 2, 0.1, 1.0, 1000))


def test_simple_bin_round_trip(native_lib, tmp_path):
    S = np.random.default_rng(0).random(12345)
    p = tmp_path / "scattering.bin"
    _native.write_simple_bin(p, S)
    raw = p.read_bytes()
    assert int.from_bytes(raw[:4], "little", signed=True) == S.size and len(raw) == 4 + 8 * S.size
    assert np.array_equal(_native.read_simple_bin(p), S)
    # Vector3 arrays (stream.bin) count Vector3 elements of 24 bytes
    v3 = np.arange(30, dtype=np.float64).reshape(10, 3)
    vec3 = np.dtype((np.float64, 3))
    _native.write_simple_bin(p, v3.view(np.dtype([("v", np.float64, 3)])).ravel())
    raw = p.read_bytes()
    assert int.from_bytes(raw[:4], "little", signed=True) == 10
    back = _native.read_simple_bin(p, np.dtype([("v", np.float64, 3)]))
    assert np.array_equal(back["v"], v3) and vec3.itemsize == 24
