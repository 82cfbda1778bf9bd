"""The reference-named host interface (cuda_solve_compat.cpp) driven in the
reference's calling order by a C++ program, compared with the oracle."""
import shutil
import subprocess

import numpy as np
import pytest

import oracle
from conftest import ROOT
from relativistic_solver_hllc_gb300 import _native

COMPAT = ROOT / "relativistic_solver_hllc_gb300" / "compat"


def build_driver(out_dir):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = out_dir / "compat_driver"
    lib_dir = _native.LIB_PATH.parent
    cmd = [gxx, "-O2", "-std=c++17", f"-I{COMPAT / 'standin'}", f"-I{ROOT / 'include'}",
           str(COMPAT / "cuda_solve_compat.cpp"), str(ROOT / "tests" / "compat" / "compat_driver.cpp"),
           f"-L{lib_dir}", "-lrts_scatter", f"-Wl,-rpath,{lib_dir}", "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_compat_shim_compiles_against_standin(native_lib, tmp_path):
    """CPU check: the shim and its calling-sequence program compile and link against the library."""
    assert build_driver(tmp_path).exists()


@pytest.mark.gpu
def test_reference_calling_sequence(native_lib, tmp_path):
    exe = build_driver(tmp_path)
    N, M = 1500, 48
    xyz, area, fa = oracle.fibonacci_directions(M)
    il = oracle.illum(12, 0.0, 1.0, N, M, independent_faces=True)
    _native.write_direction_file(tmp_path / "dirs.txt", xyz, area, fa)
    _native.write_simple_bin(tmp_path / "Illum.bin", il)
    # cell geometry files as the reference's InitDevice reads them
    nrm, fS, vol = oracle.cell_geometry(14, N)
    geo = tmp_path / "geo"
    geo.mkdir()
    _native.write_simple_bin(geo / "normals.bin", nrm.reshape(N, 12).view(np.dtype([("c", np.float64, 12)])).ravel())
    _native.write_simple_bin(geo / "squares.bin", fS.ravel())
    _native.write_simple_bin(geo / "volume.bin", vol)
    env = {**__import__("os").environ, "RTS_GEOMETRY_DIR": str(geo) + "/"}
    res = subprocess.run([str(exe), str(tmp_path / "dirs.txt"), str(tmp_path / "Illum.bin"), str(N), str(tmp_path)],
                         capture_output=True, text=True, timeout=120, env=env)
    assert res.returncode == 0, res.stderr
    ref = oracle.calculate_int_cpu(N, xyz, area, fa, il)
    for name in ("scattering.bin", "scattering_sync.bin"):
        S = _native.read_simple_bin(tmp_path / name).reshape(M, N)
        assert float(np.max(np.abs(S - ref) / ref)) <= 1e-12
    e = _native.read_simple_bin(tmp_path / "energy.bin")
    assert float(np.max(np.abs(e - oracle.energy(il, N, area, fa)) / e)) <= 1e-12
    dt = np.dtype([("v", np.float64, 3)])
    s = _native.read_simple_bin(tmp_path / "stream.bin", dt)["v"]
    assert float(np.max(np.abs(s - oracle.stream(il, N, xyz, area, fa)) / e[:, None])) <= 1e-12
    fl, im, ds, di = oracle.illum_params(il, N, xyz, area, fa, nrm, fS, vol)
    imp = _native.read_simple_bin(tmp_path / "impuls.bin", np.dtype([("m", np.float64, 9)]))["m"]
    assert float(np.max(np.abs(imp - im) / e[:, None])) <= 1e-12
    term = np.max(fS, axis=1) / vol * 4
    ds_g = _native.read_simple_bin(tmp_path / "divstream.bin")
    assert float(np.max(np.abs(ds_g - ds) / (term * np.max(np.abs(fl), axis=1)))) <= 1e-12
    assert np.array_equal(ds_g, _native.read_simple_bin(tmp_path / "divstream2.bin"))
    di_g = _native.read_simple_bin(tmp_path / "divimpuls.bin", dt)["v"]
    assert float(np.max(np.abs(di_g - di) / (term * np.max(np.abs(im), axis=1))[:, None])) <= 1e-12


def _run_driver(exe, tmp_path, xyz, area, fa, il, N, geo_seed, env_extra):
    _native.write_direction_file(tmp_path / "dirs.txt", xyz, area, fa)
    _native.write_simple_bin(tmp_path / "Illum.bin", il)
    nrm, fS, vol = oracle.cell_geometry(geo_seed, N)
    geo = tmp_path / "geo"
    geo.mkdir()
    _native.write_simple_bin(geo / "normals.bin", nrm.reshape(N, 12).view(np.dtype([("c", np.float64, 12)])).ravel())
    _native.write_simple_bin(geo / "squares.bin", fS.ravel())
    _native.write_simple_bin(geo / "volume.bin", vol)
    env = {**__import__("os").environ, "RTS_GEOMETRY_DIR": str(geo) + "/", **env_extra}
    res = subprocess.run([str(exe), str(tmp_path / "dirs.txt"), str(tmp_path / "Illum.bin"), str(N), str(tmp_path)],
                         capture_output=True, text=True, timeout=300, env=env)
    assert res.returncode == 0, res.stderr
    M = area.size
    return (_native.read_simple_bin(tmp_path / "scattering.bin").reshape(M, N),
            _native.read_simple_bin(tmp_path / "scattering_sync.bin").reshape(M, N))


@pytest.mark.gpu
def test_calling_sequence_fp64_on_golden_vectors(native_lib, tmp_path):
    """At FP64 the asynchronous pair and the synchronous call reproduce the
    reference's own CPU integral (golden vectors compiled from its source) to
    1e-12 relative."""
    exe = build_driver(tmp_path)
    g = np.load(ROOT / "tests" / "golden" / "n257_m40.npz")
    N, M = int(g["N"]), int(g["M"])
    il = oracle.illum(int(g["seed"]), float(g["mu"]), float(g["sigma"]), N, M,
                      independent_faces=bool(g["independent_faces"]))
    assert np.array_equal(il[g["pin_idx"]], g["pin_val"])
    S_async, S_sync = _run_driver(exe, tmp_path, g["xyz"], g["area"], float(g["full_area"]), il, N, 31,
                                  {"RTS_SCATTER_PRECISION": "fp64"})
    for S in (S_async, S_sync):
        assert float(np.max(np.abs(S - g["S"]) / g["S"])) <= 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp16x3", "tf32x3"])
def test_calling_sequence_at_tensor_precision(native_lib, tmp_path, prec):
    """RTS_SCATTER_PRECISION puts every scattering call of the shim on the split
    tcgen05 path: the two overlapping CalculateIntScatteringAsyncMPIStream
    calls of the source iteration ([0, M/3) on scattering stream 1, [0, M) on
    scattering stream 2, solve_module/illum/Illum_async.cpp:1019-1020) on the
    device Illum that the per-direction CudaSendIllumAsync copies filled, and
    the synchronous CalculateIntScattering; all within 1e-6 of the oracle."""
    exe = build_driver(tmp_path)
    N, M = 3000, 200
    xyz, area, fa = oracle.fibonacci_directions(M)
    il = oracle.illum(21, 0.0, 1.5, N, M, independent_faces=True)
    S_async, S_sync = _run_driver(exe, tmp_path, xyz, area, fa, il, N, 22, {"RTS_SCATTER_PRECISION": prec})
    ref = oracle.calculate_int_cpu(N, xyz, area, fa, il)
    for S in (S_async, S_sync):
        err = float(np.max(np.abs(S - ref) / ref))
        assert err <= 1e-6, err
        assert err > 1e-12  # it did take the split path
    # the rows [0, M/3) that both asynchronous calls wrote hold the same values
    # from either (different tilings of the directions, same arithmetic per
    # output), and equal the synchronous call's, which splits the cells into
    # ranges instead
    assert np.array_equal(S_async, S_sync)


@pytest.mark.gpu
def test_schedule_table_through_the_shim(native_lib, tmp_path):
    """RTS_SCATTER_TUNE at a tensor precision: the first run of the solver
    tunes the schedule at InitDevice and writes the table; the second loads
    it.  Both runs choose the same schedule, so they give the same values,
    within 1e-6 of the oracle."""
    exe = build_driver(tmp_path)
    N, M = 3000, 200
    xyz, area, fa = oracle.fibonacci_directions(M)
    il = oracle.illum(24, 0.0, 1.5, N, M, independent_faces=True)
    table = tmp_path / "schedule.txt"
    env = {"RTS_SCATTER_PRECISION": "fp16x3", "RTS_SCATTER_TUNE": str(table)}
    runs = []
    for k in range(2):
        d = tmp_path / f"run{k}"
        d.mkdir()
        runs.append(_run_driver(exe, d, xyz, area, fa, il, N, 25, env))
        assert table.exists()
        if k == 0:
            first = table.read_text()
    assert table.read_text() == first  # the second run loaded it, wrote nothing
    rows = [ln.split() for ln in first.splitlines() if ln and not ln.startswith("#")]
    assert rows and all(len(r) == 7 and int(r[0]) == M and int(r[1]) == _native.PREC_FP16X3 for r in rows)
    ref = oracle.calculate_int_cpu(N, xyz, area, fa, il)
    for S in runs[0]:
        assert float(np.max(np.abs(S - ref) / ref)) <= 1e-6
    for a, b in zip(runs[0], runs[1]):
        assert np.array_equal(a, b)
