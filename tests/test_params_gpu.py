"""Energy, flux, impulse tensor and the divergences of flux and impulse
(rts_set_geometry + rts_illum_params, the reference's d_MakeIllumParam) on the
GPU against the reference's own MakeStream / MakeDivImpuls output
(tests/golden/div_*.npz) and against the oracle at a larger size.

Tolerance: 1e-12 relative to the energy (moments) or to the largest face term
|X_f n_f| S_f / V of the divergence sums, whose face terms cancel."""
import numpy as np
import pytest

import oracle
from conftest import GOLDEN
from relativistic_solver_hllc_gb300 import STREAM_PARAMS, STREAM_SCATTERING_2, RtsError

pytestmark = pytest.mark.gpu
TOL = 1e-12


def check(ctx, il, N, M, xyz, area, fa, nrm, fS, vol, ref):
    e, fl, im, ds, di = ctx.illum_params(STREAM_PARAMS)
    ref_fl, ref_im, ref_ds, ref_di = ref
    e_ref = oracle.energy(il, N, area, fa)
    assert float(np.max(np.abs(e - e_ref) / np.abs(e_ref))) <= TOL
    assert float(np.max(np.abs(fl - ref_fl) / np.abs(e_ref)[:, None])) <= TOL
    assert float(np.max(np.abs(im.reshape(N, 9) - ref_im) / np.abs(e_ref)[:, None])) <= TOL
    term = np.max(fS, axis=1) / vol * 4
    s_fl = term * np.max(np.abs(ref_fl), axis=1) + 1e-300
    s_im = term * np.max(np.abs(ref_im), axis=1) + 1e-300
    assert float(np.max(np.abs(ds - ref_ds) / s_fl)) <= TOL
    assert float(np.max(np.abs(di - ref_di) / s_im[:, None])) <= TOL
    # the impulse tensor is symmetric
    assert np.array_equal(im, np.transpose(im, (0, 2, 1)))


@pytest.mark.parametrize("name", ["div_n40_m24", "div_n7_m5"])
def test_params_match_reference(ctx, name):
    g = np.load(GOLDEN / f"{name}.npz")
    N, M = int(g["N"]), int(g["M"])
    il = oracle.illum(int(g["seed"]), 0.0, 1.0, N, M, independent_faces=True)
    xyz, area, fa = oracle.fibonacci_directions(M)
    ctx.init(xyz, area, fa, N)
    ctx.copy_illum(il)
    ctx.set_geometry(g["normals"], g["face_areas"], g["volume"])
    check(ctx, il, N, M, xyz, area, fa, g["normals"], g["face_areas"], g["volume"],
          (g["flux"], g["impuls"], g["divstream"], g["divimpuls"]))


def test_params_match_oracle_larger(ctx):
    N, M = 3000, 146
    il = oracle.illum(41, 0.0, 1.5, N, M, independent_faces=True)
    xyz, area, fa = oracle.fibonacci_directions(M)
    nrm, fS, vol = oracle.cell_geometry(43, N)
    ctx.init(xyz, area, fa, N)
    ctx.copy_illum(il)
    ctx.set_geometry(nrm, fS, vol)
    check(ctx, il, N, M, xyz, area, fa, nrm, fS, vol, oracle.illum_params(il, N, xyz, area, fa, nrm, fS, vol))
    # the flux agrees with rts_moments
    e2, f2 = ctx.moments(STREAM_SCATTERING_2)
    e, fl, _, _, _ = ctx.illum_params(STREAM_SCATTERING_2, divergence=False)
    assert float(np.max(np.abs(e - e2) / np.abs(e2))) <= TOL
    assert float(np.max(np.abs(fl - f2) / np.abs(e2)[:, None])) <= TOL


def test_divergence_of_uniform_radiation_is_zero(ctx):
    """Face-independent intensity: both divergences vanish on a closed cell
    (sum_f n_f S_f = 0 for a real tetrahedron, so the test builds one), the
    impulse tensor's trace is the energy."""
    M = 200
    xyz, area, fa = oracle.fibonacci_directions(M)
    N = 5
    il = np.full(M * N * 4, 2.5)
    # tetrahedron (0,0,0), (1,0,0), (0,1,0), (0,0,1): outward normals and areas
    n = np.array([[0, 0, -1], [0, -1, 0], [-1, 0, 0], [1, 1, 1]], dtype=np.float64)
    n[3] /= np.sqrt(3.0)
    S = np.array([0.5, 0.5, 0.5, np.sqrt(3.0) / 2])
    nrm = np.tile(n, (N, 1, 1))
    fS = np.tile(S, (N, 1))
    vol = np.full(N, 1.0 / 6.0)
    ctx.init(xyz, area, fa, N)
    ctx.copy_illum(il)
    ctx.set_geometry(nrm, fS, vol)
    e, fl, im, ds, di = ctx.illum_params()
    assert np.allclose(e, 2.5, rtol=1e-13)
    f_exact = 2.5 * (area[:, None] * xyz.reshape(M, 3)).sum(axis=0) / fa
    assert np.max(np.abs(fl - f_exact)) <= 1e-13
    assert np.max(np.abs(ds)) <= 1e-12 and np.max(np.abs(di)) <= 1e-12
    assert np.allclose(np.trace(im, axis1=1, axis2=2), 2.5, rtol=1e-12)


def test_divergence_needs_geometry(ctx):
    M, N = 8, 10
    xyz, area, fa = oracle.fibonacci_directions(M)
    ctx.init(xyz, area, fa, N)
    with pytest.raises(RtsError):
        ctx.illum_params()
    e, fl, im, ds, di = ctx.illum_params(divergence=False)
    assert ds is None and di is None
    with pytest.raises(RtsError):
        ctx.set_geometry(np.zeros((N, 4, 3)), np.ones((N, 4)), np.zeros(N))  # volume must be > 0


def read_counted(path, per_cell):
    """int32 count, then count x per_cell FP64 (WRITE_FILE / WriteSimpleFileBin)."""
    raw = path.read_bytes()
    n = int(np.frombuffer(raw[:4], dtype=np.int32)[0])
    data = np.frombuffer(raw[4:], dtype=np.float64)
    assert data.size == n * per_cell
    return n, data.reshape(n, per_cell) if per_cell > 1 else data


def test_write_solution_files(ctx, tmp_path):
    """rts_write_solution writes the radiation part of the reference's
    WriteFileSolution: direction 0's face mean and the moments, each an int32
    count then the FP64 elements; the divergences only with the geometry."""
    N, M = 500, 64
    il = oracle.illum(9, 0.0, 1.0, N, M, independent_faces=True)
    xyz, area, fa = oracle.fibonacci_directions(M)
    ctx.init(xyz, area, fa, N)
    ctx.copy_illum(il)
    ctx.write_solution(tmp_path)
    assert not (tmp_path / "divstream.bin").exists()
    nrm, fS, vol = oracle.cell_geometry(5, N)
    ctx.set_geometry(nrm, fS, vol)
    ctx.write_solution(str(tmp_path) + "/")
    e, fl, im, ds, di = ctx.illum_params(STREAM_PARAMS)
    n, I0 = read_counted(tmp_path / "Illum.bin", 1)
    assert n == N
    faces = il[: N * 4].reshape(N, 4)
    assert np.array_equal(I0, (((faces[:, 0] + faces[:, 1]) + faces[:, 2]) + faces[:, 3]) / 4)
    for name, ref, per in (("energy.bin", e, 1), ("stream.bin", fl, 3), ("impuls.bin", im.reshape(N, 9), 9),
                           ("divstream.bin", ds, 1), ("divimpuls.bin", di, 3)):
        n, got = read_counted(tmp_path / name, per)
        assert n == N and np.array_equal(got, ref.reshape(got.shape)), name


def test_divergence_of_a_linear_stream(ctx):
    """The analytic check of the reference's TestDivStream
    (solve_module/illum/Illum_async.cpp:1351-1387): a stream (3x, 0, 0) at the
    face centres has divergence 3 on every cell.  Through Illum: I_jf =
    9 x_f (w_j)_x gives the face streams 9 x_f Q with Q = sum_j w_j (w_j)_x
    area_j / full_area (1/3 for an exact quadrature), so divstream = 9 Q_x on
    every cell of a real mesh (the divergence theorem on a linear field, with
    face centres)."""
    from relativistic_solver_hllc_gb300 import mesh_cube

    vert, pairs, normals = mesh_cube(3, 1, True)
    N, M = vert.shape[0], 146
    xyz, area, fa = oracle.fibonacci_directions(M)
    FV = [[0, 1, 3], [1, 2, 3], [2, 0, 3], [0, 2, 1]]
    centres = np.stack([vert[:, FV[f]].mean(axis=1) for f in range(4)], axis=1)  # [N][4][3]
    fS = np.stack([0.5 * np.linalg.norm(np.cross(vert[:, FV[f][1]] - vert[:, FV[f][0]],
                                                  vert[:, FV[f][2]] - vert[:, FV[f][0]]), axis=1)
                   for f in range(4)], axis=1)
    vol = np.abs(np.linalg.det(np.stack([vert[:, 1] - vert[:, 0], vert[:, 2] - vert[:, 0],
                                         vert[:, 3] - vert[:, 0]], axis=1))) / 6
    w = xyz.reshape(M, 3)
    il = 9.0 * centres[None, :, :, 0] * w[:, 0][:, None, None]  # [M][N][4]
    ctx.init(xyz, area, fa, N)
    ctx.copy_illum(np.ascontiguousarray(il).ravel())
    ctx.set_geometry(normals, fS, vol)
    _, _, _, ds, _ = ctx.illum_params()
    qx = float((w[:, 0] * w[:, 0] * area).sum() / fa)
    assert abs(qx - 1 / 3) < 1e-3
    # 1e-12 relative to the face terms 9 x_f Q_x S_f / V, which cancel to 9 Q_x
    scale = 4 * 9 * qx * np.max(np.abs(centres[:, :, 0]) * fS, axis=1) / vol
    assert float(np.max(np.abs(ds - 9 * qx) / scale)) <= 1e-12
