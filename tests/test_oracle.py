"""The oracle against the reference's own outputs (CPU only).

tests/golden/*.npz were produced by the reference's GetS / CalculateIntCPU,
IntegarteDirection(3) and GetSend / GetDisp compiled from the reference source
(oracle/build_ref.sh, tests/golden/make_golden.py).  The C restatement must
reproduce them; with FP contraction off on both sides it does so to the last
bit on x86 and to 1e-15 elsewhere.
"""
import numpy as np
import pytest

import oracle
from conftest import GOLDEN

CASES = ["tiny_n7_m3", "n64_m17", "n33_m16_part", "n130_m1", "n5_m2", "n257_m40"]


def rel_err(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


def load_case(name):
    g = np.load(GOLDEN / f"{name}.npz")
    N, M = int(g["N"]), int(g["M"])
    il = oracle.illum(int(g["seed"]), float(g["mu"]), float(g["sigma"]), N, M,
                      independent_faces=bool(g["independent_faces"]))
    return g, N, M, il


@pytest.mark.parametrize("name", CASES)
def test_generator_pins(name):
    g, N, M, il = load_case(name)
    assert rel_err(il[g["pin_idx"]], g["pin_val"]) <= 1e-15
    xyz, area, fa = oracle.fibonacci_directions(M)
    assert rel_err(xyz.ravel() + 2.0, g["xyz"].ravel() + 2.0) <= 1e-15
    assert np.array_equal(area, g["area"]) and fa == float(g["full_area"])


@pytest.mark.parametrize("name", CASES)
def test_scattering_matches_reference(name):
    g, N, M, il = load_case(name)
    xyz, area, fa = oracle.fibonacci_directions(M)
    S = oracle.calculate_int_cpu(N, xyz, area, fa, il, int(g["disp"]), int(g["size"]))
    assert S.shape == g["S"].shape
    assert rel_err(S, g["S"]) <= 1e-15


@pytest.mark.parametrize("name", CASES)
def test_moments_match_reference(name):
    g, N, M, il = load_case(name)
    xyz, area, fa = oracle.fibonacci_directions(M)
    assert rel_err(oracle.energy(il, N, area, fa), g["energy"]) <= 1e-15
    s = oracle.stream(il, N, xyz, area, fa)
    # flux components cancel; compare against the magnitude of the energy
    scale = np.abs(g["energy"])[:, None]
    assert float(np.max(np.abs(s - g["stream"]) / scale)) <= 1e-15


def divergence_scales(g):
    """Term scales of the divergence sums: face terms |X_f n_f| S_f / V
    cancel, so errors are measured against the largest term."""
    term = np.max(g["face_areas"], axis=1) / g["volume"]
    return term * np.max(np.abs(g["impuls"]), axis=1) * 4, term * np.max(np.abs(g["flux"]), axis=1) * 4 + 1e-300


@pytest.mark.parametrize("name", ["div_n40_m24", "div_n7_m5"])
def test_divergence_moments_match_reference(name):
    """orc_illum_params against the reference's MakeStream / MakeDivImpuls."""
    g = np.load(GOLDEN / f"{name}.npz")
    N, M = int(g["N"]), int(g["M"])
    il = oracle.illum(int(g["seed"]), 0.0, 1.0, N, M, independent_faces=True)
    assert np.array_equal(il[g["pin_idx"]], g["pin_val"])
    nrm, fS, vol = oracle.cell_geometry(int(g["seed"]), N)
    assert np.array_equal(nrm, g["normals"]) and np.array_equal(fS, g["face_areas"]) and np.array_equal(vol, g["volume"])
    xyz, area, fa = oracle.fibonacci_directions(M)
    fl, im, ds, di = oracle.illum_params(il, N, xyz, area, fa, nrm, fS, vol)
    e = np.abs(oracle.energy(il, N, area, fa))
    assert float(np.max(np.abs(fl - g["flux"]) / e[:, None])) <= 1e-14
    assert float(np.max(np.abs(im - g["impuls"]) / e[:, None])) <= 1e-14
    s_imp, s_flux = divergence_scales(g)
    assert float(np.max(np.abs(ds - g["divstream"]) / s_flux)) <= 1e-14
    assert float(np.max(np.abs(di - g["divimpuls"]) / s_imp[:, None])) <= 1e-14


def test_config1_sample_matches_reference():
    g = np.load(GOLDEN / "config1_sample.npz")
    N, M = int(g["N"]), int(g["M"])
    il = oracle.illum(int(g["seed"]), 0.0, 1.0, N, M)
    assert rel_err(il[g["pin_idx"]], g["pin_val"]) <= 1e-15
    xyz, area, fa = oracle.fibonacci_directions(M)
    S = oracle.calculate_int_cpu(N, xyz, area, fa, il)
    assert rel_err(S[:, g["cells"]], g["S_cells"]) <= 1e-15
    assert rel_err(S.sum(axis=1), g["row_sums"]) <= 1e-13
    assert abs(S.sum() - float(g["total"])) / float(g["total"]) <= 1e-13


def test_partition_matches_reference():
    g = np.load(GOLDEN / "partition.npz")
    off = 0
    for np_, n in zip(g["np_"], g["n"]):
        s, d = oracle.get_send_disp(int(np_), int(n))
        assert s == list(g["send"][off:off + np_])
        assert d == list(g["disp"][off:off + np_])
        off += np_


def test_matrix_form_equals_gets_form():
    """W^T Ibar with W = Gamma*area/full_area equals GetS to round-off."""
    N, M = 97, 23
    xyz, area, fa = oracle.fibonacci_directions(M)
    il = oracle.illum(3, 0.0, 1.0, N, M, independent_faces=True)
    W = oracle.weights_thomson(xyz, area, fa)
    S1 = oracle.scatter_matrix(W, oracle.face_mean(il, N, M))
    S2 = oracle.calculate_int_cpu(N, xyz, area, fa, il)
    assert rel_err(S1, S2) <= 1e-14


def test_isotropic_known_answers():
    """I = c: Thomson gives c * sum_j Gamma*area/full_area (the quadrature of
    (3/4)(1+mu^2) over the sphere, -> c as M grows); row-normalised HG gives c."""
    N, M, c = 5, 400, 2.5
    xyz, area, fa = oracle.fibonacci_directions(M)
    il = np.full(M * N * 4, c)
    S = oracle.calculate_int_cpu(N, xyz, area, fa, il)
    assert np.max(np.abs(S / c - 1.0)) < 5e-4
    W = oracle.weights_hg(xyz, area, 0.7)
    assert np.allclose(W.sum(axis=0), 1.0, rtol=0, atol=1e-14)
    S = oracle.scatter_matrix(W, np.full((M, N), c))
    assert np.max(np.abs(S / c - 1.0)) < 1e-14


def test_iteration_is_per_cell_independent():
    """The FP64 source iteration on a subset of cells equals the same
    iteration on all cells restricted to that subset."""
    N, M = 40, 16
    xyz, area, fa = oracle.fibonacci_directions(M)
    W = oracle.weights_thomson(xyz, area, fa)
    Ib = oracle.face_mean(oracle.illum(1, 0.0, 1.5, N, M), N, M)
    B = oracle.uniform(1, 2, 0.1, 1.0, N)
    S_all, r_all, _ = oracle.iterate(W, Ib, B, 0.9, 5)
    cells = np.array([3, 17, 39])
    S_sub, _, _ = oracle.iterate(W, Ib[:, cells], B[cells], 0.9, 5)
    assert np.array_equal(S_all[:, cells], S_sub)
    assert np.all(np.diff(r_all[1:]) <= 0)  # contraction: residual decreases
