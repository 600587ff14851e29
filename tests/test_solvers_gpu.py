"""Preconditioned CG, FGMRES with Ritz harvesting, the Richardson/MR smoothers,
lambda_max, the symmetric MG and the pseudofermion action on the device against
the reference's own results (tests/golden/solvers_L16.npz from make_golden.py),
plus batching and edge cases."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def case(smg_gpu):
    d = golden("solvers_L16")
    lat = smg_gpu.Lattice(int(d["L"]))
    g = smg_gpu.GaugeField(lat, d["U"])
    D = smg_gpu.DiracOp(lat, g, float(d["m"]), float(d["r"]), float(d["csw"]), 0.0)
    return d, lat, g, D


def _mg(smg, d, D):
    """The reference's 2-level hierarchy from the same seed; coarsest CG tight enough to stand in for its LU."""
    p = smg.mg_params(2, 4, 4, null_iters=int(d["null_iters"]), seed=int(d["seed"]), coarse_tol=1e-13,
                      coarse_max_iter=2000)
    return smg.MGHierarchy(D, p)


def test_lambda_max_and_smoothers(smg_gpu, case):
    d, lat, g, D = case
    lam = smg_gpu.estimate_lambda_max(D, 30)
    assert abs(lam - float(d["lam"])) / float(d["lam"]) < 1e-11
    om = float(d["omega"])
    zero = np.zeros(lat.ndof, complex)
    assert _rel(smg_gpu.richardson_smooth(D, zero, d["b"], 4, om), d["rich4"]) < 1e-12
    assert _rel(smg_gpu.richardson_smooth(D, d["x0"], d["b"], 3, om), d["rich3_x0"]) < 1e-12
    assert _rel(smg_gpu.mr_smooth(D, d["x0"], d["b"], 4), d["mr4_x0"]) < 1e-12


def test_set_symmetric_matches_reference(smg_gpu, case):
    d, lat, g, D = case
    mg = _mg(smg_gpu, d, D)
    lam0 = mg.estimate_lambda_max(0, 30)
    assert abs(lam0 - float(d["lam"])) / float(d["lam"]) < 1e-11
    om = mg.set_symmetric(0.8)
    np.testing.assert_allclose(om, d["sym_omega"], rtol=1e-11)
    out = mg.precondition(d["b"])
    assert _rel(out, d["sym_precondition"]) < 1e-9
    # Richardson smoothing makes the cycle linear: M(2b) = 2 M(b) to rounding
    assert _rel(mg.precondition(2.0 * d["b"]), 2.0 * out) < 1e-12
    # back to MR
    mg.set_symmetric(0.0)
    assert _rel(mg.precondition(d["b"]), d["sym_precondition"]) > 1e-6


def test_pcg_with_symmetric_mg_matches_reference(smg_gpu, case):
    d, lat, g, D = case
    mg = _mg(smg_gpu, d, D)
    mg.set_symmetric(0.8)
    r = smg_gpu.cg_solve_precond(D, lat.ndof, d["b"], mg, 500, 1e-10)
    assert abs(r.iterations - int(d["pcg_iters"])) <= 1, (r.iterations, int(d["pcg_iters"]))
    assert r.final_residual < 1e-10
    assert _rel(r.solution, d["pcg_x"]) < 1e-8


def test_cg_from_start_vector_matches_reference(smg_gpu, case):
    d, lat, g, D = case
    r = smg_gpu.cg_solve_precond(D, lat.ndof, d["b"], None, 2000, 1e-10, x0=d["x0"])
    assert abs(r.iterations - int(d["cgx0_iters"])) <= 1
    assert _rel(r.solution, d["cgx0_x"]) < 1e-8
    assert r.true_residual < 2e-10


def test_fgmres_mg_matches_reference(smg_gpu, case):
    d, lat, g, D = case
    mg = _mg(smg_gpu, d, D)
    r = smg_gpu.fgmres_solve_mg(D, lat.ndof, d["b"], mg, 4, 200, 1e-10, 2)
    assert r.status == 0
    assert abs(r.iterations - int(d["fgm_mg_iters"])) <= 1, (r.iterations, int(d["fgm_mg_iters"]))
    assert r.final_residual < 1e-10
    assert _rel(r.solution, d["fgm_mg_x"]) < 1e-8
    want = np.asarray(d["fgm_mg_ritz"])
    assert len(r.ritz_values) == len(want)
    np.testing.assert_allclose(np.sort(r.ritz_values), np.sort(want), rtol=1e-6)


def test_fgmres_unpreconditioned_with_deflation_matches_reference(smg_gpu, case):
    d, lat, g, D = case
    r = smg_gpu.fgmres_solve(D, lat.ndof, d["b"], None, 12, 2000, 1e-10, 4)
    assert r.status == 0
    assert abs(r.iterations - int(d["fgm_iters"])) <= 2, (r.iterations, int(d["fgm_iters"]))
    assert r.final_residual < 1e-10
    assert _rel(r.solution, d["fgm_x"]) < 1e-8
    want = np.asarray(d["fgm_ritz"])
    assert len(r.ritz_values) == len(want)
    np.testing.assert_allclose(np.sort(r.ritz_values), np.sort(want), rtol=1e-5)


def test_fgmres_batch_equals_single_and_zero_rhs(smg_gpu, case):
    """Four right-hand sides in one call (one of them zero) give each one's own solve."""
    d, lat, g, D = case
    mg = _mg(smg_gpu, d, D)
    B = np.stack([smg_gpu.random_vec(lat.ndof, 300 + j) for j in range(4)])
    B[2] = 0.0
    rb = smg_gpu.fgmres_solve_mg(D, lat.ndof, B, mg, 6, 300, 1e-10, 2)
    assert rb.status == 0
    assert np.all(rb.solution[2] == 0)
    for j in (0, 1, 3):
        rs = smg_gpu.fgmres_solve_mg(D, lat.ndof, B[j], mg, 6, 300, 1e-10, 2)
        assert _rel(rb.solution[j], rs.solution) < 1e-9
        assert sorted(rb.ritz_values[j]) == pytest.approx(sorted(rs.ritz_values), rel=1e-6)


def test_pcg_batch_equals_single(smg_gpu, case):
    d, lat, g, D = case
    mg = _mg(smg_gpu, d, D)
    mg.set_symmetric(0.8)
    B = np.stack([smg_gpu.random_vec(lat.ndof, 400 + j) for j in range(3)])
    rb = smg_gpu.cg_solve_precond(D, lat.ndof, B, mg, 500, 1e-10)
    for j in range(3):
        rs = smg_gpu.cg_solve_precond(D, lat.ndof, B[j], mg, 500, 1e-10)
        assert _rel(rb.solution[j], rs.solution) < 1e-9


def test_fermion_action_forward_backward(smg_gpu, case):
    d, lat, g, D = case
    S, X, it = smg_gpu.fermion_action(D, d["b"], 2000, 1e-10)
    assert abs(S - float(d["action"])) / abs(float(d["action"])) < 1e-10
    assert _rel(X.download(), d["action_X"]) < 1e-8
    F = smg_gpu.fermion_force(D, X)  # backward pass on the X the forward pass kept
    assert F.shape == (2, lat.V) and np.all(np.isfinite(F))


def test_fgmres_bad_arguments(smg_gpu, case):
    d, lat, g, D = case
    with pytest.raises(smg_gpu.SmgError):
        smg_gpu.fgmres_solve(D, lat.ndof, d["b"], None, 0, 100, 1e-10)
    with pytest.raises(smg_gpu.SmgError):
        smg_gpu.fgmres_solve(D, lat.ndof, d["b"], None, 8, 100, 1e-10, 9)
    with pytest.raises(smg_gpu.SmgError):
        smg_gpu.richardson_smooth(D, d["x0"], d["b"], 2, -1.0)
