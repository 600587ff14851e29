"""Even-odd (Schur complement) operator, reconstruction, log det D_ee, the
Schur CG, the e/o force and the e/o HMC trajectory on the device against the
reference's EvenOddDiracOp / eo_fermion_force / hmc_trajectory(use_eo)
(golden fixtures from tests/golden/make_golden.py)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden, rel_err_per_site

pytestmark = pytest.mark.gpu

CASES = ["eo_L16_clover_twist", "eo_L16_wilson"]


def _setup(smg, d):
    lat = smg.Lattice(int(d["L"]))
    g = smg.GaugeField(lat, d["U"])
    D = smg.DiracOp(lat, g, float(d["m"]), float(d["r"]), float(d["csw"]), float(d["mu"]))
    return lat, g, D, smg.EvenOddDiracOp(D)


@pytest.mark.parametrize("name", CASES)
def test_eo_operators_match_reference(smg_gpu, name):
    d = golden(name)
    lat, g, D, eo = _setup(smg_gpu, d)
    assert rel_err_per_site(eo.apply_schur(d["src_o"]), d["schur"]) < 1e-14
    assert rel_err_per_site(eo.apply_schur_dag(d["src_o"]), d["schur_dag"]) < 1e-14
    assert rel_err_per_site(eo.apply_schur_dag_schur(d["src_o"]), d["mdagm"]) < 1e-14
    assert rel_err_per_site(eo.apply_eo(d["src_e"]), d["hop_eo"]) < 1e-14
    assert rel_err_per_site(eo.apply_oe(d["src_o"]), d["hop_oe"]) < 1e-14
    assert rel_err_per_site(eo.reconstruct(d["src_o"], d["phi"]), d["recon"]) < 1e-14
    assert rel_err_per_site(eo.reconstruct(d["src_o"]), d["recon_full"]) < 1e-14
    assert eo.log_det_ee() == pytest.approx(float(d["logdet"]), rel=1e-13)


@pytest.mark.parametrize("name", CASES)
def test_eo_cg_and_force_match_reference(smg_gpu, name):
    d = golden(name)
    lat, g, D, eo = _setup(smg_gpu, d)
    r = eo.cg_solve(d["phi_o"], 5000, 1e-12)
    assert abs(r.iterations - int(d["cg_iters"])) <= 1
    assert np.linalg.norm(r.solution - d["cg_x"]) / np.linalg.norm(d["cg_x"]) < 1e-10
    assert r.true_residual < 2e-12
    F = eo.fermion_force(d["cg_x"]).reshape(-1)
    assert np.max(np.abs(F - d["force"])) / np.max(np.abs(d["force"])) < 1e-13


def test_eo_force_finite_differences(smg_gpu):
    """S_eo = phi_o^dag (M^dag M)^-1 phi_o - 2 log det D_ee, eps = 1e-5 on 16 seeded links
    (the reference's verify_forces with use_eo, src/hmc_forces.cpp:869-981, at a tighter bound)."""
    L, beta, m, csw, mu = 16, 4.0, 0.1, 1.0, 0.1
    U = smg_gpu.gauge_normal(L, beta, 501)
    lat = smg_gpu.Lattice(L)
    g = smg_gpu.GaugeField(lat, U)
    D = smg_gpu.DiracOp(lat, g, m, 1.0, csw, mu)
    eo = smg_gpu.EvenOddDiracOp(D)
    eta = smg_gpu.random_vec(lat.V, 502)
    phi = eo.apply_schur_dag(eta)
    x = eo.cg_solve(phi, 20000, 1e-14).solution
    F = eo.fermion_force(x)

    def action(Uv):
        g.set_links(Uv)
        D.refresh()
        xs = eo.cg_solve(phi, 20000, 1e-14).solution
        return float(np.real(np.vdot(phi, xs))) - 2.0 * eo.log_det_ee()

    rng = np.random.default_rng(503)
    eps, errs, vals = 1e-5, [], []
    for _ in range(16):
        mu_, s = int(rng.integers(2)), int(rng.integers(lat.V))
        Up, Um = U.copy(), U.copy()
        Up[mu_, s] *= np.exp(1j * eps)
        Um[mu_, s] *= np.exp(-1j * eps)
        fd = -(action(Up) - action(Um)) / (2 * eps)
        errs.append(abs(F[mu_, s] - fd))
        vals.append(abs(F[mu_, s]))
    g.set_links(U)
    D.refresh()
    assert max(errs) / max(vals) < 1e-7


def test_eo_hmc_trajectories_match_reference(smg_gpu):
    d = golden("hmc_eo_L8")
    lat = smg_gpu.Lattice(int(d["L"]))
    g = smg_gpu.GaugeField(lat, d["U"])
    p = smg_gpu.hmc_params(float(d["beta"]), tau=float(d["tau"]), n_steps=int(d["n_steps"]), omelyan=False,
                           cg_tol=float(d["cg_tol"]), c_sw=float(d["csw"]), use_eo=True)
    rng = smg_gpu.Rng(int(d["seed"]))
    for t in range(int(d["n_traj"])):
        res = smg_gpu.hmc_trajectory(g, float(d["m"]), float(d["r"]), p, rng)
        acc, dH, dKE, dSG, dSF, _, plaq, dLD = d["traj"][t]
        assert res.accepted == bool(acc)
        for got, want in ((res.dH, dH), (res.dKE, dKE), (res.dSG, dSG), (res.dSF, dSF), (res.dLD, dLD)):
            assert abs(got - want) < 1e-8 * max(1.0, abs(want)), (t, got, want)
        assert abs(res.plaquette - plaq) < 1e-12
    assert np.max(np.abs(g.U.reshape(-1) - d["U_out"])) < 1e-10


def test_eo_bad_arguments(smg_gpu):
    lat = smg_gpu.Lattice(8)
    g = smg_gpu.GaugeField(lat)
    p = smg_gpu.hmc_params(4.0, n_steps=2, use_eo=True, mixed_precision=True)
    with pytest.raises(smg_gpu.SmgError):
        smg_gpu.hmc_trajectory(g, 0.1, 1.0, p, smg_gpu.Rng(1))
