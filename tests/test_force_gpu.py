"""GPU adjoint pseudofermion force and gauge force: against the reference's
CPU force (golden fixtures), the oracle, and central finite differences of
the action (reference verify_forces, src/hmc_forces.cpp:869-981)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["cg_force_L32_config1", "cg_force_L16_wilson"])
def test_forces_match_reference(smg_gpu, name):
    d = golden(name)
    L = int(d["L"])
    lat = smg_gpu.Lattice(L)
    g = smg_gpu.GaugeField(lat, d["U"])
    D = smg_gpu.DiracOp(lat, g, float(d["m"]), float(d["r"]), float(d["csw"]), float(d["mu"]))
    F = smg_gpu.fermion_force(D, d["X"]).reshape(-1)
    scale = np.max(np.abs(d["fermion_force"]))
    assert np.max(np.abs(F - d["fermion_force"])) / scale < 1e-13
    G = smg_gpu.gauge_force(g, float(d["beta"])).reshape(-1)
    assert np.max(np.abs(G - d["gauge_force"])) / np.max(np.abs(d["gauge_force"])) < 1e-14
    assert smg_gpu.gauge_action(g, float(d["beta"])) == pytest.approx(float(d["gauge_action"]), rel=1e-13)


@pytest.mark.parametrize("L,csw,mu", [(128, 1.0, 0.0), (40, 1.0, 0.2), (24, 0.0, 0.0)])
def test_force_matches_oracle(smg_gpu, port, L, csw, mu):
    U = smg_gpu.gauge_normal(L, 4.0, L + 1)
    X = smg_gpu.random_vec(2 * L * L, L + 2)
    lat = smg_gpu.Lattice(L)
    D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat, U), 0.1, 1.0, csw, mu)
    F = smg_gpu.fermion_force(D, X).reshape(-1)
    want = port.fermion_force(U, 0.1, 1.0, csw, mu, X)
    assert np.max(np.abs(F - want)) / np.max(np.abs(want)) < 1e-13


def test_force_finite_differences(smg_gpu):
    """F = -dS/dtheta with S = phi^dag (D^dag D)^-1 phi, eps = 1e-5, 16 seeded links."""
    L, beta, m, csw = 16, 4.0, 0.1, 1.0
    U = smg_gpu.gauge_normal(L, beta, 77)
    lat = smg_gpu.Lattice(L)
    g = smg_gpu.GaugeField(lat, U)
    D = smg_gpu.DiracOp(lat, g, m, 1.0, csw, 0.0)
    eta = smg_gpu.random_vec(lat.ndof, 78)
    phi = D.apply_dag(eta)
    X = smg_gpu.cg_solve(D, lat.ndof, phi, 20000, 1e-14).solution
    F = smg_gpu.fermion_force(D, X)
    eps = 1e-5
    rng = np.random.default_rng(5)
    links = [(int(rng.integers(2)), int(rng.integers(lat.V))) for _ in range(16)]

    def action(Uv):
        g.set_links(Uv)
        D.refresh()
        x = smg_gpu.cg_solve(D, lat.ndof, phi, 20000, 1e-14).solution
        return float(np.real(np.vdot(phi, x)))

    errs, vals = [], []
    for mu, s in links:
        Up = U.copy()
        Up[mu, s] *= np.exp(1j * eps)
        Um = U.copy()
        Um[mu, s] *= np.exp(-1j * eps)
        fd = -(action(Up) - action(Um)) / (2 * eps)
        errs.append(abs(F[mu, s] - fd))
        vals.append(abs(F[mu, s]))
    g.set_links(U)
    D.refresh()
    rel = max(errs) / max(vals)
    assert rel < 1e-7, f"force vs finite differences: rel {rel:.3e}"


def test_force_finite_differences_L128_64_links(smg_gpu):
    """Differentiated-HMC check at L = 128, beta = 4, m = 0.1, c_sw = 1: eps = 1e-5 on 64
    seeded links, relative error per link below 1e-7.  S(theta') - S(theta) is formed as
    -X'^dag (A' - A) X = -[(D X')^dag dX + dX'^dag (D X) + dX'^dag dX] with dv = (D' - D) v:
    the two operators do identical arithmetic away from the perturbed link, so dv is exactly
    zero there and the difference keeps the precision of the few sites it lives on."""
    L, beta, m, csw, eps = 128, 4.0, 0.1, 1.0, 1e-5
    U = smg_gpu.gauge_normal(L, beta, 4001)
    lat = smg_gpu.Lattice(L)
    D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat, U), m, 1.0, csw, 0.0)
    eta = smg_gpu.random_vec(lat.ndof, 4002)
    phi = D.apply_dag(eta)
    X = smg_gpu.cg_solve(D, lat.ndof, phi, 50000, 1e-13).solution
    F = smg_gpu.fermion_force(D, X)
    DX = D.apply(X)
    g2 = smg_gpu.GaugeField(lat, U)
    D2 = smg_gpu.DiracOp(lat, g2, m, 1.0, csw, 0.0)
    rng = np.random.default_rng(4003)
    links = [(int(rng.integers(2)), int(rng.integers(lat.V))) for _ in range(64)]

    def delta_S(Uv):
        g2.set_links(Uv)
        D2.refresh()
        Xp = smg_gpu.cg_solve(D2, lat.ndof, phi, 50000, 1e-13).solution
        dX = D2.apply(X) - DX
        DXp = D.apply(Xp)
        dXp = D2.apply(Xp) - DXp
        return -float(np.real(np.vdot(DXp, dX) + np.vdot(dXp, DX) + np.vdot(dXp, dX)))

    rel = []
    for mu, s in links:
        Up = U.copy()
        Up[mu, s] *= np.exp(1j * eps)
        Um = U.copy()
        Um[mu, s] *= np.exp(-1j * eps)
        fd = -(delta_S(Up) - delta_S(Um)) / (2 * eps)
        rel.append(abs(F[mu, s] - fd) / abs(F[mu, s]))
    assert max(rel) < 1e-7, f"force vs finite differences at L=128: max rel {max(rel):.3e}"


@pytest.mark.parametrize("L,csw,use_eo,mu", [(8, 1.0, False, 0.0), (16, 1.0, True, 0.0), (16, 1.0, False, 0.1)])
def test_verify_forces_passes(smg_gpu, L, csw, use_eo, mu):
    """verify_forces (src/hmc_forces.cpp:869-981): the device forces against central differences at the
    reference's 20 links; the analytic values are the device force at those links."""
    lat = smg_gpu.Lattice(L)
    U = smg_gpu.gauge_normal(L, 4.0, 31 + L)
    g = smg_gpu.GaugeField(lat, U)
    chk = smg_gpu.verify_forces(g, 4.0, 0.1, 1.0, c_sw=csw, use_eo=use_eo, mu_t=mu)
    assert chk.passed and chk.n_links == 20
    assert chk.fermion_rel < 1e-4 and chk.gauge_rel < 1e-6
    V = L * L
    for t in range(20):
        assert chk.mu[t] == t % 2 and chk.site[t] == (7 * t + 13 * (t // 2)) % V
    gf = smg_gpu.gauge_force(g, 4.0)
    assert all(abs(chk.gf_ana[t] - gf[chk.mu[t], chk.site[t]]) < 1e-14 * max(1.0, abs(gf[chk.mu[t], chk.site[t]]))
               for t in range(20))
    # the links are untouched
    assert np.max(np.abs(g.U.reshape(-1) - U.reshape(-1))) == 0.0
