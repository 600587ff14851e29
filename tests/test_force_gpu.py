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
