"""The solver fixtures (tests/golden/solvers_L16.npz, produced by the reference's
own PCG, FGMRES, smoothers and action) hold what they claim: every stored
solution solves D^dag D x = b to the stated tolerance under the oracle's
operator, and the stored Richardson step count agrees with omega.  CPU only."""
from __future__ import annotations

import numpy as np

from conftest import golden


def _res(port, d, x):
    args = (d["U"], float(d["m"]), float(d["r"]), float(d["csw"]), 0.0)
    Ax = port.dirac(*args, 2, x)
    return float(np.linalg.norm(d["b"] - Ax) / np.linalg.norm(d["b"]))


def test_solver_fixture_solutions_solve_the_system(port):
    d = golden("solvers_L16")
    for key in ("pcg_x", "cgx0_x", "fgm_mg_x", "fgm_x", "action_X"):
        assert _res(port, d, d[key]) < 2e-10, key
    assert float(d["fgm_mg_res"]) < 1e-10 and float(d["fgm_res"]) < 1e-10
    S = np.real(np.vdot(d["b"], d["action_X"])).item()
    assert abs(float(d["action"]) - S) < 1e-13 * abs(S)


def test_richardson_fixture_against_oracle_operator(port):
    """Four Richardson steps from zero restated with the oracle's D^dag D."""
    d = golden("solvers_L16")
    args = (d["U"], float(d["m"]), float(d["r"]), float(d["csw"]), 0.0)
    x = np.zeros_like(d["b"])
    for _ in range(4):
        x = x + float(d["omega"]) * (d["b"] - port.dirac(*args, 2, x))
    assert np.linalg.norm(x - d["rich4"]) / np.linalg.norm(d["rich4"]) < 1e-13
    assert float(d["omega"]) == 0.8 / float(d["lam"])


def test_eo_fixture_is_the_schur_complement_of_the_oracle_operator(port):
    """D applied to (x_e, x_o) with x_e = -D_ee^-1 D_oe x_o (the fixture's reconstruct_full)
    is zero on even sites and M x_o (the fixture's apply_schur) on odd sites."""
    from conftest import golden as _g

    for name in ("eo_L16_clover_twist", "eo_L16_wilson"):
        d = _g(name)
        L = int(d["L"])
        s = np.arange(L * L)
        odd = ((s % L) + (s // L)) % 2 == 1
        Dx = port.dirac(d["U"], float(d["m"]), float(d["r"]), float(d["csw"]), float(d["mu"]), 0,
                        d["recon_full"]).reshape(-1, 2)
        scale = np.max(np.abs(d["schur"]))
        assert np.max(np.abs(Dx[~odd])) < 1e-13 * scale
        np.testing.assert_allclose(Dx[odd].reshape(-1), d["schur"], rtol=0, atol=1e-13 * scale)
        # the even half of the twisted D_ee^-1 D_oe on top of phi (reconstruct with phi)
        Dr = port.dirac(d["U"], float(d["m"]), float(d["r"]), float(d["csw"]), float(d["mu"]), 0,
                        d["recon"]).reshape(-1, 2)
        np.testing.assert_allclose(Dr[~odd], d["phi"].reshape(-1, 2)[~odd], rtol=0, atol=1e-12)
