"""HMC on the device (csrc/hmc.cu): trajectories against the reference's own
hmc_trajectory (golden fixtures from tests/golden/make_golden.py), the nested
multi-timescale integrator against a restatement driven by the oracle's
forces, integrator error scaling, and the mixed-precision solves."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

LAMBDA = 0.1932


@pytest.mark.parametrize("name", ["hmc_L8_omelyan", "hmc_L8_leapfrog"])
def test_trajectories_match_reference(smg_gpu, name):
    d = golden(name)
    L = int(d["L"])
    lat = smg_gpu.Lattice(L)
    g = smg_gpu.GaugeField(lat, d["U"])
    p = smg_gpu.hmc_params(float(d["beta"]), tau=float(d["tau"]), n_steps=int(d["n_steps"]),
                           omelyan=bool(d["omelyan"]), cg_tol=float(d["cg_tol"]), c_sw=float(d["csw"]))
    rng = smg_gpu.Rng(int(d["seed"]))
    for t in range(int(d["n_traj"])):
        res = smg_gpu.hmc_trajectory(g, float(d["m"]), float(d["r"]), p, rng)
        acc, dH, dKE, dSG, dSF, _, plaq = d["traj"][t]
        assert res.accepted == bool(acc)
        assert abs(res.dH - dH) < 1e-8 * max(1.0, abs(dH)), (t, res.dH, dH)
        assert abs(res.dKE - dKE) < 1e-8 * max(1.0, abs(dKE))
        assert abs(res.dSG - dSG) < 1e-8 * max(1.0, abs(dSG))
        assert abs(res.dSF - dSF) < 1e-8 * max(1.0, abs(dSF))
        assert abs(res.plaquette - plaq) < 1e-12
    assert np.max(np.abs(g.U.reshape(-1) - d["U_out"])) < 1e-10


def test_reversibility_matches_reference(smg_gpu):
    """reversibility_test_plain (src/hmc_trajectory.cpp:416-509): the reference's dH of the forward
    half, dH_backward = -dH_forward, and links and momenta back to rounding after the flip."""
    d = golden("reversibility_L8_omelyan")
    L = int(d["L"])
    lat = smg_gpu.Lattice(L)
    g = smg_gpu.GaugeField(lat, d["U"])
    p = smg_gpu.hmc_params(float(d["beta"]), tau=float(d["tau"]), n_steps=int(d["n_steps"]),
                           omelyan=bool(d["omelyan"]), cg_tol=float(d["cg_tol"]), c_sw=float(d["csw"]))
    res = smg_gpu.hmc_reversibility(g, float(d["m"]), float(d["r"]), p, smg_gpu.Rng(int(d["seed"])))
    gauge_delta, mom_delta, dH_f, dH_b, _ = d["result"]
    assert abs(res.dH_forward - dH_f) < 1e-8 * max(1.0, abs(dH_f))
    assert abs(res.dH_backward - dH_b) < 1e-8 * max(1.0, abs(dH_b))
    # the reference reaches 6e-14 / 2e-13 with CG to 1e-12; the residual of the solves bounds both
    assert res.gauge_delta < 1e-10 and mom_delta < 1e-10 and res.mom_delta < 1e-10
    assert abs(res.dH_forward + res.dH_backward) < 1e-8
    # the links at entry are restored
    assert np.max(np.abs(g.U.reshape(-1) - d["U"])) == 0.0


@pytest.mark.parametrize("n_inner,use_eo", [(4, False), (0, True)])
def test_reversibility_nested_and_even_odd(smg_gpu, n_inner, use_eo):
    """The nested integrator and the even-odd path are reversible to the solver tolerance."""
    L = 16
    lat = smg_gpu.Lattice(L)
    g = smg_gpu.GaugeField(lat, smg_gpu.gauge_normal(L, 4.0, 81))
    p = smg_gpu.hmc_params(4.0, tau=0.5, n_steps=4, omelyan=True, n_inner=n_inner, cg_tol=1e-12, c_sw=1.0,
                           use_eo=use_eo)
    res = smg_gpu.hmc_reversibility(g, 0.1, 1.0, p, smg_gpu.Rng(82))
    assert res.gauge_delta < 1e-10 and res.mom_delta < 1e-9
    assert abs(res.dH_forward + res.dH_backward) < 1e-7 * max(1.0, abs(res.dH_forward))


def _nested_restatement(port, rng, U, m, r, csw, beta, tau, n_outer, n_inner, tol):
    """The nested Omelyan integrator (fermion force outside, leapfrog on the gauge force inside)
    restated with the oracle's forces and solver; momenta, eta and the links in the reference's
    [mu][s] order."""
    V = U.size // 2
    pi = rng.normal(2 * V)
    e = rng.normal(4 * V)
    eta = e[1::2] + 1j * e[0::2]  # random_vec draws each entry's imaginary part first
    U = U.copy()
    phi = port.dirac(U, m, r, csw, 0.0, 1, eta)

    def ferm(U):
        X, _, _ = port.cg(U, m, r, csw, 0.0, phi, 100000, tol)
        return port.fermion_force(U, m, r, csw, 0.0, X), X

    def hamiltonian(U, pi):
        X, _, _ = port.cg(U, m, r, csw, 0.0, phi, 100000, tol)
        return 0.5 * np.sum(pi * pi) + port.gauge_action(U, beta) + np.vdot(phi, X).real

    H0 = hamiltonian(U, pi)

    def update(U, pi, s):
        return U * np.exp(1j * s * pi)

    def inner(U, pi, dt_total):
        dti = dt_total / n_inner
        pi = pi + 0.5 * dti * port.gauge_force(U, beta)
        for i in range(n_inner):
            U = update(U, pi, dti)
            pi = pi + (dti if i < n_inner - 1 else 0.5 * dti) * port.gauge_force(U, beta)
        return U, pi

    h = tau / n_outer
    F, _ = ferm(U)
    pi = pi + LAMBDA * h * F
    for o in range(n_outer):
        U, pi = inner(U, pi, 0.5 * h)
        F, _ = ferm(U)
        pi = pi + (1 - 2 * LAMBDA) * h * F
        U, pi = inner(U, pi, 0.5 * h)
        F, _ = ferm(U)
        pi = pi + (2 * LAMBDA * h if o < n_outer - 1 else LAMBDA * h) * F
    return U, hamiltonian(U, pi) - H0


def test_nested_integrator_matches_restatement(smg_gpu, port):
    L, beta, m, r, csw = 8, 4.0, 0.1, 1.0, 1.0
    U0 = smg_gpu.gauge_normal(L, beta, 71).reshape(-1)
    lat = smg_gpu.Lattice(L)
    g = smg_gpu.GaugeField(lat, U0)
    p = smg_gpu.hmc_params(beta, tau=1.0, n_steps=3, omelyan=True, n_inner=2, cg_tol=1e-12, c_sw=csw,
                           force_accept=True)
    res = smg_gpu.hmc_trajectory(g, m, r, p, smg_gpu.Rng(72))
    U_want, dH_want = _nested_restatement(port, smg_gpu.Rng(72), U0, m, r, csw, beta, 1.0, 3, 2, 1e-12)
    assert res.accepted
    assert np.max(np.abs(g.U.reshape(-1) - U_want)) < 1e-10
    assert abs(res.dH - dH_want) < 1e-8 * max(1.0, abs(dH_want))


@pytest.mark.parametrize("n_inner", [0, 4])
def test_energy_violation_scales_as_step_squared(smg_gpu, n_inner):
    """Omelyan is second order: halving the (outer) step cuts |dH| about four-fold."""
    L, beta, m, r, csw = 16, 4.0, 0.1, 1.0, 1.0
    U0 = smg_gpu.gauge_normal(L, beta, 81)
    lat = smg_gpu.Lattice(L)
    dH = []
    for n in (8, 16):
        g = smg_gpu.GaugeField(lat, U0)
        p = smg_gpu.hmc_params(beta, n_steps=n, omelyan=True, n_inner=n_inner, cg_tol=1e-12, c_sw=csw,
                               force_accept=True)
        dH.append(smg_gpu.hmc_trajectory(g, m, r, p, smg_gpu.Rng(82)).dH)
    ratio = abs(dH[0]) / abs(dH[1])
    assert 2.5 < ratio < 6.5, dH


def test_mixed_precision_trajectory_matches_fp64(smg_gpu):
    L, beta, m, r, csw = 16, 4.0, 0.1, 1.0, 1.0
    U0 = smg_gpu.gauge_normal(L, beta, 91)
    lat = smg_gpu.Lattice(L)
    out = []
    for mixed in (False, True):
        g = smg_gpu.GaugeField(lat, U0)
        p = smg_gpu.hmc_params(beta, n_steps=6, omelyan=True, n_inner=2, cg_tol=1e-10, c_sw=csw,
                               force_accept=True, mixed_precision=mixed)
        res = smg_gpu.hmc_trajectory(g, m, r, p, smg_gpu.Rng(92))
        out.append((res, g.U))
    (r64, U64), (r32, U32) = out
    assert abs(r64.dH - r32.dH) < 1e-6
    assert np.max(np.abs(U64 - U32)) < 1e-8


def test_cg_solve_mixed_reaches_fp64_tolerance(smg_gpu):
    L = 32
    U = smg_gpu.gauge_normal(L, 2.0, 31)
    lat = smg_gpu.Lattice(L)
    D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat, U), 0.1, 1.0, 1.0, 0.0)
    B = np.stack([smg_gpu.random_vec(lat.ndof, 40 + j) for j in range(4)])
    res = smg_gpu.cg_solve_mixed(D, lat.ndof, B, 10000, 1e-10)
    for j in range(4):
        Ax = D.apply_DdagD(res.solution[j])
        assert np.linalg.norm(B[j] - Ax) / np.linalg.norm(B[j]) < 1e-10
    assert res.true_residual < 1e-10


def test_hmc_bad_parameters(smg_gpu):
    lat = smg_gpu.Lattice(8)
    g = smg_gpu.GaugeField(lat)
    with pytest.raises(smg_gpu.SmgError):
        smg_gpu.hmc_trajectory(g, 0.1, 1.0, smg_gpu.hmc_params(4.0, n_steps=0), smg_gpu.Rng(1))


def test_gauge_file_round_trip_through_device(smg_gpu, tmp_path):
    """smg_gauge_save writes the device links and their plaquette; smg_gauge_load reads them back."""
    from conftest import GOLDEN

    lat = smg_gpu.Lattice(8)
    g = smg_gpu.GaugeField(lat)
    _, hdr = smg_gpu.load_gauge(GOLDEN / "gauge_L8.swng")
    lib = smg_gpu.lib()
    from schwinger_mg_gb300 import _lib as _L
    import ctypes as C

    h = _L.GaugeHeader()
    _L.check(lib.smg_gauge_load(g.h, str(GOLDEN / "gauge_L8.swng").encode(), C.byref(h)), "smg_gauge_load")
    assert abs(g.avg_plaq() - hdr["avg_plaq"]) < 1e-14
    smg_gpu.save_gauge(g, h.beta, h.mass, tmp_path / "dev.swng")
    V, h2 = smg_gpu.load_gauge(tmp_path / "dev.swng", 8)
    U, _ = smg_gpu.load_gauge(GOLDEN / "gauge_L8.swng", 8)
    np.testing.assert_allclose(V, U, rtol=0, atol=1e-15)
    assert h2["beta"] == h.beta and abs(h2["avg_plaq"] - hdr["avg_plaq"]) < 1e-14
