"""Coarse-grid deflation (TRLM eigenpairs of the level-1 operator, the deflated coarsest CG, the
low-mode solution and force, Rayleigh-Ritz after a rebuild) and the MG multi-timescale HMC,
against the reference (fixture ms_L16 from tests/golden/make_golden.py)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ms(smg_gpu):
    return golden("ms_L16")


def _hierarchy(smg, d, U=None, precision="f64", deflate=True):
    L = int(d["L"])
    lat = smg.Lattice(L)
    g = smg.GaugeField(lat, d["U"] if U is None else U)
    D = smg.DiracOp(lat, g, float(d["m"]), float(d["r"]), float(d["csw"]), 0.0)
    p = smg.mg_params(2, int(d["bs"]), int(d["k"]), null_iters=0, coarse_tol=1e-12, coarse_max_iter=200,
                      precision=precision)
    mg = smg.MGHierarchy(D, p, warm_start=d["null_vecs"])
    if deflate:
        mg.set_deflation(d["defl_vals"], d["defl_vecs"])
    return lat, g, D, mg


def test_trlm_eigenpairs_match_reference(smg_gpu, ms):
    lat, g, D, mg = _hierarchy(smg_gpu, ms, deflate=False)
    info = mg.setup_deflation(int(ms["n_defl"]))
    assert info.converged
    vals, vecs = mg.deflation
    ref_vals, ref_vecs = ms["defl_vals"], ms["defl_vecs"]
    assert np.max(np.abs(vals - ref_vals) / ref_vals) < 1e-9, (vals, ref_vals)
    # eigenvectors agree up to a phase
    overlap = np.abs(np.einsum("ij,ij->i", vecs.conj(), ref_vecs))
    assert np.min(overlap) > 1 - 1e-7, overlap
    # and are eigenvectors of the level-1 operator
    for v, lam in zip(vecs, vals):
        Av = mg.coarse_apply(1, v)
        assert np.linalg.norm(Av - lam * v) < 1e-8 * lam


def test_lowmode_solution_and_force_match_reference(smg_gpu, ms):
    lat, g, D, mg = _hierarchy(smg_gpu, ms)
    low = mg.lowmode_solution(ms["phi"])
    assert np.linalg.norm(low - ms["lowmode"]) / np.linalg.norm(ms["lowmode"]) < 1e-12
    F = smg_gpu.coarse_lowmode_force(D, mg, ms["phi"], int(ms["smooth"]))
    ref = ms["lowmode_force"]
    assert np.max(np.abs(F.reshape(-1) - ref)) / np.max(np.abs(ref)) < 1e-10
    # the raw projection (no smoothing) is the fermion force of the low-mode solution
    F0 = smg_gpu.coarse_lowmode_force(D, mg, ms["phi"], 0)
    want = smg_gpu.fermion_force(D, low)
    assert np.max(np.abs(F0 - want)) / np.max(np.abs(want)) < 1e-12


def test_cycle_with_deflated_coarsest_cg_matches_reference(smg_gpu, ms):
    """setup_sparse_coarse makes the coarsest solve CG from the deflated guess (tol 1e-12)."""
    lat, g, D, mg = _hierarchy(smg_gpu, ms)
    out = mg.precondition(ms["phi"])
    ref = ms["precondition_deflated"]
    assert np.linalg.norm(out - ref) / np.linalg.norm(ref) < 1e-9


def test_deflated_f32_hierarchy_converges(smg_gpu, ms):
    """The FP32 cycle with the deflated coarsest CG preconditions GCR to a true FP64 residual of 1e-10."""
    lat, g, D, mg = _hierarchy(smg_gpu, ms, precision="f32")
    b = smg_gpu.random_vec(lat.ndof, 5)
    res = smg_gpu.fcg_solve_mg(D, lat.ndof, b, mg, 200, 1e-10)
    assert res.true_residual < 1e-10


def test_rayleigh_ritz_after_rebuild(smg_gpu, ms):
    """rr_evolve: on an unchanged operator the space is invariant; after new links (the links of an
    accepted reference trajectory) and a rebuild the Ritz values bound the new eigenvalues from above."""
    lat, g, D, mg = _hierarchy(smg_gpu, ms)
    assert mg.deflation_rr() < 1e-8
    vals, _ = mg.deflation
    assert np.max(np.abs(vals - ms["defl_vals"]) / ms["defl_vals"]) < 1e-10
    g.set_links(ms["U_out_1"])
    D.refresh()
    mg.rebuild()
    res = mg.deflation_rr()
    rr_vals, _ = mg.deflation
    # the links moved far (two trajectories): the old space is only a rough approximation
    assert np.all(np.diff(rr_vals) >= 0) and 1e-6 < res < 1.0
    fresh = _hierarchy(smg_gpu, ms, U=ms["U_out_1"], deflate=False)[3]
    fresh.setup_deflation(int(ms["n_defl"]))
    exact, _ = fresh.deflation
    assert np.all(rr_vals >= exact * (1 - 1e-10))


@pytest.mark.parametrize("outer", [0, 1, 2, 3])
def test_multiscale_trajectories_match_reference(smg_gpu, ms, outer):
    lat, g, D, mg = _hierarchy(smg_gpu, ms)
    p = smg_gpu.ms_params(float(ms["ms_beta"]), tau=float(ms["ms_tau"]), n_outer=int(ms["ms_n_outer"]),
                          n_inner=int(ms["ms_n_inner"]), cg_maxiter=int(ms["ms_cg_maxiter"]),
                          cg_tol=float(ms["ms_cg_tol"]), inner_smooth=int(ms["ms_inner_smooth"]), outer=outer,
                          c_sw=float(ms["ms_c_sw"]))
    rng = smg_gpu.Rng(int(ms["seed"]) + 10 + outer)
    for acc, dH, dKE, dSG, dSF, _, n_low, plaq in ms[f"traj_{outer}"]:
        res = smg_gpu.hmc_mg_multiscale(g, float(ms["m"]), float(ms["r"]), p, mg, rng)
        assert res.accepted == bool(acc)
        for got, want in ((res.dH, dH), (res.dKE, dKE), (res.dSG, dSG), (res.dSF, dSF)):
            assert abs(got - want) < 1e-7 * max(1.0, abs(want)), (outer, got, want)
        assert res.lowmode_force_evals == int(n_low)
        assert abs(res.plaquette - plaq) < 1e-10
        if res.accepted:  # the MG-HMC driver's coarse rebuild and deflation update
            mg.rebuild()
            mg.deflation_rr()
    assert np.max(np.abs(g.U.reshape(-1) - ms[f"U_out_{outer}"])) < 1e-9


@pytest.mark.parametrize("outer", [0, 1, 2])
def test_multiscale_reversibility_matches_reference(smg_gpu, ms, outer):
    lat, g, D, mg = _hierarchy(smg_gpu, ms)
    p = smg_gpu.ms_params(float(ms["ms_beta"]), tau=float(ms["ms_tau"]), n_outer=int(ms["ms_n_outer"]),
                          n_inner=int(ms["ms_n_inner"]), cg_maxiter=int(ms["ms_cg_maxiter"]),
                          cg_tol=float(ms["ms_cg_tol"]), inner_smooth=int(ms["ms_inner_smooth"]), outer=outer,
                          c_sw=float(ms["ms_c_sw"]))
    res = smg_gpu.hmc_mg_multiscale_reversibility(g, float(ms["m"]), float(ms["r"]), p, mg,
                                                  smg_gpu.Rng(int(ms["seed"]) + 20 + outer))
    gd, md, dHf, dHb, _ = ms[f"rev_{outer}"]
    assert abs(res.dH_forward - dHf) < 1e-7 * max(1.0, abs(dHf))
    assert abs(res.dH_backward - dHb) < 1e-7 * max(1.0, abs(dHb))
    assert res.gauge_delta < 1e-10 and res.mom_delta < 1e-9
    assert np.max(np.abs(g.U.reshape(-1) - ms["U"])) == 0.0


def test_multiscale_bad_arguments(smg_gpu, ms):
    lat, g, D, mg = _hierarchy(smg_gpu, ms)
    other = smg_gpu.GaugeField(lat, ms["U"])
    p = smg_gpu.ms_params(4.0)
    with pytest.raises(smg_gpu.SmgError):
        smg_gpu.hmc_mg_multiscale(other, 0.1, 1.0, p, mg, smg_gpu.Rng(1))
    p.n_inner = 0
    with pytest.raises(smg_gpu.SmgError):
        smg_gpu.hmc_mg_multiscale(g, 0.1, 1.0, p, mg, smg_gpu.Rng(1))


def test_deflation_of_the_coarsest_level(smg_gpu):
    """Eigenpairs of a deeper level's operator (level 2 of three), and the cycle with the coarsest CG
    started from their deflated guess equals the undeflated cycle when the coarsest CG converges."""
    L = 32
    lat = smg_gpu.Lattice(L)
    g = smg_gpu.GaugeField(lat, smg_gpu.gauge_normal(L, 3.0, 401))
    D = smg_gpu.DiracOp(lat, g, 0.1, 1.0, 1.0, 0.0)
    p = smg_gpu.mg_params(3, 4, 4, blocks=[(4, 4), (2, 2)], null_iters=3, coarse_tol=1e-13, coarse_max_iter=2000,
                          seed=9)
    mg = smg_gpu.MGHierarchy(D, p)
    src = smg_gpu.random_vec(lat.ndof, 17)
    plain = mg.precondition(src)
    info = mg.setup_deflation(6, level=2)
    assert info.converged
    vals, vecs = mg.deflation
    assert vecs.shape == (6, mg.level_dim(2))
    for v, lam in zip(vecs, vals):
        assert np.linalg.norm(mg.coarse_apply(2, v) - lam * v) < 1e-8 * lam
    defl = mg.precondition(src)
    assert np.linalg.norm(defl - plain) / np.linalg.norm(plain) < 1e-9
    with pytest.raises(smg_gpu.SmgError):  # the low-mode solution needs a level-1 space
        mg.lowmode_solution(src)
