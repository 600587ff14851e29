"""Pins the C restatement (the oracle) to the reference.

Two anchors: the golden fixtures that tests/golden/make_golden.py produced by
running the reference's own code, and — where the reference shim is built —
the reference itself on fresh seeded inputs.  CPU only.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden

DIRAC_CASES = ["dirac_L8_wilson", "dirac_L16_clover_twist", "dirac_L32_config1"]


@pytest.mark.parametrize("name", DIRAC_CASES)
def test_port_dirac_matches_golden(port, name):
    d = golden(name)
    args = (d["U"], float(d["m"]), float(d["r"]), float(d["csw"]), float(d["mu"]))
    for op, key in enumerate(["D", "Ddag", "DdagD", "g5D"]):
        got = port.dirac(*args, op, d["src"])
        np.testing.assert_array_equal(got, d[key], err_msg=f"{name} {key}")
    np.testing.assert_array_equal(port.clover(d["U"]), d["clover"])
    assert port.avg_plaq(d["U"]) == pytest.approx(float(d["avg_plaq"]), rel=1e-14)


@pytest.mark.parametrize("name", ["cg_force_L32_config1", "cg_force_L16_wilson"])
def test_port_cg_and_forces_match_golden(port, name):
    d = golden(name)
    args = (d["U"], float(d["m"]), float(d["r"]), float(d["csw"]), float(d["mu"]))
    x, it, res = port.cg(*args, d["phi"], 10000, float(d["tol"]))
    assert abs(it - int(d["cg_iters"])) <= 1
    assert np.linalg.norm(x - d["X"]) / np.linalg.norm(d["X"]) < 1e-9
    np.testing.assert_allclose(port.fermion_force(*args, d["X"]), d["fermion_force"], rtol=0, atol=1e-13)
    np.testing.assert_array_equal(port.gauge_force(d["U"], float(d["beta"])), d["gauge_force"])
    assert port.gauge_action(d["U"], float(d["beta"])) == pytest.approx(float(d["gauge_action"]), rel=1e-13)


def test_port_mg_pieces_match_golden(port):
    d = golden("mg_L16_bs4_k4")
    L, bs, k = int(d["L"]), int(d["bs"]), int(d["k"])
    args = (d["U"], float(d["m"]), float(d["r"]), float(d["csw"]), float(d["mu"]))
    nv = port.near_null_space(*args, k, int(d["null_iters"]), d["init"])
    assert np.max(np.abs(nv - d["null_vecs"])) < 1e-10
    bv = port.prolongator_build(L, bs, k, d["null_vecs"])
    np.testing.assert_allclose(bv, d["block_vecs"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(port.restrict(L, bs, k, d["block_vecs"], d["fine_src"]), d["restrict"], atol=1e-13)
    np.testing.assert_allclose(port.prolong(L, bs, k, d["block_vecs"], d["coarse_src"]), d["prolong"], atol=1e-13)
    links = port.sparse_coarse_build(*args, bs, k, d["block_vecs"])
    np.testing.assert_allclose(links, d["links"], rtol=0, atol=1e-12)
    nbx = L // bs
    np.testing.assert_allclose(port.sparse_coarse_apply(nbx, nbx, k, d["links"], d["coarse_src"]),
                               d["coarse_apply"], atol=1e-12)
    x = port.mr_smooth(*args, d["fine_src"], np.zeros_like(d["fine_src"]), 4)
    assert np.linalg.norm(x - d["mr4"]) / np.linalg.norm(d["mr4"]) < 1e-12


def test_port_mg_cycle_and_gcr_match_golden(port):
    d = golden("mg_L16_bs4_k4")
    L, bs, k = int(d["L"]), int(d["bs"]), int(d["k"])
    p = port.mg2_params(L, bs, k, float(d["m"]), float(d["r"]), float(d["csw"]), float(d["mu"]), 3, 3, 1000, 1e-13)
    # the reference solves the coarsest level by dense LU; the oracle by CG to 1e-13
    pre = port.mg2_precondition(p, d["U"], d["block_vecs"], d["links"], d["fine_src"])
    assert np.linalg.norm(pre - d["mg_precondition"]) / np.linalg.norm(d["mg_precondition"]) < 1e-10
    # with the reference's orthogonalisation coefficient, GCR reproduces its stall
    x, it, res = port.mg2_gcr(p, d["U"], d["block_vecs"], d["links"], d["fine_src"], 200, 1e-10, 20, ref_coeff=True)
    assert it == int(d["gcr_iters"])
    assert res == pytest.approx(float(d["gcr_res"]), rel=1e-3)
    # with the projection coefficient it converges
    x, it, res = port.mg2_gcr(p, d["U"], d["block_vecs"], d["links"], d["fine_src"], 200, 1e-10, 20)
    assert res < 1e-10 and it < 60


def test_host_inputs_reproduce_reference_draws(port):
    import schwinger_mg_gb300.api as api

    d = golden("dirac_L16_clover_twist")
    L = int(d["L"])
    U = api.gauge_normal(L, float(d["beta"]), int(d["gseed"])).reshape(-1)
    np.testing.assert_array_equal(U, d["U"])
    v = api.random_vec(2 * L * L, int(d["vseed"]))
    np.testing.assert_array_equal(v, d["src"])
    m = golden("mg_L16_bs4_k4")
    n = 2 * int(m["L"]) ** 2
    first = api.random_vec(n, int(m["seed"]))
    np.testing.assert_array_equal(first, m["init"][:n])


def test_gauge_normal_statistics():
    import schwinger_mg_gb300.api as api

    U = api.gauge_normal(64, 4.0, 5)
    th = np.angle(U)
    assert np.allclose(np.abs(U), 1.0, atol=1e-15)
    assert abs(th.mean()) < 0.02 and abs(th.var() - 0.25) < 0.02


# ---- against the reference itself, fresh inputs (skipped where it is not built)

@pytest.mark.parametrize("L,m,csw,mu", [(6, 0.2, 0.0, 0.0), (12, -0.05, 1.0, 0.0), (20, 0.1, 1.5, 0.3)])
def test_port_matches_reference_dirac(port, ref, L, m, csw, mu):
    import schwinger_mg_gb300.api as api

    U = api.gauge_normal(L, 3.0, 100 + L).reshape(-1)
    src = ref.random_vecs(1, 2 * L * L, 7)
    for op in range(4):
        np.testing.assert_array_equal(port.dirac(U, m, 1.0, csw, mu, op, src), ref.dirac(U, m, 1.0, csw, mu, op, src))
    X = ref.random_vecs(1, 2 * L * L, 8)
    np.testing.assert_array_equal(port.fermion_force(U, m, 1.0, csw, mu, X), ref.fermion_force(U, m, 1.0, csw, mu, X))


def test_reference_force_verification_passes(ref):
    import schwinger_mg_gb300.api as api

    U = api.gauge_normal(8, 2.0, 3).reshape(-1)
    assert ref.verify_forces(U, 2.0, 0.1, 1.0, 1.0, 0.0, 2000, 1e-12)


def test_port_null_space_matches_reference(port, ref):
    import schwinger_mg_gb300.api as api

    L, k, iters, seed = 8, 3, 4, 77
    U = api.gauge_normal(L, 2.0, 9).reshape(-1)
    init = ref.random_vecs(k, 2 * L * L, seed)
    want = ref.near_null_space(U, 0.1, 1.0, 1.0, 0.0, k, iters, seed)
    got = port.near_null_space(U, 0.1, 1.0, 1.0, 0.0, k, iters, init)
    assert np.max(np.abs(got - want)) < 1e-11


def test_port_nlevel_cycle_matches_two_level_and_reference(port):
    d = golden("mg_L16_bs4_k4")
    L, bs, k = int(d["L"]), int(d["bs"]), int(d["k"])
    args = (float(d["m"]), float(d["r"]), float(d["csw"]), float(d["mu"]))
    p2 = port.mg2_params(L, bs, k, *args, 3, 3, 1000, 1e-13)
    two = port.mg2_precondition(p2, d["U"], d["block_vecs"], d["links"], d["fine_src"])
    pN = port.mgN_params(L, *args, [(bs, bs)], [k], [d["block_vecs"]], [None, d["links"]], 3, 3, True, 1000, 1e-13)
    nl = port.mgN_precondition(pN, d["U"], d["fine_src"])
    assert np.max(np.abs(nl - two)) / np.max(np.abs(two)) < 1e-13
    assert np.linalg.norm(nl - d["mg_precondition"]) / np.linalg.norm(d["mg_precondition"]) < 1e-10
