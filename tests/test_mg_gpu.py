"""GPU multigrid: setup pieces and the cycle against the reference
(golden fixtures from tests/golden/make_golden.py) and the oracle; GCR
convergence to a true FP64 residual of 1e-10 in FP64 and mixed precision."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def _setup(smg, d):
    L = int(d["L"])
    lat = smg.Lattice(L)
    g = smg.GaugeField(lat, d["U"])
    D = smg.DiracOp(lat, g, float(d["m"]), float(d["r"]), float(d["csw"]), float(d["mu"]))
    return lat, g, D


def _relmax(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.fixture(scope="module")
def ref_mg(smg_gpu):
    """2-level hierarchy on exactly the reference's null vectors (warm start, 0 iterations)."""
    d = golden("mg_L16_bs4_k4")
    lat, g, D = _setup(smg_gpu, d)
    p = smg_gpu.mg_params(2, int(d["bs"]), int(d["k"]), null_iters=0, coarse_tol=1e-13, coarse_max_iter=2000)
    mg = smg_gpu.MGHierarchy(D, p, warm_start=d["null_vecs"])
    return d, lat, g, D, mg


def test_prolongator_and_galerkin_match_reference(ref_mg):
    d, lat, g, D, mg = ref_mg
    assert _relmax(mg.null_vecs_l0.reshape(-1), d["null_vecs"]) < 1e-13
    assert _relmax(mg.prolongator(0), d["block_vecs"]) < 1e-13
    # direct Galerkin vs the reference's probing build (src/coarse_op.h:241-279)
    assert _relmax(mg.coarse_op(1), d["links"]) < 1e-12


def test_transfers_and_coarse_apply_match_reference(ref_mg):
    d, lat, g, D, mg = ref_mg
    assert _relmax(mg.restrict_vec(0, d["fine_src"]), d["restrict"]) < 1e-13
    assert _relmax(mg.prolong(0, d["coarse_src"]), d["prolong"]) < 1e-13
    assert _relmax(mg.coarse_apply(1, d["coarse_src"]), d["coarse_apply"]) < 1e-12


def test_cycle_matches_reference(ref_mg):
    d, lat, g, D, mg = ref_mg
    # the reference solves the coarsest level by dense LU, this path by CG to 1e-13
    out = mg.precondition(d["fine_src"])
    ref = d["mg_precondition"]
    assert np.linalg.norm(out - ref) / np.linalg.norm(ref) < 1e-9


def test_gcr_reference_coefficient_reproduces_reference_stall(smg_gpu, ref_mg):
    d, lat, g, D, mg = ref_mg
    r = smg_gpu.fcg_solve_mg(D, lat.ndof, d["fine_src"], mg, 200, 1e-10, 20, reference_coefficient=True)
    assert r.iterations == int(d["gcr_iters"])
    assert r.final_residual == pytest.approx(float(d["gcr_res"]), rel=0.05)


def test_gcr_converges_and_matches_cg(smg_gpu, port, ref_mg):
    d, lat, g, D, mg = ref_mg
    r = smg_gpu.fcg_solve_mg(D, lat.ndof, d["fine_src"], mg, 200, 1e-10, 20)
    assert r.status == 0 and r.true_residual < 1e-10
    x_cg, _, _ = port.cg(d["U"], float(d["m"]), 1.0, float(d["csw"]), 0.0, d["fine_src"], 5000, 1e-13)
    assert np.linalg.norm(r.solution - x_cg) / np.linalg.norm(x_cg) < 1e-8
    # the oracle's GCR with the projection coefficient takes the same number of steps
    p = port.mg2_params(int(d["L"]), int(d["bs"]), int(d["k"]), float(d["m"]), 1.0, float(d["csw"]), 0.0, 3, 3,
                        2000, 1e-13)
    _, it_o, _ = port.mg2_gcr(p, d["U"], d["block_vecs"], d["links"], d["fine_src"], 200, 1e-10, 20)
    assert abs(r.iterations - it_o) <= 1


def test_null_space_from_seed_matches_reference(smg_gpu):
    d = golden("mg_L16_bs4_k4")
    lat, g, D = _setup(smg_gpu, d)
    p = smg_gpu.mg_params(2, int(d["bs"]), int(d["k"]), null_iters=int(d["null_iters"]), seed=int(d["seed"]))
    mg = smg_gpu.MGHierarchy(D, p)
    assert _relmax(mg.null_vecs_l0.reshape(-1), d["null_vecs"]) < 1e-9


@pytest.mark.parametrize("levels,prec", [(2, "f64"), (2, "f32"), (3, "f32")])
def test_chiral_mg_gcr_true_residual(smg_gpu, levels, prec):
    """4x4 aggregates, 8 null vectors split by chirality, then 2x2: GCR to a true FP64 residual of 1e-10."""
    L = 64
    U = smg_gpu.gauge_normal(L, 6.0, 4242)
    lat = smg_gpu.Lattice(L)
    D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat, U), -0.05, 1.0, 1.0, 0.0)
    p = smg_gpu.mg_params(levels, 4, 8, blocks=[(4, 4), (2, 2)], chiral_split=True, null_iters=4,
                          pre_smooth=4, post_smooth=4, coarse_max_iter=60, coarse_tol=1e-2, precision=prec,
                          seed=7)
    mg = smg_gpu.MGHierarchy(D, p)
    assert mg.level_dims(1) == (16, 16, 16)
    b = smg_gpu.random_vec(lat.ndof, 99)
    r = smg_gpu.fcg_solve_mg(D, lat.ndof, b, mg, 300, 1e-10, 20)
    assert r.status == 0, r
    assert r.true_residual < 1e-10
    Ax = D.apply_DdagD(r.solution)
    assert np.linalg.norm(b - Ax) / np.linalg.norm(b) < 1e-10


@pytest.mark.parametrize("nrhs,levels", [(4, 2), (16, 3)])
def test_multi_rhs_cycle_equals_single(smg_gpu, nrhs, levels):
    """The batched cycle (aggregate-blocked transfers from 8 RHS up) equals one cycle per RHS."""
    L = 32
    U = smg_gpu.gauge_normal(L, 4.0, 17)
    lat = smg_gpu.Lattice(L)
    D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat, U), 0.05, 1.0, 1.0, 0.0)
    p = smg_gpu.mg_params(levels, 4, 4, blocks=[(4, 4), (2, 2)], chiral_split=True, null_iters=3, coarse_tol=1e-6,
                          coarse_max_iter=500)
    mg = smg_gpu.MGHierarchy(D, p)
    B = np.stack([smg_gpu.random_vec(lat.ndof, 300 + j) for j in range(nrhs)])
    multi = mg.precondition(B)
    for j in (0, nrhs - 1):
        single = mg.precondition(B[j])
        assert np.linalg.norm(multi[j] - single) / np.linalg.norm(single) < 1e-10


def test_mg_bad_parameters(smg_gpu):
    lat = smg_gpu.Lattice(16)
    D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat), 0.1)
    with pytest.raises(smg_gpu.SmgError):
        smg_gpu.MGHierarchy(D, smg_gpu.mg_params(2, 8, 4))  # 2 x 2 coarse lattice
    with pytest.raises(smg_gpu.SmgError):
        smg_gpu.MGHierarchy(D, smg_gpu.mg_params(2, 3, 4))  # 3 does not divide 16


@pytest.mark.parametrize("chiral,k", [(False, 4), (True, 4)])
def test_three_level_cycle_matches_oracle(smg_gpu, port, chiral, k):
    """The GPU's 3-level W-cycle against the oracle's restatement of mg_cycle on the same hierarchy."""
    L = 32
    U = smg_gpu.gauge_normal(L, 3.0, 555)
    lat = smg_gpu.Lattice(L)
    D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat, U), 0.05, 1.0, 1.0, 0.0)
    blocks = [(4, 4), (2, 2)]
    p = smg_gpu.mg_params(3, 4, k, blocks=blocks, chiral_split=chiral, null_iters=3, coarse_tol=1e-13,
                          coarse_max_iter=3000, seed=11)
    mg = smg_gpu.MGHierarchy(D, p)
    ncs = [mg.level_dims(1)[2], mg.level_dims(2)[2]]
    po = port.mgN_params(L, 0.05, 1.0, 1.0, 0.0, blocks, ncs, [mg.prolongator(0), mg.prolongator(1)],
                         [None, mg.coarse_op(1), mg.coarse_op(2)], 3, 3, True, 3000, 1e-13)
    b = smg_gpu.random_vec(lat.ndof, 5)
    got = mg.precondition(b)
    want = port.mgN_precondition(po, U, b)
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-9


def test_rebuild_after_gauge_change(smg_gpu):
    """rebuild_deeper_levels: after new links, every coarse operator is the Galerkin product of the
    new operator with the existing prolongators (2 levels: equal to a fresh build on the same null
    vectors; level 2: A2 = P1^dag A1 P1 through the host transfer entry points)."""
    L = 32
    U1 = smg_gpu.gauge_normal(L, 3.0, 301)
    U2 = smg_gpu.gauge_normal(L, 3.0, 302)
    lat = smg_gpu.Lattice(L)
    g = smg_gpu.GaugeField(lat, U1)
    D = smg_gpu.DiracOp(lat, g, 0.1, 1.0, 1.0, 0.0)
    p = smg_gpu.mg_params(3, 4, 4, blocks=[(4, 4), (2, 2)], null_iters=3, coarse_tol=1e-13, coarse_max_iter=2000,
                          seed=3)
    mg = smg_gpu.MGHierarchy(D, p)
    nv = mg.null_vecs_l0.copy()
    g.set_links(U2)
    D.refresh()
    mg.rebuild()
    # level 1: the fresh hierarchy on U2 with the same null vectors has the same prolongator
    g2 = smg_gpu.GaugeField(lat, U2)
    D2 = smg_gpu.DiracOp(lat, g2, 0.1, 1.0, 1.0, 0.0)
    fresh = smg_gpu.MGHierarchy(D2, smg_gpu.mg_params(2, 4, 4, null_iters=0, coarse_tol=1e-13, seed=3),
                                warm_start=nv)
    assert np.max(np.abs(mg.coarse_op(1) - fresh.coarse_op(1))) / np.max(np.abs(fresh.coarse_op(1))) < 1e-12
    # level 2 is the Galerkin product of the rebuilt level-1 operator
    nx, ny, nd = mg.level_dims(2)
    rng = np.random.default_rng(5)
    xc = rng.standard_normal(nx * ny * nd) + 1j * rng.standard_normal(nx * ny * nd)
    want = mg.restrict_vec(1, mg.coarse_apply(1, mg.prolong(1, xc)))
    got = mg.coarse_apply(2, xc)
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-12


def test_rebuild_f32_cycle_matches_fresh_hierarchy(smg_gpu):
    """An F32 hierarchy rebuilt after new links applies the same cycle as one built on the new links
    from the same null vectors (its FP32 copies and captured cycle are refreshed in place)."""
    L = 32
    lat = smg_gpu.Lattice(L)
    g = smg_gpu.GaugeField(lat, smg_gpu.gauge_normal(L, 3.0, 303))
    D = smg_gpu.DiracOp(lat, g, 0.1, 1.0, 1.0, 0.0)
    p = smg_gpu.mg_params(2, 4, 4, null_iters=3, coarse_tol=1e-10, coarse_max_iter=500, precision="f32", seed=7)
    mg = smg_gpu.MGHierarchy(D, p)
    src = smg_gpu.random_vec(lat.ndof, 11)
    mg.precondition(src)  # one cycle on the old links before the rebuild
    U2 = smg_gpu.gauge_normal(L, 3.0, 304)
    g.set_links(U2)
    D.refresh()
    mg.rebuild()
    g2 = smg_gpu.GaugeField(lat, U2)
    D2 = smg_gpu.DiracOp(lat, g2, 0.1, 1.0, 1.0, 0.0)
    fresh = smg_gpu.MGHierarchy(
        D2, smg_gpu.mg_params(2, 4, 4, null_iters=0, coarse_tol=1e-10, coarse_max_iter=500, precision="f32", seed=7),
        warm_start=mg.null_vecs_l0)
    a, b = mg.precondition(src), fresh.precondition(src)
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-4
