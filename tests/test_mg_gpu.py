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


@pytest.mark.parametrize("nrhs,levels,k,chiral,prec", [(4, 2, 4, True, "f64"), (16, 3, 4, True, "f64"),
                                                       (32, 3, 4, True, "f64"), (32, 3, 16, False, "f64"),
                                                       (32, 3, 4, True, "f32"), (32, 3, 16, False, "f32")])
def test_multi_rhs_cycle_equals_single(smg_gpu, nrhs, levels, k, chiral, prec):
    """The batched cycle equals one cycle per RHS: aggregate-blocked transfers from 8 RHS up (8 and 16
    coarse dofs, FP64 and FP32) against the one-thread-per-output transfers of a single RHS.  The F32
    cases keep the coarse operators on the CUDA cores, so that only rounding order differs."""
    L = 32
    U = smg_gpu.gauge_normal(L, 4.0, 17)
    lat = smg_gpu.Lattice(L)
    D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat, U), 0.05, 1.0, 1.0, 0.0)
    p = smg_gpu.mg_params(levels, 4, k, blocks=[(4, 4), (2, 2)], chiral_split=chiral, null_iters=3, coarse_tol=1e-6,
                          coarse_max_iter=500, precision=prec, tensor_cores=False)
    mg = smg_gpu.MGHierarchy(D, p)
    B = np.stack([smg_gpu.random_vec(lat.ndof, 300 + j) for j in range(nrhs)])
    multi = mg.precondition(B)
    tol = 1e-10 if prec == "f64" else 2e-4
    for j in (0, nrhs - 1):
        single = mg.precondition(B[j])
        assert np.linalg.norm(multi[j] - single) / np.linalg.norm(single) < tol


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


def test_three_level_reference_blocking_matches_reference(smg_gpu):
    """The reference's three-level hierarchy (golden mg3_L48_k4): level 2 blocks 4k consecutive level-1
    dofs (CoarseProlongator, src/prolongator.h:149-228), which is the 4 x 1 aggregate of level-1 sites,
    with the dense intermediate operator P^dag A_1 P (src/multigrid.cpp:640-687).  The GPU hierarchy is
    built from the same seed: null vectors, level-1 block vectors, level-2 operator, W-cycle and the
    reference-coefficient GCR are compared."""
    d = golden("mg3_L48_k4")
    lat, g, D = _setup(smg_gpu, d)
    k = int(d["k"])
    p = smg_gpu.mg_params(3, int(d["bs"]), k, blocks=[(int(d["bs"]), int(d["bs"])), (4, 1)],
                          null_iters=int(d["null_iters"]), seed=int(d["seed"]), w_cycle=True, pre_smooth=3,
                          post_smooth=3, coarse_tol=1e-14, coarse_max_iter=5000)
    mg = smg_gpu.MGHierarchy(D, p)
    n1 = int(d["L"]) // int(d["bs"])
    assert mg.level_dims(2) == (n1 // 4, n1, k)
    assert _relmax(mg.null_vecs_l0.reshape(-1), d["null_vecs"].reshape(-1)) < 1e-9
    assert _relmax(mg.prolongator(1), d["block_vecs1"]) < 1e-8
    assert _relmax(mg.coarse_op(2), d["links2"]) < 1e-8
    out = mg.precondition(d["fine_src"])
    ref = d["mg_precondition"]
    assert np.linalg.norm(out - ref) / np.linalg.norm(ref) < 1e-8
    r = smg_gpu.fcg_solve_mg(D, lat.ndof, d["fine_src"], mg, 200, 1e-10, 20, reference_coefficient=True)
    assert r.iterations == int(d["gcr_iters"])
    assert r.final_residual == pytest.approx(float(d["gcr_res"]), rel=0.05)


def test_chiral_coarse_links_match_oracle(smg_gpu, port):
    """Nc = 16 (8 null vectors split by chirality): the GPU's direct Galerkin links against the oracle's
    probing build (SparseCoarseOp::build, src/coarse_op.h:241-279) on the GPU's own block vectors, and the
    whole three-level hierarchy against the oracle's CPU set-up from the same seed."""
    L = 32
    U = smg_gpu.gauge_normal(L, 6.0, 4242)
    lat = smg_gpu.Lattice(L)
    args = (-0.05, 1.0, 1.0, 0.0)
    D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat, U), *args)
    p = smg_gpu.mg_params(3, 4, 8, blocks=[(4, 4), (2, 2)], chiral_split=True, null_iters=2, seed=7)
    mg = smg_gpu.MGHierarchy(D, p)
    assert mg.level_dims(1) == (8, 8, 16)
    bv = mg.prolongator(0)
    assert _relmax(mg.coarse_op(1), port.sparse_coarse_build(U, *args, 4, 16, bv)) < 1e-12
    bvs, links, null0 = port.mgN_setup(L, U, *args, [(4, 4), (2, 2)], [8, 8], 2, 7, chiral_split=True)
    assert _relmax(mg.null_vecs_l0.reshape(-1), null0.reshape(-1)) < 1e-10
    assert _relmax(bv, bvs[0]) < 1e-10
    assert _relmax(mg.coarse_op(1), links[1]) < 1e-10
    assert _relmax(mg.coarse_op(2), links[2]) < 1e-8


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_config2_two_level_chiral_L256(smg_gpu, prec):
    """The two-level configuration at L = 256 (beta = 6, m = -0.05, c_sw = 1): 4 x 4 aggregates, 8 null
    vectors split by chirality (16 coarse dofs), 2 inverse iterations, 4 MR steps, coarsest CG <= 50
    iterations to 5e-2.  Plain FP64 and the FP32 hierarchy inside FP64 defect correction both reach a
    true FP64 residual of 1e-10; the mixed solve takes at most 15 % more GCR iterations."""
    L = 256
    U = smg_gpu.gauge_normal(L, 6.0, 2025)
    lat = smg_gpu.Lattice(L)
    D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat, U), -0.05, 1.0, 1.0, 0.0)
    b = smg_gpu.random_vec(lat.ndof, 2026)
    its = {}
    for pr in ("f64", prec):
        p = smg_gpu.mg_params(2, 4, 8, chiral_split=True, null_iters=2, pre_smooth=4, post_smooth=4, w_cycle=False,
                              coarse_max_iter=50, coarse_tol=5e-2, precision=pr, seed=2025)
        mg = smg_gpu.MGHierarchy(D, p)
        assert mg.level_dims(1) == (64, 64, 16)
        r = smg_gpu.fcg_solve_mg(D, lat.ndof, b, mg, 1000, 1e-10, 20)
        assert r.status == 0, r
        assert r.true_residual < 1e-10
        its[pr] = r.iterations
    Ax = D.apply_DdagD(r.solution)
    assert np.linalg.norm(b - Ax) / np.linalg.norm(b) < 1e-10
    assert its[prec] <= 1.15 * its["f64"] + 1


def test_config2_settings_match_oracle_iterations(smg_gpu, port):
    """The same settings at L = 64: the GPU's FP64 hierarchy and GCR against the oracle's CPU set-up and
    GCR from the same seeds (the oracle's GCR stops on the recursive residual)."""
    L = 64
    U = smg_gpu.gauge_normal(L, 6.0, 2025)
    lat = smg_gpu.Lattice(L)
    args = (-0.05, 1.0, 1.0, 0.0)
    D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat, U), *args)
    p = smg_gpu.mg_params(2, 4, 8, chiral_split=True, null_iters=2, pre_smooth=4, post_smooth=4, w_cycle=False,
                          coarse_max_iter=50, coarse_tol=5e-2, precision="f64", seed=2025)
    mg = smg_gpu.MGHierarchy(D, p)
    b = smg_gpu.random_vec(lat.ndof, 2026)
    r = smg_gpu.fcg_solve_mg(D, lat.ndof, b, mg, 1000, 1e-10, 20)
    bvs, links, _ = port.mgN_setup(L, U, *args, [(4, 4)], [8], 2, 2025, chiral_split=True)
    assert _relmax(mg.coarse_op(1), links[1]) < 1e-9
    po = port.mgN_params(L, *args, [(4, 4)], [16], bvs, links, 4, 4, False, 50, 5e-2)
    _, it_o, res_o, _ = port.mgN_gcr(po, U, b, 1000, 1e-10, 20)
    assert r.status == 0 and r.true_residual < 1e-10
    assert abs(r.iterations - it_o) <= 2


def test_gcr_in_the_cycle_graph_fields_across_rhs_counts(smg_gpu):
    """The GCR keeps its residual and preconditioned vector in the captured cycle's own input and output
    fields: solves of 8, then 32, then again 8 right-hand sides on one FP32 hierarchy recapture the cycle
    for each count, each reaches a true residual of 1e-10, and the two 8-RHS solves agree bit for bit
    (after a first pass over both counts has fixed the stencil's timed launch shapes)."""
    L = 32
    lat = smg_gpu.Lattice(L)
    D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat, smg_gpu.gauge_normal(L, 6.0, 17)), -0.05, 1.0, 1.0, 0.0)
    mg = smg_gpu.MGHierarchy(D, smg_gpu.mg_params(2, 4, 8, null_iters=3, pre_smooth=4, post_smooth=4,
                                                  w_cycle=False, coarse_tol=1e-6, precision="f32", seed=3))
    B32 = np.stack([smg_gpu.random_vec(lat.ndof, 200 + j) for j in range(32)])
    # the stencil's launch shape is chosen by timing on its first use per RHS count; a first solve does
    # that, so the compared solves run the same kernels
    smg_gpu.fcg_solve_mg(D, lat.ndof, B32[:8], mg, 300, 1e-10, 10)
    smg_gpu.fcg_solve_mg(D, lat.ndof, B32, mg, 300, 1e-10, 10)
    r8a = smg_gpu.fcg_solve_mg(D, lat.ndof, B32[:8], mg, 300, 1e-10, 10)
    r32 = smg_gpu.fcg_solve_mg(D, lat.ndof, B32, mg, 300, 1e-10, 10)
    r8b = smg_gpu.fcg_solve_mg(D, lat.ndof, B32[:8], mg, 300, 1e-10, 10)
    for r in (r8a, r32, r8b):
        assert r.status == 0 and r.true_residual < 1e-10
    assert r8a.iterations == r8b.iterations
    assert np.array_equal(r8a.solution, r8b.solution)
    j = 5
    assert np.linalg.norm(B32[j] - D.apply_DdagD(r32.solution[j])) / np.linalg.norm(B32[j]) < 1e-10
