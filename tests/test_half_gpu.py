"""FP16 fields with one FP32 scale per site (SMG_F16) and the MG cycle whose
fine smoother keeps its work vectors in them: storage error bounded by the
site scale, the operator on FP16 fields against FP64, and mixed MG-GCR
solves that still reach a true FP64 residual of 1e-10."""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_f16_round_trip_error_is_bounded_by_the_site_scale(smg_gpu):
    L, nrhs = 32, 8
    lat = smg_gpu.Lattice(L)
    rng = np.random.default_rng(3)
    # magnitudes spread over six decades across sites, equal within a site
    mag = 10.0 ** rng.uniform(-3, 3, size=lat.V)
    B = np.stack([smg_gpu.random_vec(lat.ndof, 10 + j) * np.repeat(mag, 2) for j in range(nrhs)])
    f = smg_gpu.Field(lat, nrhs, "f16", data=B)
    got = f.download().reshape(nrhs, lat.V, 2)
    want = B.reshape(nrhs, lat.V, 2)
    site_max = np.max(np.maximum(np.abs(want.real), np.abs(want.imag)), axis=(0, 2))
    err = np.max(np.maximum(np.abs((got - want).real), np.abs((got - want).imag)), axis=(0, 2))
    assert np.all(err <= 2.0 ** -11 * site_max * 1.001)


def test_f16_nrhs_must_be_a_power_of_two(smg_gpu):
    lat = smg_gpu.Lattice(16)
    with pytest.raises(smg_gpu.SmgError):
        smg_gpu.Field(lat, 12, "f16")


@pytest.mark.parametrize("nrhs,mu", [(8, 0.0), (32, 0.0), (32, 0.1)])
def test_operator_on_f16_fields(smg_gpu, nrhs, mu):
    """32 RHS without twist is the specialised smoother stencil (FP16 spin projections); with a twist,
    and at 8 RHS, the generic FP16 stencil."""
    L = 64
    U = smg_gpu.gauge_normal(L, 6.0, 21)
    lat = smg_gpu.Lattice(L)
    D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat, U), -0.05, 1.0, 1.0, mu)
    B = np.stack([smg_gpu.random_vec(lat.ndof, 30 + j) for j in range(nrhs)])
    for op in (0, 1):
        want = D.apply_op(op, B)
        f16 = smg_gpu.Field(lat, nrhs, "f16", data=B)
        got = D.apply_op(op, f16).download().reshape(want.shape)
        assert np.linalg.norm(got - want) / np.linalg.norm(want) < 2e-3


@pytest.mark.parametrize("nrhs,levels", [(8, 2), (32, 3)])
def test_half_smoother_cycle_and_solve(smg_gpu, nrhs, levels):
    L = 64
    U = smg_gpu.gauge_normal(L, 6.0, 41)
    lat = smg_gpu.Lattice(L)
    D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat, U), -0.05, 1.0, 1.0, 0.0)
    kw = dict(blocks=[(4, 4), (2, 2)], chiral_split=False, null_iters=4, pre_smooth=4, post_smooth=4,
              w_cycle=False, coarse_max_iter=20, coarse_tol=5e-2, precision="f32", seed=9)
    mg32 = smg_gpu.MGHierarchy(D, smg_gpu.mg_params(levels, 4, 16, **kw))
    mg16 = smg_gpu.MGHierarchy(D, smg_gpu.mg_params(levels, 4, 16, smoother_half=True, **kw))
    B = np.stack([smg_gpu.random_vec(lat.ndof, 50 + j) for j in range(nrhs)])
    b32 = smg_gpu.Field(lat, nrhs, "f32", data=B)
    c32 = mg32.precondition(b32).download()
    c16 = mg16.precondition(b32).download()
    assert np.linalg.norm(c16 - c32) / np.linalg.norm(c32) < 2e-2
    r = smg_gpu.fcg_solve_mg(D, lat.ndof, B, mg16, 300, 1e-10, 20)
    assert r.status == 0 and r.true_residual < 1e-10
    for j in (0, nrhs - 1):
        assert np.linalg.norm(B[j] - D.apply_DdagD(r.solution[j])) / np.linalg.norm(B[j]) < 1e-10


def test_half_coarsest_cg_cycle_and_solve(smg_gpu):
    """The coarsest-level CG with its residual and search direction in FP16 with one FP32 scale per
    coarse site (coarse_half; tensor-core apply on FP16 inputs): the cycle stays within the FP16
    rounding of the FP32-vector cycle, and the mixed solve reaches a true FP64 residual of 1e-10 in at
    most a few more iterations."""
    L, nrhs = 64, 32
    U = smg_gpu.gauge_normal(L, 6.0, 43)
    lat = smg_gpu.Lattice(L)
    D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat, U), -0.05, 1.0, 1.0, 0.0)
    kw = dict(blocks=[(4, 4), (2, 2)], chiral_split=False, null_iters=4, pre_smooth=4, post_smooth=4,
              w_cycle=False, coarse_max_iter=20, coarse_tol=5e-2, precision="f32", seed=11, smoother_half=True)
    mg32 = smg_gpu.MGHierarchy(D, smg_gpu.mg_params(3, 4, 16, **kw))
    mg16 = smg_gpu.MGHierarchy(D, smg_gpu.mg_params(3, 4, 16, coarse_half=True, **kw))
    assert mg16.level_dims(2) == (8, 8, 16)
    B = np.stack([smg_gpu.random_vec(lat.ndof, 70 + j) for j in range(nrhs)])
    b32 = smg_gpu.Field(lat, nrhs, "f32", data=B)
    c32 = mg32.precondition(b32).download()
    c16 = mg16.precondition(b32).download()
    assert np.linalg.norm(c16 - c32) / np.linalg.norm(c32) < 2e-2
    r32 = smg_gpu.fcg_solve_mg(D, lat.ndof, B, mg32, 300, 1e-10, 20)
    r16 = smg_gpu.fcg_solve_mg(D, lat.ndof, B, mg16, 300, 1e-10, 20)
    assert r16.status == 0 and r16.true_residual < 1e-10
    assert r16.iterations <= 1.1 * r32.iterations + 2
    for j in (0, nrhs - 1):
        assert np.linalg.norm(B[j] - D.apply_DdagD(r16.solution[j])) / np.linalg.norm(B[j]) < 1e-10


_CCG_CHILD = r"""
import sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import schwinger_mg_gb300 as smg
L, nrhs = 64, 32
lat = smg.Lattice(L)
D = smg.DiracOp(lat, smg.GaugeField(lat, smg.gauge_normal(L, 6.0, 43)), -0.05, 1.0, 1.0, 0.0)
nvec = int(sys.argv[3]) if len(sys.argv) > 3 else 16
chiral = len(sys.argv) > 4 and sys.argv[4] == "1"
nvec1 = int(sys.argv[5]) if len(sys.argv) > 5 else nvec
mg = smg.MGHierarchy(D, smg.mg_params(3, 4, nvec, blocks=[(4, 4), (2, 2)], n_vecs=[nvec, nvec1],
                                       chiral_split=chiral, null_iters=4,
                                       pre_smooth=4, post_smooth=4, w_cycle=False, coarse_max_iter=20,
                                       coarse_tol=5e-2, precision="f32", seed=11, smoother_half=True,
                                       coarse_half=True))
B = np.stack([smg.random_vec(lat.ndof, 70 + j) for j in range(nrhs)])
c = mg.precondition(smg.Field(lat, nrhs, "f32", data=B)).download()
r = smg.fcg_solve_mg(D, lat.ndof, B, mg, 300, 1e-10, 20)
np.savez(sys.argv[2], c=c, iters=r.iterations, res=r.true_residual)
"""


def _ccg_run(tmp_path: Path, name: str, persistent: bool, *args: str, **switches: str) -> dict:
    root = Path(__file__).resolve().parents[1]
    out = tmp_path / f"{name}.npz"
    env = dict(os.environ, SMG_CCG_PERSISTENT="1" if persistent else "0", **switches)
    subprocess.run([sys.executable, "-c", _CCG_CHILD, str(root), str(out), *args], env=env, check=True,
                   timeout=600)
    with np.load(out) as z:
        return {k: z[k] for k in z.files}


def test_persistent_coarsest_cg_matches_per_iteration_kernels(tmp_path):
    """The coarsest CG as one cooperative launch (k_ccg_tc: p formed on the fly from the FP16 r and the
    previous p, two grid barriers per iteration) against the per-iteration kernels (apply, update, p
    update) on the same hierarchy and right-hand sides, each in its own process: the cycles agree to
    the FP16 and BF16 rounding of the search direction, the solves reach 1e-10 in as many iterations
    up to two."""
    per = _ccg_run(tmp_path, "per_iteration", False)
    pst = _ccg_run(tmp_path, "persistent", True)
    assert np.linalg.norm(pst["c"] - per["c"]) / np.linalg.norm(per["c"]) < 1e-2
    assert float(pst["res"]) < 1e-10 and float(per["res"]) < 1e-10
    assert abs(int(pst["iters"]) - int(per["iters"])) <= 2


@pytest.mark.parametrize("nvec,chiral,nvec1", [(16, "0", 16), (8, "0", 8), (16, "1", 16), (16, "0", 8),
                                               (16, "0", 32)])
def test_packed_transfers_match_generic_kernels(tmp_path, nvec, chiral, nvec1):
    """The transfers with packed FP32 FMAs (level 0: k_restrict0_h, k_prolong0_ring; level 1:
    k_restrict_c16p, k_prolong_c16p; the prolongations with the pre-smoothing x pass folded in)
    against the generic aggregate kernels and separate x passes, each
    in its own process, for 8, 16 and (chirally split) 32 coarse dofs at level 0 and 8, 16 and 32 at
    level 1 (the level-1 kernels serve 16-dof sites, so with nvec 16 unsplit): the same arithmetic in FP32 up
    to the order of the sums, so the cycles agree to the FP16 rounding downstream, and the solves
    reach 1e-10 in as many iterations up to 3 % (a flexible solve with a preconditioner that differs
    in its last bits: 110 against 112 iterations with 8 null vectors)."""
    args = (str(nvec), chiral, str(nvec1))
    gen = _ccg_run(tmp_path, "generic", True, *args, SMG_TRANSFER_PACKED="0")
    pk = _ccg_run(tmp_path, "packed", True, *args, SMG_TRANSFER_PACKED="1")
    assert np.linalg.norm(pk["c"] - gen["c"]) / np.linalg.norm(gen["c"]) < 3e-3  # measured <= 5.1e-4
    assert float(pk["res"]) < 1e-10 and float(gen["res"]) < 1e-10
    assert abs(int(pk["iters"]) - int(gen["iters"])) <= max(1, int(0.03 * int(gen["iters"])))
