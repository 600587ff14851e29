"""Many independent lattices of uneven size in one batch (smg_batch_*): every
lattice's right-hand sides reach a true FP64 residual of 1e-10 with the mixed
MG-GCR, the accumulated pseudofermion force equals the sum of the per-RHS
forces from the single-lattice API, and the host-I/O solve returns the same."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cases(smg):
    rng = np.random.default_rng(11)
    out = []
    for k, L in enumerate([32, 16, 24, 20, 28]):
        beta = float(rng.uniform(2, 8))
        m = float(rng.uniform(-0.05, 0.2))
        U = smg.gauge_normal(L, beta, 700 + k)
        nrhs = 2 + k % 3
        B = np.stack([smg.random_vec(2 * L * L, 800 + 10 * k + j) for j in range(nrhs)])
        out.append((L, beta, m, U, B))
    return out


def test_batch_solves_and_forces(smg_gpu):
    cases = _cases(smg_gpu)
    batch = smg_gpu.LatticeBatch(n_workers=4)
    for L, beta, m, U, B in cases:
        batch.add(L, U, m, c_sw=1.0, nrhs=B.shape[0])
    p = smg_gpu.mg_params(2, 4, 8, null_iters=4, pre_smooth=4, post_smooth=4, coarse_max_iter=60, coarse_tol=1e-2,
                          precision="f32", seed=5)
    batch.setup(p)
    for i, (L, beta, m, U, B) in enumerate(cases):
        batch.bind(i, B)
    st, sec = batch.solve(500, 1e-10, 20, with_force=True)
    assert st == 0 and sec > 0
    for i, (L, beta, m, U, B) in enumerate(cases):
        s, r, _ = batch.result(i)
        assert s == 0 and r.true_residual < 1e-10, (i, s, r.true_residual)
        X, F = batch.download(i)
        lat = smg_gpu.Lattice(L)
        D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat, U), m, 1.0, 1.0, 0.0)
        for j in range(B.shape[0]):
            assert np.linalg.norm(B[j] - D.apply_DdagD(X[j])) / np.linalg.norm(B[j]) < 1e-10
        want = sum(smg_gpu.fermion_force(D, X[j]) for j in range(B.shape[0]))
        assert np.max(np.abs(F - want)) / np.max(np.abs(want)) < 1e-13
    # host I/O inside the call gives the same solutions and forces
    outs = []
    for i, (L, beta, m, U, B) in enumerate(cases):
        xo = np.zeros(B.size, dtype=np.complex128)
        fo = np.zeros(2 * L * L)
        batch.bind(i, B, xo, fo)
        outs.append((xo, fo))
    st, _ = batch.solve(500, 1e-10, 20, with_force=True, host_io=True)
    assert st == 0
    for i, (xo, fo) in enumerate(outs):
        X, F = batch.download(i)
        np.testing.assert_array_equal(xo.reshape(X.shape), X)
        np.testing.assert_array_equal(fo.reshape(F.shape), F)
    batch.close()


def test_batch_rejects_solve_before_setup(smg_gpu):
    batch = smg_gpu.LatticeBatch(n_workers=2)
    L = 16
    batch.add(L, smg_gpu.gauge_normal(L, 4.0, 1), 0.1, nrhs=1)
    st, _ = batch.solve(10, 1e-10)
    assert st != 0
    batch.close()
