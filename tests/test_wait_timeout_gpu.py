"""A bounded device wait made to run out on purpose: the coarsest-level CG kernel's grid barrier
(a cooperative launch, every block co-resident) polls at most smg_mg_set_wait_limit times before
it gives up, raises the hierarchy's error flag and returns.  With a bound of 0 polls a waiting
block gives up at once, the cycle reports SMG_TIMEOUT, and with the default bound restored the
same hierarchy gives the same cycle as before and a converged solve: the context stays usable.
No GPU fault, trap or endless wait is involved."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_grid_barrier_wait_runs_out_and_reports_timeout(smg_gpu):
    from schwinger_mg_gb300 import _lib

    L = 64
    lat = smg_gpu.Lattice(L)
    D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat, smg_gpu.gauge_normal(L, 6.0, 11)), -0.05, 1.0, 1.0, 0.0)
    # two levels with 8 coarse dofs and one right-hand side: the coarsest CG runs as the persistent kernel
    p = smg_gpu.mg_params(2, 4, 8, null_iters=2, w_cycle=False, coarse_max_iter=200, coarse_tol=1e-12, seed=3)
    mg = smg_gpu.MGHierarchy(D, p)
    b = smg_gpu.random_vec(lat.ndof, 12)
    y0 = mg.precondition(b)
    lib = smg_gpu.lib()
    assert lib.smg_mg_set_wait_limit(mg.h, 0) == _lib.OK
    with pytest.raises(_lib.SmgError) as e:
        mg.precondition(b)
    assert e.value.status == _lib.TIMEOUT
    assert lib.smg_mg_set_wait_limit(mg.h, -1) == _lib.OK
    y1 = mg.precondition(b)
    assert np.max(np.abs(y1 - y0)) <= 1e-13 * np.max(np.abs(y0))
    r = smg_gpu.fcg_solve_mg(D, lat.ndof, b, mg, 300, 1e-10, 20)
    assert r.status == 0 and r.true_residual < 1e-10


def test_persistent_tensor_core_cg_wait_runs_out_and_reports_timeout(smg_gpu):
    """The same bound on the coarsest CG of 32 right-hand sides that runs as one cooperative
    tensor-core launch (FP16 vectors): its grid barriers give up at once with a bound of 0 polls, every
    CTA leaves (bulk copies and MMAs drained, tensor memory freed), the cycle reports SMG_TIMEOUT, and
    the restored bound gives the same cycle bit for bit."""
    from schwinger_mg_gb300 import _lib

    L, nrhs = 64, 32
    lat = smg_gpu.Lattice(L)
    D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat, smg_gpu.gauge_normal(L, 6.0, 13)), -0.05, 1.0, 1.0, 0.0)
    p = smg_gpu.mg_params(3, 4, 16, blocks=[(4, 4), (2, 2)], chiral_split=False, null_iters=3, pre_smooth=2,
                          post_smooth=2, w_cycle=False, coarse_max_iter=20, coarse_tol=5e-2, precision="f32",
                          seed=5, smoother_half=True, coarse_half=True)
    mg = smg_gpu.MGHierarchy(D, p)
    B = np.stack([smg_gpu.random_vec(lat.ndof, 40 + j) for j in range(nrhs)])
    b = smg_gpu.Field(lat, nrhs, "f32", data=B)
    y0 = mg.precondition(b).download()
    lib = smg_gpu.lib()
    assert lib.smg_mg_set_wait_limit(mg.h, 0) == _lib.OK
    with pytest.raises(_lib.SmgError) as e:
        mg.precondition(b)
    assert e.value.status == _lib.TIMEOUT
    assert lib.smg_mg_set_wait_limit(mg.h, -1) == _lib.OK
    y1 = mg.precondition(b).download()
    assert np.array_equal(y1, y0)
