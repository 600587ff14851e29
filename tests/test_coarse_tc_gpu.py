"""Tensor-core coarse-operator apply (coarse_tc.cu): the BF16 x BF16 -> FP32
MMA path against an exact emulation in numpy (operands rounded to BF16 the
same way, products summed in FP64), against the FP32 CUDA-core kernel, the
fused reductions, and a 32-RHS MG-GCR solve that uses it on every coarse level."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DX = [0, 1, -1, 0, 0, 1, 1, -1, -1]
DY = [0, 0, 0, 1, -1, 1, -1, 1, -1]


def bf16(a):
    """Round float32 values to the nearest BF16 (ties to even), returned as float32."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32)


def bf16c(z):
    return bf16(z.real.astype(np.float32)).astype(np.float64) + 1j * bf16(z.imag.astype(np.float32)).astype(np.float64)


def stencil(links, x, nx, ny, nd):
    """y[s][i][r] = sum_d sum_j L[s][d](i, j) x[s + delta_d][j][r]; links [s][d][i][j], x [s][j][r]."""
    Lk = links.reshape(ny, nx, 9, nd, nd)
    X = x.reshape(ny, nx, nd, -1)
    y = np.zeros(X.shape, dtype=np.complex128)
    for d in range(9):
        Xn = np.roll(X, shift=(-DY[d], -DX[d]), axis=(0, 1))
        y += np.einsum("yxij,yxjr->yxir", Lk[:, :, d], Xn)
    return y.reshape(nx * ny, nd, -1)


@pytest.fixture(scope="module")
def hier(smg_gpu):
    L = 64
    U = smg_gpu.gauge_normal(L, 6.0, 4242)
    lat = smg_gpu.Lattice(L)
    D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat, U), -0.05, 1.0, 1.0, 0.0)
    p = smg_gpu.mg_params(3, 4, 8, blocks=[(4, 4), (2, 2)], chiral_split=True, null_iters=3, pre_smooth=4,
                          post_smooth=4, coarse_max_iter=60, coarse_tol=1e-2, precision="f32", seed=7)
    mg = smg_gpu.MGHierarchy(D, p)
    return lat, D, mg


def _rand(shape, seed):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


def test_emulation_matches_fp64_host_apply(hier):
    lat, D, mg = hier
    nx, ny, nd = mg.level_dims(1)
    v = _rand((nx * ny, nd, 1), 1).astype(np.complex128)
    want = mg.coarse_apply(1, v.reshape(-1))
    got = stencil(mg.coarse_op(1), v, nx, ny, nd).reshape(-1)
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-13


@pytest.mark.parametrize("level,nrhs", [(1, 32), (2, 32), (1, 64)])
def test_tensor_core_apply_matches_bf16_emulation(hier, level, nrhs):
    lat, D, mg = hier
    nx, ny, nd = mg.level_dims(level)
    assert nd == 16 and nx % 8 == 0
    x = _rand((nx * ny, nd, nrhs), 10 + level + nrhs)
    y = mg.coarse_apply_batch(level, x, engine="tensor")
    # exact product of the BF16-rounded operands (links rounded from FP64 through FP32)
    links = mg.coarse_op(level).astype(np.complex64).astype(np.complex128)
    ye = stencil(bf16c(links), bf16c(x.astype(np.complex128)), nx, ny, nd)
    rel = np.linalg.norm(y - ye) / np.linalg.norm(ye)
    assert rel < 1e-5, rel  # FP32 accumulation of 288 products per output; a layout error gives O(1)
    assert np.max(np.abs(y - ye)) / np.max(np.abs(ye)) < 1e-4
    # against the FP32 CUDA-core kernel: BF16 operand rounding only
    yc = mg.coarse_apply_batch(level, x, engine="cuda")
    assert np.linalg.norm(y - yc) / np.linalg.norm(yc) < 1e-2


@pytest.mark.parametrize("level", [1, 2])
def test_tensor_core_fused_reductions(hier, level):
    lat, D, mg = hier
    nx, ny, nd = mg.level_dims(level)
    x = _rand((nx * ny, nd, 32), 77)
    w = _rand((nx * ny, nd, 32), 78)
    y, n2 = mg.coarse_apply_batch(level, x, engine="tensor", dots=True)
    y = y.astype(np.complex128)
    assert np.allclose(n2, np.sum(np.abs(y) ** 2, axis=(0, 1)), rtol=1e-5)
    y2, dot, n2b = mg.coarse_apply_batch(level, x, engine="tensor", w=w, dots=True)
    assert np.array_equal(y2, y.astype(np.complex64))
    want = np.sum(np.conj(y) * w.astype(np.complex128), axis=(0, 1))
    assert np.allclose(dot, want, rtol=1e-5, atol=1e-5 * np.max(np.abs(want)))
    assert np.allclose(n2b, n2, rtol=1e-12)


def test_tensor_core_engine_refuses_unsupported_shape(smg_gpu, hier):
    lat, D, mg = hier
    nx, ny, nd = mg.level_dims(1)
    with pytest.raises(smg_gpu.SmgError):
        mg.coarse_apply_batch(1, _rand((nx * ny, nd, 16), 3), engine="tensor")  # 16 rhs


def test_batched_mg_gcr_with_tensor_cores(smg_gpu, hier):
    """32 right-hand sides, every coarse apply of the cycle on the tensor cores: each
    solution reaches a true FP64 residual of 1e-10 in about as many iterations as
    with the FP32 CUDA-core coarse operators."""
    lat, D, mg = hier
    B = np.stack([smg_gpu.random_vec(lat.ndof, 500 + j) for j in range(32)])
    r = smg_gpu.fcg_solve_mg(D, lat.ndof, B, mg, 400, 1e-10, 20)
    assert r.status == 0, r
    X = r.solution
    for j in (0, 13, 31):
        Ax = D.apply_DdagD(X[j])
        assert np.linalg.norm(B[j] - Ax) / np.linalg.norm(B[j]) < 1e-10
    p = mg.params
    p.tensor_cores = 0
    mg_c = smg_gpu.MGHierarchy(D, p)
    rc = smg_gpu.fcg_solve_mg(D, lat.ndof, B, mg_c, 400, 1e-10, 20)
    assert rc.status == 0
    assert r.iterations <= rc.iterations + 4, (r.iterations, rc.iterations)
