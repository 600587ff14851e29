"""GPU BLAS-1 and CG parity (reference src/linalg.cpp, src/solvers.cpp:16-78)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nrhs,prec,tol", [(1, "f64", 1e-13), (5, "f64", 1e-13), (32, "f32", 1e-5)])
def test_blas(smg_gpu, nrhs, prec, tol):
    lat = smg_gpu.Lattice(64)
    a = np.stack([smg_gpu.random_vec(lat.ndof, 10 + j) for j in range(nrhs)])
    b = np.stack([smg_gpu.random_vec(lat.ndof, 50 + j) for j in range(nrhs)])
    fa = smg_gpu.Field(lat, nrhs, prec, data=a)
    fb = smg_gpu.Field(lat, nrhs, prec, data=b)
    want_dot = np.einsum("ij,ij->i", a.conj(), b)
    np.testing.assert_allclose(smg_gpu.dot(fa, fb), want_dot, rtol=tol)
    np.testing.assert_allclose(smg_gpu.norm(fa), np.linalg.norm(a, axis=1), rtol=tol)
    alpha = (np.arange(nrhs) + 1) * (0.5 - 0.25j)
    smg_gpu.axpy(alpha, fa, fb)
    np.testing.assert_allclose(fb.download().reshape(nrhs, -1), b + alpha[:, None] * a, rtol=tol, atol=tol)
    smg_gpu.scale(fa, 2.0)
    np.testing.assert_allclose(fa.download().reshape(nrhs, -1), 2 * a, rtol=tol, atol=tol)


def test_blas_deterministic(smg_gpu):
    lat = smg_gpu.Lattice(128)
    fa = smg_gpu.Field(lat, 1, "f64", data=smg_gpu.random_vec(lat.ndof, 1))
    vals = {float(smg_gpu.norm(fa)[0]) for _ in range(5)}
    assert len(vals) == 1


def test_cg_config1_matches_reference(smg_gpu):
    """Config 1: L=32, beta=2, m=0.1, c_sw=1, CG on D^dag D to 1e-10."""
    d = golden("cg_force_L32_config1")
    L = int(d["L"])
    lat = smg_gpu.Lattice(L)
    D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat, d["U"]), float(d["m"]), float(d["r"]), float(d["csw"]),
                        float(d["mu"]))
    res = smg_gpu.cg_solve(D, lat.ndof, d["phi"], 10000, 1e-10)
    assert abs(res.iterations - int(d["cg_iters"])) <= 2
    assert res.final_residual < 1e-10
    assert res.true_residual < 2e-10
    assert np.linalg.norm(res.solution - d["X"]) / np.linalg.norm(d["X"]) < 1e-8


def test_cg_multi_rhs_and_zero_rhs(smg_gpu, port):
    L = 32
    U = smg_gpu.gauge_normal(L, 2.0, 9)
    lat = smg_gpu.Lattice(L)
    D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat, U), 0.1, 1.0, 1.0, 0.0)
    B = np.stack([smg_gpu.random_vec(lat.ndof, 200 + j) for j in range(4)])
    B[2] = 0.0  # a zero right-hand side returns x = 0 (solvers.cpp:23)
    res = smg_gpu.cg_solve(D, lat.ndof, B, 5000, 1e-10)
    X = res.solution.reshape(4, -1)
    assert np.all(X[2] == 0)
    for j in (0, 1, 3):
        x_o, it_o, _ = port.cg(U, 0.1, 1.0, 1.0, 0.0, B[j], 5000, 1e-10)
        assert np.linalg.norm(X[j] - x_o) / np.linalg.norm(x_o) < 1e-8
    assert res.true_residual < 2e-10


def test_cg_f32(smg_gpu):
    d = golden("cg_force_L32_config1")
    lat = smg_gpu.Lattice(int(d["L"]))
    D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat, d["U"]), float(d["m"]), 1.0, float(d["csw"]), 0.0)
    res = smg_gpu.cg_solve(D, lat.ndof, d["phi"], 10000, 1e-5, precision="f32")
    assert res.final_residual < 1e-5
    assert np.linalg.norm(res.solution - d["X"]) / np.linalg.norm(d["X"]) < 1e-3


def test_cg_not_converged_status(smg_gpu):
    d = golden("cg_force_L32_config1")
    lat = smg_gpu.Lattice(int(d["L"]))
    D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat, d["U"]), float(d["m"]), 1.0, float(d["csw"]), 0.0)
    res = smg_gpu.cg_solve(D, lat.ndof, d["phi"], 10, 1e-10)
    assert res.iterations == 10 and res.final_residual > 1e-10
    with pytest.raises(smg_gpu.SmgError) as e:
        smg_gpu.cg_solve(D, lat.ndof, d["phi"], 10, 1e-10, raise_on_failure=True)
    assert e.value.status == 1


def test_cg_nonfinite_rhs(smg_gpu):
    lat = smg_gpu.Lattice(8)
    D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat), 0.1)
    b = smg_gpu.random_vec(lat.ndof, 1)
    b[5] = np.nan
    with pytest.raises(smg_gpu.SmgError) as e:
        smg_gpu.cg_solve(D, lat.ndof, b, 100, 1e-10)
    assert e.value.status == 3


@pytest.mark.parametrize("prec", ["f64", "f32", "f16"])
def test_pinned_host_transfers_match_pageable(smg_gpu, prec):
    """Uploads and downloads with page-locked host buffers (read and written by the layout kernels in
    place) give the same fields and host images as with pageable numpy buffers (staged on the device)."""
    torch = pytest.importorskip("torch")
    import ctypes as C

    from schwinger_mg_gb300 import _lib

    lat = smg_gpu.Lattice(32)
    nrhs = 8
    B = np.stack([smg_gpu.random_vec(lat.ndof, 900 + j) for j in range(nrhs)])
    ref = smg_gpu.Field(lat, nrhs, prec, data=B)
    pin_in = torch.empty(B.size * 2, dtype=torch.float64).pin_memory()
    pin_in.numpy()[:] = B.reshape(-1).view(np.float64)
    pin_out = torch.zeros_like(pin_in).pin_memory()
    dp = C.POINTER(C.c_double)
    f = smg_gpu.Field(lat, nrhs, prec)
    lib = smg_gpu.lib()
    assert lib.smg_field_upload_async(f.h, C.cast(pin_in.data_ptr(), dp)) == _lib.OK
    assert lib.smg_field_download_async(f.h, C.cast(pin_out.data_ptr(), dp)) == _lib.OK
    f.ctx.synchronize()
    want = ref.download()
    assert np.array_equal(f.download(), want)
    assert np.array_equal(pin_out.numpy().view(np.complex128).reshape(want.shape), want)
