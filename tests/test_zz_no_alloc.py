"""smg_blas_dot_noalloc, the dot product for callers that cannot allocate
device memory, against the existing smg_blas_dot entry point.

The file name sorts last so that a run stopping at the first failure has
already run every other test.  It must pass both alone in a fresh process and
after the rest of the suite."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dot_noalloc(lib, a_ptr, b_ptr, n, nrhs, out_ptr, stream):
    fn = lib.smg_blas_dot_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_void_p, C.c_void_p]
    return fn(a_ptr, b_ptr, n, nrhs, out_ptr, stream)


def test_dot_noalloc_matches_blas_dot_twice(smg_gpu):
    import torch

    smg = smg_gpu
    lib = smg.lib()
    ctx = smg.Context.default()
    lat = smg.Lattice(64)
    fa = smg.Field(lat, 1, "f64", data=smg.random_vec(lat.ndof, 11))
    fb = smg.Field(lat, 1, "f64", data=smg.random_vec(lat.ndof, 12))
    want = smg.dot(fa, fb)[0]  # existing entry point
    pa = lib.smg_field_device_ptr(fa.h)
    pb = lib.smg_field_device_ptr(fb.h)
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    stream = lib.smg_context_stream(ctx.h)
    for _ in range(2):  # the shared scratch keeps the previous call's contents
        out.fill_(0.0)
        torch.cuda.synchronize()
        st = _dot_noalloc(lib, pa, pb, lat.ndof, 1, out.data_ptr(), stream)
        assert st == 0
        ctx.synchronize()
        got = complex(*out.cpu().tolist())
        assert abs(got - want) / abs(want) < 1e-13


def test_dot_noalloc_several_vectors_and_limit(smg_gpu):
    import torch

    smg = smg_gpu
    lib = smg.lib()
    rng = np.random.default_rng(3)
    nrhs, n = 5, 10007
    a = rng.standard_normal((nrhs, n)) + 1j * rng.standard_normal((nrhs, n))
    b = rng.standard_normal((nrhs, n)) + 1j * rng.standard_normal((nrhs, n))
    ta = torch.from_numpy(a.view(np.float64).copy()).cuda()
    tb = torch.from_numpy(b.view(np.float64).copy()).cuda()
    out = torch.zeros(2 * nrhs, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    assert _dot_noalloc(lib, ta.data_ptr(), tb.data_ptr(), n, nrhs, out.data_ptr(), None) == 0
    torch.cuda.synchronize()
    got = out.cpu().numpy().view(np.complex128)
    np.testing.assert_allclose(got, np.einsum("ij,ij->i", a.conj(), b), rtol=1e-13)
    # beyond the scratch: rejected, nothing launched
    assert _dot_noalloc(lib, ta.data_ptr(), tb.data_ptr(), n, 17, out.data_ptr(), None) == 4
