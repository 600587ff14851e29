"""GPU parity of the Wilson-clover Dirac operator against the reference
(golden fixtures) and the oracle, through the C ABI."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden, rel_err_per_site

pytestmark = pytest.mark.gpu

OPS = ["D", "Ddag", "DdagD", "g5D"]
# FP64: per-site relative error bound demanded of the FP64 dslash
TOL_F64_SITE = 1e-14
# FP32 storage and arithmetic: relative to the field norm
TOL_F32 = 2e-6


def _make(smg, d):
    L = int(d["L"])
    lat = smg.Lattice(L)
    g = smg.GaugeField(lat, d["U"])
    D = smg.DiracOp(lat, g, float(d["m"]), float(d["r"]), float(d["csw"]), float(d["mu"]))
    return lat, g, D


@pytest.mark.parametrize("name", ["dirac_L8_wilson", "dirac_L16_clover_twist", "dirac_L32_config1"])
def test_f64_ops_match_reference_per_site(smg_gpu, name):
    d = golden(name)
    lat, g, D = _make(smg_gpu, d)
    for op, key in enumerate(OPS):
        got = D.apply_op(op, d["src"])
        err = rel_err_per_site(got, d[key])
        assert err < TOL_F64_SITE, f"{name} {key}: per-site rel err {err:.3e}"


@pytest.mark.parametrize("name", ["dirac_L16_clover_twist", "dirac_L32_config1"])
def test_clover_and_plaquette_match_reference(smg_gpu, name):
    d = golden(name)
    lat, g, D = _make(smg_gpu, d)
    np.testing.assert_allclose(D.clover_field, d["clover"], rtol=0, atol=1e-15)
    assert g.avg_plaq() == pytest.approx(float(d["avg_plaq"]), rel=1e-14)
    np.testing.assert_array_equal(g.U.reshape(-1), d["U"])


@pytest.mark.parametrize("L,m,csw,mu", [(64, -0.05, 1.0, 0.0), (128, 0.1, 1.0, 0.15), (96, 0.2, 0.0, 0.0)])
def test_f64_ops_match_oracle_larger(smg_gpu, port, L, m, csw, mu):
    U = smg_gpu.gauge_normal(L, 6.0, 7 * L)
    src = smg_gpu.random_vec(2 * L * L, L)
    lat = smg_gpu.Lattice(L)
    D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat, U), m, 1.0, csw, mu)
    for op in range(4):
        got = D.apply_op(op, src)
        want = port.dirac(U, m, 1.0, csw, mu, op, src)
        assert rel_err_per_site(got, want) < TOL_F64_SITE


def test_f32_ops_match_reference(smg_gpu):
    d = golden("dirac_L32_config1")
    lat, g, D = _make(smg_gpu, d)
    src = smg_gpu.Field(lat, 1, "f32", data=d["src"])
    for op, key in enumerate(OPS):
        got = D.apply_op(op, src).download()
        err = np.linalg.norm(got - d[key]) / np.linalg.norm(d[key])
        assert err < TOL_F32, f"{key}: {err:.3e}"


@pytest.mark.parametrize("nrhs,prec", [(3, "f64"), (8, "f64"), (32, "f32"), (12, "f32")])
def test_multi_rhs_equals_single_rhs(smg_gpu, nrhs, prec):
    L = 32
    U = smg_gpu.gauge_normal(L, 2.0, 5)
    lat = smg_gpu.Lattice(L)
    D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat, U), 0.05, 1.0, 1.0, 0.1)
    srcs = np.stack([smg_gpu.random_vec(lat.ndof, 100 + j) for j in range(nrhs)])
    multi = D.apply_op(2, smg_gpu.Field(lat, nrhs, prec, data=srcs)).download()
    tol = 1e-15 if prec == "f64" else 1e-7  # the launch shape (row kernel or tile) may differ with nrhs
    for j in (0, nrhs // 2, nrhs - 1):
        single = D.apply_op(2, smg_gpu.Field(lat, 1, prec, data=srcs[j])).download()
        assert rel_err_per_site(multi[j], single) < tol


def test_gamma5_hermiticity_full_size(smg_gpu):
    """<a, D b> = <D^dag a, b> on the 512 x 512 lattice (size-independent property)."""
    L = 512
    U = smg_gpu.gauge_normal(L, 6.0, 3)
    lat = smg_gpu.Lattice(L)
    D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat, U), -0.05, 1.0, 1.0, 0.0)
    a = smg_gpu.Field(lat, 1, "f64", data=smg_gpu.random_vec(lat.ndof, 1))
    b = smg_gpu.Field(lat, 1, "f64", data=smg_gpu.random_vec(lat.ndof, 2))
    Db = D.apply(b)
    Dda = D.apply_dag(a)
    lhs = smg_gpu.dot(a, Db)[0]
    rhs = smg_gpu.dot(Dda, b)[0]
    assert abs(lhs - rhs) / abs(lhs) < 1e-12
    # linearity: D(a + 2b) = D a + 2 D b
    ab = smg_gpu.Field(lat, 1, "f64", data=a.download() + 2 * b.download())
    lin = D.apply(ab).download() - D.apply(a).download() - 2 * Db.download()
    assert np.linalg.norm(lin) / np.linalg.norm(Db.download()) < 1e-13


def test_bad_arguments_raise(smg_gpu):
    lat = smg_gpu.Lattice(8)
    D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat), 0.1)
    a = smg_gpu.Field(lat, 1, "f64")
    b = smg_gpu.Field(lat, 2, "f64")
    with pytest.raises(smg_gpu.SmgError) as e:
        D.apply(a, b)
    assert e.value.status == 4
    with pytest.raises(smg_gpu.SmgError):
        D.apply(a, a)
    with pytest.raises(smg_gpu.SmgError):
        smg_gpu.Field(smg_gpu.Lattice(7), 1, "f64")


@pytest.mark.parametrize("variant", [0, 1, 2, 3, 4, 5, 6, 7])
@pytest.mark.parametrize("nrhs,prec", [(8, "f32"), (32, "f32"), (4, "f64"), (16, "f64")])
def test_stencil_launch_variants_agree(smg_gpu, port, monkeypatch, variant, nrhs, prec):
    """Every launch shape the stencil autotuner can pick (row kernel, shared-memory tiles of 2, 4, 8
    rows) gives the reference operator on every right-hand side; a fresh context plans afresh."""
    monkeypatch.setenv("SMG_DSLASH_VARIANT", str(variant))
    ctx = smg_gpu.Context(0)
    L, m, csw, mu = 48, 0.05, 1.0, 0.1
    U = smg_gpu.gauge_normal(L, 3.0, 61)
    lat = smg_gpu.Lattice(L)
    D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat, U, ctx), m, 1.0, csw, mu)
    B = np.stack([smg_gpu.random_vec(lat.ndof, 90 + j) for j in range(nrhs)])
    src = smg_gpu.Field(lat, nrhs, prec, ctx, data=B)
    tol = 1e-14 if prec == "f64" else 3e-6
    for op, dag in ((0, False), (1, True)):
        out = D.apply_op(op, src).download().reshape(nrhs, -1)
        for j in (0, nrhs // 2, nrhs - 1):
            want = port.dirac(U, m, 1.0, csw, mu, op, B[j])
            assert rel_err_per_site(out[j], want) < tol, (variant, op, j)


def test_apply_delta_D_matches_reference(smg_gpu):
    d = golden("delta_L16")
    L = int(d["L"])
    lat = smg_gpu.Lattice(L)
    D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat, d["U"]), float(d["m"]), float(d["r"]), float(d["csw"]),
                        float(d["mu"]))
    got = D.apply_delta_D(d["src"], d["pi"], float(d["dt"]))
    assert rel_err_per_site(got, d["delta"]) < 1e-13


def test_apply_delta_D_is_the_operator_difference_without_clover(smg_gpu):
    """With c_sw = 0 only the hops depend on the links: D(U') v - D(U) v = apply_delta_D v."""
    L, dt = 24, 0.1
    U = smg_gpu.gauge_normal(L, 3.0, 71)
    pi = np.random.default_rng(72).standard_normal((2, L * L))
    lat = smg_gpu.Lattice(L)
    D0 = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat, U), 0.1, 1.0, 0.0, 0.2)
    D1 = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat, U * np.exp(1j * dt * pi)), 0.1, 1.0, 0.0, 0.2)
    v = smg_gpu.random_vec(lat.ndof, 73)
    want = D1.apply(v) - D0.apply(v)
    got = D0.apply_delta_D(v, pi, dt)
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-13
