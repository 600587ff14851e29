"""The coarse-deflation fixture (tests/golden/ms_L16.npz, produced by the reference's
setup_sparse_coarse with TRLM) holds what it claims, checked with the oracle's C
restatement on the CPU: the stored pairs are the lowest eigenpairs of the level-1
operator P^dag D^dag D P built from the stored null vectors, and the stored low-mode
solution is P sum_i v_i v_i^dag / lambda_i P^dag phi."""
from __future__ import annotations

import numpy as np

from conftest import golden


def _coarse(port, d):
    L, bs, k = int(d["L"]), int(d["bs"]), int(d["k"])
    bv = port.prolongator_build(L, bs, k, d["null_vecs"])
    links = port.sparse_coarse_build(d["U"], float(d["m"]), float(d["r"]), float(d["csw"]), 0.0, bs, k, bv)
    nbx = L // bs
    return L, bs, k, nbx, bv, links


def test_deflation_pairs_are_the_lowest_eigenpairs(port):
    d = golden("ms_L16")
    L, bs, k, nbx, bv, links = _coarse(port, d)
    dim = nbx * nbx * k
    vals, vecs = d["defl_vals"], d["defl_vecs"]
    for v, lam in zip(vecs, vals):
        Av = port.sparse_coarse_apply(nbx, nbx, k, links, v)
        assert np.linalg.norm(Av - lam * v) < 1e-8 * lam
    A = np.stack([port.sparse_coarse_apply(nbx, nbx, k, links, e) for e in np.eye(dim, dtype=np.complex128)], axis=1)
    assert np.max(np.abs(A - A.conj().T)) < 1e-12 * np.max(np.abs(A))
    exact = np.linalg.eigvalsh(A)[: len(vals)]
    assert np.max(np.abs(exact - vals) / exact) < 1e-9


def test_lowmode_fixture_is_the_deflated_projection(port):
    d = golden("ms_L16")
    L, bs, k, nbx, bv, links = _coarse(port, d)
    c = port.restrict(L, bs, k, bv, d["phi"])
    xc = sum((np.vdot(v, c) / lam) * v for v, lam in zip(d["defl_vecs"], d["defl_vals"]))
    low = port.prolong(L, bs, k, bv, xc)
    assert np.linalg.norm(low - d["lowmode"]) / np.linalg.norm(d["lowmode"]) < 1e-12


def test_reversibility_fixtures_are_reversible():
    """The reference's own reversibility results: dH_fwd = -dH_bwd, links and momenta back to rounding."""
    for name, keys in (("reversibility_L8_omelyan", ["result"]), ("ms_L16", ["rev_0", "rev_1", "rev_2"])):
        d = golden(name)
        for key in keys:
            gd, md, dHf, dHb, _ = d[key]
            assert gd < 1e-12 and md < 1e-12
            assert abs(dHf + dHb) < 1e-9 * max(1.0, abs(dHf))
