"""Pins the oracle's own inputs and CPU hierarchy set-up (oracle/inputs.cpp,
orc_mgN_setup) to the reference: the seeded generators, the two-level build
(golden mg_L16_bs4_k4) and the three-level build with the reference's default
coarse blocking — CoarseProlongator over 4k consecutive coarse dofs and the
dense intermediate operator (golden mg3_L48_k4).  CPU only.  These are what
the benchmark's reference arm runs, so it needs no GPU and no product code."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def test_inputs_match_reference_generators(port, ref):
    # random_vec (src/linalg.cpp:44-48): k vectors from one std::mt19937
    v = ref.random_vecs(1, 1000, 77)
    np.testing.assert_array_equal(port.random_vec(1000, 77), v.reshape(-1))


def test_inputs_match_golden_links(port):
    d = golden("mg_L16_bs4_k4")
    U = port.gauge_normal(int(d["L"]), float(d["beta"]), int(d["gseed"]))
    np.testing.assert_array_equal(U.reshape(-1), d["U"])


def test_two_level_setup_matches_reference(port):
    d = golden("mg_L16_bs4_k4")
    L, bs, k = int(d["L"]), int(d["bs"]), int(d["k"])
    bvs, links, null0 = port.mgN_setup(L, d["U"], float(d["m"]), float(d["r"]), float(d["csw"]), float(d["mu"]),
                                       [(bs, bs)], [k], int(d["null_iters"]), int(d["seed"]))
    assert _rel(null0.reshape(-1), d["null_vecs"].reshape(-1)) < 1e-13
    assert _rel(bvs[0], d["block_vecs"]) < 1e-13
    # direct Galerkin product against the reference's probing build (src/coarse_op.h:241-279)
    assert _rel(links[1], d["links"]) < 1e-13


def test_three_level_setup_matches_reference_blocking(port):
    """The reference's level-2 blocking of 4k consecutive level-1 dofs is the 4 x 1 aggregate."""
    d = golden("mg3_L48_k4")
    L, bs, k = int(d["L"]), int(d["bs"]), int(d["k"])
    args = (float(d["m"]), float(d["r"]), float(d["csw"]), float(d["mu"]))
    bvs, links, null0 = port.mgN_setup(L, d["U"], *args, [(bs, bs), (4, 1)], [k, k], int(d["null_iters"]),
                                       int(d["seed"]))
    assert _rel(null0.reshape(-1), d["null_vecs"].reshape(-1)) < 1e-12
    assert _rel(bvs[1], d["block_vecs1"]) < 1e-11
    assert _rel(links[2], d["links2"]) < 1e-11
    # W-cycle with the coarsest level solved to 1e-14 against the reference's dense LU
    p = port.mgN_params(L, *args, [(bs, bs), (4, 1)], [k, k], bvs, links, 3, 3, True, 5000, 1e-14)
    out = port.mgN_precondition(p, d["U"], d["fine_src"])
    assert np.linalg.norm(out - d["mg_precondition"]) / np.linalg.norm(d["mg_precondition"]) < 1e-10


def test_chiral_split_setup_matches_probing(port):
    """Chirality-split block vectors (2k per aggregate) and the direct Galerkin operator against the
    probing build on the same block vectors; a third level on 2 x 2 aggregates against P^dag A_1 P."""
    L, k = 24, 4
    U = port.gauge_normal(L, 6.0, 5)
    args = (-0.05, 1.0, 1.0, 0.0)
    bvs, links, _ = port.mgN_setup(L, U, *args, [(4, 4), (2, 2)], [k, k], 3, 9, chiral_split=True)
    assert _rel(links[1], port.sparse_coarse_build(U, *args, 4, 2 * k, bvs[0])) < 1e-13
    # level 2: dense P^dag A_1 P with the level-1 block vectors
    n1, nd1 = L // 4, 2 * k
    A1 = _dense(links[1], n1, n1, nd1)
    P = np.zeros((n1 * n1 * nd1, (n1 // 2) ** 2 * 2 * k), complex)
    bv = bvs[1].reshape((n1 // 2) ** 2, 2 * k, 4, nd1)
    for B in range((n1 // 2) ** 2):
        x0, y0 = (B % (n1 // 2)) * 2, (B // (n1 // 2)) * 2
        for loc in range(4):
            s = (x0 + loc % 2) + n1 * (y0 + loc // 2)
            P[s * nd1:(s + 1) * nd1, B * 2 * k:(B + 1) * 2 * k] = bv[B, :, loc, :].T
    assert _rel(_dense(links[2], n1 // 2, n1 // 2, 2 * k), P.conj().T @ A1 @ P) < 1e-13
    # chirality: the first k block vectors live on spin 0 only, the last k on spin 1 only
    b0 = bvs[0].reshape(-1, 2 * k, 16, 2)
    assert np.max(np.abs(b0[:, :k, :, 1])) == 0 and np.max(np.abs(b0[:, k:, :, 0])) == 0


def _dense(links, nx, ny, k):
    dx = [0, 1, -1, 0, 0, 1, 1, -1, -1]
    dy = [0, 0, 0, 1, -1, 1, -1, 1, -1]
    lk = links.reshape(nx * ny, 9, k, k)
    A = np.zeros((nx * ny * k, nx * ny * k), complex)
    for b in range(nx * ny):
        bx, by = b % nx, b // nx
        for d in range(9):
            nb = (bx + dx[d]) % nx + nx * ((by + dy[d]) % ny)
            A[b * k:(b + 1) * k, nb * k:(nb + 1) * k] += lk[b, d]
    return A


@pytest.mark.parametrize("trunc", [10])
def test_cpu_three_level_gcr_converges(port, trunc):
    """The reference arm's solve path end to end on the CPU: seeded inputs, set-up, N-level GCR."""
    L = 32
    U = port.gauge_normal(L, 6.0, 20240)
    args = (-0.05, 1.0, 1.0, 0.0)
    bvs, links, _ = port.mgN_setup(L, U, *args, [(4, 4), (2, 2)], [8, 8], 4, 20240)
    p = port.mgN_params(L, *args, [(4, 4), (2, 2)], [8, 8], bvs, links, 4, 4, False, 20, 5e-2)
    b = port.random_vec(2 * L * L, 20241)
    x, it, res, _ = port.mgN_gcr(p, U, b, 300, 1e-10, trunc)
    assert res < 1e-10 and it < 300
    Ax = port.dirac(U, *args, 2, x)
    assert np.linalg.norm(b - Ax) / np.linalg.norm(b) < 2e-10
