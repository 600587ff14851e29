"""Neighbour, even-odd and aggregate index maps, bit-exact against the
reference's definitions (src/lattice.h:4-42, src/prolongator.h:35-58) —
including the device site index q = parity * V/2 + s // 2 that the CUDA
kernels use (csrc/smg_internal.h site_q/site_coords)."""
from __future__ import annotations

import numpy as np
import pytest


def ref_lattice_maps(L):
    """Literal restatement of Lattice (src/lattice.h:15-41)."""
    V = L * L
    idx = lambda x, y: ((x % L + L) % L) + L * ((y % L + L) % L)
    even, odd, eo = [], [], [0] * V
    for s in range(V):
        if ((s % L) + (s // L)) % 2 == 0:
            eo[s] = len(even)
            even.append(s)
        else:
            eo[s] = len(odd)
            odd.append(s)
    nb = {
        "xp": [idx(s % L + 1, s // L) for s in range(V)],
        "xm": [idx(s % L - 1, s // L) for s in range(V)],
        "yp": [idx(s % L, s // L + 1) for s in range(V)],
        "ym": [idx(s % L, s // L - 1) for s in range(V)],
    }
    return np.array(even), np.array(odd), np.array(eo), {k: np.array(v) for k, v in nb.items()}


def device_site_q(L, s):
    """Python restatement of csrc/smg_internal.h site_q."""
    x, y = s % L, s // L
    parity = (x + y) & 1
    return parity * (L * L // 2) + ((x + L * y) >> 1)


def device_site_coords(L, q):
    Vh, Lh = L * L // 2, L // 2
    parity = (q >= Vh).astype(int)
    cb = q - parity * Vh
    y = cb // Lh
    x = 2 * (cb - y * Lh) + ((y + parity) & 1)
    return x, y, parity


@pytest.mark.parametrize("L", [4, 6, 8, 16, 96])
def test_lattice_maps_bit_exact(L):
    from schwinger_mg_gb300 import Lattice

    lat = Lattice(L)
    even, odd, eo, nb = ref_lattice_maps(L)
    np.testing.assert_array_equal(lat.even_sites, even)
    np.testing.assert_array_equal(lat.odd_sites, odd)
    np.testing.assert_array_equal(lat.eo_index, eo)
    s = np.arange(L * L)
    for k in ("xp", "xm", "yp", "ym"):
        np.testing.assert_array_equal(getattr(lat, k)(s), nb[k])


@pytest.mark.parametrize("L", [4, 8, 32, 96, 384, 512])
def test_device_site_index_is_eo_index(L):
    even, odd, eo, _ = ref_lattice_maps(L) if L <= 96 else (None, None, None, None)
    s = np.arange(L * L)
    q = device_site_q(L, s)
    par = ((s % L) + (s // L)) % 2
    # q within a parity equals the reference's eo_index
    if eo is not None:
        np.testing.assert_array_equal(q - par * (L * L // 2), eo)
    # q is a bijection and site_coords inverts it
    assert np.array_equal(np.sort(q), s)
    x, y, p = device_site_coords(L, q)
    np.testing.assert_array_equal(x, s % L)
    np.testing.assert_array_equal(y, s // L)
    np.testing.assert_array_equal(p, par)


@pytest.mark.parametrize("L,bs", [(16, 4), (32, 4), (24, 2)])
def test_block_maps_bit_exact(L, bs):
    """site_to_block / site_to_local of the geometric Prolongator (prolongator.h:50-57)."""
    s = np.arange(L * L)
    x, y = s % L, s // L
    nbx = L // bs
    blk = (x // bs) + nbx * (y // bs)
    loc = (x % bs) + bs * (y % bs)
    # each block holds bs*bs sites, each local index once
    counts = np.bincount(blk, minlength=nbx * nbx)
    assert np.all(counts == bs * bs)
    for b in (0, nbx * nbx - 1):
        assert sorted(loc[blk == b].tolist()) == list(range(bs * bs))
