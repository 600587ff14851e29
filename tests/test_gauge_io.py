"""Gauge configuration files in the reference's "SWNG" and raw formats
(save_gauge / load_gauge, src/hmc_forces.cpp:18-62; GaugeField::save / load,
src/gauge.h:38-57).  The fixtures tests/golden/gauge_L8.{swng,raw} were written
by the reference itself (make_golden.py); the host entry points need no GPU."""
from __future__ import annotations

import struct

import numpy as np
import pytest

from conftest import GOLDEN

L, BETA, MASS, GSEED = 8, 3.0, 0.05, 81


def _links():
    from schwinger_mg_gb300.api import gauge_normal

    return gauge_normal(L, BETA, GSEED)


def test_read_reference_swng():
    import schwinger_mg_gb300 as smg

    U, hdr = smg.load_gauge(GOLDEN / "gauge_L8.swng", L)
    assert hdr["L"] == L and hdr["beta"] == BETA and hdr["mass"] == MASS
    want = _links()
    np.testing.assert_allclose(U, want / np.abs(want), rtol=0, atol=1e-15)
    raw = (GOLDEN / "gauge_L8.swng").read_bytes()
    magic, l, beta, mass, plaq = struct.unpack("<IIddd", raw[:32])
    assert magic == 0x53574E47 and l == L and hdr["avg_plaq"] == plaq


def test_write_is_byte_identical_to_reference(tmp_path):
    import schwinger_mg_gb300 as smg

    ref_bytes = (GOLDEN / "gauge_L8.swng").read_bytes()
    plaq = struct.unpack("<d", ref_bytes[24:32])[0]
    smg.save_gauge(_links(), BETA, MASS, tmp_path / "g.swng", avg_plaq=plaq)
    assert (tmp_path / "g.swng").read_bytes() == ref_bytes
    smg.save_gauge_raw(_links(), tmp_path / "g.raw")
    assert (tmp_path / "g.raw").read_bytes() == (GOLDEN / "gauge_L8.raw").read_bytes()
    np.testing.assert_array_equal(smg.load_gauge_raw(GOLDEN / "gauge_L8.raw", L), _links())


def test_load_normalises_and_checks(tmp_path):
    import schwinger_mg_gb300 as smg

    U = 1.5 * _links()
    smg.save_gauge(U, BETA, MASS, tmp_path / "s.swng")
    V, _ = smg.load_gauge(tmp_path / "s.swng")
    np.testing.assert_allclose(np.abs(V), 1.0, rtol=0, atol=1e-15)
    with pytest.raises(smg.SmgError):  # lattice size mismatch
        smg.load_gauge(tmp_path / "s.swng", 16)
    bad = bytearray((tmp_path / "s.swng").read_bytes())
    bad[0] ^= 0xFF
    (tmp_path / "bad.swng").write_bytes(bytes(bad))
    with pytest.raises(smg.SmgError):  # bad magic number
        smg.load_gauge(tmp_path / "bad.swng")
    (tmp_path / "short.swng").write_bytes(bytes(bad[:100]))
    with pytest.raises(smg.SmgError):
        smg.load_gauge(tmp_path / "missing.swng")
    with pytest.raises(smg.SmgError):  # V mismatch in the raw header
        smg.load_gauge_raw(GOLDEN / "gauge_L8.raw", 16)


def test_reference_reads_our_file(ref, tmp_path):
    import schwinger_mg_gb300 as smg

    smg.save_gauge(_links(), BETA, MASS, tmp_path / "o.swng", avg_plaq=0.5)
    U, hdr = ref.load_gauge(L, tmp_path / "o.swng")
    assert U is not None and list(hdr) == [BETA, MASS, 0.5]
    np.testing.assert_allclose(U.reshape(2, -1), _links(), rtol=0, atol=1e-15)


def test_reading_links_needs_the_callers_size():
    """The links are read only into a buffer whose lattice size the caller states: with L_expected <= 0
    the header alone is returned, and asking for the links as well is a bad argument."""
    import ctypes as C

    import schwinger_mg_gb300 as smg
    from schwinger_mg_gb300 import _lib

    lib = smg.lib()
    path = str(GOLDEN / "gauge_L8.swng").encode()
    hdr = _lib.GaugeHeader()
    assert lib.smg_host_gauge_read_swng(path, 0, C.byref(hdr), None) == 0 and hdr.L == L
    U = np.empty(4 * L * L)
    bad = lib.smg_host_gauge_read_swng(path, 0, C.byref(hdr), U.ctypes.data_as(C.POINTER(C.c_double)))
    assert bad == _lib.BAD_ARG
    assert lib.smg_host_gauge_read_swng(path, L, C.byref(hdr), U.ctypes.data_as(C.POINTER(C.c_double))) == 0
