"""Shared fixtures.  GPU tests are marked `gpu`; everything else runs on CPU."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def port():
    from oracle import oracle as O

    O.build(ref=False) if not O.PORT_SO.exists() else None
    return O.port()


@pytest.fixture(scope="session")
def ref():
    from oracle import oracle as O

    r = O.ref()
    if r is None:
        pytest.skip("reference shim not built (reference tree absent)")
    return r


def golden(name: str) -> dict:
    with np.load(GOLDEN / f"{name}.npz") as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def smg_gpu():
    """The product package with a live GPU context; fails loudly if the CUDA library is missing."""
    import schwinger_mg_gb300 as smg

    smg.lib()  # raises SmgLibraryError when libsmg_gpu.so is absent
    smg.Context.default()
    return smg


def rel_err_per_site(got: np.ndarray, want: np.ndarray) -> float:
    """max over sites of |got(s) - want(s)| / |want(s)| with |.| the 2-spinor norm."""
    g = got.reshape(-1, 2)
    w = want.reshape(-1, 2)
    num = np.linalg.norm(g - w, axis=1)
    den = np.linalg.norm(w, axis=1)
    return float(np.max(num / den))
