"""The C ABI library loads on a machine without a GPU and exports every symbol
include/smg_gpu.h declares; host-only entry points work; device entry points
fail with a status instead of crashing when no GPU is present."""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols() -> set[str]:
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        for m in re.finditer(r"SMG_API\s+[\w\s\*]+?\b(smg_\w+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "smg_dirac_apply" in names and "smg_cg_solve" in names and "smg_fermion_force" in names
    assert len(names) >= 40


def test_library_exports_every_declared_symbol():
    from schwinger_mg_gb300 import _lib

    lib = _lib.lib()
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_python_binding_covers_header():
    from schwinger_mg_gb300 import _lib

    assert declared_symbols() == set(_lib.exported_symbols())


def test_version_and_status_strings():
    from schwinger_mg_gb300 import _lib

    lib = _lib.lib()
    assert b"sm_103a" in lib.smg_version()
    assert lib.smg_status_string(_lib.BAD_ARG) == b"bad argument"


def test_host_generators_reject_bad_arguments():
    from schwinger_mg_gb300 import _lib

    lib = _lib.lib()
    buf = np.empty(8)
    p = buf.ctypes.data_as(C.POINTER(C.c_double))
    assert lib.smg_host_gauge_normal(1, 2.0, 0, p) == _lib.BAD_ARG
    assert lib.smg_host_gauge_normal(4, -1.0, 0, p) == _lib.BAD_ARG
    assert lib.smg_host_random_vec(-1, 0, p) == _lib.BAD_ARG


def test_null_handles_are_bad_arguments():
    from schwinger_mg_gb300 import _lib

    lib = _lib.lib()
    assert lib.smg_dirac_apply(None, 0, None, None) == _lib.BAD_ARG
    assert lib.smg_cg_solve(None, None, None, 10, 1e-10, None) == _lib.BAD_ARG
    assert lib.smg_field_upload(None, None) == _lib.BAD_ARG


def test_context_without_gpu_reports_device_error():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from schwinger_mg_gb300 import _lib

    h = C.c_void_p()
    st = _lib.lib().smg_context_create(0, None, C.byref(h))
    assert st == _lib.DEVICE_ERROR


def test_cpp_dropin_header_compiles(tmp_path):
    """include/smg_gpu.hpp (the reference's C++ call shapes over the C ABI) compiles as C++17."""
    import shutil
    import subprocess

    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    src = tmp_path / "use.cpp"
    src.write_text(
        '#include "smg_gpu.hpp"\n'
        "double use(const smg::DiracOp& D, smg::MGHierarchy& mg, const smg::Vec& b) {\n"
        "    smg::Vec x(b.size());\n"
        "    smg::mr_smooth(D, x, b, 4);\n"
        "    smg::richardson_smooth(D, x, b, 4, 0.8 / smg::estimate_lambda_max(D, 30));\n"
        "    mg.set_symmetric(0.8);\n"
        "    auto c = smg::cg_solve_precond(D, D.lat.ndof, b, mg, 100, 1e-10);\n"
        "    auto f = smg::fgmres_solve_mg(D, D.lat.ndof, b, &mg, 30, 300, 1e-10);\n"
        "    smg::PseudofermionAction act(D, &mg);\n"
        "    double S = act.forward(b, 1000, 1e-10);\n"
        "    std::array<smg::RVec, 2> F;\n"
        "    act.backward(F);\n"
        "    return S + c.final_residual + f.final_residual + F[0][0];\n"
        "}\n"
        "double use_hmc(smg::GaugeField& g, smg::DiracOp& D, smg::MGHierarchy& mg, const smg::Vec& phi) {\n"
        "    smg_hmc_params hp; smg_hmc_params_default(&hp);\n"
        "    smg_ms_params mp; smg_ms_params_default(&mp);\n"
        "    smg::Rng rng(1);\n"
        "    auto t = smg::hmc_trajectory(g, 0.1, 1.0, hp, rng);\n"
        "    auto r = smg::reversibility_test_plain(g, 0.1, 1.0, hp, rng);\n"
        "    D.refresh(); mg.rebuild(); mg.setup_deflation(4); double rr = mg.deflation_rr();\n"
        "    smg::Vec low = mg.lowmode_solution(phi);\n"
        "    std::array<smg::RVec, 2> F; smg::coarse_lowmode_force(D, mg, phi, F, 3);\n"
        "    auto m = smg::hmc_trajectory_mg_multiscale(g, 0.1, 1.0, mp, mg, rng);\n"
        "    auto mr = smg::reversibility_test_mg_multiscale(g, 0.1, 1.0, mp, mg, rng);\n"
        "    bool ok = smg::verify_forces(g, 4.0, 0.1, 1.0, 1000, 1e-12, 1.0, true);\n"
        "    return t.dH + r.dH_forward + rr + low[0].real() + F[0][0] + m.dH + mr.dH_forward + (ok ? 1 : 0);\n"
        "}\n")
    r = subprocess.run([gxx, "-std=c++17", "-fsyntax-only", "-I", str(ROOT / "include"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
