"""The C++ drop-in header (include/smg_gpu.hpp) used the way the reference's own drivers call
its API: a small program compiled with g++ against libsmg_gpu.so runs D, CG, build_full_mg,
coarse deflation, an HMC trajectory, the multiscale trajectory and both reversibility tests on
the GPU and prints what the test checks."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]

PROGRAM = r'''
#include <cmath>
#include <cstdio>
#include <vector>
#include "smg_gpu.hpp"

int main() {
    const int L = 16;
    smg::Lattice lat(L);
    smg::GaugeField g(lat);
    std::vector<double> U(4 * (size_t)lat.V);
    if (smg_host_gauge_normal(L, 4.0, 7, U.data()) != SMG_OK) return 2;
    for (int mu = 0; mu < 2; ++mu)
        for (int s = 0; s < lat.V; ++s)
            g.U[mu][s] = smg::cx(U[2 * ((size_t)mu * lat.V + s)], U[2 * ((size_t)mu * lat.V + s) + 1]);
    g.sync();
    smg::DiracOp D(lat, g, 0.1, 1.0, 1.0);
    std::vector<double> bh(2 * (size_t)lat.ndof);
    if (smg_host_random_vec(lat.ndof, 11, bh.data()) != SMG_OK) return 3;
    smg::Vec b(lat.ndof);
    for (int i = 0; i < lat.ndof; ++i) b[i] = smg::cx(bh[2 * i], bh[2 * i + 1]);
    auto cg = smg::cg_solve(D, lat.ndof, b, 1000, 1e-10);
    smg::Vec Ax;
    D.apply_DdagD(cg.solution, Ax);
    double rn = 0, bn = 0;
    for (int i = 0; i < lat.ndof; ++i) { rn += std::norm(b[i] - Ax[i]); bn += std::norm(b[i]); }
    std::printf("cg %d %.3e\n", cg.iterations, std::sqrt(rn / bn));
    smg::MGConfig mc;
    auto mg = smg::build_full_mg(D, mc, 5);
    auto info = mg->setup_deflation(4);
    std::vector<double> vals;
    std::vector<smg::Vec> vecs;
    mg->deflation(vals, vecs);
    std::printf("defl %d %zu %.6e\n", info.converged, vals.size(), vals.empty() ? 0.0 : vals[0]);
    auto fg = smg::fcg_solve_mg(D, lat.ndof, b, *mg, 200, 1e-10);
    std::printf("gcr %d %.3e\n", fg.iterations, fg.final_residual);
    smg_hmc_params hp;
    smg_hmc_params_default(&hp);
    hp.c_sw = 1.0;
    hp.tau = 0.5;
    hp.n_steps = 5;
    hp.cg_tol = 1e-12;
    smg::Rng rng(21);
    auto rev = smg::reversibility_test_plain(g, 0.1, 1.0, hp, rng);
    std::printf("rev %.3e %.3e %.6e %.6e\n", rev.gauge_delta, rev.mom_delta, rev.dH_forward, rev.dH_backward);
    const double plaq0 = g.avg_plaq();
    auto tr = smg::hmc_trajectory(g, 0.1, 1.0, hp, rng);
    double hp_plaq = 0;
    for (int mu = 0; mu < 1; ++mu)
        for (int s = 0; s < lat.V; ++s) hp_plaq += std::abs(g.U[mu][s]);
    std::printf("hmc %d %.6e %.6f %.6f %.6f\n", tr.accepted, tr.dH, plaq0, tr.plaquette, hp_plaq / lat.V);
    D.refresh();
    mg->rebuild();
    mg->deflation_rr();
    smg_ms_params mp;
    smg_ms_params_default(&mp);
    mp.beta = 4.0;
    mp.tau = 0.2;
    mp.n_outer = 2;
    mp.n_inner = 2;
    mp.c_sw = 1.0;
    mp.cg_tol = 1e-12;
    auto ms = smg::hmc_trajectory_mg_multiscale(g, 0.1, 1.0, mp, *mg, rng);
    std::printf("ms %d %.6e %d\n", ms.accepted, ms.dH, ms.lowmode_force_evals);
    auto mrev = smg::reversibility_test_mg_multiscale(g, 0.1, 1.0, mp, *mg, rng);
    std::printf("msrev %.3e %.3e %.6e %.6e\n", mrev.gauge_delta, mrev.mom_delta, mrev.dH_forward, mrev.dH_backward);
    return 0;
}
'''


def test_cpp_dropin_program_runs(smg_gpu, tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    lib_dir = ROOT / "schwinger_mg_gb300"
    src = tmp_path / "dropin.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "dropin"
    r = subprocess.run([gxx, "-std=c++17", "-O1", "-I", str(ROOT / "include"), str(src), "-L", str(lib_dir),
                        "-lsmg_gpu", f"-Wl,-rpath,{lib_dir}", "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout + run.stderr
    out = {line.split()[0]: line.split()[1:] for line in run.stdout.splitlines()}
    assert float(out["cg"][1]) < 1e-9
    assert int(out["defl"][0]) == 1 and int(out["defl"][1]) == 4 and float(out["defl"][2]) > 0
    assert float(out["gcr"][1]) < 1e-10
    gd, md, f, bwd = map(float, out["rev"])
    assert gd < 1e-10 and md < 1e-9 and abs(f + bwd) < 1e-7 * max(1.0, abs(f))
    assert abs(float(out["hmc"][4]) - 1.0) < 1e-12  # host links pulled back: unit modulus
    assert int(out["ms"][2]) > 0
    gd, md, f, bwd = map(float, out["msrev"])
    assert gd < 1e-10 and md < 1e-9 and abs(f + bwd) < 1e-7 * max(1.0, abs(f))
