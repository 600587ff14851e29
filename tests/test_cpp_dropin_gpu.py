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


# The reference's own calling code (the style of src/mode_studies.cpp and src/multigrid.cpp) with only the
# include and the namespace changed: OpApply from as_DdagD_op, build_full_mg(D, mcfg, scfg, rng),
# fcg_solve_mg / cg_solve / fgmres_solve_mg on the OpApply, Prolongator + SparseCoarseOp as
# setup_sparse_coarse builds them, EvenOddDiracOp.
REFERENCE_STYLE = r'''
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>
#include "smg_gpu.hpp"      // was: lattice.h gauge.h dirac.h mg_builder.h solvers.h prolongator.h coarse_op.h
using namespace smg;         // the reference's types live in the global namespace

static double rel_res(const OpApply& A, const Vec& b, const Vec& x) {
    Vec Ax(b.size());
    A(x, Ax);
    double r = 0, n = 0;
    for (size_t i = 0; i < b.size(); ++i) { r += std::norm(b[i] - Ax[i]); n += std::norm(b[i]); }
    return std::sqrt(r / n);
}

int main(int argc, char** argv) {
    const int L = 32;
    Lattice lat(L);
    GaugeField gauge(lat);
    std::mt19937 grng(2024);
    std::normal_distribution<double> theta(0.0, std::sqrt(1.0 / 6.0));
    for (int mu = 0; mu < 2; ++mu)
        for (int s = 0; s < lat.V; ++s) gauge.U[mu][s] = std::polar(1.0, theta(grng));
    DiracOp D(lat, gauge, -0.05, 1.0, 1.0);
    OpApply A = D.as_DdagD_op();

    MGConfig mcfg;
    mcfg.mg_levels = 2;
    mcfg.k_null = 8;
    SolverConfig scfg;
    std::mt19937 rng(42);
    MGHierarchy mg = build_full_mg(D, mcfg, scfg, rng);
    Vec b = random_vec(lat.ndof, rng);

    FCGResult r = fcg_solve_mg(A, lat.ndof, b, mg, 500, 1e-10);
    std::printf("gcr %d %.3e\n", r.iterations, rel_res(A, b, r.solution));
    CGResult c = cg_solve(A, lat.ndof, b, 5000, 1e-10);
    std::printf("cg %d %.3e\n", c.iterations, rel_res(A, b, c.solution));
    FGMRESResult f = fgmres_solve_mg(A, lat.ndof, b, mg, 30, 500, 1e-10);
    std::printf("fgmres %d %.3e %zu\n", f.iterations, rel_res(A, b, f.solution), f.ritz_pairs.size());
    auto precond = mg.as_precond();
    FCGResult r2 = fcg_solve(A, lat.ndof, b, precond, 500, 1e-10, 20);
    std::printf("fcg %d %.3e\n", r2.iterations, rel_res(A, b, r2.solution));

    // a host lambda is not a device operator: the device solvers refuse it
    OpApply host = [&D](const Vec& s, Vec& d) { D.apply_DdagD(s, d); };
    int refused = 0;
    try { cg_solve(host, lat.ndof, b, 10, 1e-10); } catch (const Error& e) { refused = e.status == SMG_UNSUPPORTED; }
    std::printf("refused %d\n", refused);

    // setup_sparse_coarse's pieces: Prolongator from the null vectors, SparseCoarseOp by Galerkin
    std::vector<Vec> nv = mg.null_vectors();
    Prolongator P(lat, 4, 4, mcfg.k_null);
    P.build_from_vectors(nv);
    SparseCoarseOp Ac;
    Ac.build(P, A, lat.ndof);
    Vec xc = random_vec(Ac.dim, rng);
    Vec y1, Ap(lat.ndof);
    Ac.apply_to(xc, y1);
    A(P.prolong(xc), Ap);
    Vec y2 = P.restrict_vec(Ap);
    double e = 0, n = 0;
    for (int i = 0; i < Ac.dim; ++i) { e += std::norm(y1[i] - y2[i]); n += std::norm(y2[i]); }
    Vec back = P.restrict_vec(P.prolong(xc));
    double pe = 0;
    for (int i = 0; i < Ac.dim; ++i) pe = std::max(pe, std::abs(back[i] - xc[i]));
    Vec bc = P.restrict_vec(b);
    Vec xs = Ac.solve(bc, 2000, 1e-12);
    Vec ys;
    Ac.apply_to(xs, ys);
    double sr = 0, sn = 0;
    for (int i = 0; i < Ac.dim; ++i) { sr += std::norm(ys[i] - bc[i]); sn += std::norm(bc[i]); }
    std::printf("coarse %d %.3e %.3e %.3e\n", Ac.dim, std::sqrt(e / n), pe, std::sqrt(sr / sn));

    // EvenOddDiracOp: D applied to (x_e, x_o) with x_e = -D_ee^-1 D_oe x_o is (0, M x_o)
    EvenOddDiracOp eo(D);
    Vec xo(2 * (size_t)lat.V_half);
    for (auto& v : xo) v = cx(theta(grng), theta(grng));
    Vec full = eo.reconstruct_full(xo), Dfull(lat.ndof), Mx;
    D.apply(full, Dfull);
    eo.apply_schur(xo, Mx);
    Vec De = eo.gather_even(Dfull), Do = eo.gather_odd(Dfull);
    double ee = 0, eo_ = 0, mn = 0;
    for (size_t i = 0; i < Mx.size(); ++i) { ee += std::norm(De[i]); eo_ += std::norm(Do[i] - Mx[i]); mn += std::norm(Mx[i]); }
    std::printf("eo %.3e %.3e %.6e\n", std::sqrt(ee / mn), std::sqrt(eo_ / mn), eo.log_det_ee());

    if (argc > 1) {  // the hierarchy's null vectors for the caller to compare
        FILE* fp = std::fopen(argv[1], "wb");
        for (const Vec& v : nv) std::fwrite(v.data(), sizeof(cx), v.size(), fp);
        std::fclose(fp);
    }
    return 0;
}
'''


def test_reference_style_program_runs(smg_gpu, tmp_path):
    """The reference's calling code with only the include and namespace changed compiles, solves on the
    GPU, refuses host callbacks, and build_full_mg with the caller's std::mt19937(42) gives the hierarchy
    the library builds from seed 42 (the same draws)."""
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    import numpy as np

    lib_dir = ROOT / "schwinger_mg_gb300"
    src = tmp_path / "refstyle.cpp"
    src.write_text(REFERENCE_STYLE)
    exe = tmp_path / "refstyle"
    r = subprocess.run([gxx, "-std=c++17", "-O1", "-I", str(ROOT / "include"), str(src), "-L", str(lib_dir),
                        "-lsmg_gpu", f"-Wl,-rpath,{lib_dir}", "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    nvf = tmp_path / "nv.bin"
    run = subprocess.run([str(exe), str(nvf)], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout + run.stderr
    out = {line.split()[0]: line.split()[1:] for line in run.stdout.splitlines()}
    for key in ("gcr", "cg", "fgmres", "fcg"):
        assert float(out[key][1]) < 1e-9, (key, out[key])
    assert out["gcr"] == out["fcg"]  # fcg_solve with as_precond is fcg_solve_mg
    assert int(out["refused"][0]) == 1
    dim, gal, pp, sol = out["coarse"]
    assert int(dim) == 8 * 8 * 8 and float(gal) < 1e-12 and float(pp) < 1e-12 and float(sol) < 1e-10
    e_even, e_odd, _ = map(float, out["eo"])
    assert e_even < 1e-13 and e_odd < 1e-13
    # the same hierarchy from the library's own draws with seed 42 on the same links (theta ~ N(0, 1/6)
    # from std::mt19937(2024), mu-major)
    L = 32
    nv = np.fromfile(nvf, dtype=np.complex128).reshape(8, -1)
    lat = smg_gpu.Lattice(L)
    D = smg_gpu.DiracOp(lat, smg_gpu.GaugeField(lat, smg_gpu.gauge_normal(L, 6.0, 2024)), -0.05, 1.0, 1.0, 0.0)
    mg = smg_gpu.MGHierarchy(D, smg_gpu.mg_params(2, 4, 8, null_iters=20, seed=42))
    ref = mg.null_vecs_l0
    assert np.max(np.abs(nv - ref)) < 1e-8 * np.max(np.abs(ref))
