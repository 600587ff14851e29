"""Generates the golden fixtures in tests/golden/ from the reference's own code.

Runs the reference C++ sources (compiled by oracle/Makefile into
oracle/_ref/libsmg_ref.so through oracle/ref_shim.cpp) on seeded inputs and
stores inputs and outputs as compressed .npz files.  The GPU machine has no copy of
the reference, so the GPU parity tests read these fixtures there.

    python tests/golden/make_golden.py

Inputs: gauge links from smg_host_gauge_normal (theta ~ N(0, 1/beta),
std::mt19937) and sources from the reference's random_vec with a stated seed.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle as O  # noqa: E402
from schwinger_mg_gb300.api import gauge_normal  # noqa: E402

OUT = Path(__file__).resolve().parent


def dirac_case(ref, name, L, beta, m, r, csw, mu, gseed, vseed):
    U = gauge_normal(L, beta, gseed).reshape(-1)
    n = 2 * L * L
    src = ref.random_vecs(1, n, vseed)
    d = dict(L=L, beta=beta, m=m, r=r, csw=csw, mu=mu, gseed=gseed, vseed=vseed, U=U, src=src,
             clover=ref.clover(U), avg_plaq=ref.avg_plaq(U))
    for op, key in enumerate(["D", "Ddag", "DdagD", "g5D"]):
        d[key] = ref.dirac(U, m, r, csw, mu, op, src)
    np.savez_compressed(OUT / f"{name}.npz", **d)
    print("wrote", name)


def cg_force_case(ref, name, L, beta, m, r, csw, mu, gseed, vseed, tol=1e-10):
    U = gauge_normal(L, beta, gseed).reshape(-1)
    n = 2 * L * L
    eta = ref.random_vecs(1, n, vseed)
    phi = ref.dirac(U, m, r, csw, mu, 1, eta)  # phi = D^dag eta (hmc_trajectory.cpp:32-36)
    X, it, res = ref.cg(U, m, r, csw, mu, phi, 10000, tol)
    F = ref.fermion_force(U, m, r, csw, mu, X)
    G = ref.gauge_force(U, beta)
    np.savez_compressed(OUT / f"{name}.npz", L=L, beta=beta, m=m, r=r, csw=csw, mu=mu, gseed=gseed, vseed=vseed,
                        U=U, eta=eta, phi=phi, X=X, cg_iters=it, cg_res=res, tol=tol, fermion_force=F,
                        gauge_force=G, gauge_action=ref.gauge_action(U, beta))
    print("wrote", name, "cg iters", it)


def mg_case(ref, name, L, beta, m, r, csw, mu, gseed, bs, k, null_iters, seed):
    U = gauge_normal(L, beta, gseed).reshape(-1)
    n = 2 * L * L
    params = O.RefMGParams(2, bs, k, 0, null_iters, 1, 3, 3, 0)
    init = ref.random_vecs(k, n, seed)                       # the vectors compute_near_null_space draws
    nv = ref.near_null_space(U, m, r, csw, mu, k, null_iters, seed)
    bv = ref.prolongator_build(L, bs, k, nv)
    links = ref.sparse_coarse_build(U, m, r, csw, mu, bs, k, bv)
    nbx = L // bs
    csrc = ref.random_vecs(1, nbx * nbx * k, seed + 1)
    capply = ref.sparse_coarse_apply(nbx, nbx, k, links, csrc)
    fsrc = ref.random_vecs(1, n, seed + 2)
    restr = ref.restrict(L, bs, k, bv, fsrc)
    prol = ref.prolong(L, bs, k, bv, csrc)
    mr = ref.mr_smooth(U, m, r, csw, mu, fsrc, np.zeros(n, complex), 4)
    # 2-level hierarchy on exactly these null vectors: dense coarse LU solve
    pre = ref.mg_precondition(U, m, r, csw, mu, O.RefMGParams(2, bs, k, 0, 0, 1, 3, 3, 0), seed, fsrc, warm=nv)
    x, it, res = ref.mg_gcr(U, m, r, csw, mu, O.RefMGParams(2, bs, k, 0, 0, 1, 3, 3, 0), seed, fsrc, 200, 1e-10, 20,
                            warm=nv)
    np.savez_compressed(OUT / f"{name}.npz", L=L, beta=beta, m=m, r=r, csw=csw, mu=mu, gseed=gseed, bs=bs, k=k,
                        null_iters=null_iters, seed=seed, U=U, init=init, null_vecs=nv, block_vecs=bv, links=links,
                        coarse_src=csrc, coarse_apply=capply, fine_src=fsrc, restrict=restr, prolong=prol,
                        mr4=mr, mg_precondition=pre, gcr_x=x, gcr_iters=it, gcr_res=res)
    print("wrote", name, "gcr iters", it, "res", res)


def hmc_case(ref, name, L, beta, m, r, csw, gseed, seed, n_steps, omelyan, n_traj, tau=1.0):
    """Trajectories of the reference's hmc_trajectory (full lattice, clover) from one rng."""
    U = gauge_normal(L, beta, gseed).reshape(-1)
    U_out, out = ref.hmc_trajectories(U, m, r, beta, tau, n_steps, omelyan, 10000, 1e-12, csw, 0.0, 0, seed, n_traj)
    np.savez_compressed(OUT / f"{name}.npz", L=L, beta=beta, m=m, r=r, csw=csw, gseed=gseed, seed=seed,
                        n_steps=n_steps, omelyan=omelyan, tau=tau, n_traj=n_traj, cg_tol=1e-12, U=U, U_out=U_out,
                        traj=out)
    print("wrote", name, out[:, :2].tolist())


def reversibility_case(ref, name, L, beta, m, r, csw, gseed, seed, n_steps, omelyan, tau=1.0):
    """The reference's reversibility_test_plain (forward, momentum flip, backward)."""
    U = gauge_normal(L, beta, gseed).reshape(-1)
    out = ref.hmc_reversibility(U, m, r, beta, tau, n_steps, omelyan, 10000, 1e-12, csw, 0.0, seed)
    np.savez_compressed(OUT / f"{name}.npz", L=L, beta=beta, m=m, r=r, csw=csw, gseed=gseed, seed=seed,
                        n_steps=n_steps, omelyan=omelyan, tau=tau, cg_tol=1e-12, U=U, result=out)
    print("wrote", name, out.tolist())


def ms_case(ref, name, L, beta, m, r, csw, gseed, seed, bs=4, k=4, n_defl=6, null_iters=5, smooth=3):
    """Coarse deflation (TRLM on the level-1 operator), the low-mode solution and force, and the
    MG multi-timescale HMC (trajectories for each outer integrator, reversibility) of the
    reference, on one hierarchy built from mt19937(seed)."""
    U = gauge_normal(L, beta, gseed).reshape(-1)
    n = 2 * L * L
    cdim = (L // bs) ** 2 * k
    params = O.RefMGParams(2, bs, k, 0, null_iters, 1, 3, 3, n_defl)
    phi = ref.random_vecs(1, n, seed + 1)
    nv, vals, vecs, low, force = ref.ms_setup(U, m, r, csw, 0.0, params, seed, phi, smooth, cdim)
    # one cycle whose coarsest solve is the deflated CG (setup_sparse_coarse wires it, src/multigrid.cpp:780-790)
    pre = ref.mg_precondition(U, m, r, csw, 0.0, O.RefMGParams(2, bs, k, 0, 0, 1, 3, 3, n_defl), seed, phi, warm=nv)
    out = dict(L=L, beta=beta, m=m, r=r, csw=csw, gseed=gseed, seed=seed, bs=bs, k=k, n_defl=n_defl, smooth=smooth,
               U=U, null_vecs=nv, defl_vals=vals, defl_vecs=vecs, phi=phi, lowmode=low, lowmode_force=force,
               precondition_deflated=pre)
    ms = dict(beta=beta, tau=0.2, n_outer=4, n_inner=3, cg_maxiter=500, cg_tol=1e-12, inner_smooth=smooth, c_sw=csw,
              mu_t=0.0)
    for t, n_traj in ((0, 2), (1, 2), (2, 1), (3, 1)):
        q = O.RefMSParams(ms["beta"], ms["tau"], ms["n_outer"], ms["n_inner"], ms["cg_maxiter"], ms["cg_tol"],
                          ms["inner_smooth"], t, ms["c_sw"], ms["mu_t"])
        U_out, traj = ref.ms_trajectories(U, m, r, params, seed, q, seed + 10 + t, n_traj)
        out[f"traj_{t}"] = traj
        out[f"U_out_{t}"] = U_out
        if t < 3:
            out[f"rev_{t}"] = ref.ms_reversibility(U, m, r, params, seed, q, seed + 20 + t)
        print(name, "outer", t, traj[:, :2].tolist(), out.get(f"rev_{t}", np.zeros(5))[:4].tolist())
    out.update({f"ms_{key}": v for key, v in ms.items()})
    np.savez_compressed(OUT / f"{name}.npz", **out)
    print("wrote", name, "defl vals", vals.tolist())


def solvers_case(ref, name, L, beta, m, r, csw, gseed, seed, null_iters=5):
    """PCG (plain with a start vector, and with the symmetric MG), FGMRES (with MG and
    unpreconditioned, Ritz harvesting on), the Richardson/MR smoothers, lambda_max,
    set_symmetric and the pseudofermion action, all from the reference."""
    U = gauge_normal(L, beta, gseed).reshape(-1)
    n = 2 * L * L
    b = ref.random_vecs(1, n, seed + 1)
    x0 = ref.random_vecs(1, n, seed + 2)
    lam = ref.estimate_lambda_max(U, m, r, csw, 0.0, 30)
    omega = 0.8 / lam
    rich = ref.richardson_smooth(U, m, r, csw, 0.0, b, np.zeros(n, complex), 4, omega)
    rich_x0 = ref.richardson_smooth(U, m, r, csw, 0.0, b, x0, 3, omega)
    mr_x0 = ref.mr_smooth(U, m, r, csw, 0.0, b, x0, 4)
    params = O.RefMGParams(2, 4, 4, 0, null_iters, 1, 3, 3, 0)
    pre_sym, om = ref.mg_precondition_sym(U, m, r, csw, 0.0, params, seed, 0.8, b)
    pcg_x, pcg_it, pcg_res = ref.cg_precond(U, m, r, csw, 0.0, params, seed, 0.8, b, None, 500, 1e-10)
    cgx0_x, cgx0_it, cgx0_res = ref.cg_precond(U, m, r, csw, 0.0, None, 0, 0.0, b, x0, 2000, 1e-10)
    fm_x, fm_it, fm_res, fm_ritz = ref.fgmres(U, m, r, csw, 0.0, params, seed, b, 4, 200, 1e-10, 2)
    fp_x, fp_it, fp_res, fp_ritz = ref.fgmres(U, m, r, csw, 0.0, None, 0, b, 12, 2000, 1e-10, 4)
    S, X = ref.fermion_action(U, m, r, csw, 0.0, b, 2000, 1e-10)
    np.savez_compressed(OUT / f"{name}.npz", L=L, beta=beta, m=m, r=r, csw=csw, gseed=gseed, seed=seed,
                        null_iters=null_iters, U=U, b=b, x0=x0, lam=lam, omega=omega, rich4=rich, rich3_x0=rich_x0,
                        mr4_x0=mr_x0, sym_omega=om, sym_precondition=pre_sym, pcg_x=pcg_x, pcg_iters=pcg_it,
                        pcg_res=pcg_res, cgx0_x=cgx0_x, cgx0_iters=cgx0_it, cgx0_res=cgx0_res, fgm_mg_x=fm_x,
                        fgm_mg_iters=fm_it, fgm_mg_res=fm_res, fgm_mg_ritz=fm_ritz, fgm_x=fp_x, fgm_iters=fp_it,
                        fgm_res=fp_res, fgm_ritz=fp_ritz, action=S, action_X=X)
    print("wrote", name, "lambda", lam, "pcg", pcg_it, "cg x0", cgx0_it, "fgmres mg", fm_it, fm_ritz, "fgmres",
          fp_it, fp_ritz)


def eo_case(ref, name, L, beta, m, r, csw, mu, gseed, seed):
    """EvenOddDiracOp operators, reconstruction, log det D_ee, the Schur CG and the e/o force."""
    U = gauge_normal(L, beta, gseed).reshape(-1)
    V = L * L
    src_o = ref.random_vecs(1, V, seed)        # half vectors: V/2 sites x 2 spins
    src_e = ref.random_vecs(1, V, seed + 1)
    phi = ref.random_vecs(1, 2 * V, seed + 2)
    d = dict(L=L, beta=beta, m=m, r=r, csw=csw, mu=mu, gseed=gseed, seed=seed, U=U, src_o=src_o, src_e=src_e,
             phi=phi)
    for op, key in enumerate(["schur", "schur_dag", "mdagm", "hop_eo", "hop_oe"]):
        d[key] = ref.eo_apply(U, m, r, csw, mu, op, src_e if op == 3 else src_o)
    d["recon"] = ref.eo_reconstruct(U, m, r, csw, mu, src_o, phi)
    d["recon_full"] = ref.eo_reconstruct(U, m, r, csw, mu, src_o, None)
    d["logdet"] = ref.eo_logdet(U, m, r, csw, mu)
    phi_o = ref.eo_apply(U, m, r, csw, mu, 1, src_o)  # phi_o = M^dag eta_o
    x_o, it, res = ref.eo_cg(U, m, r, csw, mu, phi_o, 5000, 1e-12)
    d.update(phi_o=phi_o, cg_x=x_o, cg_iters=it, cg_res=res, force=ref.eo_force(U, m, r, csw, mu, x_o))
    np.savez_compressed(OUT / f"{name}.npz", **d)
    print("wrote", name, "eo cg iters", it)


def hmc_eo_case(ref, name, L, beta, m, r, csw, gseed, seed, n_steps, n_traj, tau=1.0):
    """Trajectories of the reference's even-odd hmc_trajectory (leapfrog, Schur CG, log det D_ee)."""
    U = gauge_normal(L, beta, gseed).reshape(-1)
    U_out, out = ref.hmc_trajectories(U, m, r, beta, tau, n_steps, 0, 10000, 1e-12, csw, 0.0, 0, seed, n_traj,
                                      use_eo=True)
    np.savez_compressed(OUT / f"{name}.npz", L=L, beta=beta, m=m, r=r, csw=csw, gseed=gseed, seed=seed,
                        n_steps=n_steps, tau=tau, n_traj=n_traj, cg_tol=1e-12, U=U, U_out=U_out, traj=out)
    print("wrote", name, out[:, :2].tolist())


def delta_case(ref, name, L, beta, m, r, csw, mu, gseed, seed, dt):
    """DiracOp::apply_delta_D with Gaussian momenta."""
    U = gauge_normal(L, beta, gseed).reshape(-1)
    pi = np.random.default_rng(seed).standard_normal(2 * L * L)
    src = ref.random_vecs(1, 2 * L * L, seed + 1)
    out = ref.apply_delta_D(U, m, r, csw, mu, pi, dt, src)
    np.savez_compressed(OUT / f"{name}.npz", L=L, beta=beta, m=m, r=r, csw=csw, mu=mu, gseed=gseed, seed=seed, dt=dt,
                        U=U, pi=pi, src=src, delta=out)
    print("wrote", name)


def gauge_files_case(ref, name, L, beta, mass, gseed):
    """A configuration written by the reference's save_gauge ("SWNG") and GaugeField::save (raw)."""
    U = gauge_normal(L, beta, gseed).reshape(-1)
    assert ref.save_gauge(U, beta, mass, OUT / f"{name}.swng", OUT / f"{name}.raw")
    print("wrote", name)


def sparse_from_dense(A, nx, ny, k):
    """SparseCoarseOp links [site][dir][i * k + j] of a dense 9-point coarse operator (checked exact)."""
    dx = [0, 1, -1, 0, 0, 1, 1, -1, -1]
    dy = [0, 0, 0, 1, -1, 1, -1, 1, -1]
    lk = np.zeros((nx * ny, 9, k, k), complex)
    back = np.zeros_like(A)
    for b in range(nx * ny):
        bx, by = b % nx, b // nx
        for d in range(9):
            nb = (bx + dx[d]) % nx + nx * ((by + dy[d]) % ny)
            lk[b, d] = A[b * k:(b + 1) * k, nb * k:(nb + 1) * k]
            back[b * k:(b + 1) * k, nb * k:(nb + 1) * k] += lk[b, d]
    assert np.max(np.abs(back - A)) <= 1e-14 * np.max(np.abs(A)), "not a 9-point operator"
    return lk.reshape(-1)


def mg3_case(ref, name, L, beta, m, r, csw, mu, gseed, bs, k, null_iters, seed):
    """Three levels with the reference's default coarse blocking (4k consecutive coarse dofs,
    CoarseProlongator, src/prolongator.h:149-228) and its dense intermediate operator
    (src/multigrid.cpp:640-687); W-cycle, 3 + 3 MR steps, dense LU on the coarsest level."""
    U = gauge_normal(L, beta, gseed).reshape(-1)
    n = 2 * L * L
    params = O.RefMGParams(3, bs, k, 0, null_iters, 1, 3, 3, 0)
    nv, bv1, A1, A2 = ref.mg3_export(U, m, r, csw, mu, params, seed)
    n1 = L // bs
    # 4k consecutive dofs of the lexicographic level-1 vector = 4 x 1 aggregates of level-1 sites
    links2 = sparse_from_dense(A2, n1 // 4, n1, k)
    fsrc = ref.random_vecs(1, n, seed + 2)
    pre = ref.mg_precondition(U, m, r, csw, mu, params, seed, fsrc)
    x, it, res = ref.mg_gcr(U, m, r, csw, mu, params, seed, fsrc, 200, 1e-10, 20)
    np.savez_compressed(OUT / f"{name}.npz", L=L, beta=beta, m=m, r=r, csw=csw, mu=mu, gseed=gseed, bs=bs, k=k,
                        null_iters=null_iters, seed=seed, U=U, null_vecs=nv, block_vecs1=bv1, links2=links2,
                        fine_src=fsrc, mg_precondition=pre, gcr_iters=it, gcr_res=res)
    print("wrote", name, "gcr iters", it, "res", res)


CASES = {
    "dirac_L8_wilson": lambda ref: dirac_case(ref, "dirac_L8_wilson", 8, 2.0, 0.3, 1.0, 0.0, 0.0, 11, 12),
    "dirac_L16_clover_twist": lambda ref: dirac_case(ref, "dirac_L16_clover_twist", 16, 2.0, -0.05, 1.0, 1.0, 0.2,
                                                     21, 22),
    "dirac_L32_config1": lambda ref: dirac_case(ref, "dirac_L32_config1", 32, 2.0, 0.1, 1.0, 1.0, 0.0, 31, 32),
    "cg_force_L32_config1": lambda ref: cg_force_case(ref, "cg_force_L32_config1", 32, 2.0, 0.1, 1.0, 1.0, 0.0, 31,
                                                      33),
    "cg_force_L16_wilson": lambda ref: cg_force_case(ref, "cg_force_L16_wilson", 16, 4.0, 0.2, 1.0, 0.0, 0.0, 41, 42),
    "mg_L16_bs4_k4": lambda ref: mg_case(ref, "mg_L16_bs4_k4", 16, 2.0, 0.1, 1.0, 1.0, 0.0, 51, 4, 4, 5, 52),
    "hmc_L8_omelyan": lambda ref: hmc_case(ref, "hmc_L8_omelyan", 8, 4.0, 0.1, 1.0, 1.0, 61, 62, 5, 1, 3),
    "hmc_L8_leapfrog": lambda ref: hmc_case(ref, "hmc_L8_leapfrog", 8, 4.0, 0.1, 1.0, 1.0, 63, 64, 8, 0, 2),
    "solvers_L16": lambda ref: solvers_case(ref, "solvers_L16", 16, 2.0, 0.1, 1.0, 1.0, 71, 72),
    "gauge_L8": lambda ref: gauge_files_case(ref, "gauge_L8", 8, 3.0, 0.05, 81),
    "eo_L16_clover_twist": lambda ref: eo_case(ref, "eo_L16_clover_twist", 16, 2.0, 0.1, 1.0, 1.0, 0.2, 91, 92),
    "eo_L16_wilson": lambda ref: eo_case(ref, "eo_L16_wilson", 16, 4.0, 0.2, 1.0, 0.0, 0.0, 93, 94),
    "reversibility_L8_omelyan": lambda ref: reversibility_case(ref, "reversibility_L8_omelyan", 8, 4.0, 0.1, 1.0,
                                                               1.0, 71, 72, 5, 1),
    "ms_L16": lambda ref: ms_case(ref, "ms_L16", 16, 4.0, 0.1, 1.0, 1.0, 111, 112),
    "hmc_eo_L8": lambda ref: hmc_eo_case(ref, "hmc_eo_L8", 8, 4.0, 0.1, 1.0, 1.0, 95, 96, 6, 3),
    "delta_L16": lambda ref: delta_case(ref, "delta_L16", 16, 3.0, 0.1, 1.0, 1.0, 0.1, 97, 98, 0.05),
    "mg3_L48_k4": lambda ref: mg3_case(ref, "mg3_L48_k4", 48, 6.0, -0.05, 1.0, 1.0, 0.0, 121, 4, 4, 5, 122),
}


def main():
    """python make_golden.py [case ...]: regenerates the named fixtures (all without arguments)."""
    O.build(ref=True)
    ref = O.ref()
    if ref is None:
        raise SystemExit("the reference shim is needed to generate fixtures")
    names = sys.argv[1:] or list(CASES)
    for nm in names:
        CASES[nm](ref)


if __name__ == "__main__":
    main()
