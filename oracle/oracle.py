"""ORACLE TEST INFRASTRUCTURE — not part of the product.

ctypes loaders for the two CPU checkers:

* ``port()`` — oracle/_build/libsmg_oracle.so, the plain-C restatement of the
  reference path (smg_oracle.c).  Builds anywhere gcc and OpenMP exist, so it
  is the checker on the GPU machine and the CPU baseline of bench.py.
* ``ref()``  — oracle/_ref/libsmg_ref.so, the reference's own C++ sources
  compiled by oracle/Makefile with the ref_shim.cpp entry points.  Exists only
  where the reference tree was present at build time; ``ref()`` returns None
  otherwise.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.  Arrays are numpy complex128 in the reference layouts
(spinor v[2*s+spin], links U[mu][s], force F[mu][s]).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PORT_SO = HERE / "_build" / "libsmg_oracle.so"
REF_SO = HERE / "_ref" / "libsmg_ref.so"
# the reference's src/ directory, only from the environment (the reference shim is built only when it is set)
REF_SRC = Path(os.environ["SMG_REFERENCE_SRC"]) if os.environ.get("SMG_REFERENCE_SRC") else None

_dp = C.POINTER(C.c_double)


def build(ref: bool | None = None) -> None:
    """Compiles the C restatement and, when the reference tree exists, the reference shim."""
    targets = ["oracle"]
    if ref is None:
        ref = REF_SRC is not None and (REF_SRC / "dirac.h").exists()
    if ref:
        targets.append("ref")
    args = [f"REF={REF_SRC}"] if REF_SRC is not None else []
    subprocess.run(["make", "-s", "-j8", "-C", str(HERE), *args, *targets], check=True)


def _p(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def _c(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.complex128)


class RefMGParams(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("levels", "block_size", "k_null", "coarse_block", "null_iters", "w_cycle",
                                         "pre_smooth", "post_smooth", "n_defl")]


class RefMSParams(C.Structure):
    _fields_ = [("beta", C.c_double), ("tau", C.c_double), ("n_outer", C.c_int), ("n_inner", C.c_int),
                ("cg_maxiter", C.c_int), ("cg_tol", C.c_double), ("inner_smooth", C.c_int), ("outer_type", C.c_int),
                ("c_sw", C.c_double), ("mu_t", C.c_double)]


class OrcMG2Params(C.Structure):
    _fields_ = [("L", C.c_int), ("bs", C.c_int), ("k", C.c_int), ("m", C.c_double), ("r", C.c_double),
                ("csw", C.c_double), ("mu", C.c_double), ("pre_smooth", C.c_int), ("post_smooth", C.c_int),
                ("coarse_max_iter", C.c_int), ("coarse_tol", C.c_double)]


MAXL = 6


class OrcMGNParams(C.Structure):
    _fields_ = [("n_levels", C.c_int), ("L", C.c_int), ("m", C.c_double), ("r", C.c_double), ("csw", C.c_double),
                ("mu", C.c_double), ("block", (C.c_int * 2) * (MAXL - 1)), ("nc", C.c_int * (MAXL - 1)),
                ("block_vecs", C.POINTER(C.c_double) * (MAXL - 1)), ("links", C.POINTER(C.c_double) * MAXL),
                ("pre_smooth", C.c_int), ("post_smooth", C.c_int), ("w_cycle", C.c_int),
                ("coarse_max_iter", C.c_int), ("coarse_tol", C.c_double)]


class OrcMGNSetupParams(C.Structure):
    _fields_ = [("n_levels", C.c_int), ("L", C.c_int), ("m", C.c_double), ("r", C.c_double), ("csw", C.c_double),
                ("mu", C.c_double), ("block", (C.c_int * 2) * (MAXL - 1)), ("nvec", C.c_int * (MAXL - 1)),
                ("chiral_split", C.c_int), ("null_iters", C.c_int), ("null_mr_steps", C.c_int), ("seed", C.c_uint32)]


class _Lib:
    """Common numpy-facing wrappers; `prefix` is 'orc_' (port) or 'ref_' (reference)."""

    def __init__(self, path: Path, prefix: str):
        self.lib = C.CDLL(str(path))
        self.prefix = prefix
        self.is_ref = prefix == "ref_"
        f = self._f
        f("clover").restype = None
        f("avg_plaq").restype = C.c_double
        f("dirac").restype = None
        f("cg").restype = C.c_int
        f("gauge_force").restype = None
        f("gauge_action").restype = C.c_double
        f("fermion_force").restype = None
        f("mr_smooth").restype = None
        f("near_null_space").restype = None
        f("prolongator_build").restype = None
        f("prolong").restype = None
        f("restrict").restype = None
        f("sparse_coarse_build").restype = None
        f("sparse_coarse_apply").restype = None

    def _f(self, name):
        return getattr(self.lib, self.prefix + name)

    # -- geometry helpers
    @staticmethod
    def _L(U):
        V = U.size // 2
        L = int(round(V ** 0.5))
        assert L * L == V
        return L

    def clover(self, U):
        U = _c(U)
        L = self._L(U)
        out = np.empty(L * L)
        self._f("clover")(C.c_int(L), _p(U), _p(out))
        return out

    def avg_plaq(self, U):
        U = _c(U)
        return self._f("avg_plaq")(C.c_int(self._L(U)), _p(U))

    def dirac(self, U, m, r, csw, mu, op, src):
        U = _c(U)
        src = _c(src)
        dst = np.empty_like(src)
        self._f("dirac")(C.c_int(self._L(U)), _p(U), C.c_double(m), C.c_double(r), C.c_double(csw),
                         C.c_double(mu), C.c_int(op), _p(src), _p(dst))
        return dst

    def cg(self, U, m, r, csw, mu, b, max_iter, tol):
        U = _c(U)
        b = _c(b)
        x = np.empty_like(b)
        res = C.c_double(0)
        it = self._f("cg")(C.c_int(self._L(U)), _p(U), C.c_double(m), C.c_double(r), C.c_double(csw),
                           C.c_double(mu), _p(b), _p(x), C.c_int(max_iter), C.c_double(tol), C.byref(res))
        return x, it, res.value

    def gauge_force(self, U, beta):
        U = _c(U)
        F = np.empty(U.size)
        self._f("gauge_force")(C.c_int(self._L(U)), _p(U), C.c_double(beta), _p(F))
        return F

    def gauge_action(self, U, beta):
        U = _c(U)
        return self._f("gauge_action")(C.c_int(self._L(U)), _p(U), C.c_double(beta))

    def fermion_force(self, U, m, r, csw, mu, X):
        U = _c(U)
        X = _c(X)
        F = np.empty(U.size)
        self._f("fermion_force")(C.c_int(self._L(U)), _p(U), C.c_double(m), C.c_double(r), C.c_double(csw),
                                 C.c_double(mu), _p(X), _p(F))
        return F

    def mr_smooth(self, U, m, r, csw, mu, b, x0, niter):
        U = _c(U)
        b = _c(b)
        x = _c(x0).copy()
        self._f("mr_smooth")(C.c_int(self._L(U)), _p(U), C.c_double(m), C.c_double(r), C.c_double(csw),
                             C.c_double(mu), _p(b), _p(x), C.c_int(niter))
        return x

    def prolongator_build(self, L, bs, k, null_vecs):
        nv = _c(null_vecs)
        nb = (L // bs) ** 2
        out = np.empty(nb * k * 2 * bs * bs, dtype=np.complex128)
        self._f("prolongator_build")(C.c_int(L), C.c_int(bs), C.c_int(k), _p(nv), _p(out))
        return out

    def prolong(self, L, bs, k, bv, coarse):
        bv = _c(bv)
        coarse = _c(coarse)
        fine = np.empty(2 * L * L, dtype=np.complex128)
        self._f("prolong")(C.c_int(L), C.c_int(bs), C.c_int(k), _p(bv), _p(coarse), _p(fine))
        return fine

    def restrict(self, L, bs, k, bv, fine):
        bv = _c(bv)
        fine = _c(fine)
        coarse = np.empty((L // bs) ** 2 * k, dtype=np.complex128)
        self._f("restrict")(C.c_int(L), C.c_int(bs), C.c_int(k), _p(bv), _p(fine), _p(coarse))
        return coarse

    def sparse_coarse_build(self, U, m, r, csw, mu, bs, k, bv):
        U = _c(U)
        bv = _c(bv)
        L = self._L(U)
        nb = (L // bs) ** 2
        links = np.empty(nb * 9 * k * k, dtype=np.complex128)
        self._f("sparse_coarse_build")(C.c_int(L), _p(U), C.c_double(m), C.c_double(r), C.c_double(csw),
                                       C.c_double(mu), C.c_int(bs), C.c_int(k), _p(bv), _p(links))
        return links

    def sparse_coarse_apply(self, nbx, nby, k, links, src):
        links = _c(links)
        src = _c(src)
        dst = np.empty_like(src)
        self._f("sparse_coarse_apply")(C.c_int(nbx), C.c_int(nby), C.c_int(k), _p(links), _p(src), _p(dst))
        return dst


class Port(_Lib):
    def __init__(self):
        super().__init__(PORT_SO, "orc_")
        self.lib.orc_get_threads.restype = C.c_int
        self.lib.orc_mg2_gcr.restype = C.c_int
        self.lib.orc_sparse_coarse_cg.restype = C.c_int

    def time_dirac(self, U, m, r, csw, mu, op, srcs, reps):
        """Seconds for `reps` applications of op to every row of srcs (nrhs x 2V)."""
        U = _c(U)
        srcs = _c(srcs)
        nrhs = srcs.size // (U.size)
        dst = np.empty_like(srcs)
        self.lib.orc_time_dirac.restype = C.c_double
        t = self.lib.orc_time_dirac(C.c_int(self._L(U)), _p(U), C.c_double(m), C.c_double(r), C.c_double(csw),
                                    C.c_double(mu), C.c_int(op), C.c_int(nrhs), _p(srcs), _p(dst), C.c_int(reps))
        return t, dst

    def time_cg(self, U, m, r, csw, mu, b, max_iter, tol):
        U, b = _c(U), _c(b)
        x = np.empty_like(b)
        it = C.c_int(0)
        self.lib.orc_time_cg.restype = C.c_double
        t = self.lib.orc_time_cg(C.c_int(self._L(U)), _p(U), C.c_double(m), C.c_double(r), C.c_double(csw),
                                 C.c_double(mu), _p(b), _p(x), C.c_int(max_iter), C.c_double(tol), C.byref(it))
        return t, x, it.value

    def mgN_params(self, L, m, r, csw, mu, blocks, ncs, block_vecs, links, pre, post, w_cycle, coarse_max_iter,
                   coarse_tol):
        """Builds orc_mgN_params; the returned object keeps the arrays alive."""
        p = OrcMGNParams()
        p.n_levels = len(blocks) + 1
        p.L, p.m, p.r, p.csw, p.mu = L, m, r, csw, mu
        keep = []
        for l, (b, nc, bv) in enumerate(zip(blocks, ncs, block_vecs)):
            p.block[l][0], p.block[l][1] = b
            p.nc[l] = nc
            a = _c(bv)
            keep.append(a)
            p.block_vecs[l] = _p(a)
        for l, lk in enumerate(links):
            if lk is None:
                continue
            a = _c(lk)
            keep.append(a)
            p.links[l] = _p(a)
        p.pre_smooth, p.post_smooth, p.w_cycle = pre, post, int(w_cycle)
        p.coarse_max_iter, p.coarse_tol = coarse_max_iter, coarse_tol
        p._keep = keep
        return p

    def mgN_precondition(self, p, U, b):
        U, b = _c(U), _c(b)
        out = np.empty_like(b)
        self.lib.orc_mgN_precondition(C.byref(p), _p(U), _p(b), _p(out))
        return out

    def mgN_gcr(self, p, U, b, max_iter, tol, trunc):
        U, b = _c(U), _c(b)
        x = np.empty_like(b)
        res, sec = C.c_double(0), C.c_double(0)
        self.lib.orc_mgN_gcr.restype = C.c_int
        it = self.lib.orc_mgN_gcr(C.byref(p), _p(U), _p(b), _p(x), C.c_int(max_iter), C.c_double(tol),
                                  C.c_int(trunc), C.byref(res), C.byref(sec))
        return x, it, res.value, sec.value

    def random_vec(self, n: int, seed: int) -> np.ndarray:
        """random_vec(n, std::mt19937(seed)) (oracle/inputs.cpp)."""
        v = np.empty(n, dtype=np.complex128)
        self.lib.orc_random_vec(C.c_long(n), C.c_uint32(seed), _p(v))
        return v

    def gauge_normal(self, L: int, beta: float, seed: int) -> np.ndarray:
        """Links U[mu][s] = exp(i theta), theta ~ N(0, 1/beta) from std::mt19937(seed) (oracle/inputs.cpp)."""
        U = np.empty(2 * L * L, dtype=np.complex128)
        self.lib.orc_gauge_normal(C.c_int(L), C.c_double(beta), C.c_uint32(seed), _p(U))
        return U.reshape(2, L * L)

    def mgN_setup(self, L, U, m, r, csw, mu, blocks, nvecs, null_iters, seed, chiral_split=False, null_mr_steps=5):
        """The hierarchy built on the CPU (orc_mgN_setup): (block_vecs per transfer, links per level with
        links[0] = None, level-0 null vectors), in the layouts orc_mgN_params takes."""
        n_levels = len(blocks) + 1
        p = OrcMGNSetupParams()
        p.n_levels, p.L, p.m, p.r, p.csw, p.mu = n_levels, L, m, r, csw, mu
        for l, (b, k) in enumerate(zip(blocks, nvecs)):
            p.block[l][0], p.block[l][1] = b
            p.nvec[l] = k
        p.chiral_split, p.null_iters, p.null_mr_steps, p.seed = int(chiral_split), null_iters, null_mr_steps, seed
        nx = ny = L
        nd = 2
        bvs, links = [], [None]
        for (ax, ay), k in zip(blocks, nvecs):
            nc = 2 * k if chiral_split else k
            bvs.append(np.empty(nx * ny * nd * nc, dtype=np.complex128))
            nx, ny, nd = nx // ax, ny // ay, nc
            links.append(np.empty(nx * ny * 9 * nd * nd, dtype=np.complex128))
        null0 = np.empty(nvecs[0] * 2 * L * L, dtype=np.complex128)
        bv_arr = (_dp * (MAXL - 1))(*[_p(b) for b in bvs])
        lk_arr = (_dp * MAXL)(None, *[_p(a) for a in links[1:]])
        U = _c(U)
        self.lib.orc_mgN_setup.restype = C.c_int
        rc = self.lib.orc_mgN_setup(C.byref(p), _p(U), bv_arr, lk_arr, _p(null0))
        if rc != 0:
            raise ValueError(f"orc_mgN_setup: bad geometry ({rc})")
        return bvs, links, null0.reshape(nvecs[0], -1)

    def set_threads(self, n: int) -> None:
        self.lib.orc_set_threads(C.c_int(n))

    def threads(self) -> int:
        return self.lib.orc_get_threads()

    def near_null_space(self, U, m, r, csw, mu, k, iters, init):
        U = _c(U)
        init = _c(init)
        out = np.empty_like(init)
        self.lib.orc_near_null_space(C.c_int(self._L(U)), _p(U), C.c_double(m), C.c_double(r), C.c_double(csw),
                                     C.c_double(mu), C.c_int(k), C.c_int(iters), _p(init), _p(out))
        return out

    def sparse_coarse_cg(self, nbx, nby, k, links, b, max_iter, tol):
        links = _c(links)
        b = _c(b)
        x = np.empty_like(b)
        it = self.lib.orc_sparse_coarse_cg(C.c_int(nbx), C.c_int(nby), C.c_int(k), _p(links), _p(b), _p(x),
                                           C.c_int(max_iter), C.c_double(tol))
        return x, it

    @staticmethod
    def mg2_params(L, bs, k, m, r, csw, mu, pre, post, coarse_max_iter, coarse_tol):
        return OrcMG2Params(L, bs, k, m, r, csw, mu, pre, post, coarse_max_iter, coarse_tol)

    def mg2_precondition(self, p, U, bv, links, b):
        U, bv, links, b = _c(U), _c(bv), _c(links), _c(b)
        out = np.empty_like(b)
        self.lib.orc_mg2_precondition(C.byref(p), _p(U), _p(bv), _p(links), _p(b), _p(out))
        return out

    def mg2_gcr(self, p, U, bv, links, b, max_iter, tol, trunc, ref_coeff=False):
        U, bv, links, b = _c(U), _c(bv), _c(links), _c(b)
        x = np.empty_like(b)
        res = C.c_double(0)
        it = self.lib.orc_mg2_gcr(C.byref(p), _p(U), _p(bv), _p(links), _p(b), _p(x), C.c_int(max_iter),
                                  C.c_double(tol), C.c_int(trunc), C.c_int(int(ref_coeff)), C.byref(res))
        return x, it, res.value


class Ref(_Lib):
    def __init__(self):
        super().__init__(REF_SO, "ref_")
        self.lib.ref_verify_forces.restype = C.c_int
        self.lib.ref_mg_gcr.restype = C.c_int
        self.lib.ref_set_verbosity(C.c_int(0))

    def random_vecs(self, k, n, seed):
        out = np.empty(k * n, dtype=np.complex128)
        self.lib.ref_random_vecs(C.c_int(k), C.c_int(n), C.c_uint(seed), _p(out))
        return out

    def near_null_space(self, U, m, r, csw, mu, k, iters, seed):
        U = _c(U)
        L = self._L(U)
        out = np.empty(k * 2 * L * L, dtype=np.complex128)
        self.lib.ref_near_null_space(C.c_int(L), _p(U), C.c_double(m), C.c_double(r), C.c_double(csw),
                                     C.c_double(mu), C.c_int(k), C.c_int(iters), C.c_uint(seed), _p(out))
        return out

    def dense_coarse_build(self, U, m, r, csw, mu, bs, k, bv):
        U, bv = _c(U), _c(bv)
        L = self._L(U)
        dim = (L // bs) ** 2 * k
        mat = np.empty(dim * dim, dtype=np.complex128)
        self.lib.ref_dense_coarse_build(C.c_int(L), _p(U), C.c_double(m), C.c_double(r), C.c_double(csw),
                                        C.c_double(mu), C.c_int(bs), C.c_int(k), _p(bv), _p(mat))
        return mat.reshape(dim, dim).T  # stored column-major

    def mg3_export(self, U, m, r, csw, mu, params: RefMGParams, seed):
        """The reference's three-level hierarchy: (level-0 null vectors, level-1 CoarseProlongator block vectors
        [block][k][block_k], dense level-1 operator, dense level-2 operator), the dense matrices as [row][col]."""
        U = _c(U)
        L = self._L(U)
        k = params.k_null
        dim1 = (L // params.block_size) ** 2 * k
        cb = params.coarse_block if params.coarse_block > 0 else 4 * k
        dim2 = dim1 // cb * k
        null0 = np.empty(k * 2 * L * L, dtype=np.complex128)
        bv1 = np.empty(dim1 // cb * k * cb, dtype=np.complex128)
        A1 = np.empty(dim1 * dim1, dtype=np.complex128)
        A2 = np.empty(dim2 * dim2, dtype=np.complex128)
        self.lib.ref_mg3_export(C.c_int(L), _p(U), C.c_double(m), C.c_double(r), C.c_double(csw), C.c_double(mu),
                                C.byref(params), C.c_uint(seed), _p(null0), _p(bv1), _p(A1), _p(A2))
        return null0.reshape(k, -1), bv1, A1.reshape(dim1, dim1).T.copy(), A2.reshape(dim2, dim2).T.copy()

    def verify_forces(self, U, beta, m, r, csw, mu, max_iter, tol, use_eo=False):
        U = _c(U)
        return self.lib.ref_verify_forces(C.c_int(self._L(U)), _p(U), C.c_double(beta), C.c_double(m),
                                          C.c_double(r), C.c_double(csw), C.c_double(mu), C.c_int(max_iter),
                                          C.c_double(tol), C.c_int(int(use_eo))) == 1

    def mg_precondition(self, U, m, r, csw, mu, params: RefMGParams, seed, b, warm=None):
        U, b = _c(U), _c(b)
        out = np.empty_like(b)
        wp = _p(_c(warm)) if warm is not None else None
        keep = _c(warm) if warm is not None else None
        if keep is not None:
            wp = _p(keep)
        self.lib.ref_mg_precondition(C.c_int(self._L(U)), _p(U), C.c_double(m), C.c_double(r), C.c_double(csw),
                                     C.c_double(mu), C.byref(params), C.c_uint(seed), wp, _p(b), _p(out))
        return out

    def mg_gcr(self, U, m, r, csw, mu, params: RefMGParams, seed, b, max_iter, tol, trunc, warm=None):
        U, b = _c(U), _c(b)
        x = np.empty_like(b)
        res = C.c_double(0)
        keep = _c(warm) if warm is not None else None
        wp = _p(keep) if keep is not None else None
        it = self.lib.ref_mg_gcr(C.c_int(self._L(U)), _p(U), C.c_double(m), C.c_double(r), C.c_double(csw),
                                 C.c_double(mu), C.byref(params), C.c_uint(seed), wp, _p(b), _p(x),
                                 C.c_int(max_iter), C.c_double(tol), C.c_int(trunc), C.byref(res))
        return x, it, res.value

    def hmc_trajectories(self, U, m, r, beta, tau, n_steps, omelyan, cg_maxiter, cg_tol, csw, mu, force_accept,
                         seed, n_traj, use_eo=False):
        """The reference's hmc_trajectory n_traj times with one std::mt19937(seed); returns the
        final links and per trajectory (accepted, dH, dKE, dSG, dSF, cg iterations, plaquette)
        and, with use_eo, dLD as an eighth column."""
        U = _c(U).copy()
        out = np.zeros(8 * n_traj)
        self.lib.ref_hmc_trajectories(C.c_int(self._L(U)), _p(U), C.c_double(m), C.c_double(r), C.c_double(beta),
                                      C.c_double(tau), C.c_int(n_steps), C.c_int(omelyan), C.c_int(cg_maxiter),
                                      C.c_double(cg_tol), C.c_double(csw), C.c_double(mu), C.c_int(force_accept),
                                      C.c_uint(seed), C.c_int(n_traj), _p(out), C.c_int(int(use_eo)))
        return U, out.reshape(n_traj, 8)[:, :8 if use_eo else 7]

    def ms_setup(self, U, m, r, csw, mu, params: RefMGParams, seed, phi, smooth, cdim):
        """A reference hierarchy with TRLM coarse deflation: (null vectors, deflation values,
        deflation vectors, low-mode solution of phi, coarse_lowmode_force(phi, smooth))."""
        U, phi = _c(U), _c(phi)
        L = self._L(U)
        n = 2 * L * L
        nv = np.zeros((params.k_null, n), dtype=np.complex128)
        vals = np.zeros(params.n_defl)
        vecs = np.zeros((params.n_defl, cdim), dtype=np.complex128)
        low = np.zeros(n, dtype=np.complex128)
        force = np.zeros(2 * L * L)
        self.lib.ref_ms_setup(C.c_int(L), _p(U), C.c_double(m), C.c_double(r), C.c_double(csw), C.c_double(mu),
                              C.byref(params), C.c_uint(seed), _p(phi), C.c_int(smooth), _p(nv),
                              vals.ctypes.data_as(C.POINTER(C.c_double)), _p(vecs), _p(low),
                              force.ctypes.data_as(C.POINTER(C.c_double)))
        return nv, vals, vecs, low, force

    def ms_trajectories(self, U, m, r, params: RefMGParams, mg_seed, ms: RefMSParams, seed, n_traj):
        """hmc_trajectory_mg_multiscale n_traj times (deflation evolved between accepted
        trajectories); returns the final links and per trajectory (accepted, dH, dKE, dSG, dSF,
        CG iterations, low-mode evaluations, plaquette)."""
        U = _c(U).copy()
        out = np.zeros(9 * n_traj)
        self.lib.ref_ms_trajectories(C.c_int(self._L(U)), _p(U), C.c_double(m), C.c_double(r), C.byref(params),
                                     C.c_uint(mg_seed), C.byref(ms), C.c_uint(seed), C.c_int(n_traj),
                                     out.ctypes.data_as(C.POINTER(C.c_double)))
        return U, out.reshape(n_traj, 9)[:, :8]

    def ms_reversibility(self, U, m, r, params: RefMGParams, mg_seed, ms: RefMSParams, seed):
        U = _c(U)
        out = np.zeros(5)
        self.lib.ref_ms_reversibility(C.c_int(self._L(U)), _p(U), C.c_double(m), C.c_double(r), C.byref(params),
                                      C.c_uint(mg_seed), C.byref(ms), C.c_uint(seed),
                                      out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def hmc_reversibility(self, U, m, r, beta, tau, n_steps, omelyan, cg_maxiter, cg_tol, csw, mu, seed):
        """The reference's reversibility_test_plain with std::mt19937(seed): (gauge_delta,
        mom_delta, dH_forward, dH_backward, total CG iterations)."""
        U = _c(U)
        out = np.zeros(5)
        self.lib.ref_hmc_reversibility(C.c_int(self._L(U)), _p(U), C.c_double(m), C.c_double(r), C.c_double(beta),
                                       C.c_double(tau), C.c_int(n_steps), C.c_int(omelyan), C.c_int(cg_maxiter),
                                       C.c_double(cg_tol), C.c_double(csw), C.c_double(mu), C.c_uint(seed), _p(out))
        return out

    def apply_delta_D(self, U, m, r, csw, mu, pi, dt, src):
        U, src = _c(U), _c(src)
        pi = np.ascontiguousarray(pi, dtype=np.float64).reshape(-1)
        out = np.empty_like(src)
        self.lib.ref_apply_delta_D(C.c_int(self._L(U)), _p(U), C.c_double(m), C.c_double(r), C.c_double(csw),
                                   C.c_double(mu), pi.ctypes.data_as(C.POINTER(C.c_double)), C.c_double(dt), _p(src),
                                   _p(out))
        return out

    def eo_apply(self, U, m, r, csw, mu, op, src):
        U, src = _c(U), _c(src)
        L = self._L(U)
        out = np.empty(L * L, dtype=np.complex128)
        self.lib.ref_eo_apply(C.c_int(L), _p(U), C.c_double(m), C.c_double(r), C.c_double(csw), C.c_double(mu),
                              C.c_int(op), _p(src), _p(out))
        return out

    def eo_reconstruct(self, U, m, r, csw, mu, x_o, phi=None):
        U, x_o = _c(U), _c(x_o)
        L = self._L(U)
        out = np.empty(2 * L * L, dtype=np.complex128)
        keep = _c(phi) if phi is not None else None
        self.lib.ref_eo_reconstruct(C.c_int(L), _p(U), C.c_double(m), C.c_double(r), C.c_double(csw),
                                    C.c_double(mu), _p(x_o), _p(keep) if keep is not None else None, _p(out))
        return out

    def eo_logdet(self, U, m, r, csw, mu):
        U = _c(U)
        f = self.lib.ref_eo_logdet
        f.restype = C.c_double
        return f(C.c_int(self._L(U)), _p(U), C.c_double(m), C.c_double(r), C.c_double(csw), C.c_double(mu))

    def eo_cg(self, U, m, r, csw, mu, phi_o, max_iter, tol):
        U, phi_o = _c(U), _c(phi_o)
        x = np.empty_like(phi_o)
        res = C.c_double(0)
        f = self.lib.ref_eo_cg
        f.restype = C.c_int
        it = f(C.c_int(self._L(U)), _p(U), C.c_double(m), C.c_double(r), C.c_double(csw), C.c_double(mu),
               _p(phi_o), _p(x), C.c_int(max_iter), C.c_double(tol), C.byref(res))
        return x, it, res.value

    def eo_force(self, U, m, r, csw, mu, x_o):
        U, x_o = _c(U), _c(x_o)
        L = self._L(U)
        F = np.empty(2 * L * L)
        self.lib.ref_eo_force(C.c_int(L), _p(U), C.c_double(m), C.c_double(r), C.c_double(csw), C.c_double(mu),
                              _p(x_o), _p(F))
        return F

    def richardson_smooth(self, U, m, r, csw, mu, b, x0, niter, omega):
        U, b = _c(U), _c(b)
        x = _c(x0).copy()
        self.lib.ref_richardson_smooth(C.c_int(self._L(U)), _p(U), C.c_double(m), C.c_double(r), C.c_double(csw),
                                       C.c_double(mu), _p(b), _p(x), C.c_int(niter), C.c_double(omega))
        return x

    def estimate_lambda_max(self, U, m, r, csw, mu, niter):
        U = _c(U)
        f = self.lib.ref_estimate_lambda_max
        f.restype = C.c_double
        return f(C.c_int(self._L(U)), _p(U), C.c_double(m), C.c_double(r), C.c_double(csw), C.c_double(mu),
                 C.c_int(niter))

    def mg_precondition_sym(self, U, m, r, csw, mu, params: RefMGParams, seed, damping, b):
        """set_symmetric(damping) then precondition(b); returns (M b, omegas)."""
        U, b = _c(U), _c(b)
        out = np.empty_like(b)
        om = np.zeros(max(1, params.levels - 1))
        self.lib.ref_mg_precondition_sym(C.c_int(self._L(U)), _p(U), C.c_double(m), C.c_double(r),
                                         C.c_double(csw), C.c_double(mu), C.byref(params), C.c_uint(seed),
                                         C.c_double(damping), _p(b), _p(out), _p(om))
        return out, om

    def cg_precond(self, U, m, r, csw, mu, params, seed, damping, b, x0, max_iter, tol):
        """cg_solve / cg_solve_x0 / cg_solve_precond / cg_solve_x0_precond; params None: no MG."""
        U, b = _c(U), _c(b)
        x = np.empty_like(b)
        keep = _c(x0) if x0 is not None else None
        res = C.c_double(0)
        f = self.lib.ref_cg_precond
        f.restype = C.c_int
        it = f(C.c_int(self._L(U)), _p(U), C.c_double(m), C.c_double(r), C.c_double(csw), C.c_double(mu),
               C.c_int(int(params is not None)), C.byref(params) if params is not None else None, C.c_uint(seed),
               C.c_double(damping), _p(b), _p(keep) if keep is not None else None, _p(x), C.c_int(max_iter),
               C.c_double(tol), C.byref(res))
        return x, it, res.value

    def fgmres(self, U, m, r, csw, mu, params, seed, b, restart, max_iter, tol, n_ritz):
        """fgmres_solve_mg (params given) or fgmres_solve_generic with the identity; returns
        (x, iterations, final residual, ritz values)."""
        U, b = _c(U), _c(b)
        x = np.empty_like(b)
        res = C.c_double(0)
        ritz = np.zeros(3 * max(1, n_ritz))
        nr = C.c_int(0)
        f = self.lib.ref_fgmres
        f.restype = C.c_int
        it = f(C.c_int(self._L(U)), _p(U), C.c_double(m), C.c_double(r), C.c_double(csw), C.c_double(mu),
               C.c_int(int(params is not None)), C.byref(params) if params is not None else None, C.c_uint(seed),
               _p(b), _p(x), C.c_int(restart), C.c_int(max_iter), C.c_double(tol), C.c_int(n_ritz), C.byref(res),
               _p(ritz), C.byref(nr))
        return x, it, res.value, ritz[:nr.value].copy()

    def fermion_action(self, U, m, r, csw, mu, phi, max_iter, tol):
        U, phi = _c(U), _c(phi)
        X = np.empty_like(phi)
        f = self.lib.ref_fermion_action
        f.restype = C.c_double
        S = f(C.c_int(self._L(U)), _p(U), C.c_double(m), C.c_double(r), C.c_double(csw), C.c_double(mu), _p(phi),
              C.c_int(max_iter), C.c_double(tol), _p(X))
        return S, X

    def save_gauge(self, U, beta, mass, swng_path, raw_path):
        """save_gauge and GaugeField::save of the links U into the two files."""
        U = _c(U)
        f = self.lib.ref_save_gauge
        f.restype = C.c_int
        return f(C.c_int(self._L(U)), _p(U), C.c_double(beta), C.c_double(mass), str(swng_path).encode(),
                 str(raw_path).encode()) == 1

    def load_gauge(self, L, path):
        U = np.empty(2 * L * L, dtype=np.complex128)
        hdr = np.zeros(3)
        f = self.lib.ref_load_gauge
        f.restype = C.c_int
        ok = f(C.c_int(L), str(path).encode(), _p(U), _p(hdr)) == 1
        return (U, hdr) if ok else (None, None)

    def pseudofermion(self, U, m, r, csw, mu, seed):
        U = _c(U)
        L = self._L(U)
        phi = np.empty(2 * L * L, dtype=np.complex128)
        self.lib.ref_pseudofermion(C.c_int(L), _p(U), C.c_double(m), C.c_double(r), C.c_double(csw),
                                   C.c_double(mu), C.c_uint(seed), _p(phi))
        return phi


_port = None
_ref = None


def port() -> Port:
    global _port
    if _port is None:
        if not PORT_SO.exists():
            build(ref=False)
        _port = Port()
    return _port


def ref() -> Ref | None:
    global _ref
    if _ref is None:
        if not REF_SO.exists():
            return None
        _ref = Ref()
    return _ref
