"""Python mirror of the reference's operator and solver API over libsmg_gpu.

Names, argument meaning and result fields follow the reference
(cpviolator/Schwinger_MG): ``Lattice`` (src/lattice.h), ``GaugeField``
(src/gauge.h), ``DiracOp`` (src/dirac.h), ``cg_solve`` and ``CGResult``
(src/solvers.h), ``fermion_force`` / ``gauge_force`` / ``gauge_action``
(src/hmc.h).  Host vectors are numpy complex128 arrays in the reference's
layout (spinor ``v[2*s+spin]``, links ``U[mu][s]``); every computation runs on
the GPU through the C ABI, and a failure raises ``SmgError`` instead of the
reference's asserts and warnings.
"""
from __future__ import annotations

import ctypes as C
import weakref
from dataclasses import dataclass

import numpy as np

from . import _lib as _L

_dp = C.POINTER(C.c_double)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def _as_c128(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.complex128)


PRECISIONS = {"f64": _L.F64, "f32": _L.F32, "f16": _L.F16}


class _Handle:
    """Owns one C handle.  A dependent (e.g. a DiracOp on a GaugeField) is
    registered with its owner and is always released before it, also when the
    garbage collector finalises both in arbitrary order."""

    h = None

    def _adopt(self, h, owner: "_Handle | None", destroy) -> None:
        self.h = h
        self._destroy = destroy
        self._dependents = weakref.WeakSet()
        self._owner = owner
        if owner is not None:
            owner._dependents.add(self)

    def release(self) -> None:
        h = self.h
        if not h:
            return
        for dep in list(getattr(self, "_dependents", ())):
            dep.release()
        self.h = None
        if _L._lib is not None:
            self._destroy(h)

    def __del__(self):
        self.release()


class Context:
    """One CUDA device + stream; all objects made from it enqueue on that stream."""

    _default: "Context | None" = None

    def __init__(self, device: int = 0, stream: int | None = None):
        lib = _L.lib()
        h = C.c_void_p()
        _L.check(lib.smg_context_create(device, C.c_void_p(stream) if stream else None, C.byref(h)),
                 "smg_context_create")
        self.h = h
        self.device = device

    @classmethod
    def default(cls) -> "Context":
        if cls._default is None:
            cls._default = Context(0)
        return cls._default

    def synchronize(self) -> None:
        _L.check(_L.lib().smg_context_synchronize(self.h), "smg_context_synchronize", self.h)

    def set_stream(self, stream: int) -> None:
        _L.check(_L.lib().smg_context_set_stream(self.h, C.c_void_p(stream)), "smg_context_set_stream", self.h)

    def timer_begin(self) -> None:
        _L.check(_L.lib().smg_timer_begin(self.h), "smg_timer_begin", self.h)

    def timer_end(self) -> float:
        """Milliseconds of device time on this context's stream since timer_begin."""
        v = C.c_double()
        _L.check(_L.lib().smg_timer_end(self.h, C.byref(v)), "smg_timer_end", self.h)
        return v.value

    @property
    def kernel_launches(self) -> int:
        return int(_L.lib().smg_context_kernel_launches(self.h))

    def close(self) -> None:
        if getattr(self, "h", None):
            _L.lib().smg_context_destroy(self.h)
            self.h = None


class Lattice:
    """Geometry and even-odd maps (reference src/lattice.h:4-42), computed on the host."""

    def __init__(self, L: int):
        self.L = L
        self.V = L * L
        self.ndof = 2 * L * L
        self.V_half = L * L // 2
        s = np.arange(self.V)
        par = ((s % L) + (s // L)) % 2
        self.even_sites = s[par == 0].astype(np.int32)
        self.odd_sites = s[par == 1].astype(np.int32)
        self.eo_index = np.empty(self.V, dtype=np.int32)
        self.eo_index[self.even_sites] = np.arange(self.even_sites.size, dtype=np.int32)
        self.eo_index[self.odd_sites] = np.arange(self.odd_sites.size, dtype=np.int32)

    def idx(self, x, y):
        L = self.L
        return ((x % L + L) % L) + L * ((y % L + L) % L)

    def xp(self, s):
        return self.idx(s % self.L + 1, s // self.L)

    def xm(self, s):
        return self.idx(s % self.L - 1, s // self.L)

    def yp(self, s):
        return self.idx(s % self.L, s // self.L + 1)

    def ym(self, s):
        return self.idx(s % self.L, s // self.L - 1)

    def parity(self, s):
        return ((s % self.L) + (s // self.L)) % 2


class GaugeField(_Handle):
    """U(1) links U[mu][s] resident on the device (reference src/gauge.h:10-36)."""

    def __init__(self, lat: Lattice, U=None, ctx: Context | None = None):
        self.lat = lat
        self.ctx = ctx or Context.default()
        if U is None:
            U = np.ones(2 * lat.V, dtype=np.complex128)
        U = _as_c128(U).reshape(-1)
        if U.size != 2 * lat.V:
            raise ValueError("U must hold 2*V complex links")
        h = C.c_void_p()
        _L.check(_L.lib().smg_gauge_create(self.ctx.h, lat.L, _ptr(U.view(np.float64)), C.byref(h)),
                 "smg_gauge_create", self.ctx.h)
        self._adopt(h, None, _L.lib().smg_gauge_destroy)

    @property
    def U(self) -> np.ndarray:
        out = np.empty(2 * self.lat.V, dtype=np.complex128)
        _L.check(_L.lib().smg_gauge_get(self.h, _ptr(out.view(np.float64))), "smg_gauge_get", self.ctx.h)
        return out.reshape(2, self.lat.V)

    def set_links(self, U) -> None:
        U = _as_c128(U).reshape(-1)
        _L.check(_L.lib().smg_gauge_set(self.h, _ptr(U.view(np.float64))), "smg_gauge_set", self.ctx.h)

    def avg_plaq(self) -> float:
        v = C.c_double()
        _L.check(_L.lib().smg_gauge_avg_plaq(self.h, C.byref(v)), "smg_gauge_avg_plaq", self.ctx.h)
        return v.value


class Field(_Handle):
    """nrhs spinors of an L x L lattice resident on the device."""

    def __init__(self, lat: Lattice, nrhs: int = 1, precision: str = "f64", ctx: Context | None = None, data=None):
        self.lat = lat
        self.nrhs = nrhs
        self.precision = precision
        self.ctx = ctx or Context.default()
        h = C.c_void_p()
        _L.check(_L.lib().smg_field_create(self.ctx.h, lat.L, nrhs, PRECISIONS[precision], C.byref(h)),
                 "smg_field_create", self.ctx.h)
        self._adopt(h, None, _L.lib().smg_field_destroy)
        if data is not None:
            self.upload(data)

    def upload(self, data) -> "Field":
        a = _as_c128(data).reshape(-1)
        if a.size != self.nrhs * self.lat.ndof:
            raise ValueError(f"expected {self.nrhs * self.lat.ndof} complex values, got {a.size}")
        _L.check(_L.lib().smg_field_upload(self.h, _ptr(a.view(np.float64))), "smg_field_upload", self.ctx.h)
        return self

    def download(self) -> np.ndarray:
        out = np.empty(self.nrhs * self.lat.ndof, dtype=np.complex128)
        _L.check(_L.lib().smg_field_download(self.h, _ptr(out.view(np.float64))), "smg_field_download", self.ctx.h)
        return out if self.nrhs == 1 else out.reshape(self.nrhs, self.lat.ndof)

    def zero(self) -> None:
        _L.check(_L.lib().smg_field_zero(self.h), "smg_field_zero", self.ctx.h)

    def copy_from(self, other: "Field") -> None:
        _L.check(_L.lib().smg_field_copy(other.h, self.h), "smg_field_copy", self.ctx.h)


def dot(a: Field, b: Field) -> np.ndarray:
    """sum conj(a) b per right-hand side (reference src/linalg.cpp:8-18)."""
    out = np.empty(2 * a.nrhs)
    _L.check(_L.lib().smg_blas_dot(a.h, b.h, _ptr(out)), "smg_blas_dot", a.ctx.h)
    return out[0::2] + 1j * out[1::2]


def norm(a: Field) -> np.ndarray:
    out = np.empty(a.nrhs)
    _L.check(_L.lib().smg_blas_norm(a.h, _ptr(out)), "smg_blas_norm", a.ctx.h)
    return out


def axpy(alpha, x: Field, y: Field) -> None:
    al = np.broadcast_to(np.asarray(alpha, dtype=np.complex128), (x.nrhs,)).copy()
    _L.check(_L.lib().smg_blas_axpy(_ptr(al.view(np.float64)), x.h, y.h), "smg_blas_axpy", x.ctx.h)


def scale(v: Field, alpha) -> None:
    al = np.broadcast_to(np.asarray(alpha, dtype=np.complex128), (v.nrhs,)).copy()
    _L.check(_L.lib().smg_blas_scale(_ptr(al.view(np.float64)), v.h), "smg_blas_scale", v.ctx.h)


class DiracOp(_Handle):
    """Wilson-clover Dirac operator (reference src/dirac.h:8-183) on the device."""

    def __init__(self, lat: Lattice, gauge: GaugeField, mass: float, r: float = 1.0, c_sw: float = 0.0,
                 mu_t: float = 0.0):
        self.lat = lat
        self.gauge = gauge
        self.mass, self.r, self.c_sw, self.mu_t = mass, r, c_sw, mu_t
        self.ctx = gauge.ctx
        h = C.c_void_p()
        _L.check(_L.lib().smg_dirac_create(gauge.h, mass, r, c_sw, mu_t, C.byref(h)), "smg_dirac_create",
                 self.ctx.h)
        self._adopt(h, gauge, _L.lib().smg_dirac_destroy)

    def refresh(self) -> None:
        """Recomputes the clover term after the gauge links changed."""
        _L.check(_L.lib().smg_dirac_refresh(self.h), "smg_dirac_refresh", self.ctx.h)

    @property
    def clover_field(self) -> np.ndarray:
        out = np.empty(self.lat.V)
        _L.check(_L.lib().smg_dirac_get_clover(self.h, _ptr(out)), "smg_dirac_get_clover", self.ctx.h)
        return out

    def apply_op(self, op: int, src, dst=None):
        """Applies op to a Field (device in, device out) or to host arrays."""
        if isinstance(src, Field):
            if dst is None:
                dst = Field(self.lat, src.nrhs, src.precision, self.ctx)
            _L.check(_L.lib().smg_dirac_apply(self.h, op, src.h, dst.h), "smg_dirac_apply", self.ctx.h)
            return dst
        a = _as_c128(src)
        nrhs = a.size // self.lat.ndof
        fs = Field(self.lat, nrhs, "f64", self.ctx, data=a)
        fd = Field(self.lat, nrhs, "f64", self.ctx)
        _L.check(_L.lib().smg_dirac_apply(self.h, op, fs.h, fd.h), "smg_dirac_apply", self.ctx.h)
        out = fd.download().reshape(a.shape)
        if dst is not None:
            dst[...] = out
            return dst
        return out

    def apply(self, src, dst=None):
        return self.apply_op(_L.OP_D, src, dst)

    def apply_delta_D(self, src, pi, dt: float) -> np.ndarray:
        """(D(e^{i dt pi} U) - D(U)) src through the hopping terms (reference src/dirac.h:154-174)."""
        a = _as_c128(src)
        nrhs = a.size // self.lat.ndof
        p = np.ascontiguousarray(pi, dtype=np.float64).reshape(-1)
        fs = Field(self.lat, nrhs, "f64", self.ctx, data=a)
        fd = Field(self.lat, nrhs, "f64", self.ctx)
        _L.check(_L.lib().smg_dirac_apply_delta(self.h, _ptr(p), dt, fs.h, fd.h), "smg_dirac_apply_delta", self.ctx.h)
        return fd.download().reshape(a.shape)

    def apply_dag(self, src, dst=None):
        return self.apply_op(_L.OP_DDAG, src, dst)

    def apply_DdagD(self, src, dst=None):
        return self.apply_op(_L.OP_DDAGD, src, dst)

    def apply_g5D(self, src, dst=None):
        return self.apply_op(_L.OP_G5D, src, dst)


class EvenOddDiracOp:
    """EvenOddDiracOp (reference src/dirac.h:190-553) on host half-lattice vectors:
    a half vector holds 2 * V/2 complex values in the reference's even_sites /
    odd_sites order.  Each call moves the halves into device fields, runs the
    sm_103a kernels and copies the result back."""

    def __init__(self, D: DiracOp):
        self.D = D
        self.lat = D.lat
        self.ctx = D.ctx

    # host-side layout helpers (scatter / gather_even / gather_odd, dirac.h:449-485)
    def scatter(self, half_e, half_o) -> np.ndarray:
        full = np.zeros((self.lat.V, 2), dtype=np.complex128)
        if half_e is not None:
            full[self.lat.even_sites] = _as_c128(half_e).reshape(-1, 2)
        if half_o is not None:
            full[self.lat.odd_sites] = _as_c128(half_o).reshape(-1, 2)
        return full.reshape(-1)

    def gather_even(self, full) -> np.ndarray:
        return _as_c128(full).reshape(-1, 2)[self.lat.even_sites].reshape(-1)

    def gather_odd(self, full) -> np.ndarray:
        return _as_c128(full).reshape(-1, 2)[self.lat.odd_sites].reshape(-1)

    def _run(self, op, half_e, half_o, out_parity):
        fs = Field(self.lat, 1, "f64", self.ctx, data=self.scatter(half_e, half_o))
        fd = Field(self.lat, 1, "f64", self.ctx)
        _L.check(_L.lib().smg_eo_apply(self.D.h, op, fs.h, fd.h), "smg_eo_apply", self.ctx.h)
        full = fd.download()
        return self.gather_odd(full) if out_parity else self.gather_even(full)

    def apply_schur(self, src_o):
        return self._run(_L.EO_SCHUR, None, src_o, 1)

    def apply_schur_dag(self, src_o):
        return self._run(_L.EO_SCHUR_DAG, None, src_o, 1)

    def apply_schur_dag_schur(self, src_o):
        return self._run(_L.EO_SCHUR_DAG_SCHUR, None, src_o, 1)

    def apply_eo(self, src_e):
        return self._run(_L.EO_HOP_EO, src_e, None, 1)

    def apply_oe(self, src_o):
        return self._run(_L.EO_HOP_OE, None, src_o, 0)

    def reconstruct(self, x_o, phi=None) -> np.ndarray:
        """Full solution from x_o: x_e = D_ee^-1 (phi_e - D_oe x_o) (reconstruct /
        reconstruct_full, dirac.h:499-540); returns the full vector."""
        fx = Field(self.lat, 1, "f64", self.ctx, data=self.scatter(None, x_o))
        fp = Field(self.lat, 1, "f64", self.ctx, data=_as_c128(phi)) if phi is not None else None
        _L.check(_L.lib().smg_eo_reconstruct(self.D.h, fp.h if fp is not None else None, fx.h),
                 "smg_eo_reconstruct", self.ctx.h)
        return fx.download()

    def log_det_ee(self) -> float:
        v = C.c_double(0)
        _L.check(_L.lib().smg_eo_logdet_ee(self.D.h, C.byref(v)), "smg_eo_logdet_ee", self.ctx.h)
        return v.value

    def generate_pseudofermion_eo(self, rng: "Rng") -> np.ndarray:
        """phi_o = M^dag eta_o with eta_o = random_vec(V, rng) (dirac.h:491-497)."""
        d = rng.normal(2 * self.lat.V)
        eta = d[1::2] + 1j * d[0::2]  # random_vec draws each entry's imaginary part first
        return self.apply_schur_dag(eta)

    def cg_solve(self, phi_o, max_iter: int, tol: float) -> "CGResult":
        """cg_solve on M^dag M over odd-site half vectors."""
        b = _as_c128(phi_o).reshape(-1)
        fb = Field(self.lat, 1, "f64", self.ctx, data=self.scatter(None, b))
        fx = Field(self.lat, 1, "f64", self.ctx)
        res = _L.SolveResult()
        st = _L.lib().smg_eo_cg_solve(self.D.h, fb.h, fx.h, max_iter, tol, C.byref(res))
        if st not in (_L.OK, _L.NOT_CONVERGED):
            _L.check(st, "smg_eo_cg_solve", self.ctx.h)
        return CGResult(self.gather_odd(fx.download()), res.iterations, res.final_residual, res.true_residual)

    def fermion_force(self, x_o) -> np.ndarray:
        """eo_fermion_force (src/hmc_forces.cpp:812-867) at x_o; returns F[mu][s]."""
        fx = Field(self.lat, 1, "f64", self.ctx, data=self.scatter(None, x_o))
        out = np.empty(2 * self.lat.V)
        _L.check(_L.lib().smg_eo_fermion_force(self.D.h, fx.h, _ptr(out)), "smg_eo_fermion_force", self.ctx.h)
        return out.reshape(2, self.lat.V)


@dataclass
class CGResult:
    """Mirrors CGResult / FCGResult (reference src/solvers.h:25-35) plus the FP64 true residual."""
    solution: np.ndarray
    iterations: int
    final_residual: float
    true_residual: float = float("nan")


def cg_solve(A: DiracOp, n: int, rhs, max_iter: int, tol: float, precision: str = "f64",
             raise_on_failure: bool = False) -> CGResult:
    """CG on D^dag D from x = 0 (reference src/solvers.cpp:75-78); `A` is the DiracOp."""
    b = _as_c128(rhs)
    nrhs = b.size // A.lat.ndof
    if n != A.lat.ndof:
        raise ValueError("n must equal 2*V")
    fb = Field(A.lat, nrhs, precision, A.ctx, data=b)
    fx = Field(A.lat, nrhs, precision, A.ctx)
    res = _L.SolveResult()
    st = _L.lib().smg_cg_solve(A.h, fb.h, fx.h, max_iter, tol, C.byref(res))
    if st != _L.OK and (raise_on_failure or st not in (_L.NOT_CONVERGED,)):
        _L.check(st, "smg_cg_solve", A.ctx.h)
    return CGResult(fx.download().reshape(b.shape), res.iterations, res.final_residual, res.true_residual)


def cg_solve_mixed(A: DiracOp, n: int, rhs, max_iter: int, tol: float) -> CGResult:
    """CG on D^dag D to a true FP64 residual below tol with FP32 CG inside FP64
    defect correction (same result contract as cg_solve in FP64)."""
    b = _as_c128(rhs)
    nrhs = b.size // A.lat.ndof
    if n != A.lat.ndof:
        raise ValueError("n must equal 2*V")
    fb = Field(A.lat, nrhs, "f64", A.ctx, data=b)
    fx = Field(A.lat, nrhs, "f64", A.ctx)
    res = _L.SolveResult()
    st = _L.lib().smg_cg_solve_mixed(A.h, fb.h, fx.h, max_iter, tol, C.byref(res))
    if st not in (_L.OK, _L.NOT_CONVERGED):
        _L.check(st, "smg_cg_solve_mixed", A.ctx.h)
    return CGResult(fx.download().reshape(b.shape), res.iterations, res.final_residual, res.true_residual)


def cg_solve_precond(A: DiracOp, n: int, rhs, precond: "MGHierarchy | None", max_iter: int, tol: float,
                     x0=None, precision: str = "f64") -> CGResult:
    """Preconditioned CG on D^dag D (reference cg_solve_precond / cg_solve_x0 /
    cg_solve_x0_precond, src/solvers.cpp:16-96): `precond` is an MGHierarchy
    (one cycle per iteration) or None; `x0` an optional start vector."""
    b = _as_c128(rhs)
    if n != A.lat.ndof:
        raise ValueError("n must equal 2*V")
    nrhs = b.size // A.lat.ndof
    fb = Field(A.lat, nrhs, precision, A.ctx, data=b)
    fx = Field(A.lat, nrhs, precision, A.ctx, data=_as_c128(x0) if x0 is not None else None)
    res = _L.SolveResult()
    st = _L.lib().smg_cg_solve_precond(A.h, precond.h if precond is not None else None, fb.h, fx.h,
                                       int(x0 is not None), max_iter, tol, C.byref(res))
    if st not in (_L.OK, _L.NOT_CONVERGED):
        _L.check(st, "smg_cg_solve_precond", A.ctx.h)
    return CGResult(fx.download().reshape(b.shape), res.iterations, res.final_residual, res.true_residual)


def mr_smooth(D: DiracOp, x, b, niter: int) -> np.ndarray:
    """mr_smooth (reference src/smoother.cpp:9-23) on D^dag D from the start vector x."""
    bb = _as_c128(b)
    nrhs = bb.size // D.lat.ndof
    fb = Field(D.lat, nrhs, "f64", D.ctx, data=bb)
    fx = Field(D.lat, nrhs, "f64", D.ctx, data=_as_c128(x))
    _L.check(_L.lib().smg_mr_smooth(D.h, fb.h, fx.h, niter), "smg_mr_smooth", D.ctx.h)
    return fx.download().reshape(bb.shape)


def richardson_smooth(D: DiracOp, x, b, niter: int, omega: float) -> np.ndarray:
    """richardson_smooth_op (reference src/smoother.cpp:64-73) on D^dag D from the start vector x."""
    bb = _as_c128(b)
    nrhs = bb.size // D.lat.ndof
    fb = Field(D.lat, nrhs, "f64", D.ctx, data=bb)
    fx = Field(D.lat, nrhs, "f64", D.ctx, data=_as_c128(x))
    _L.check(_L.lib().smg_richardson_smooth(D.h, fb.h, fx.h, niter, omega), "smg_richardson_smooth", D.ctx.h)
    return fx.download().reshape(bb.shape)


def estimate_lambda_max(D: DiracOp, niter: int = 30) -> float:
    """estimate_lambda_max of D^dag D (reference src/smoother.cpp:43-60)."""
    v = C.c_double(0)
    _L.check(_L.lib().smg_estimate_lambda_max(D.h, niter, C.byref(v)), "smg_estimate_lambda_max", D.ctx.h)
    return v.value


def fermion_action(D: DiracOp, phi, max_iter: int, tol: float, precond: "MGHierarchy | None" = None):
    """Forward pass (fermion_action / fermion_action_precond, src/hmc_forces.cpp:113-131):
    returns (S = Re <phi, X>, X = (D^dag D)^-1 phi as a device Field, iterations).
    fermion_force(D, X) is the backward pass."""
    p = _as_c128(phi)
    nrhs = p.size // D.lat.ndof
    fp = Field(D.lat, nrhs, "f64", D.ctx, data=p)
    fx = Field(D.lat, nrhs, "f64", D.ctx)
    S = np.zeros(nrhs)
    res = _L.SolveResult()
    _L.check(_L.lib().smg_fermion_action(D.h, precond.h if precond is not None else None, fp.h, fx.h, max_iter, tol,
                                         _ptr(S), C.byref(res)), "smg_fermion_action", D.ctx.h)
    return (S[0] if nrhs == 1 else S), fx, res.iterations


def fermion_force(D: DiracOp, X) -> np.ndarray:
    """F[mu][s] = -dS/dtheta for S = phi^dag (D^dag D)^-1 phi at X = (D^dag D)^-1 phi
    (reference src/hmc_forces.cpp:134-495)."""
    fx = X if isinstance(X, Field) else Field(D.lat, 1, "f64", D.ctx, data=X)
    out = np.empty(2 * D.lat.V)
    _L.check(_L.lib().smg_fermion_force(D.h, fx.h, _ptr(out)), "smg_fermion_force", D.ctx.h)
    return out.reshape(2, D.lat.V)


def gauge_force(g: GaugeField, beta: float) -> np.ndarray:
    out = np.empty(2 * g.lat.V)
    _L.check(_L.lib().smg_gauge_force(g.h, beta, _ptr(out)), "smg_gauge_force", g.ctx.h)
    return out.reshape(2, g.lat.V)


def gauge_action(g: GaugeField, beta: float) -> float:
    v = C.c_double()
    _L.check(_L.lib().smg_gauge_action(g.h, beta, C.byref(v)), "smg_gauge_action", g.ctx.h)
    return v.value


# ---------------------------------------------------------------- HMC
class Rng(_Handle):
    """The reference's std::mt19937 threaded through HMC trajectories."""

    def __init__(self, seed: int):
        h = C.c_void_p()
        _L.check(_L.lib().smg_rng_create(seed, C.byref(h)), "smg_rng_create")
        self.ctx = None
        self._adopt(h, None, _L.lib().smg_rng_destroy)

    def uniform(self) -> float:
        v = C.c_double()
        _L.check(_L.lib().smg_rng_uniform(self.h, C.byref(v)), "smg_rng_uniform")
        return v.value

    def normal(self, n: int) -> np.ndarray:
        """n draws of one fresh std::normal_distribution (as MomentumField::randomise)."""
        out = np.empty(n)
        _L.check(_L.lib().smg_rng_normal(self.h, n, _ptr(out)), "smg_rng_normal")
        return out


def hmc_params(beta: float, tau: float = 1.0, n_steps: int = 10, omelyan: bool = True, n_inner: int = 0,
               cg_maxiter: int = 10000, cg_tol: float = 1e-10, c_sw: float = 0.0, mu_t: float = 0.0,
               force_accept: bool = False, mixed_precision: bool = False, use_eo: bool = False) -> _L.HMCParams:
    """smg_hmc_params from the reference's HMCParams fields (src/hmc.h:107-119); n_inner > 0
    selects the nested integrator with n_inner gauge-force steps between fermion-force kicks;
    use_eo the reference's even-odd (Schur complement) trajectory."""
    p = _L.HMCParams()
    _L.check(_L.lib().smg_hmc_params_default(C.byref(p)), "smg_hmc_params_default")
    p.beta, p.tau, p.n_steps, p.omelyan, p.n_inner = beta, tau, n_steps, int(omelyan), n_inner
    p.cg_maxiter, p.cg_tol, p.c_sw, p.mu_t = cg_maxiter, cg_tol, c_sw, mu_t
    p.force_accept, p.mixed_precision, p.use_eo = int(force_accept), int(mixed_precision), int(use_eo)
    return p


@dataclass
class HMCResult:
    """HMCResult (reference src/hmc.h:121-129) plus the plaquette and the number of solves."""
    accepted: bool
    dH: float
    dKE: float
    dSG: float
    dSF: float
    total_cg_iters: int
    solves: int
    plaquette: float
    dLD: float = 0.0


def hmc_trajectory(g: GaugeField, mass: float, wilson_r: float, params: _L.HMCParams, rng: Rng) -> HMCResult:
    """One HMC trajectory on the device (reference hmc_trajectory, src/hmc_trajectory.cpp:38-235);
    the links of `g` are updated in place (restored on rejection)."""
    r = _L.HMCResult()
    _L.check(_L.lib().smg_hmc_trajectory(g.h, mass, wilson_r, C.byref(params), rng.h, C.byref(r)),
             "smg_hmc_trajectory", g.ctx.h)
    return HMCResult(bool(r.accepted), r.dH, r.dKE, r.dSG, r.dSF, r.total_cg_iters, r.solves, r.plaquette, r.dLD)


@dataclass
class ReversibilityResult:
    """ReversibilityResult (reference src/hmc.h:402-408) plus the number of solves."""
    gauge_delta: float
    mom_delta: float
    dH_forward: float
    dH_backward: float
    total_cg_iters: int
    solves: int


def hmc_reversibility(g: GaugeField, mass: float, wilson_r: float, params: _L.HMCParams,
                      rng: Rng) -> ReversibilityResult:
    """reversibility_test_plain (reference src/hmc_trajectory.cpp:416-509): forward molecular
    dynamics, momentum flip, backward; the links of `g` are restored afterwards."""
    r = _L.ReversibilityResult()
    _L.check(_L.lib().smg_hmc_reversibility(g.h, mass, wilson_r, C.byref(params), rng.h, C.byref(r)),
             "smg_hmc_reversibility", g.ctx.h)
    return ReversibilityResult(r.gauge_delta, r.mom_delta, r.dH_forward, r.dH_backward, r.total_cg_iters, r.solves)


def coarse_lowmode_force(D: DiracOp, mg: MGHierarchy, phi, smooth_iters: int = 0) -> np.ndarray:
    """coarse_lowmode_force (reference src/hmc_multiscale.cpp:237-276); returns F[mu][s]."""
    f = Field(D.lat, 1, "f64", D.ctx, data=phi)
    out = np.empty(2 * D.lat.V)
    _L.check(_L.lib().smg_coarse_lowmode_force(D.h, mg.h, f.h, smooth_iters, _ptr(out)), "smg_coarse_lowmode_force",
             D.ctx.h)
    return out.reshape(2, D.lat.V)


def verify_forces(g: GaugeField, beta: float, mass: float, wilson_r: float = 1.0, max_iter: int = 10000,
                  tol: float = 1e-12, c_sw: float = 0.0, use_eo: bool = False, err_threshold: float = 1e-4,
                  mu_t: float = 0.0) -> _L.ForceCheck:
    """verify_forces (reference src/hmc_forces.cpp:869-981) on the device: analytic gauge and
    fermion forces against central differences at the reference's 20 links; `.passed` is its
    return value, the per-link values are in gf_ana/gf_num/ff_ana/ff_num."""
    out = _L.ForceCheck()
    _L.check(_L.lib().smg_verify_forces(g.h, beta, mass, wilson_r, max_iter, tol, c_sw, int(use_eo), err_threshold,
                                        mu_t, C.byref(out)), "smg_verify_forces", g.ctx.h)
    return out


OUTER_INTEGRATORS = {"leapfrog": 0, "omelyan": 1, "fgi": 2, "fgi_qpqpq": 3}


def ms_params(beta: float, tau: float = 1.0, n_outer: int = 4, n_inner: int = 5, cg_maxiter: int = 500,
              cg_tol: float = 1e-10, inner_smooth: int = 3, outer="leapfrog", c_sw: float = 0.0,
              mu_t: float = 0.0) -> _L.MSParams:
    """smg_ms_params from MGMultiScaleParams (reference src/hmc.h:338-357)."""
    p = _L.MSParams()
    _L.check(_L.lib().smg_ms_params_default(C.byref(p)), "smg_ms_params_default")
    p.beta, p.tau, p.n_outer, p.n_inner = beta, tau, n_outer, n_inner
    p.cg_maxiter, p.cg_tol, p.inner_smooth = cg_maxiter, cg_tol, inner_smooth
    p.outer_type = OUTER_INTEGRATORS[outer] if isinstance(outer, str) else int(outer)
    p.c_sw, p.mu_t = c_sw, mu_t
    return p


@dataclass
class MSResult:
    """MGMultiScaleResult (reference src/hmc.h:359-367) plus the plaquette and the number of solves."""
    accepted: bool
    dH: float
    dKE: float
    dSG: float
    dSF: float
    highmode_cg_iters: int
    lowmode_force_evals: int
    solves: int
    plaquette: float


def hmc_mg_multiscale(g: GaugeField, mass: float, wilson_r: float, params: _L.MSParams, mg: MGHierarchy,
                      rng: Rng) -> MSResult:
    """hmc_trajectory_mg_multiscale (reference src/hmc_multiscale.cpp:340-886) on the device."""
    r = _L.MSResult()
    _L.check(_L.lib().smg_hmc_mg_multiscale(g.h, mass, wilson_r, C.byref(params), mg.h, rng.h, C.byref(r)),
             "smg_hmc_mg_multiscale", g.ctx.h)
    return MSResult(bool(r.accepted), r.dH, r.dKE, r.dSG, r.dSF, r.highmode_cg_iters, r.lowmode_force_evals, r.solves,
                    r.plaquette)


def hmc_mg_multiscale_reversibility(g: GaugeField, mass: float, wilson_r: float, params: _L.MSParams,
                                    mg: MGHierarchy, rng: Rng) -> ReversibilityResult:
    """reversibility_test_mg_multiscale (reference src/hmc_multiscale.cpp:963-1000)."""
    r = _L.ReversibilityResult()
    _L.check(_L.lib().smg_hmc_mg_multiscale_reversibility(g.h, mass, wilson_r, C.byref(params), mg.h, rng.h,
                                                          C.byref(r)),
             "smg_hmc_mg_multiscale_reversibility", g.ctx.h)
    return ReversibilityResult(r.gauge_delta, r.mom_delta, r.dH_forward, r.dH_backward, r.total_cg_iters, r.solves)


# ---------------------------------------------------------------- host inputs
def save_gauge(g: "GaugeField | np.ndarray", beta: float, mass: float, path, avg_plaq: float | None = None) -> None:
    """save_gauge (reference src/hmc_forces.cpp:18-35): the "SWNG" file.  `g` is a
    device GaugeField (its plaquette goes into the header) or host links [2][V]."""
    p = str(path).encode()
    if isinstance(g, GaugeField):
        _L.check(_L.lib().smg_gauge_save(g.h, beta, mass, p), "smg_gauge_save", g.ctx.h)
        return
    U = _as_c128(g).reshape(-1)
    L = int(round((U.size // 2) ** 0.5))
    _L.check(_L.lib().smg_host_gauge_write_swng(p, L, _ptr(U.view(np.float64)), beta, mass,
                                                float(avg_plaq if avg_plaq is not None else 0.0)),
             "smg_host_gauge_write_swng")


def load_gauge(path, L: int = 0):
    """load_gauge (reference src/hmc_forces.cpp:37-62): returns (links [2][V] divided by their
    modulus, header dict).  L > 0 checks the lattice size like the reference."""
    p = str(path).encode()
    hdr = _L.GaugeHeader()
    _L.check(_L.lib().smg_host_gauge_read_swng(p, L, C.byref(hdr), None), "smg_host_gauge_read_swng")
    n = int(hdr.L)
    U = np.empty(2 * n * n, dtype=np.complex128)
    _L.check(_L.lib().smg_host_gauge_read_swng(p, n, C.byref(hdr), _ptr(U.view(np.float64))),
             "smg_host_gauge_read_swng")
    return U.reshape(2, n * n), dict(L=n, beta=hdr.beta, mass=hdr.mass, avg_plaq=hdr.avg_plaq)


def save_gauge_raw(U, path) -> None:
    """GaugeField::save (reference src/gauge.h:38-46): int32 V, then the links."""
    U = _as_c128(U).reshape(-1)
    L = int(round((U.size // 2) ** 0.5))
    _L.check(_L.lib().smg_host_gauge_write_raw(str(path).encode(), L, _ptr(U.view(np.float64))),
             "smg_host_gauge_write_raw")


def load_gauge_raw(path, L: int) -> np.ndarray:
    """GaugeField::load (reference src/gauge.h:48-57)."""
    U = np.empty(2 * L * L, dtype=np.complex128)
    _L.check(_L.lib().smg_host_gauge_read_raw(str(path).encode(), L, _ptr(U.view(np.float64))),
             "smg_host_gauge_read_raw")
    return U.reshape(2, L * L)


def gauge_normal(L: int, beta: float, seed: int) -> np.ndarray:
    """U = exp(i theta), theta ~ N(0, 1/beta) from std::mt19937(seed); shape (2, V)."""
    out = np.empty(2 * L * L, dtype=np.complex128)
    _L.check(_L.lib().smg_host_gauge_normal(L, beta, seed, _ptr(out.view(np.float64))), "smg_host_gauge_normal")
    return out.reshape(2, L * L)


def random_vec(n: int, seed: int) -> np.ndarray:
    """random_vec(n, std::mt19937(seed)) (reference src/linalg.cpp:44-48)."""
    out = np.empty(n, dtype=np.complex128)
    _L.check(_L.lib().smg_host_random_vec(n, seed, _ptr(out.view(np.float64))), "smg_host_random_vec")
    return out


# ---------------------------------------------------------------- multigrid
def mg_params(n_levels: int = 2, block_size: int = 4, k_null: int = 4, coarse_block=(4, 1), null_iters: int = 20,
              w_cycle: bool = True, pre_smooth: int = 3, post_smooth: int = 3, chiral_split: bool = False,
              blocks=None, n_vecs=None, null_mr_steps: int = 5, coarse_max_iter: int = 200,
              coarse_tol: float = 1e-12, precision: str = "f64", seed: int = 42,
              tensor_cores: bool = True, smoother_half: bool = False, coarse_half: bool = False) -> _L.MGParams:
    """smg_mg_params from the reference's build_mg_hierarchy arguments
    (src/multigrid.cpp:595-602).  `blocks` / `n_vecs` override the per-level
    aggregate shapes and null-vector counts.  `tensor_cores` lets an F32
    hierarchy apply its batched coarse operators on the tensor cores;
    `smoother_half` keeps its fine smoother's work vectors in FP16 with
    per-site scales; `coarse_half` does the same (scales per coarse site and
    half of the 32 right-hand sides) for the coarsest-level CG's residual and
    search directions and the intermediate levels' MR residuals."""
    p = _L.MGParams()
    _L.check(_L.lib().smg_mg_params_default(C.byref(p)), "smg_mg_params_default")
    p.n_levels = n_levels
    for l in range(_L.MAX_LEVELS - 1):
        b = (blocks[l] if blocks is not None and l < len(blocks) else
             ((block_size, block_size) if l == 0 else tuple(coarse_block)))
        p.block[l][0], p.block[l][1] = int(b[0]), int(b[1])
        p.n_vec[l] = int(n_vecs[l] if n_vecs is not None and l < len(n_vecs) else k_null)
    p.chiral_split = int(chiral_split)
    p.null_iters = null_iters
    p.null_mr_steps = null_mr_steps
    p.pre_smooth, p.post_smooth = pre_smooth, post_smooth
    p.w_cycle = int(w_cycle)
    p.coarse_max_iter, p.coarse_tol = coarse_max_iter, coarse_tol
    p.precision = PRECISIONS[precision]
    p.seed = seed
    p.tensor_cores = int(tensor_cores)
    p.smoother_half = int(smoother_half)
    p.coarse_half = int(coarse_half)
    return p


class MGHierarchy(_Handle):
    """MG preconditioner for D^dag D (MGHierarchy, reference src/multigrid.h:41-107)."""

    def __init__(self, D: DiracOp, params: _L.MGParams | None = None, warm_start=None):
        self.D = D
        self.ctx = D.ctx
        self.params = params if params is not None else mg_params()
        h = C.c_void_p()
        warm = None
        if warm_start is not None:
            warm = _as_c128(warm_start).reshape(-1)
            if warm.size != self.params.n_vec[0] * D.lat.ndof:
                raise ValueError("warm_start must hold n_vec[0] fine vectors")
        wp = _ptr(warm.view(np.float64)) if warm is not None else None
        _L.check(_L.lib().smg_mg_create(D.h, C.byref(self.params), wp, C.byref(h)), "smg_mg_create", self.ctx.h)
        self._adopt(h, D, _L.lib().smg_mg_destroy)

    @property
    def n_levels(self) -> int:
        return self.params.n_levels

    def level_dims(self, level: int):
        nx, ny, nd = C.c_int(), C.c_int(), C.c_int()
        _L.check(_L.lib().smg_mg_level_dims(self.h, level, C.byref(nx), C.byref(ny), C.byref(nd)),
                 "smg_mg_level_dims", self.ctx.h)
        return nx.value, ny.value, nd.value

    def level_dim(self, level: int) -> int:
        nx, ny, nd = self.level_dims(level)
        return nx * ny * nd

    @property
    def null_vecs_l0(self) -> np.ndarray:
        k = self.params.n_vec[0]
        out = np.empty(k * self.D.lat.ndof, dtype=np.complex128)
        _L.check(_L.lib().smg_mg_null_vectors(self.h, _ptr(out.view(np.float64))), "smg_mg_null_vectors", self.ctx.h)
        return out.reshape(k, -1)

    def prolongator(self, level: int = 0) -> np.ndarray:
        """block_vecs in the reference layout [block][k][local dof]."""
        n = self.level_dim(level) * self.level_dims(level + 1)[2]
        out = np.empty(n, dtype=np.complex128)
        _L.check(_L.lib().smg_mg_get_prolongator(self.h, level, _ptr(out.view(np.float64))),
                 "smg_mg_get_prolongator", self.ctx.h)
        return out

    def coarse_op(self, level: int = 1) -> np.ndarray:
        """SparseCoarseOp::link layout [site][dir][ki*k + kj]."""
        nx, ny, nd = self.level_dims(level)
        out = np.empty(nx * ny * 9 * nd * nd, dtype=np.complex128)
        _L.check(_L.lib().smg_mg_get_coarse_op(self.h, level, _ptr(out.view(np.float64))), "smg_mg_get_coarse_op",
                 self.ctx.h)
        return out

    def _host_op(self, fn, level, v, out_dim):
        v = _as_c128(v).reshape(-1)
        out = np.empty(out_dim, dtype=np.complex128)
        _L.check(getattr(_L.lib(), fn)(self.h, level, _ptr(v.view(np.float64)), _ptr(out.view(np.float64))), fn,
                 self.ctx.h)
        return out

    def prolong(self, level: int, coarse):
        return self._host_op("smg_mg_prolong_host", level, coarse, self.level_dim(level))

    def restrict_vec(self, level: int, fine):
        return self._host_op("smg_mg_restrict_host", level, fine, self.level_dim(level + 1))

    def coarse_apply(self, level: int, v):
        return self._host_op("smg_mg_coarse_apply_host", level, v, self.level_dim(level))

    def coarse_apply_batch(self, level: int, v, engine: str = "cuda", w=None, dots: bool = False):
        """Batched coarse operator of an F32 hierarchy on a complex64 array
        [site][dof][rhs] (sites lexicographic on the coarse lattice).  engine
        "cuda" (FP32 CUDA cores) or "tensor" (BF16 tensor cores, FP32
        accumulation).  With dots, also returns per rhs ||Av||^2, or
        (<Av, w>, ||Av||^2) when w is given."""
        nx, ny, nd = self.level_dims(level)
        a = np.ascontiguousarray(v, dtype=np.complex64)
        nrhs = a.size // (nx * ny * nd)
        if a.size != nx * ny * nd * nrhs:
            raise ValueError("input size is not a multiple of the coarse vector size")
        out = np.empty_like(a)
        fp = C.POINTER(C.c_float)
        wa = None if w is None else np.ascontiguousarray(w, dtype=np.complex64)
        k = 3 if wa is not None else 1
        d = np.zeros(nrhs * k) if dots else None
        _L.check(_L.lib().smg_mg_coarse_apply_batch(
            self.h, level, nrhs, {"cuda": 0, "tensor": 1}[engine], a.ctypes.data_as(fp),
            None if wa is None else wa.ctypes.data_as(fp), out.ctypes.data_as(fp),
            None if d is None else d.ctypes.data_as(C.POINTER(C.c_double))), "smg_mg_coarse_apply_batch", self.ctx.h)
        if not dots:
            return out
        d = d.reshape(nrhs, k)
        if wa is None:
            return out, d[:, 0]
        return out, d[:, 0] + 1j * d[:, 1], d[:, 2]

    def precondition(self, b):
        """One MG cycle x = M^-1 b (MGHierarchy::precondition, src/multigrid.cpp:155)."""
        if isinstance(b, Field):
            x = Field(self.D.lat, b.nrhs, b.precision, self.ctx)
            _L.check(_L.lib().smg_mg_precondition(self.h, b.h, x.h), "smg_mg_precondition", self.ctx.h)
            return x
        a = _as_c128(b)
        nrhs = a.size // self.D.lat.ndof
        prec = "f64" if self.params.precision == _L.F64 else "f32"
        fb = Field(self.D.lat, nrhs, prec, self.ctx, data=a)
        fx = Field(self.D.lat, nrhs, prec, self.ctx)
        _L.check(_L.lib().smg_mg_precondition(self.h, fb.h, fx.h), "smg_mg_precondition", self.ctx.h)
        return fx.download().reshape(a.shape)


    def setup_deflation(self, n_ev: int, n_kr: int = 0, max_restarts: int = 100, tol: float = 1e-10,
                        allow_unconverged: bool = False, level: int = 1) -> _L.DeflationInfo:
        """SparseCoarseOp::setup_deflation (src/coarse_op.cpp:10-54, TRLM): the n_ev lowest
        eigenpairs of the level-1 operator (or of `level`); when that level is the coarsest, the
        coarsest CG of every cycle starts from the deflated guess."""
        info = _L.DeflationInfo()
        self._defl_level = level
        st = _L.lib().smg_mg_setup_deflation_level(self.h, level, n_ev, n_kr, max_restarts, tol, C.byref(info))
        if not (allow_unconverged and st == _L.NOT_CONVERGED):
            _L.check(st, "smg_mg_setup_deflation", self.ctx.h)
        return info

    def set_deflation(self, vals, vecs) -> None:
        """Installs eigenpairs (vectors in the reference's coarse layout, one per row)."""
        vals = np.ascontiguousarray(vals, dtype=np.float64).reshape(-1)
        vecs = _as_c128(vecs).reshape(len(vals), -1)
        self._defl_level = 1
        _L.check(_L.lib().smg_mg_set_deflation(self.h, len(vals), _ptr(vals), _ptr(vecs.view(np.float64))),
                 "smg_mg_set_deflation", self.ctx.h)

    @property
    def deflation(self):
        """(eigenvalues, eigenvectors [n][level-1 dim]) of the deflation space."""
        n = C.c_int()
        _L.check(_L.lib().smg_mg_get_deflation(self.h, C.byref(n), None, None), "smg_mg_get_deflation", self.ctx.h)
        vals = np.empty(n.value)
        vecs = np.empty((n.value, self.level_dim(getattr(self, "_defl_level", 1))), dtype=np.complex128)
        if n.value:
            _L.check(_L.lib().smg_mg_get_deflation(self.h, C.byref(n), _ptr(vals), _ptr(vecs.view(np.float64))),
                     "smg_mg_get_deflation", self.ctx.h)
        return vals, vecs

    def deflation_rr(self) -> float:
        """rr_evolve (src/eigen_evolve.cpp:48-105) of the deflation space on the current level-1
        operator; returns the largest relative eigen-residual."""
        out = C.c_double()
        _L.check(_L.lib().smg_mg_deflation_rr(self.h, C.byref(out)), "smg_mg_deflation_rr", self.ctx.h)
        return out.value

    def lowmode_solution(self, phi) -> np.ndarray:
        """CoarseDeflState::lowmode_solution (src/hmc.h:312-323): P sum_i v_i v_i^dag / lambda_i P^dag phi."""
        lat = self.D.lat
        f = Field(lat, 1, "f64", self.ctx, data=phi)
        x = Field(lat, 1, "f64", self.ctx)
        _L.check(_L.lib().smg_mg_lowmode_solution(self.h, f.h, x.h), "smg_mg_lowmode_solution", self.ctx.h)
        return x.download()

    def rebuild(self) -> None:
        """rebuild_deeper_levels (src/multigrid.cpp:158-193): the coarse operators from the current
        links of the Dirac operator (refresh it after changing its gauge field) and the existing
        prolongators."""
        _L.check(_L.lib().smg_mg_rebuild(self.h), "smg_mg_rebuild", self.ctx.h)

    def estimate_lambda_max(self, level: int = 0, niter: int = 30) -> float:
        """estimate_lambda_max (src/smoother.cpp:43-60) of the level operator."""
        v = C.c_double(0)
        _L.check(_L.lib().smg_mg_estimate_lambda_max(self.h, level, niter, C.byref(v)),
                 "smg_mg_estimate_lambda_max", self.ctx.h)
        return v.value

    def set_symmetric(self, damping: float = 0.8) -> np.ndarray:
        """MGHierarchy::set_symmetric (src/multigrid.cpp:144-152): Richardson
        smoothing with omega = damping / lambda_max per level; returns the omegas."""
        om = np.zeros(max(1, self.n_levels - 1))
        _L.check(_L.lib().smg_mg_set_symmetric(self.h, damping, _ptr(om)), "smg_mg_set_symmetric", self.ctx.h)
        return om


def build_mg_hierarchy(D: DiracOp, n_levels: int, block_size: int, k_null: int, coarse_block_agg: int,
                       null_iters: int, seed: int, w_cycle: bool = True, pre_smooth: int = 3, post_smooth: int = 3,
                       warm_start=None, **kw) -> MGHierarchy:
    """build_mg_hierarchy (reference src/multigrid.cpp:595-687).  The
    reference's rng argument is `seed` (std::mt19937(seed)); its deeper-level
    linear blocking of coarse_block_agg = 4*k_null dofs is the 4 x 1 aggregate."""
    agg = max(1, coarse_block_agg // max(1, k_null))
    p = mg_params(n_levels, block_size, k_null, (agg, 1), null_iters, w_cycle, pre_smooth, post_smooth, seed=seed,
                  **kw)
    return MGHierarchy(D, p, warm_start)


def build_full_mg(D: DiracOp, mg_levels: int = 1, block_size: int = 4, k_null: int = 4, coarse_block: int = 0,
                  w_cycle: bool = True, pre_smooth: int = 3, post_smooth: int = 3, seed: int = 42, warm_start=None,
                  **kw) -> MGHierarchy:
    """build_full_mg (reference src/mg_builder.cpp:3-31) with the trlm null-space
    path: 20 inverse iterations, or 5 when warm-started."""
    cb = coarse_block if coarse_block > 0 else 4 * k_null
    iters = 5 if warm_start is not None else 20
    return build_mg_hierarchy(D, max(2, mg_levels), block_size, k_null, cb, iters, seed, w_cycle, pre_smooth,
                              post_smooth, warm_start, **kw)


@dataclass
class FCGResult:
    """FCGResult (reference src/solvers.h:31-35) plus the FP64 true residual."""
    solution: np.ndarray
    iterations: int
    final_residual: float
    true_residual: float = float("nan")
    status: int = 0


def fcg_solve(A: DiracOp, n: int, rhs, precond: "MGHierarchy | None", max_iter: int, tol: float, trunc: int = 30,
              precision: str = "f64", reference_coefficient: bool = False) -> FCGResult:
    """Truncated GCR on D^dag D (reference fcg_solve, src/solvers.cpp:223-300);
    `precond` is an MGHierarchy (one cycle per iteration) or None."""
    b = _as_c128(rhs)
    if n != A.lat.ndof:
        raise ValueError("n must equal 2*V")
    nrhs = b.size // A.lat.ndof
    fb = Field(A.lat, nrhs, precision, A.ctx, data=b)
    fx = Field(A.lat, nrhs, precision, A.ctx)
    res = _L.SolveResult()
    st = _L.lib().smg_gcr_solve(A.h, precond.h if precond is not None else None, fb.h, fx.h, max_iter, tol, trunc,
                                int(reference_coefficient), C.byref(res))
    if st not in (_L.OK, _L.NOT_CONVERGED):
        _L.check(st, "smg_gcr_solve", A.ctx.h)
    return FCGResult(fx.download().reshape(b.shape), res.iterations, res.final_residual, res.true_residual, st)


def fcg_solve_mg(A: DiracOp, n: int, rhs, mg: MGHierarchy, max_iter: int, tol: float, truncation: int = 20,
                 **kw) -> FCGResult:
    """fcg_solve_mg (reference src/solvers.cpp:803-811)."""
    return fcg_solve(A, n, rhs, mg, max_iter, tol, truncation, **kw)


@dataclass
class FGMRESResult:
    """FGMRESResult (reference src/solvers.h:18-23): Ritz values per right-hand
    side stand in for ritz_pairs (the vectors stay on the device)."""
    solution: np.ndarray
    iterations: int
    final_residual: float
    ritz_values: list
    status: int = 0


def fgmres_solve(A: DiracOp, n: int, rhs, precond: "MGHierarchy | None", restart: int, max_iter: int, tol: float,
                 n_ritz_harvest: int = 4, precision: str = "f64") -> FGMRESResult:
    """Restarted flexible GMRES on D^dag D (reference fgmres_solve_generic,
    src/solvers.cpp:555-773) with one MG cycle per step (`precond`) or none."""
    b = _as_c128(rhs)
    if n != A.lat.ndof:
        raise ValueError("n must equal 2*V")
    nrhs = b.size // A.lat.ndof
    fb = Field(A.lat, nrhs, precision, A.ctx, data=b)
    fx = Field(A.lat, nrhs, precision, A.ctx)
    res = _L.SolveResult()
    vals = np.zeros(nrhs * 3 * max(1, n_ritz_harvest))
    cnt = (C.c_int * nrhs)()
    st = _L.lib().smg_fgmres_solve(A.h, precond.h if precond is not None else None, fb.h, fx.h, restart, max_iter,
                                   tol, n_ritz_harvest, C.byref(res), _ptr(vals), cnt)
    if st not in (_L.OK, _L.NOT_CONVERGED):
        _L.check(st, "smg_fgmres_solve", A.ctx.h)
    vals = vals.reshape(nrhs, -1)
    ritz = [list(vals[j, :cnt[j]]) for j in range(nrhs)]
    return FGMRESResult(fx.download().reshape(b.shape), res.iterations, res.true_residual,
                        ritz[0] if nrhs == 1 else ritz, st)


def fgmres_solve_mg(A: DiracOp, n: int, rhs, mg: MGHierarchy, restart: int, max_iter: int, tol: float,
                    n_ritz_harvest: int = 4, **kw) -> FGMRESResult:
    """fgmres_solve_mg (reference src/solvers.cpp:776-787)."""
    return fgmres_solve(A, n, rhs, mg, restart, max_iter, tol, n_ritz_harvest, **kw)


class LatticeBatch:
    """Independent lattices of uneven size solved together on one GPU (smg_batch_*):
    one stream per lattice, n_workers host threads over one largest-first queue."""

    def __init__(self, n_workers: int = 8, device: int = 0):
        h = C.c_void_p()
        _L.check(_L.lib().smg_batch_create(device, n_workers, C.byref(h)), "smg_batch_create")
        self.h = h
        self.lattices = []  # (L, nrhs)
        self._keep = []

    def add(self, L: int, U, mass: float, c_sw: float = 0.0, wilson_r: float = 1.0, mu_t: float = 0.0,
            nrhs: int = 1) -> int:
        Ua = _as_c128(U).reshape(-1)
        i = C.c_int(0)
        _L.check(_L.lib().smg_batch_add(self.h, L, _ptr(Ua.view(np.float64)), mass, wilson_r, c_sw, mu_t, nrhs,
                                        C.byref(i)), "smg_batch_add")
        self.lattices.append((L, nrhs))
        return i.value

    def setup(self, params: _L.MGParams) -> None:
        _L.check(_L.lib().smg_batch_setup(self.h, C.byref(params)), "smg_batch_setup")

    def bind(self, i: int, rhs, x_out: np.ndarray | None = None, force_out: np.ndarray | None = None) -> None:
        """rhs: host array (nrhs, 2V) complex, uploaded now; x_out / force_out: host arrays the
        host_io solves write (kept referenced by the batch)."""
        r = _as_c128(rhs).reshape(-1)
        self._keep += [r, x_out, force_out]
        _L.check(_L.lib().smg_batch_bind_host(self.h, i, _ptr(r.view(np.float64)),
                                              _ptr(x_out.view(np.float64)) if x_out is not None else None,
                                              _ptr(force_out) if force_out is not None else None),
                 "smg_batch_bind_host")

    def solve(self, max_iter: int, tol: float, trunc: int = 20, with_force: bool = True,
              host_io: bool = False) -> tuple[int, float]:
        sec = C.c_double(0)
        st = _L.lib().smg_batch_solve(self.h, max_iter, tol, trunc, int(with_force), int(host_io), C.byref(sec))
        return st, sec.value

    def result(self, i: int):
        r = _L.SolveResult()
        st = C.c_int(0)
        sec = C.c_double(0)
        _L.check(_L.lib().smg_batch_result(self.h, i, C.byref(r), C.byref(st), C.byref(sec)), "smg_batch_result")
        return st.value, r, sec.value

    def download(self, i: int):
        L, nrhs = self.lattices[i]
        x = np.empty(nrhs * 2 * L * L, dtype=np.complex128)
        F = np.empty(2 * L * L)
        _L.check(_L.lib().smg_batch_download(self.h, i, _ptr(x.view(np.float64)), _ptr(F)), "smg_batch_download")
        return x.reshape(nrhs, 2 * L * L), F.reshape(2, L * L)

    @property
    def kernel_launches(self) -> int:
        n = C.c_uint64(0)
        _L.check(_L.lib().smg_batch_kernel_launches(self.h, C.byref(n)), "smg_batch_kernel_launches")
        return n.value

    def close(self) -> None:
        if self.h:
            _L.lib().smg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
