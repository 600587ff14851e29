"""ctypes binding of libsmg_gpu.so (the C ABI declared in include/smg_gpu.h).

The library is loaded from this package directory only.  There is no CPU
fallback: if the shared object is missing or fails to load, every call raises
``SmgLibraryError`` naming the cause.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libsmg_gpu.so"

# smg_status codes (include/smg_gpu.h)
OK, NOT_CONVERGED, BREAKDOWN, NONFINITE, BAD_ARG, DEVICE_ERROR, TIMEOUT, NO_MEMORY, UNSUPPORTED, IO_ERROR = range(10)
F64, F32, F16 = 0, 1, 2
OP_D, OP_DDAG, OP_DDAGD, OP_G5D = 0, 1, 2, 3
EO_SCHUR, EO_SCHUR_DAG, EO_SCHUR_DAG_SCHUR, EO_HOP_EO, EO_HOP_OE = 0, 1, 2, 3, 4


class SmgLibraryError(RuntimeError):
    pass


class SmgError(RuntimeError):
    def __init__(self, status: int, where: str, msg: str):
        super().__init__(f"{where}: {msg} (status {status})")
        self.status = status


class SolveResult(C.Structure):
    _fields_ = [("iterations", C.c_int), ("final_residual", C.c_double), ("true_residual", C.c_double),
                ("operator_applications", C.c_int)]


MAX_LEVELS = 6


class GaugeHeader(C.Structure):
    """smg_gauge_header = the reference's GaugeHeader (src/hmc.h:19-25)."""
    _fields_ = [("magic", C.c_uint32), ("L", C.c_uint32), ("beta", C.c_double), ("mass", C.c_double),
                ("avg_plaq", C.c_double)]


class HMCParams(C.Structure):
    """smg_hmc_params (include/smg_gpu.h)."""
    _fields_ = [("beta", C.c_double), ("tau", C.c_double), ("n_steps", C.c_int), ("omelyan", C.c_int),
                ("n_inner", C.c_int), ("cg_maxiter", C.c_int), ("cg_tol", C.c_double), ("c_sw", C.c_double),
                ("mu_t", C.c_double), ("force_accept", C.c_int), ("mixed_precision", C.c_int),
                ("use_eo", C.c_int)]


class HMCResult(C.Structure):
    """smg_hmc_result (include/smg_gpu.h)."""
    _fields_ = [("accepted", C.c_int), ("dH", C.c_double), ("dKE", C.c_double), ("dSG", C.c_double),
                ("dSF", C.c_double), ("total_cg_iters", C.c_int), ("solves", C.c_int), ("plaquette", C.c_double),
                ("dLD", C.c_double)]


class ReversibilityResult(C.Structure):
    """smg_reversibility_result (include/smg_gpu.h)."""
    _fields_ = [("gauge_delta", C.c_double), ("mom_delta", C.c_double), ("dH_forward", C.c_double),
                ("dH_backward", C.c_double), ("total_cg_iters", C.c_int), ("solves", C.c_int)]


class DeflationInfo(C.Structure):
    """smg_deflation_info (include/smg_gpu.h)."""
    _fields_ = [("converged", C.c_int), ("restarts", C.c_int), ("iterations", C.c_int), ("n_kr", C.c_int)]


class MSParams(C.Structure):
    """smg_ms_params (include/smg_gpu.h)."""
    _fields_ = [("beta", C.c_double), ("tau", C.c_double), ("n_outer", C.c_int), ("n_inner", C.c_int),
                ("cg_maxiter", C.c_int), ("cg_tol", C.c_double), ("inner_smooth", C.c_int), ("outer_type", C.c_int),
                ("c_sw", C.c_double), ("mu_t", C.c_double)]


class MSResult(C.Structure):
    """smg_ms_result (include/smg_gpu.h)."""
    _fields_ = [("accepted", C.c_int), ("dH", C.c_double), ("dKE", C.c_double), ("dSG", C.c_double),
                ("dSF", C.c_double), ("highmode_cg_iters", C.c_int), ("lowmode_force_evals", C.c_int),
                ("solves", C.c_int), ("plaquette", C.c_double)]


class ForceCheck(C.Structure):
    """smg_force_check (include/smg_gpu.h)."""
    _fields_ = [("passed", C.c_int), ("gauge_passed", C.c_int), ("fermion_passed", C.c_int),
                ("gauge_max_err", C.c_double), ("gauge_rel", C.c_double), ("fermion_max_err", C.c_double),
                ("fermion_rel", C.c_double), ("n_links", C.c_int), ("mu", C.c_int * 20), ("site", C.c_int * 20),
                ("gf_ana", C.c_double * 20), ("gf_num", C.c_double * 20), ("ff_ana", C.c_double * 20),
                ("ff_num", C.c_double * 20)]


class MGParams(C.Structure):
    """smg_mg_params (include/smg_gpu.h)."""
    _fields_ = [("n_levels", C.c_int), ("block", (C.c_int * 2) * (MAX_LEVELS - 1)),
                ("n_vec", C.c_int * (MAX_LEVELS - 1)), ("chiral_split", C.c_int), ("null_iters", C.c_int),
                ("null_mr_steps", C.c_int), ("pre_smooth", C.c_int), ("post_smooth", C.c_int), ("w_cycle", C.c_int),
                ("coarse_max_iter", C.c_int), ("coarse_tol", C.c_double), ("precision", C.c_int),
                ("seed", C.c_uint32), ("tensor_cores", C.c_int), ("smoother_half", C.c_int),
                ("coarse_half", C.c_int)]


_vp = C.c_void_p
_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_st = C.c_int

_SIGS = {
    "smg_version": (C.c_char_p, []),
    "smg_status_string": (C.c_char_p, [C.c_int]),
    "smg_context_create": (_st, [C.c_int, _vp, C.POINTER(_vp)]),
    "smg_context_destroy": (_st, [_vp]),
    "smg_context_synchronize": (_st, [_vp]),
    "smg_context_set_stream": (_st, [_vp, _vp]),
    "smg_context_stream": (_vp, [_vp]),
    "smg_last_error": (C.c_char_p, [_vp]),
    "smg_context_kernel_launches": (C.c_uint64, [_vp]),
    "smg_timer_begin": (_st, [_vp]),
    "smg_timer_end": (_st, [_vp, _dp]),
    "smg_gauge_create": (_st, [_vp, C.c_int, _dp, C.POINTER(_vp)]),
    "smg_gauge_destroy": (_st, [_vp]),
    "smg_gauge_set": (_st, [_vp, _dp]),
    "smg_gauge_get": (_st, [_vp, _dp]),
    "smg_gauge_L": (C.c_int, [_vp]),
    "smg_gauge_avg_plaq": (_st, [_vp, _dp]),
    "smg_gauge_action": (_st, [_vp, C.c_double, _dp]),
    "smg_gauge_force": (_st, [_vp, C.c_double, _dp]),
    "smg_dirac_create": (_st, [_vp, C.c_double, C.c_double, C.c_double, C.c_double, C.POINTER(_vp)]),
    "smg_dirac_destroy": (_st, [_vp]),
    "smg_dirac_refresh": (_st, [_vp]),
    "smg_dirac_get_clover": (_st, [_vp, _dp]),
    "smg_dirac_apply": (_st, [_vp, C.c_int, _vp, _vp]),
    "smg_field_create": (_st, [_vp, C.c_int, C.c_int, C.c_int, C.POINTER(_vp)]),
    "smg_field_destroy": (_st, [_vp]),
    "smg_field_upload": (_st, [_vp, _dp]),
    "smg_field_download": (_st, [_vp, _dp]),
    "smg_field_upload_async": (_st, [_vp, _dp]),
    "smg_field_download_async": (_st, [_vp, _dp]),
    "smg_field_zero": (_st, [_vp]),
    "smg_field_copy": (_st, [_vp, _vp]),
    "smg_field_nrhs": (C.c_int, [_vp]),
    "smg_field_L": (C.c_int, [_vp]),
    "smg_field_precision": (C.c_int, [_vp]),
    "smg_field_device_ptr": (_vp, [_vp]),
    "smg_field_bytes": (C.c_size_t, [_vp]),
    "smg_blas_dot": (_st, [_vp, _vp, _dp]),
    "smg_blas_norm": (_st, [_vp, _dp]),
    "smg_blas_axpy": (_st, [_dp, _vp, _vp]),
    "smg_blas_scale": (_st, [_dp, _vp]),
    "smg_blas_dot_noalloc": (_st, [_vp, _vp, C.c_int64, C.c_int, _vp, _vp]),
    "smg_cg_solve": (_st, [_vp, _vp, _vp, C.c_int, C.c_double, C.POINTER(SolveResult)]),
    "smg_cg_solve_mixed": (_st, [_vp, _vp, _vp, C.c_int, C.c_double, C.POINTER(SolveResult)]),
    "smg_rng_create": (_st, [C.c_uint32, C.POINTER(_vp)]),
    "smg_rng_destroy": (_st, [_vp]),
    "smg_rng_uniform": (_st, [_vp, _dp]),
    "smg_rng_normal": (_st, [_vp, C.c_int64, _dp]),
    "smg_hmc_params_default": (_st, [C.POINTER(HMCParams)]),
    "smg_hmc_trajectory": (_st, [_vp, C.c_double, C.c_double, C.POINTER(HMCParams), _vp, C.POINTER(HMCResult)]),
    "smg_hmc_reversibility": (_st, [_vp, C.c_double, C.c_double, C.POINTER(HMCParams), _vp,
                                    C.POINTER(ReversibilityResult)]),
    "smg_fermion_force": (_st, [_vp, _vp, _dp]),
    "smg_mg_params_default": (_st, [C.POINTER(MGParams)]),
    "smg_mg_create": (_st, [_vp, C.POINTER(MGParams), _dp, C.POINTER(_vp)]),
    "smg_mg_destroy": (_st, [_vp]),
    "smg_mg_level_dims": (_st, [_vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "smg_mg_null_vectors": (_st, [_vp, _dp]),
    "smg_mg_get_prolongator": (_st, [_vp, C.c_int, _dp]),
    "smg_mg_get_coarse_op": (_st, [_vp, C.c_int, _dp]),
    "smg_mg_precondition": (_st, [_vp, _vp, _vp]),
    "smg_mg_prolong_host": (_st, [_vp, C.c_int, _dp, _dp]),
    "smg_mg_restrict_host": (_st, [_vp, C.c_int, _dp, _dp]),
    "smg_mg_coarse_apply_host": (_st, [_vp, C.c_int, _dp, _dp]),
    "smg_mg_time_coarse_apply": (_st, [_vp, C.c_int, C.c_int, C.c_int, _dp, _dp]),
    "smg_mg_time_smoother": (_st, [_vp, _vp, C.c_int, _dp, _dp]),
    "smg_mg_time_coarse_solve": (_st, [_vp, C.c_int, _dp, C.POINTER(C.c_int)]),
    "smg_mg_create_from_starts": (_st, [_vp, _vp, C.POINTER(_dp), C.POINTER(_vp)]),
    "smg_mg_n_null_vectors": (_st, [_vp, C.POINTER(C.c_int)]),
    "smg_mg_set_wait_limit": (_st, [_vp, C.c_longlong]),
    "smg_prolongator_create": (_st, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, _dp, C.POINTER(_vp)]),
    "smg_prolongator_destroy": (_st, [_vp]),
    "smg_prolongator_get_block_vecs": (_st, [_vp, _dp]),
    "smg_prolongator_prolong": (_st, [_vp, _dp, _dp]),
    "smg_prolongator_restrict": (_st, [_vp, _dp, _dp]),
    "smg_coarse_op_create": (_st, [_vp, _vp, C.POINTER(_vp)]),
    "smg_coarse_op_destroy": (_st, [_vp]),
    "smg_coarse_op_dims": (_st, [_vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "smg_coarse_op_get_links": (_st, [_vp, _dp]),
    "smg_coarse_op_apply": (_st, [_vp, _dp, _dp]),
    "smg_coarse_op_solve": (_st, [_vp, _dp, _dp, C.c_int, C.c_double]),
    "smg_coarse_op_setup_deflation": (_st, [_vp, C.c_int, C.c_int, C.c_int, C.c_double, _vp]),
    "smg_mg_coarse_apply_batch": (_st, [_vp, C.c_int, C.c_int, C.c_int, _fp, _fp, _fp, _dp]),
    "smg_gcr_solve": (_st, [_vp, _vp, _vp, _vp, C.c_int, C.c_double, C.c_int, C.c_int, C.POINTER(SolveResult)]),
    "smg_cg_solve_precond": (_st, [_vp, _vp, _vp, _vp, C.c_int, C.c_int, C.c_double, C.POINTER(SolveResult)]),
    "smg_mr_smooth": (_st, [_vp, _vp, _vp, C.c_int]),
    "smg_richardson_smooth": (_st, [_vp, _vp, _vp, C.c_int, C.c_double]),
    "smg_estimate_lambda_max": (_st, [_vp, C.c_int, _dp]),
    "smg_mg_rebuild": (_st, [_vp]),
    "smg_verify_forces": (_st, [_vp, C.c_double, C.c_double, C.c_double, C.c_int, C.c_double, C.c_double, C.c_int,
                                C.c_double, C.c_double, C.POINTER(ForceCheck)]),
    "smg_mg_setup_deflation": (_st, [_vp, C.c_int, C.c_int, C.c_int, C.c_double, C.POINTER(DeflationInfo)]),
    "smg_mg_setup_deflation_level": (_st, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                           C.POINTER(DeflationInfo)]),
    "smg_mg_set_deflation": (_st, [_vp, C.c_int, _dp, _dp]),
    "smg_mg_get_deflation": (_st, [_vp, C.POINTER(C.c_int), _dp, _dp]),
    "smg_mg_deflation_rr": (_st, [_vp, _dp]),
    "smg_mg_lowmode_solution": (_st, [_vp, _vp, _vp]),
    "smg_coarse_lowmode_force": (_st, [_vp, _vp, _vp, C.c_int, _dp]),
    "smg_ms_params_default": (_st, [C.POINTER(MSParams)]),
    "smg_hmc_mg_multiscale": (_st, [_vp, C.c_double, C.c_double, C.POINTER(MSParams), _vp, _vp,
                                    C.POINTER(MSResult)]),
    "smg_hmc_mg_multiscale_reversibility": (_st, [_vp, C.c_double, C.c_double, C.POINTER(MSParams), _vp, _vp,
                                                  C.POINTER(ReversibilityResult)]),
    "smg_mg_estimate_lambda_max": (_st, [_vp, C.c_int, C.c_int, _dp]),
    "smg_mg_set_symmetric": (_st, [_vp, C.c_double, _dp]),
    "smg_fgmres_solve": (_st, [_vp, _vp, _vp, _vp, C.c_int, C.c_int, C.c_double, C.c_int, C.POINTER(SolveResult),
                               _dp, C.POINTER(C.c_int)]),
    "smg_fermion_action": (_st, [_vp, _vp, _vp, _vp, C.c_int, C.c_double, _dp, C.POINTER(SolveResult)]),
    "smg_dirac_apply_delta": (_st, [_vp, _dp, C.c_double, _vp, _vp]),
    "smg_eo_apply": (_st, [_vp, C.c_int, _vp, _vp]),
    "smg_eo_reconstruct": (_st, [_vp, _vp, _vp]),
    "smg_eo_logdet_ee": (_st, [_vp, _dp]),
    "smg_eo_cg_solve": (_st, [_vp, _vp, _vp, C.c_int, C.c_double, C.POINTER(SolveResult)]),
    "smg_eo_fermion_force": (_st, [_vp, _vp, _dp]),
    "smg_batch_create": (_st, [C.c_int, C.c_int, C.POINTER(_vp)]),
    "smg_batch_destroy": (_st, [_vp]),
    "smg_batch_add": (_st, [_vp, C.c_int, _dp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int,
                            C.POINTER(C.c_int)]),
    "smg_batch_setup": (_st, [_vp, C.POINTER(MGParams)]),
    "smg_batch_bind_host": (_st, [_vp, C.c_int, _dp, _dp, _dp]),
    "smg_batch_solve": (_st, [_vp, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, _dp]),
    "smg_batch_result": (_st, [_vp, C.c_int, C.POINTER(SolveResult), C.POINTER(C.c_int), _dp]),
    "smg_batch_download": (_st, [_vp, C.c_int, _dp, _dp]),
    "smg_batch_kernel_launches": (_st, [_vp, C.POINTER(C.c_uint64)]),
    "smg_host_gauge_write_swng": (_st, [C.c_char_p, C.c_int, _dp, C.c_double, C.c_double, C.c_double]),
    "smg_host_gauge_read_swng": (_st, [C.c_char_p, C.c_int, C.POINTER(GaugeHeader), _dp]),
    "smg_host_gauge_write_raw": (_st, [C.c_char_p, C.c_int, _dp]),
    "smg_host_gauge_read_raw": (_st, [C.c_char_p, C.c_int, _dp]),
    "smg_gauge_save": (_st, [_vp, C.c_double, C.c_double, C.c_char_p]),
    "smg_gauge_load": (_st, [_vp, C.c_char_p, C.POINTER(GaugeHeader)]),
    "smg_host_gauge_normal": (_st, [C.c_int, C.c_double, C.c_uint32, _dp]),
    "smg_host_random_vec": (_st, [C.c_int64, C.c_uint32, _dp]),
}

_lib = None
_load_error: str | None = None


def exported_symbols() -> list[str]:
    return sorted(_SIGS)


def lib():
    """Returns the loaded library, raising SmgLibraryError if it is unavailable."""
    global _lib, _load_error
    if _lib is not None:
        return _lib
    if _load_error is not None:
        raise SmgLibraryError(_load_error)
    if not LIB_PATH.exists():
        _load_error = (f"{LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; g.build()\"` "
                       "(there is no CPU fallback)")
        raise SmgLibraryError(_load_error)
    try:
        L = C.CDLL(str(LIB_PATH))
    except OSError as e:
        _load_error = f"loading {LIB_PATH} failed: {e}"
        raise SmgLibraryError(_load_error) from e
    for name, (res, args) in _SIGS.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(status: int, where: str, ctx=None) -> int:
    if status == OK:
        return status
    L = lib()
    msg = L.smg_status_string(status).decode()
    if ctx is not None:
        detail = L.smg_last_error(ctx).decode()
        if detail:
            msg = f"{msg}: {detail}"
    raise SmgError(status, where, msg)
