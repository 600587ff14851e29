"""GB300-native (sm_103a) Wilson-clover Dirac operator and multigrid solve path
for the 2D U(1) lattice Schwinger model, behind the operator and solver API of
cpviolator/Schwinger_MG.

The compute runs in libsmg_gpu.so (hand-written CUDA for sm_103a, C ABI in
include/smg_gpu.h); this package is the Python mirror of that API.
"""
from ._lib import SmgError, SmgLibraryError, lib  # noqa: F401
from .api import (  # noqa: F401
    CGResult,
    FCGResult,
    FGMRESResult,
    cg_solve_precond,
    estimate_lambda_max,
    fermion_action,
    fgmres_solve,
    fgmres_solve_mg,
    mr_smooth,
    richardson_smooth,
    HMCResult,
    ReversibilityResult,
    Rng,
    cg_solve_mixed,
    hmc_params,
    hmc_reversibility,
    hmc_mg_multiscale,
    hmc_mg_multiscale_reversibility,
    ms_params,
    MSResult,
    coarse_lowmode_force,
    verify_forces,
    hmc_trajectory,
    MGHierarchy,
    build_full_mg,
    build_mg_hierarchy,
    fcg_solve,
    fcg_solve_mg,
    mg_params,
    Context,
    DiracOp,
    EvenOddDiracOp,
    Field,
    GaugeField,
    Lattice,
    LatticeBatch,
    axpy,
    cg_solve,
    dot,
    fermion_force,
    gauge_action,
    gauge_force,
    gauge_normal,
    load_gauge,
    load_gauge_raw,
    save_gauge,
    save_gauge_raw,
    norm,
    random_vec,
    scale,
)

__version__ = "0.1.0"
