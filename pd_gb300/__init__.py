"""GB300-native Projective Dynamics substep (pd_ipc's per-substep loop) behind a C ABI.

The compute path is the in-tree CUDA library ``pd_gb300/_lib/libpd_gb300.so`` (built by
``pd_gb300.build``); this package only binds it. There is no CPU fallback: importing the
bindings raises if the library is missing.
"""
from .api import (  # noqa: F401
    PD_OK,
    PD_ERR_INVALID_ARGUMENT,
    PD_ERR_STATE,
    PD_ERR_FACTORIZATION,
    PD_ERR_CUDA,
    PD_ERR_UNSUPPORTED,
    PD_ERR_NO_MEMORY,
    PD_PRECISION_FP64_EXACT,
    PD_PRECISION_FP64,
    PD_PRECISION_FP32_PROJECTION,
    PD_PRECISION_FP32_SOLVE,
    PD_PRECISION_MIXED,
    PD_SOLVE_LEVELS,
    PD_SOLVE_SUPERNODAL,
    PD_SOLVE_SUPERNODAL32,
    PD_SOLVE_DENSE32,
    PD_SOLVE_DENSE32_TEAM,
    PD_SOLVE_SUPERNODAL32_CORRECTION,
    PD_SOLVE_DENSE64_TEAM,
    PD_HOST_STATE_NONE,
    PD_HOST_STATE_COPIES,
    PD_HOST_STATE_GRAPH,
    PD_CHEB_OFF,
    PD_CHEB_RHO,
    PD_CHEB_INTERVAL,
    PdError,
    SceneConfig,
    GridScene,
    Simulator,
    GpuDirectSolver,
    load_library,
    make_grid,
    make_obj,
)
