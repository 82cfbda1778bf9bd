"""GB300-native scattering integral of relativistic_solver_hllc's
radiation-transport source iteration.

The compute path is librts_scatter.so (hand-written CUDA for sm_103a behind the
C ABI in include/rts_scatter.h).  This package builds it in-tree and binds it
with ctypes; there is no CPU fallback anywhere in it.
"""
from ._native import (  # noqa: F401
    PHASE_CUSTOM,
    PHASE_HG,
    PHASE_THOMSON,
    PREC_BF16X3,
    PREC_FP16X3,
    PREC_TF32X3,
    PREC_FP64,
    PRECISIONS,
    STREAM_PARAMS,
    STREAM_SCATTERING_1,
    STREAM_SCATTERING_2,
    TUNE_BIAS,
    TUNE_FLUSH,
    BOUND_FREE,
    BOUND_INNER,
    BOUND_LOCK,
    BOUND_OUTSOURCE,
    LOCX0_DTYPE,
    MEDIUM_ABSORPTION,
    MEDIUM_SCATTERING,
    Batch,
    Context,
    Medium,
    RtsError,
    header_symbols,
    load_library,
    medium,
    medium_gas,
    mesh_cube,
)
from .build import build_library  # noqa: F401
