"""femtc_gb300: GB300-native (sm_103a) matrix-free hexahedral operator action.

The product is libfemtc_gpu.so (C ABI, include/femtc_gpu.h) with its C++
drop-in header include/femtc_gpu/operators.hpp.  This package builds it
in-tree and binds it with ctypes for Python callers, tests and benchmarks.
"""
from ._lib import (  # noqa: F401
    Application, BATCH_SPLIT, BATCH_TUNE, Batch, NOT_CONVERGED, SERVE_FIFO, SERVE_SHORTEST_FIRST, batch_apply_static, Problem, Server, solve, solve_bytes,
    BF16X3, EXACT, F16X2, F32, F64, F64E, FP64_STORAGE, HELMHOLTZ, MASS, REFERENCE, STIFFNESS,
    DTYPE_NAMES, helmholtz_apply, helmholtz_geometry,
    MASS_AFFINE, STIFFNESS_AFFINE, affine_apply, affine_tables,
    assembled_apply, assembled_work_bytes, dofmap_transpose,
    FemtcError, apply, apply_contractions, apply_host, autotune, autotune_host, gemm_blocked, gemm_micro, geometry, check, device_status, get_tile_config, load,
    even_odd_used, operator_launches, set_even_odd, set_host_path, set_tile_config, supported, tabulate, tile_db_load, tile_db_save,
)
from .buildlib import build, lib_path  # noqa: F401
