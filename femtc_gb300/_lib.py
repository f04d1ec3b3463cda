"""ctypes binding of libfemtc_gpu.so (the C ABI in include/femtc_gpu.h).

This module only marshals arguments: device buffers are passed as raw
pointers (torch tensors are accepted for convenience and contribute their
data_ptr()), tables as host arrays.  Loading fails loudly when the library
is missing; there is no fallback implementation.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from . import buildlib as _build

F64, F32, F16X2, BF16X3 = 0, 1, 2, 3
EXACT, REFERENCE = 0, 1
MASS, STIFFNESS = 0, 1

DTYPE_NAMES = {F64: "f64", F32: "f32", F16X2: "f16x2", BF16X3: "bf16x3"}

_lock = threading.Lock()
_lib = None


class FemtcError(RuntimeError):
    """A femtc C-ABI call returned a non-zero status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"femtc status {status}: {message}")
        self.status = status


def _declare(lib: ctypes.CDLL) -> None:
    c_int, c_size, vp = ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p
    dp = ctypes.POINTER(ctypes.c_double)
    sigs = {
        "femtc_version": ([], c_int),
        "femtc_last_error": ([], ctypes.c_char_p),
        "femtc_device_status": ([], c_int),
        "femtc_supported": ([c_int] * 5, c_int),
        "femtc_mass_apply": ([c_int] * 4 + [vp] * 4 + [c_size, vp], c_int),
        "femtc_stiffness_apply": ([c_int] * 4 + [vp] * 4 + [c_size, vp], c_int),
        "femtc_mass_apply_host": ([c_int] * 4 + [vp] * 4 + [c_size], c_int),
        "femtc_stiffness_apply_host": ([c_int] * 4 + [vp] * 4 + [c_size], c_int),
        "femtc_set_tile_config": ([c_int] * 7, c_int),
        "femtc_get_tile_config": ([c_int] * 5 + [ctypes.POINTER(c_int)] * 2, c_int),
        "femtc_tabulate": ([c_int, c_int, dp, dp, dp, dp], c_int),
    }
    for name, (args, res) in sigs.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load (building first if needed) the in-tree libfemtc_gpu.so."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.lib_path()
        if not os.path.exists(path):
            if not build_if_missing:
                raise FemtcError(-3, f"{path} is missing; run femtc_gb300.build.build()")
            path = _build.build()
        lib = ctypes.CDLL(path)
        _declare(lib)
        _lib = lib
        return lib


def check(status: int) -> None:
    if status != 0:
        msg = load().femtc_last_error().decode(errors="replace")
        raise FemtcError(status, msg)


def ptr(x) -> int | None:
    """Raw address of a torch tensor, numpy array or integer (None -> NULL)."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    raise TypeError(f"cannot take the address of {type(x)}")


def host_tables(tables, dtype: int) -> np.ndarray:
    want = np.float64 if dtype == F64 else np.float32
    return np.ascontiguousarray(np.asarray(tables), dtype=want)


def stream_ptr(stream) -> int | None:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream  # torch.cuda.Stream


def tabulate(degree: int, nquad: int):
    """(tables[2*Q*N], points[Q], weights[Q], nodes[N]) in FP64 (host)."""
    n = degree + 1
    tab = np.zeros(2 * nquad * n)
    x = np.zeros(nquad)
    w = np.zeros(nquad)
    z = np.zeros(n)
    dp = ctypes.POINTER(ctypes.c_double)
    check(load().femtc_tabulate(
        degree, nquad, tab.ctypes.data_as(dp), x.ctypes.data_as(dp),
        w.ctypes.data_as(dp), z.ctypes.data_as(dp)))
    return tab, x, w, z


def apply(op: int, dtype: int, semantics: int, degree: int, nquad: int,
          tables, u, y, geo, ncells: int, stream=None) -> None:
    """Device-resident operator action through femtc_{mass,stiffness}_apply."""
    lib = load()
    tab = host_tables(tables, dtype)
    fn = lib.femtc_mass_apply if op == MASS else lib.femtc_stiffness_apply
    check(fn(dtype, semantics, degree, nquad, tab.ctypes.data, ptr(u), ptr(y),
             ptr(geo), ncells, stream_ptr(stream)))


def apply_host(op: int, dtype: int, semantics: int, degree: int, nquad: int,
               tables, u, y, geo, ncells: int) -> None:
    """Host-buffer drop-in path (copies in, applies, copies out)."""
    lib = load()
    tab = host_tables(tables, dtype)
    fn = lib.femtc_mass_apply_host if op == MASS else lib.femtc_stiffness_apply_host
    check(fn(dtype, semantics, degree, nquad, tab.ctypes.data, ptr(u), ptr(y),
             ptr(geo), ncells))


def supported(op: int, dtype: int, semantics: int, degree: int, nquad: int) -> bool:
    return bool(load().femtc_supported(op, dtype, semantics, degree, nquad))


def set_tile_config(op, dtype, semantics, degree, nquad, cb, geo_staged) -> None:
    check(load().femtc_set_tile_config(op, dtype, semantics, degree, nquad, cb, geo_staged))


def get_tile_config(op, dtype, semantics, degree, nquad):
    cb, st = ctypes.c_int(), ctypes.c_int()
    check(load().femtc_get_tile_config(op, dtype, semantics, degree, nquad,
                                       ctypes.byref(cb), ctypes.byref(st)))
    return cb.value, st.value


def device_status() -> int:
    s = load().femtc_device_status()
    if s < 0:
        check(s)
    return s
