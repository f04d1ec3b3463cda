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

F64, F32, F16X2, BF16X3, F64E = 0, 1, 2, 3, 4
EXACT, REFERENCE = 0, 1
MASS, STIFFNESS, HELMHOLTZ = 0, 1, 2
MASS_AFFINE, STIFFNESS_AFFINE = 3, 4  # one geometry set per cell (affine cells)

DTYPE_NAMES = {F64: "f64", F32: "f32", F16X2: "f16x2", BF16X3: "bf16x3", F64E: "f64e"}
FP64_STORAGE = (F64, F64E)

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
        "femtc_operator_launches": ([], ctypes.c_longlong),
        "femtc_last_error": ([], ctypes.c_char_p),
        "femtc_device_status": ([], c_int),
        "femtc_bounded_wait_check": ([c_int, vp], c_int),
        "femtc_supported": ([c_int] * 5, c_int),
        "femtc_mass_apply": ([c_int] * 4 + [vp] * 4 + [c_size, vp], c_int),
        "femtc_stiffness_apply": ([c_int] * 4 + [vp] * 4 + [c_size, vp], c_int),
        "femtc_helmholtz_apply": ([c_int] * 3 + [vp] * 4 + [c_size, vp], c_int),
        "femtc_set_even_odd": ([c_int], c_int),
        "femtc_even_odd_used": ([c_int] * 5 + [vp], c_int),
        "femtc_helmholtz_geometry": ([c_int, ctypes.c_double, vp, ctypes.c_double, vp, vp, c_size, vp],
                                     c_int),
        "femtc_affine_apply": ([c_int] * 4 + [vp] * 4 + [c_size, vp], c_int),
        "femtc_assembled_apply": ([c_int] * 5 + [vp] * 4 + [c_size] + [vp] * 3 + [c_size, vp, vp],
                                  c_int),
        "femtc_assembled_work_bytes": ([c_int, c_int, c_size], c_size),
        "femtc_dofmap_transpose": ([vp, c_size, c_int, c_size, vp, vp], c_int),
        "femtc_affine_apply_host": ([c_int] * 4 + [vp] * 4 + [c_size], c_int),
        "femtc_mass_apply_host": ([c_int] * 4 + [vp] * 4 + [c_size], c_int),
        "femtc_stiffness_apply_host": ([c_int] * 4 + [vp] * 4 + [c_size], c_int),
        "femtc_set_tile_config": ([c_int] * 9, c_int),
        "femtc_get_tile_config": ([c_int] * 5 + [ctypes.POINTER(c_int)] * 4, c_int),
        "femtc_autotune": ([c_int] * 5 + [vp] * 4 + [c_size, vp] + [ctypes.POINTER(c_int)] * 3
                           + [ctypes.POINTER(ctypes.c_float)], c_int),
        "femtc_autotune_host": ([c_int] * 5 + [vp] * 4 + [c_size] + [ctypes.POINTER(c_int)] * 3
                                + [ctypes.POINTER(ctypes.c_float)], c_int),
        "femtc_tile_db_save": ([ctypes.c_char_p], c_int),
        "femtc_tile_db_load": ([ctypes.c_char_p], c_int),
        "femtc_tabulate": ([c_int, c_int, dp, dp, dp, dp], c_int),
        "femtc_set_host_path": ([c_int], c_int),
        "femtc_gemm_blocked": ([c_int] * 4 + [vp] * 3 + [c_size, vp], c_int),
        "femtc_gemm_micro": ([c_int] * 7 + [vp] * 3 + [c_size] * 4 + [vp], c_int),
        "femtc_apply_contractions": ([c_int] * 4 + [vp] * 5 + [c_size, vp], c_int),
        "femtc_geometry": ([c_int, c_int, vp, vp, c_int, vp, vp, c_size, vp], c_int),
        "femtc_batch_create": ([c_int, vp, c_int, c_int, ctypes.POINTER(vp)], c_int),
        "femtc_batch_launch": ([vp, vp], c_int),
        "femtc_batch_launch_eager": ([vp, vp], c_int),
        "femtc_batch_info": ([vp, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(c_int),
                              ctypes.POINTER(c_int), ctypes.POINTER(ctypes.c_longlong)], c_int),
        "femtc_batch_layout": ([vp, c_int, c_int, ctypes.POINTER(c_int), ctypes.POINTER(c_int)], c_int),
        "femtc_batch_threads": ([vp], c_int),
        "femtc_batch_plan": ([vp, ctypes.POINTER(c_int), ctypes.POINTER(c_int)], c_int),
        "femtc_batch_destroy": ([vp], None),
        "femtc_batch_apply_static": ([c_int, vp, c_int, vp], c_int),
        "femtc_solve_bytes": ([c_int, c_int, c_size], c_size),
        "femtc_solve": ([vp, vp, vp], c_int),
        "femtc_server_create": ([c_size, c_int, ctypes.POINTER(vp)], c_int),
        "femtc_server_submit": ([vp, vp, ctypes.POINTER(ctypes.c_longlong)], c_int),
        "femtc_server_submit_apply": ([vp, vp, ctypes.POINTER(ctypes.c_longlong)], c_int),
        "femtc_server_wait": ([vp, ctypes.c_longlong, ctypes.c_double, vp], c_int),
        "femtc_server_get_stats": ([vp, vp], c_int),
        "femtc_server_set_policy": ([vp, c_int], c_int),
        "femtc_server_destroy": ([vp], None),
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
    want = np.float64 if dtype in FP64_STORAGE else np.float32
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
    """Device-resident operator action through femtc_{mass,stiffness}_apply
    (affine forms: femtc_affine_apply, exact semantics, tables with the
    weights appended -- see affine_tables)."""
    lib = load()
    tab = host_tables(tables, dtype)
    if op in (MASS_AFFINE, STIFFNESS_AFFINE):
        if semantics != EXACT:
            raise ValueError("affine forms: exact semantics only")
        check(lib.femtc_affine_apply(op, dtype, degree, nquad, tab.ctypes.data, ptr(u), ptr(y),
                                     ptr(geo), ncells, stream_ptr(stream)))
        return
    fn = lib.femtc_mass_apply if op == MASS else lib.femtc_stiffness_apply
    check(fn(dtype, semantics, degree, nquad, tab.ctypes.data, ptr(u), ptr(y),
             ptr(geo), ncells, stream_ptr(stream)))


def dofmap_transpose(dofmap, ndofs: int):
    """CSR transpose (offsets[ndofs+1], entries) of a [ncells, N^3] int32 DOF
    map, on the host (femtc_dofmap_transpose)."""
    dm = np.ascontiguousarray(dofmap, dtype=np.int32)
    ncells, n3 = dm.shape
    offsets = np.empty(ndofs + 1, dtype=np.int32)
    entries = np.empty(dm.size, dtype=np.int32)
    check(load().femtc_dofmap_transpose(dm.ctypes.data, ncells, n3, ndofs, offsets.ctypes.data,
                                        entries.ctypes.data))
    return offsets, entries


def assembled_work_bytes(dtype: int, degree: int, ncells: int) -> int:
    return int(load().femtc_assembled_work_bytes(dtype, degree, ncells))


def assembled_apply(op: int, dtype: int, semantics: int, degree: int, nquad: int, tables,
                    dofmap, offsets, entries, ndofs: int, x, y, geo, ncells: int, work,
                    stream=None) -> None:
    """Global-DOF action y = sum_c P_c^T A_c P_c x (femtc_assembled_apply);
    dofmap, offsets, entries, x, y, geo and work are device buffers."""
    tab = host_tables(tables, dtype)
    check(load().femtc_assembled_apply(op, dtype, semantics, degree, nquad, tab.ctypes.data,
                                       ptr(dofmap), ptr(offsets), ptr(entries), ndofs, ptr(x),
                                       ptr(y), ptr(geo), ncells, ptr(work), stream_ptr(stream)))


def affine_tables(tables, weights) -> np.ndarray:
    """The affine forms' tables: Phi, Gamma (2*Q*N) then the Q 1D weights."""
    return np.concatenate([np.asarray(tables, dtype=np.float64).reshape(-1),
                           np.asarray(weights, dtype=np.float64).reshape(-1)])


def affine_apply(op: int, dtype: int, degree: int, nquad: int, tables, weights, u, y, cgeo,
                 ncells: int, stream=None) -> None:
    """Operator action on affine cells (femtc_affine_apply): cgeo holds one
    detJ (MASS_AFFINE) or one detJ J^-1 J^-T [zz,yz,xz,yy,xy,xx]
    (STIFFNESS_AFFINE) per cell; the 1D quadrature weights enter through the
    backward tables."""
    apply(op, dtype, EXACT, degree, nquad, affine_tables(tables, weights), u, y, cgeo, ncells,
          stream)


def helmholtz_apply(dtype: int, degree: int, nquad: int, tables, u, y, geo8, ncells: int,
                    stream=None) -> None:
    """y = alpha M u + beta K u in one pass (femtc_helmholtz_apply); geo8 is
    the interleaved [ncells][Q^3][8] geometry of helmholtz_geometry."""
    tab = host_tables(tables, dtype)
    check(load().femtc_helmholtz_apply(dtype, degree, nquad, tab.ctypes.data, ptr(u), ptr(y),
                                       ptr(geo8), ncells, stream_ptr(stream)))


def helmholtz_geometry(nquad: int, alpha: float, dw, beta: float, G, geo8, ncells: int,
                       stream=None) -> None:
    """geo8 = [beta G, alpha dw, 0] per quadrature point (FP32 device buffers)."""
    check(load().femtc_helmholtz_geometry(nquad, alpha, ptr(dw), beta, ptr(G), ptr(geo8), ncells,
                                          stream_ptr(stream)))


def apply_host(op: int, dtype: int, semantics: int, degree: int, nquad: int,
               tables, u, y, geo, ncells: int) -> None:
    """Host-buffer drop-in path (copies in, applies, copies out)."""
    lib = load()
    tab = host_tables(tables, dtype)
    if op in (MASS_AFFINE, STIFFNESS_AFFINE):
        if semantics != EXACT:
            raise ValueError("affine forms: exact semantics only")
        check(lib.femtc_affine_apply_host(op, dtype, degree, nquad, tab.ctypes.data, ptr(u),
                                          ptr(y), ptr(geo), ncells))
        return
    fn = lib.femtc_mass_apply_host if op == MASS else lib.femtc_stiffness_apply_host
    check(fn(dtype, semantics, degree, nquad, tab.ctypes.data, ptr(u), ptr(y),
             ptr(geo), ncells))


def set_even_odd(enable: bool) -> None:
    """Even-odd contractions for symmetric tables (FP64, exact); on by default."""
    check(load().femtc_set_even_odd(1 if enable else 0))


def even_odd_used(op: int, dtype: int, semantics: int, degree: int, nquad: int, tables) -> bool:
    """Whether a launch with these tables runs the even-odd kernels."""
    tab = host_tables(tables, dtype)
    rc = load().femtc_even_odd_used(op, dtype, semantics, degree, nquad, tab.ctypes.data)
    check(min(rc, 0))
    return rc == 1


def operator_launches() -> int:
    """Operator kernels launched by the library so far in this process."""
    return int(load().femtc_operator_launches())


def set_host_path(mode: int) -> None:
    """0 auto (zero-copy for pinned buffers), 1 staging copies, 2 zero-copy only."""
    check(load().femtc_set_host_path(mode))


def supported(op: int, dtype: int, semantics: int, degree: int, nquad: int) -> bool:
    return bool(load().femtc_supported(op, dtype, semantics, degree, nquad))


def set_tile_config(op, dtype, semantics, degree, nquad, cb, geo_staged, threads=256,
                    lanes=0) -> None:
    check(load().femtc_set_tile_config(op, dtype, semantics, degree, nquad, cb, geo_staged,
                                       threads, lanes))


def get_tile_config(op, dtype, semantics, degree, nquad):
    """(cells per tile, geometry staged, threads per CTA, lanes per slab)."""
    cb, st, nt, ln = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    check(load().femtc_get_tile_config(op, dtype, semantics, degree, nquad,
                                       ctypes.byref(cb), ctypes.byref(st), ctypes.byref(nt),
                                       ctypes.byref(ln)))
    return cb.value, st.value, nt.value, ln.value


def autotune(op, dtype, semantics, degree, nquad, tables, u, y, geo, ncells, stream=None):
    """Measure tile shapes on these buffers and keep the fastest.
    Returns (cb, geo_staged, threads, ms)."""
    cb, st, nt = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    ms = ctypes.c_float()
    tab = host_tables(tables, dtype)
    check(load().femtc_autotune(op, dtype, semantics, degree, nquad, tab.ctypes.data, ptr(u),
                                ptr(y), ptr(geo), ncells, stream_ptr(stream), ctypes.byref(cb),
                                ctypes.byref(st), ctypes.byref(nt), ctypes.byref(ms)))
    return cb.value, st.value, nt.value, ms.value


def autotune_host(op, dtype, semantics, degree, nquad, tables, u, y, geo, ncells):
    """Tile tuning of the zero-copy host path on pinned host buffers.
    Returns (cb, geo_staged, threads, ms)."""
    cb, st, nt = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    ms = ctypes.c_float()
    tab = host_tables(tables, dtype)
    check(load().femtc_autotune_host(op, dtype, semantics, degree, nquad, tab.ctypes.data,
                                     ptr(u), ptr(y), ptr(geo), ncells, ctypes.byref(cb),
                                     ctypes.byref(st), ctypes.byref(nt), ctypes.byref(ms)))
    return cb.value, st.value, nt.value, ms.value


def tile_db_save(path: str) -> None:
    check(load().femtc_tile_db_save(path.encode()))


def tile_db_load(path: str) -> int:
    n = load().femtc_tile_db_load(path.encode())
    if n < 0:
        check(n)
    return n


def device_status() -> int:
    s = load().femtc_device_status()
    if s < 0:
        check(s)
    return s


def gemm_blocked(dtype: int, k: int, m: int, n: int, a, b, c, batch: int, stream=None) -> None:
    """Batched linalg::gemm_blocked on the device (a: host table)."""
    tab = host_tables(a, dtype)
    check(load().femtc_gemm_blocked(dtype, k, m, n, tab.ctypes.data, ptr(b), ptr(c), batch,
                                    stream_ptr(stream)))


def gemm_micro(dtype: int, k: int, m: int, nc: int, lda: int, ldb: int, ldc: int, a, b, c,
               batch: int = 1, strides=(0, 0, 0), stream=None) -> None:
    """Batched linalg::gemm_micro on the device: C += A B (a, b, c device
    buffers; strides in elements between items)."""
    check(load().femtc_gemm_micro(dtype, k, m, nc, lda, ldb, ldc, ptr(a), ptr(b), ptr(c), batch,
                                  strides[0], strides[1], strides[2], stream_ptr(stream)))


def apply_contractions(dtype: int, na: int, nb: int, tr: bool, i0, i1, i2, b, a, ncells: int,
                       stream=None) -> None:
    """Batched tmm apply_contractions on the device (tables: host)."""
    t = [host_tables(x, dtype) for x in (i0, i1, i2)]
    check(load().femtc_apply_contractions(dtype, na, nb, int(bool(tr)), t[0].ctypes.data,
                                          t[1].ctypes.data, t[2].ctypes.data, ptr(b), ptr(a),
                                          ncells, stream_ptr(stream)))


def geometry(out_dtype: int, nquad: int, weights, J, dw, G, ncells: int, per_point: bool = False,
             stream=None) -> None:
    """FP64 quadrature factors detJ*w and/or G from Jacobians (device J)."""
    w = np.ascontiguousarray(weights, dtype=np.float64)
    check(load().femtc_geometry(out_dtype, nquad, w.ctypes.data, ptr(J), int(bool(per_point)),
                                ptr(dw), ptr(G), ncells, stream_ptr(stream)))


class BatchItem(ctypes.Structure):
    """femtc_batch_item (include/femtc_gpu.h)."""
    _fields_ = [("op", ctypes.c_int), ("degree", ctypes.c_int), ("nquad", ctypes.c_int),
                ("tables", ctypes.c_void_p), ("u", ctypes.c_void_p), ("y", ctypes.c_void_p),
                ("geo", ctypes.c_void_p), ("ncells", ctypes.c_size_t)]


BATCH_TUNE = 1
BATCH_SPLIT = 2


def batch_apply_static(dtype: int, meshes, stream=None) -> None:
    """femtc_batch_apply_static: the batched launch with its schedule in the
    library's fixed device array (no device allocation); meshes as for Batch."""
    tabs = [host_tables(m[3], dtype) for m in meshes]
    arr = (BatchItem * len(tabs))()
    for i, m in enumerate(meshes):
        op, degree, nquad, _, u, y, geo, ncells = m
        arr[i] = BatchItem(op, degree, nquad, tabs[i].ctypes.data, ptr(u), ptr(y), ptr(geo), ncells)
    check(load().femtc_batch_apply_static(dtype, ctypes.cast(arr, ctypes.c_void_p), len(tabs),
                                          stream_ptr(stream)))


class Batch:
    """A batched persistent launch over many meshes (femtc_batch_*).

    meshes: iterable of (op, degree, nquad, tables, u, y, geo, ncells) with
    device tensors; the tables are kept alive here until the batch is built.
    tune: tile shapes measured on the meshes, and the split plan where it is
    faster (femtc_batch_plan); split: the split plan in any case.
    """

    def __init__(self, dtype: int, meshes, tune: bool = False, split: bool = False):
        lib = load()
        self._tabs = [host_tables(m[3], dtype) for m in meshes]
        arr = (BatchItem * len(self._tabs))()
        for i, m in enumerate(meshes):
            op, degree, nquad, _, u, y, geo, ncells = m
            arr[i] = BatchItem(op, degree, nquad, self._tabs[i].ctypes.data, ptr(u), ptr(y),
                               ptr(geo), ncells)
        h = ctypes.c_void_p()
        check(lib.femtc_batch_create(dtype, ctypes.cast(arr, ctypes.c_void_p), len(self._tabs),
                                     (BATCH_TUNE if tune else 0) | (BATCH_SPLIT if split else 0),
                                     ctypes.byref(h)))
        self.handle = h

    def launch(self, stream=None) -> None:
        check(load().femtc_batch_launch(self.handle, stream_ptr(stream)))

    def launch_eager(self, stream=None) -> None:
        check(load().femtc_batch_launch_eager(self.handle, stream_ptr(stream)))

    def info(self):
        nt, ctas, smem, nd = ctypes.c_longlong(), ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong()
        check(load().femtc_batch_info(self.handle, ctypes.byref(nt), ctypes.byref(ctas),
                                      ctypes.byref(smem), ctypes.byref(nd)))
        threads = load().femtc_batch_threads(self.handle)
        check(min(threads, 0))
        kern, solo = ctypes.c_int(), ctypes.c_int()
        check(load().femtc_batch_plan(self.handle, ctypes.byref(kern), ctypes.byref(solo)))
        return {"tiles": nt.value, "ctas": ctas.value, "threads": threads, "smem": smem.value,
                "dofs": nd.value, "batch_kernels": kern.value, "single_launches": solo.value}

    def layout(self, op: int, degree: int):
        cb, st = ctypes.c_int(), ctypes.c_int()
        check(load().femtc_batch_layout(self.handle, op, degree, ctypes.byref(cb), ctypes.byref(st)))
        return cb.value, st.value

    def close(self) -> None:
        if self.handle:
            load().femtc_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


NOT_CONVERGED, TIMEOUT, NOMEM = -6, -7, -4


class SolveRequest(ctypes.Structure):
    """femtc_solve_request (include/femtc_gpu.h)."""
    _fields_ = [("degree", ctypes.c_int), ("nquad", ctypes.c_int), ("ncells", ctypes.c_size_t),
                ("alpha", ctypes.c_double), ("beta", ctypes.c_double), ("J", ctypes.c_void_p),
                ("b", ctypes.c_void_p), ("x", ctypes.c_void_p), ("rtol", ctypes.c_double),
                ("inner_rtol", ctypes.c_double), ("max_outer", ctypes.c_int),
                ("max_inner", ctypes.c_int), ("inner_dtype", ctypes.c_int)]


class SolveResult(ctypes.Structure):
    """femtc_solve_result (include/femtc_gpu.h)."""
    _fields_ = [("status", ctypes.c_int), ("outer_iters", ctypes.c_int),
                ("inner_iters", ctypes.c_int), ("relres", ctypes.c_double),
                ("bnorm", ctypes.c_double), ("ms_total", ctypes.c_double),
                ("t_submit_ms", ctypes.c_double), ("t_admit_ms", ctypes.c_double),
                ("t_done_ms", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ApplyRequest(ctypes.Structure):
    """femtc_apply_request (include/femtc_gpu.h)."""
    _fields_ = [("op", ctypes.c_int), ("dtype", ctypes.c_int), ("semantics", ctypes.c_int),
                ("degree", ctypes.c_int), ("nquad", ctypes.c_int), ("ncells", ctypes.c_size_t),
                ("tables", ctypes.c_void_p), ("u", ctypes.c_void_p), ("geo", ctypes.c_void_p),
                ("y", ctypes.c_void_p)]


class Application:
    """Host data of one served operator application y = A u (keeps the
    arrays alive; y holds the result once the request completes)."""

    def __init__(self, op, dtype, semantics, degree, nquad, tables, u, geo):
        st = np.float64 if dtype in FP64_STORAGE else np.float32
        self.tables = host_tables(tables, dtype)
        self.u = np.ascontiguousarray(u, dtype=st)
        self.geo = np.ascontiguousarray(geo, dtype=st)
        self.y = np.zeros_like(self.u)
        self.req = ApplyRequest(op, dtype, semantics, degree, nquad, self.u.shape[0],
                                self.tables.ctypes.data, self.u.ctypes.data,
                                self.geo.ctypes.data, self.y.ctypes.data)


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_longlong), ("completed", ctypes.c_longlong),
                ("rejected", ctypes.c_longlong), ("queued", ctypes.c_longlong),
                ("active", ctypes.c_longlong), ("in_use_bytes", ctypes.c_size_t),
                ("peak_in_use_bytes", ctypes.c_size_t), ("max_concurrent", ctypes.c_int)]


class Problem:
    """Host data of one (alpha M + beta K) x = b solve (keeps arrays alive)."""

    def __init__(self, degree, nquad, J, b, alpha=1.0, beta=1.0, rtol=1e-8, inner_dtype=F32,
                 inner_rtol=1e-4, max_outer=20, max_inner=2000):
        self.J = np.ascontiguousarray(J, dtype=np.float64).reshape(-1, 9)
        self.b = np.ascontiguousarray(b, dtype=np.float64).reshape(self.J.shape[0], -1)
        self.x = np.zeros_like(self.b)
        self.req = SolveRequest(degree, nquad, self.J.shape[0], alpha, beta, self.J.ctypes.data,
                                self.b.ctypes.data, self.x.ctypes.data, rtol, inner_rtol,
                                max_outer, max_inner, inner_dtype)


def solve_bytes(degree: int, nquad: int, ncells: int) -> int:
    return int(load().femtc_solve_bytes(degree, nquad, ncells))


def solve(problem: "Problem", stream=None, raise_on_error: bool = True) -> dict:
    """Synchronous solve; returns the result as a dict, problem.x holds x."""
    res = SolveResult()
    rc = load().femtc_solve(ctypes.byref(problem.req), ctypes.byref(res), stream_ptr(stream))
    if rc != 0 and raise_on_error and rc != NOT_CONVERGED:
        check(rc)
    out = res.as_dict()
    out["rc"] = rc
    return out


SERVE_FIFO, SERVE_SHORTEST_FIRST = 0, 1


class Server:
    """Continuous-batching solve server (femtc_server_*); policy: admission
    order, SERVE_SHORTEST_FIRST (default, with aging) or SERVE_FIFO."""

    def __init__(self, hbm_budget_bytes: int, max_active: int,
                 policy: int = SERVE_SHORTEST_FIRST):
        h = ctypes.c_void_p()
        check(load().femtc_server_create(hbm_budget_bytes, max_active, ctypes.byref(h)))
        self.handle = h
        self._live = {}
        check(load().femtc_server_set_policy(h, policy))

    def submit(self, problem: "Problem") -> int:
        t = ctypes.c_longlong()
        check(load().femtc_server_submit(self.handle, ctypes.byref(problem.req), ctypes.byref(t)))
        self._live[t.value] = problem
        return t.value

    def submit_apply(self, app: "Application") -> int:
        """Queue an operator application (femtc_server_submit_apply)."""
        t = ctypes.c_longlong()
        check(load().femtc_server_submit_apply(self.handle, ctypes.byref(app.req),
                                               ctypes.byref(t)))
        self._live[t.value] = app
        return t.value

    def wait(self, ticket: int, timeout_s: float = 600.0) -> dict:
        res = SolveResult()
        rc = load().femtc_server_wait(self.handle, ticket, timeout_s, ctypes.byref(res))
        if rc == TIMEOUT:
            raise FemtcError(rc, load().femtc_last_error().decode())
        self._live.pop(ticket, None)
        out = res.as_dict()
        out["rc"] = rc
        return out

    def stats(self) -> dict:
        st = ServerStats()
        check(load().femtc_server_get_stats(self.handle, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in st._fields_}

    def close(self) -> None:
        if self.handle:
            load().femtc_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
