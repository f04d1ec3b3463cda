"""CPU oracle (test infrastructure only -- the checker, never the product).

Loads oracle/liboracle.so (the FP64 C restatement of the reference's
per-cell algorithm, femtc_oracle.c) and, when it was built from the
reference sources, oracle/_ref/*.so (the reference's own templates).
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
import this package.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
EXACT, REFERENCE = 0, 1
_lock = threading.Lock()
_lib = None
_ref = {}


def build(ref: bool = True) -> None:
    """make -C oracle (liboracle.so, and _ref/ when the reference exists)."""
    targets = ["liboracle.so"] + (["ref"] if ref else [])
    r = subprocess.run(["make", "-C", HERE, *targets], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")


def _d(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def lib() -> ctypes.CDLL:
    global _lib
    with _lock:
        if _lib is None:
            path = os.path.join(HERE, "liboracle.so")
            if not os.path.exists(path):
                build(ref=False)
            L = ctypes.CDLL(path)
            vp, i, sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t
            dbl = ctypes.c_double
            L.oracle_mass.argtypes = [i, i, i, vp, vp, vp, vp, sz, i]
            L.oracle_stiffness.argtypes = [i, i, i, vp, vp, vp, vp, sz, i]
            L.oracle_gemm_blocked.argtypes = [i, i, i, vp, vp, vp]
            L.oracle_gemm_blocked_batched.argtypes = [i, i, i, vp, vp, vp, sz]
            L.oracle_apply_contractions.argtypes = [i, i, i, vp, vp, vp, vp, vp, sz]
            L.oracle_helmholtz.argtypes = [i, i, vp, vp, vp, vp, dbl, dbl, vp, sz, i]
            L.oracle_helmholtz_diagonal.argtypes = [i, i, vp, vp, vp, dbl, dbl, vp, sz]
            L.oracle_cg.argtypes = [i, i, vp, vp, vp, dbl, dbl, vp, vp, sz, dbl, i,
                                    ctypes.POINTER(dbl)]
            for f in (L.oracle_mass, L.oracle_stiffness, L.oracle_helmholtz,
                      L.oracle_helmholtz_diagonal, L.oracle_cg):
                f.restype = ctypes.c_int
            _lib = L
        return _lib


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def mass(sem, degree, nquad, tables, u, d, nthreads=0):
    u, d, t = _f64(u), _f64(d), _f64(tables)
    ncells = u.shape[0]
    y = np.empty_like(u)
    rc = lib().oracle_mass(sem, degree + 1, nquad, t.ctypes.data, u.ctypes.data,
                           d.ctypes.data, y.ctypes.data, ncells, nthreads)
    if rc != 0:
        raise RuntimeError(f"oracle_mass rc={rc}")
    return y


def stiffness(sem, degree, nquad, tables, u, g, nthreads=0):
    u, g, t = _f64(u), _f64(g), _f64(tables)
    ncells = u.shape[0]
    y = np.empty_like(u)
    rc = lib().oracle_stiffness(sem, degree + 1, nquad, t.ctypes.data, u.ctypes.data,
                                g.ctypes.data, y.ctypes.data, ncells, nthreads)
    if rc != 0:
        raise RuntimeError(f"oracle_stiffness rc={rc}")
    return y


def gemm_blocked(k, m, n, a, b):
    a, b = _f64(a), _f64(b)
    c = np.empty(m * n)
    lib().oracle_gemm_blocked(k, m, n, a.ctypes.data, b.ctypes.data, c.ctypes.data)
    return c


def gemm_blocked_batched(k, m, n, a, b, ncells):
    a, b = _f64(a), _f64(b)
    c = np.empty(ncells * m * n)
    lib().oracle_gemm_blocked_batched(k, m, n, a.ctypes.data, b.ctypes.data, c.ctypes.data, ncells)
    return c


def apply_contractions(na, nb, tr, i0, i1, i2, b, ncells):
    i0, i1, i2, b = _f64(i0), _f64(i1), _f64(i2), _f64(b)
    a = np.empty(ncells * na ** 3)
    lib().oracle_apply_contractions(na, nb, int(bool(tr)), i0.ctypes.data, i1.ctypes.data,
                                    i2.ctypes.data, b.ctypes.data, a.ctypes.data, ncells)
    return a


def helmholtz(degree, nquad, tables, u, d, g, alpha, beta, nthreads=0):
    u, d, g, t = _f64(u), _f64(d), _f64(g), _f64(tables)
    y = np.empty_like(u)
    rc = lib().oracle_helmholtz(degree + 1, nquad, t.ctypes.data, u.ctypes.data, d.ctypes.data,
                                g.ctypes.data, alpha, beta, y.ctypes.data, u.shape[0], nthreads)
    if rc != 0:
        raise RuntimeError(f"oracle_helmholtz rc={rc}")
    return y


def helmholtz_diagonal(degree, nquad, tables, d, g, alpha, beta, ncells):
    d, g, t = _f64(d), _f64(g), _f64(tables)
    out = np.empty(ncells * (degree + 1) ** 3)
    lib().oracle_helmholtz_diagonal(degree + 1, nquad, t.ctypes.data, d.ctypes.data, g.ctypes.data,
                                    alpha, beta, out.ctypes.data, ncells)
    return out


def cg(degree, nquad, tables, d, g, alpha, beta, b, rtol, maxit):
    d, g, t, b = _f64(d), _f64(g), _f64(tables), _f64(b)
    x = np.empty_like(b)
    rel = ctypes.c_double()
    it = lib().oracle_cg(degree + 1, nquad, t.ctypes.data, d.ctypes.data, g.ctypes.data, alpha,
                         beta, b.ctypes.data, x.ctypes.data, b.size // (degree + 1) ** 3, rtol,
                         maxit, ctypes.byref(rel))
    return x, it, rel.value


# ----------------------------------------------------------------- _ref --
def ref_available() -> bool:
    return all(os.path.exists(os.path.join(HERE, "_ref", f))
               for f in ("libfemtc_ref_mass.so", "libfemtc_ref_stiffness.so"))


def _reflib(name):
    with _lock:
        if name not in _ref:
            L = ctypes.CDLL(os.path.join(HERE, "_ref", f"libfemtc_ref_{name}.so"))
            vp, i, sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t
            if name == "mass":
                L.ref_mass_f64.argtypes = [i, vp, vp, vp, vp, sz]
                L.ref_mass_f32.argtypes = [i, vp, vp, vp, vp, sz]
                L.ref_gemm_blocked_f64.argtypes = [i, i, vp, vp, vp]
            else:
                L.ref_stiffness_f64.argtypes = [i, vp, vp, vp, vp, sz]
                L.ref_stiffness_f32.argtypes = [i, vp, vp, vp, vp, sz]
            _ref[name] = L
        return _ref[name]


def ref_mass(degree, tables, u, d, dtype=np.float64):
    """The reference's own mass_operator<T,P,kij,0,0> (src/mass.hpp:10-49)."""
    u = np.ascontiguousarray(u, dtype=dtype).copy()
    d = np.ascontiguousarray(d, dtype=dtype)
    t = np.ascontiguousarray(tables, dtype=dtype)
    y = np.zeros_like(u)
    L = _reflib("mass")
    fn = L.ref_mass_f64 if dtype == np.float64 else L.ref_mass_f32
    rc = fn(degree, t.ctypes.data, u.ctypes.data, y.ctypes.data, d.ctypes.data, u.shape[0])
    if rc != 0:
        raise RuntimeError("reference mass: degree not built")
    return y


def ref_stiffness(degree, tables, u, g, dtype=np.float64):
    """The reference's own stiffness_operator<T,P,kij,0,0> (src/stiffness.hpp:34-99)."""
    u = np.ascontiguousarray(u, dtype=dtype).copy()
    g = np.ascontiguousarray(g, dtype=dtype)
    t = np.ascontiguousarray(tables, dtype=dtype)
    y = np.zeros_like(u)
    L = _reflib("stiffness")
    fn = L.ref_stiffness_f64 if dtype == np.float64 else L.ref_stiffness_f32
    rc = fn(degree, t.ctypes.data, u.ctypes.data, y.ctypes.data, g.ctypes.data, u.shape[0])
    if rc != 0:
        raise RuntimeError("reference stiffness: degree not built")
    return y


def ref_gemm_blocked(degree, blocked, a, b):
    n = degree + 1
    a, b = _f64(a), _f64(b)
    c = np.zeros(n * n * n)
    _reflib("mass").ref_gemm_blocked_f64(degree, int(blocked), a.ctypes.data, b.ctypes.data,
                                         c.ctypes.data)
    return c
