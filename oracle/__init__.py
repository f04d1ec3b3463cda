"""CPU oracle (test infrastructure only -- the checker, never the product).

Loads oracle/liboracle.so (the FP64 C restatement of the reference's
per-cell algorithm, femtc_oracle.c) and, when it was built from the
reference sources, oracle/_ref/*.so (the reference's own templates).
oracle/liboracle_fast.so is the same C source built with the reference's
recommended -Ofast and native-ISA flags: bench.py times the CPU baseline and
the reference arm on it (fast=True); parity checks use the IEEE build.
tabulate() restates the GLL-to-Gauss basis tables with numpy, so the CPU
arm needs nothing from the GPU library.
Only tests/, __graft_entry__.smoke() and bench.py's CPU legs import this
package.
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
_fast = None
_ref = {}
# Where the reference sources lie in the build container (absent on GPU
# hosts, where only the oracle's own C source is built).
REFERENCE_DIR = os.environ.get("FEMTC_REFERENCE_DIR", "/root/reference")


def build(ref: bool = True) -> None:
    """make -C oracle: liboracle.so, liboracle_fast.so, and _ref/ when the
    reference sources exist."""
    targets = ["liboracle.so", "liboracle_fast.so"] + (["ref"] if ref else [])
    cmd = ["make", "-C", HERE, *targets]
    if ref:
        cmd.append(f"REF={REFERENCE_DIR}")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")


def _d(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _open(name: str) -> ctypes.CDLL:
    path = os.path.join(HERE, name)
    if not os.path.exists(path):
        build(ref=False)
    L = ctypes.CDLL(path)
    _declare(L)
    return L


def lib() -> ctypes.CDLL:
    """The parity build (IEEE arithmetic)."""
    global _lib
    with _lock:
        if _lib is None:
            _lib = _open("liboracle.so")
        return _lib


def fast_lib() -> ctypes.CDLL:
    """The timing build (-Ofast, native ISA): the CPU baseline."""
    global _fast
    with _lock:
        if _fast is None:
            _fast = _open("liboracle_fast.so")
        return _fast


def fast_flags() -> str:
    """Compiler and flags of the timing build."""
    fast_lib()
    try:
        with open(os.path.join(HERE, "liboracle_fast.flags")) as f:
            return f.read().strip()
    except OSError:
        return "unknown"


def _declare(L: ctypes.CDLL) -> None:
    vp, i, sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t
    dbl = ctypes.c_double
    L.oracle_mass.argtypes = [i, i, i, vp, vp, vp, vp, sz, i]
    L.oracle_stiffness.argtypes = [i, i, i, vp, vp, vp, vp, sz, i]
    L.oracle_gemm_blocked.argtypes = [i, i, i, vp, vp, vp]
    L.oracle_gemm_blocked_batched.argtypes = [i, i, i, vp, vp, vp, sz]
    L.oracle_gemm_micro.argtypes = [i, i, i, i, i, i, vp, vp, vp]
    L.oracle_apply_contractions.argtypes = [i, i, i, vp, vp, vp, vp, vp, sz]
    L.oracle_helmholtz.argtypes = [i, i, vp, vp, vp, vp, dbl, dbl, vp, sz, i]
    L.oracle_helmholtz_diagonal.argtypes = [i, i, vp, vp, vp, dbl, dbl, vp, sz]
    L.oracle_cg.argtypes = [i, i, vp, vp, vp, dbl, dbl, vp, vp, sz, dbl, i,
                            ctypes.POINTER(dbl)]
    for f in (L.oracle_mass, L.oracle_stiffness, L.oracle_helmholtz,
              L.oracle_helmholtz_diagonal, L.oracle_cg):
        f.restype = ctypes.c_int


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def mass(sem, degree, nquad, tables, u, d, nthreads=0, fast=False):
    """y = B^T D B u per cell (src/mass.hpp:10-49; exact or reference
    semantics).  fast=True runs the timing build."""
    u, d, t = _f64(u), _f64(d), _f64(tables)
    ncells = u.shape[0]
    y = np.empty_like(u)
    rc = (fast_lib() if fast else lib()).oracle_mass(sem, degree + 1, nquad, t.ctypes.data, u.ctypes.data,
                           d.ctypes.data, y.ctypes.data, ncells, nthreads)
    if rc != 0:
        raise RuntimeError(f"oracle_mass rc={rc}")
    return y


def stiffness(sem, degree, nquad, tables, u, g, nthreads=0, fast=False):
    """y = sum_d D_d^T (G D u)_d per cell (src/stiffness.hpp:34-99; exact or
    reference semantics).  fast=True runs the timing build."""
    u, g, t = _f64(u), _f64(g), _f64(tables)
    ncells = u.shape[0]
    y = np.empty_like(u)
    rc = (fast_lib() if fast else lib()).oracle_stiffness(sem, degree + 1, nquad, t.ctypes.data, u.ctypes.data,
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


def gemm_micro(k, m, nc, lda, ldb, ldc, a, b, c):
    """c += a.b as linalg::gemm_micro (src/linalg.hpp:45-94): a column-major
    (lda), b and c row-major (ldb, ldc).  Returns the updated copy of c."""
    a, b = _f64(a), _f64(b)
    c = _f64(c).copy()
    lib().oracle_gemm_micro(k, m, nc, lda, ldb, ldc, a.ctypes.data, b.ctypes.data, c.ctypes.data)
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


# ------------------------------------------------------------ tabulation --
def tabulate(degree: int, nquad: int):
    """(tables[2*Q*N], points[Q], weights[Q], nodes[N]) in FP64: Lagrange
    basis on the P+1 Gauss-Lobatto-Legendre nodes of [0,1] and its
    derivative, at the Q Gauss-Legendre points of [0,1], in the layout
    Phi(q,i) = tables[q + i*Q], Gamma(q,i) = tables[Q*N + q + i*Q].
    Independent of the GPU library: Gauss points and weights from numpy's
    leggauss; GLL nodes are the endpoints and the roots of L_P' (numpy's
    legder/legroots, polished by Newton steps on L_P'); the basis and its
    derivative from the Lagrange product formula."""
    from numpy.polynomial import legendre as L
    t, w = L.leggauss(nquad)
    x, w = 0.5 * (t + 1.0), 0.5 * w
    cP = np.zeros(degree + 1)
    cP[-1] = 1.0
    d1, d2 = L.legder(cP), L.legder(cP, 2)
    r = np.sort(np.real(L.legroots(d1))) if degree > 1 else np.zeros(0)
    for _ in range(3):
        r = r - L.legval(r, d1) / L.legval(r, d2)
    z = np.concatenate([[0.0], 0.5 * (r + 1.0), [1.0]])
    n = degree + 1
    phi = np.empty((n, nquad))
    dphi = np.empty((n, nquad))
    for i in range(n):
        others = [j for j in range(n) if j != i]
        fac = [(x - z[j]) / (z[i] - z[j]) for j in others]
        phi[i] = np.prod(fac, axis=0)
        acc = np.zeros(nquad)
        for a, m in enumerate(others):
            rest = [fac[b] for b in range(len(others)) if b != a]
            acc += (np.prod(rest, axis=0) if rest else 1.0) / (z[i] - z[m])
        dphi[i] = acc
    tables = np.concatenate([phi.reshape(-1), dphi.reshape(-1)])
    return tables, x, w, z


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
