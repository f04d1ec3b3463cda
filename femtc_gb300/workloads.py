"""Seeded synthetic inputs for the operator workloads (host, numpy, FP64).

The reference ships no meshes or basis tables (bench_mass.cpp:72-88 fills
phi, U and detJ with std::rand()); these generators produce inputs with the
shapes and value distributions of the benchmark workloads:

  mass_p3      : P=3, Q=5, 4096 cells, D = detJ*w, detJ ~ U(0.5,1.5) per point,
                 u ~ U(-1,1)
  stiffness_p4 : P=4, Q=6, 32768 cells, affine J = I + 0.1 N(0,1) (redrawn while
                 det < 0.2), G = detJ w J^-1 J^-T (6 components), u ~ U(-1,1)
  stiffness_p6 : P=6, Q=8, 131072 cells, same geometry, u ~ N(0,1) plus
                 sin(pi x) sin(pi y) sin(pi z) at the cell's GLL nodes

make_affine(name) gives the same degree, Q and cell count on affine cells
(J = I + 0.1 N(0,1) per cell, u ~ U(-1,1)) with one geometry set per cell:
detJ (mass) or detJ J^-1 J^-T (stiffness), for the affine operator forms.

Layouts follow include/femtc_gpu.h.  Seeds are fixed per workload.  The
basis tables come from the library's femtc_tabulate unless the caller passes
another `tabulate(degree, nquad)` with the same result (a CPU-only caller
that must not load the GPU library).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import _lib


@dataclass
class Workload:
    name: str
    op: int
    degree: int
    nquad: int
    ncells: int
    tables: np.ndarray  # FP64, 2*Q*N
    u: np.ndarray       # FP64 [ncells, N^3]
    geo: np.ndarray     # FP64 mass [ncells, Q^3]; stiffness [ncells, Q^3, 6];
                        # affine forms: [ncells] or [ncells, 6]
    seed: int
    weights: np.ndarray | None = None  # affine forms: the Q 1D quadrature weights

    @property
    def affine(self) -> bool:
        return self.op in (_lib.MASS_AFFINE, _lib.STIFFNESS_AFFINE)

    @property
    def base_op(self) -> int:
        """MASS or STIFFNESS: the operator the workload applies."""
        return self.op - _lib.MASS_AFFINE if self.affine else self.op

    def op_tables(self) -> np.ndarray:
        """The tables the library's entry point for this workload takes."""
        return _lib.affine_tables(self.tables, self.weights) if self.affine else self.tables

    def point_geometry(self, k: int | None = None) -> np.ndarray:
        """Per-point factors of the first k cells (all by default): the
        geometry the per-point operator takes for the same action."""
        g = self.geo[:k]
        if not self.affine:
            return g
        w3 = tensor_weights(self.weights)
        if self.base_op == _lib.MASS:
            return np.ascontiguousarray(g[:, None] * w3[None])
        return np.ascontiguousarray(g[:, None, :] * w3[None, :, None])

    @property
    def n(self) -> int:
        return self.degree + 1

    @property
    def ndofs(self) -> int:
        return self.ncells * self.n ** 3


def tensor_weights(w: np.ndarray) -> np.ndarray:
    """w[q0]*w[q1]*w[q2] in [q0][q1][q2] order, flattened."""
    return np.einsum("i,j,k->ijk", w, w, w).reshape(-1)


def random_jacobians(rng: np.random.Generator, ncells: int) -> np.ndarray:
    """J = I + 0.1 N(0,1), redrawn while det(J) < 0.2."""
    J = np.eye(3)[None] + 0.1 * rng.standard_normal((ncells, 3, 3))
    while True:
        bad = np.linalg.det(J) < 0.2
        if not bad.any():
            return J
        J[bad] = np.eye(3)[None] + 0.1 * rng.standard_normal((int(bad.sum()), 3, 3))


def geometry_from_jacobians(J: np.ndarray, w3: np.ndarray) -> np.ndarray:
    """G[c, q, 6] = detJ_c w_q (J_c^-1 J_c^-T) in the order [zz,yz,xz,yy,xy,xx]."""
    Jinv = np.linalg.inv(J)
    K = np.einsum("cij,ckj->cik", Jinv, Jinv)  # J^-1 J^-T, symmetric
    det = np.linalg.det(J)
    comps = np.stack([K[:, 2, 2], K[:, 1, 2], K[:, 0, 2], K[:, 1, 1], K[:, 0, 1], K[:, 0, 0]], axis=1)
    comps = comps * det[:, None]
    return comps[:, None, :] * w3[None, :, None]


def _spec(name: str):
    """(degree, nquad, op, cells, seed) of a named workload."""
    if name == "mass_p3":
        return 3, 5, _lib.MASS, 4096, 1001
    if name == "stiffness_p4":
        return 4, 6, _lib.STIFFNESS, 32768, 1002
    if name == "stiffness_p6":
        return 6, 8, _lib.STIFFNESS, 131072, 1003
    raise ValueError(f"unknown workload {name}")


def make(name: str, ncells: int | None = None, seed: int | None = None,
         tabulate=None) -> Workload:
    degree, nquad, op, nc, sd = _spec(name)
    return make_custom(name, op, degree, nquad, ncells or nc, sd if seed is None else seed,
                       smooth=(name == "stiffness_p6"), tabulate=tabulate)


def make_affine(name: str, ncells: int | None = None, seed: int | None = None,
                tabulate=None) -> Workload:
    """The named workload's degree, Q and cell count on affine cells, with
    one geometry set per cell (the affine operator forms)."""
    degree, nquad, op, nc, sd = _spec(name)
    ncells = ncells or nc
    rng = np.random.default_rng(sd if seed is None else seed)
    tables, _, w, _ = (tabulate or _lib.tabulate)(degree, nquad)
    J = random_jacobians(rng, ncells)
    if op == _lib.MASS:
        geo, aop = np.linalg.det(J), _lib.MASS_AFFINE
    else:
        geo = geometry_from_jacobians(J, np.ones(1)).reshape(ncells, 6)
        aop = _lib.STIFFNESS_AFFINE
    u = rng.uniform(-1.0, 1.0, size=(ncells, (degree + 1) ** 3))
    return Workload(name + "_affine", aop, degree, nquad, ncells, tables, np.ascontiguousarray(u),
                    np.ascontiguousarray(geo), sd if seed is None else seed, weights=w)


def make_custom(name: str, op: int, degree: int, nquad: int, ncells: int, seed: int,
                smooth: bool = False, tabulate=None) -> Workload:
    rng = np.random.default_rng(seed)
    n = degree + 1
    tables, x, w, z = (tabulate or _lib.tabulate)(degree, nquad)
    w3 = tensor_weights(w)
    if op == _lib.MASS:
        detj = rng.uniform(0.5, 1.5, size=(ncells, nquad ** 3))
        geo = detj * w3[None, :]
        u = rng.uniform(-1.0, 1.0, size=(ncells, n ** 3))
    else:
        J = random_jacobians(rng, ncells)
        geo = geometry_from_jacobians(J, w3)
        if smooth:
            u = rng.standard_normal((ncells, n ** 3))
            # cell origins on a lattice, affine map x = x0 + J xi
            side = int(np.ceil(ncells ** (1.0 / 3.0)))
            idx = np.arange(ncells)
            x0 = np.stack([idx // (side * side), (idx // side) % side, idx % side], axis=1) / side
            xi = np.stack(np.meshgrid(z, z, z, indexing="ij"), axis=-1).reshape(-1, 3)
            X = x0[:, None, :] + np.einsum("cij,pj->cpi", J, xi) / side
            u += np.sin(np.pi * X[..., 0]) * np.sin(np.pi * X[..., 1]) * np.sin(np.pi * X[..., 2])
        else:
            u = rng.uniform(-1.0, 1.0, size=(ncells, n ** 3))
    return Workload(name, op, degree, nquad, ncells, tables, np.ascontiguousarray(u),
                    np.ascontiguousarray(geo), seed)


def box_dofmap(nx: int, ny: int, nz: int, degree: int):
    """DOF map of an nx x ny x nz box of hexahedra of degree P with shared
    (continuous) DOFs: cells in lexicographic order (x slowest), local DOF
    (i0, i1, i2) of cell (cx, cy, cz) -> global grid point
    (cx P + i0, cy P + i1, cz P + i2) of the (nx P + 1)(ny P + 1)(nz P + 1)
    grid, numbered with the last index fastest.  Returns (dofmap int32
    [ncells, N^3], ndofs)."""
    p, n = degree, degree + 1
    gy, gz = ny * p + 1, nz * p + 1
    cx, cy, cz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    i0, i1, i2 = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    gx_ = cx.reshape(-1, 1) * p + i0.reshape(1, -1)
    gy_ = cy.reshape(-1, 1) * p + i1.reshape(1, -1)
    gz_ = cz.reshape(-1, 1) * p + i2.reshape(1, -1)
    dofmap = (gx_ * gy + gy_) * gz + gz_
    return np.ascontiguousarray(dofmap, dtype=np.int32), (nx * p + 1) * gy * gz


def random_reference_inputs(op: int, degree: int, ncells: int, seed: int):
    """Inputs like the reference's own benchmark (bench_mass.cpp:72-88):
    random tables, U, and detJ/G, all U(0,1), Q = N.  Returns
    (tables[2*N*N], u[ncells,N^3], geo)."""
    rng = np.random.default_rng(seed)
    n = degree + 1
    tables = rng.uniform(0.0, 1.0, size=2 * n * n)
    u = rng.uniform(0.0, 1.0, size=(ncells, n ** 3))
    if op == _lib.MASS:
        geo = rng.uniform(0.0, 1.0, size=(ncells, n ** 3))
    else:
        geo = rng.uniform(0.0, 1.0, size=(ncells, n ** 3, 6))
    return tables, u, geo


def batch64_spec(seed: int = 1004, nmeshes: int = 64):
    """The batching workload: 64 meshes, degree P ~ U{1..7}, Q = P+2, cell
    counts log-uniform in [1e3, 1e5], half mass and half stiffness.
    Returns [(op, degree, ncells)]."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(nmeshes):
        degree = int(rng.integers(1, 8))
        ncells = int(round(10 ** rng.uniform(3.0, 5.0)))
        op = _lib.MASS if i < nmeshes // 2 else _lib.STIFFNESS
        out.append((op, degree, ncells))
    return out
