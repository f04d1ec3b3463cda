"""Generate the golden vectors in this directory from the reference itself.

Runs the reference's own kernel templates (IgorBaratta/femtc
src/mass.hpp:10-49, src/stiffness.hpp:34-99, src/linalg.hpp:101-182),
compiled from the reference sources by oracle/Makefile into oracle/_ref/,
on seeded inputs drawn like the reference's benchmark drivers
(bench_mass.cpp:72-88: tables, U and detJ/G uniform in [0,1], Q = N).

Usage (in a checkout that has the reference sources):
    make -C oracle ref && python tests/golden/make_golden.py
Writes reference_ops.npz (operator outputs, P = 1..7, FP64 and FP32) and
reference_gemm.npz (gemm_blocked outputs, P = 1..8).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402

NCELLS = 3


def main() -> None:
    if not oracle.ref_available():
        raise SystemExit("oracle/_ref is not built: run `make -C oracle ref` with the reference present")
    out = {}
    for P in range(1, 8):
        n = P + 1
        for op, name in ((0, "mass"), (1, "stiffness")):
            rng = np.random.default_rng(7000 + 10 * P + op)
            tables = rng.uniform(0.0, 1.0, size=2 * n * n)
            u = rng.uniform(0.0, 1.0, size=(NCELLS, n ** 3))
            geo = rng.uniform(0.0, 1.0, size=(NCELLS, n ** 3) if op == 0 else (NCELLS, n ** 3, 6))
            for dt, tag in ((np.float64, "f64"), (np.float32, "f32")):
                if op == 0:
                    y = oracle.ref_mass(P, tables[: n * n], u, geo, dtype=dt)
                else:
                    y = oracle.ref_stiffness(P, tables, u, geo, dtype=dt)
                out[f"{name}_P{P}_{tag}_y"] = y
            out[f"{name}_P{P}_tables"] = tables
            out[f"{name}_P{P}_u"] = u
            out[f"{name}_P{P}_geo"] = geo
    np.savez_compressed(os.path.join(HERE, "reference_ops.npz"), **out)

    g = {}
    for P in range(1, 9):
        n = P + 1
        rng = np.random.default_rng(8000 + P)
        a = rng.uniform(0.0, 1.0, size=n * n)
        b = rng.uniform(0.0, 1.0, size=n * n * n)
        g[f"P{P}_a"] = a
        g[f"P{P}_b"] = b
        g[f"P{P}_c_blocked"] = oracle.ref_gemm_blocked(P, 1, a, b)
        g[f"P{P}_c_plain"] = oracle.ref_gemm_blocked(P, 0, a, b)
    np.savez_compressed(os.path.join(HERE, "reference_gemm.npz"), **g)
    print("wrote", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    main()
