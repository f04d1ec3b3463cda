"""The C++ drop-in header: compiles (CPU) and, on a GPU, runs the reference's
benchmark call sequence through it and matches the oracle."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "drop_in_driver.cpp")


def compile_driver(femtc, out):
    lib = femtc.lib_path()
    exe = os.path.join(out, "drop_in_driver")
    cmd = ["g++", "-std=c++20", "-O2", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"), SRC,
           "-o", exe, "-L", os.path.dirname(lib), "-lfemtc_gpu", f"-Wl,-rpath,{os.path.dirname(lib)}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_header_compiles(femtc, tmp_path):
    exe = compile_driver(femtc, str(tmp_path))
    assert os.path.exists(exe)


@pytest.mark.gpu
@pytest.mark.parametrize("op", ["mass", "stiffness"])
@pytest.mark.parametrize("dtype", ["double", "float"])
@pytest.mark.parametrize("degree", [1, 3, 4, 7, 8, 12, 15, 25])
def test_drop_in_matches_oracle(femtc, orc, dev, tmp_path, op, dtype, degree):
    """Degrees 1..7 run the slab kernels, 8..25 the general-degree kernel
    (shared-memory work buffers up to about N = 16, a device workspace
    above).  FP32 tolerance: 2e-6 to degree 7; sums of up to 26^3 positive
    products at the higher degrees are allowed 1e-5."""
    exe = compile_driver(femtc, str(tmp_path))
    ncells = 129 if degree <= 15 else 37
    r = subprocess.run([exe, op, str(degree), str(ncells), dtype, str(tmp_path)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    npdt = np.float64 if dtype == "double" else np.float32
    rd = lambda f: np.fromfile(os.path.join(tmp_path, f), dtype=npdt).astype(np.float64)
    n = degree + 1
    phi, U, geo = rd("phi.bin"), rd("U.bin").reshape(ncells, -1), rd("geo.bin")
    tables = np.concatenate([phi, np.zeros(2 * n * n - phi.size)])
    if op == "mass":
        ref = orc.mass(orc.REFERENCE, degree, n, tables, U, geo.reshape(ncells, -1))
    else:
        ref = orc.stiffness(orc.REFERENCE, degree, n, tables, U, geo.reshape(ncells, -1))
    tol = 1e-12 if dtype == "double" else (2e-6 if degree <= 7 else 1e-5)
    assert femtc.supported(0 if op == "mass" else 1, 0 if dtype == "double" else 1,
                           femtc.REFERENCE, degree, degree + 1)
    for f in ("W_dispatch.bin", "W_template.bin"):
        W = rd(f).reshape(ncells, -1)
        assert np.abs(W - ref).max() / np.abs(ref).max() <= tol


@pytest.mark.gpu
@pytest.mark.parametrize("op", ["affine_mass", "affine_stiffness"])
@pytest.mark.parametrize("dtype", ["double", "float"])
@pytest.mark.parametrize("degree", [1, 4, 7])
def test_drop_in_affine_matches_oracle(femtc, orc, dev, tmp_path, op, dtype, degree):
    """The header's affine operators against the oracle on the expanded
    per-point factors (Q = P+2, tabulated tables)."""
    from femtc_gb300 import workloads as W
    exe = compile_driver(femtc, str(tmp_path))
    ncells = 133
    r = subprocess.run([exe, op, str(degree), str(ncells), dtype, str(tmp_path)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    npdt = np.float64 if dtype == "double" else np.float32
    rd = lambda f: np.fromfile(os.path.join(tmp_path, f), dtype=npdt).astype(np.float64)
    n, q = degree + 1, degree + 2
    tab, U, geo = rd("tables.bin"), rd("U.bin").reshape(ncells, -1), rd("geo.bin")
    w3 = W.tensor_weights(tab[2 * q * n:])
    if op == "affine_mass":
        ref = orc.mass(orc.EXACT, degree, q, tab[:2 * q * n], U, geo[:, None] * w3[None])
    else:
        g = geo.reshape(ncells, 6)
        ref = orc.stiffness(orc.EXACT, degree, q, tab[:2 * q * n], U,
                            g[:, None, :] * w3[None, :, None])
    tol = 1e-12 if dtype == "double" else 2e-6
    Wt = rd("W_template.bin").reshape(ncells, -1)
    assert np.abs(Wt - ref).max() / np.abs(ref).max() <= tol
