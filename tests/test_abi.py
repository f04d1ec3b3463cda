"""CPU: the C-ABI library loads, exports every symbol include/*.h declares,
and rejects bad arguments before touching a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            txt = open(os.path.join(inc, f)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            syms |= set(re.findall(r"\b(femtc_[a-z0-9_]+)\s*\(", txt))
    return sorted(syms)


def test_exports_every_declared_symbol(femtc):
    lib = femtc.load()
    syms = declared_symbols()
    assert "femtc_mass_apply" in syms and "femtc_stiffness_apply" in syms
    for s in syms:
        assert hasattr(lib, s), f"{s} declared in include/ but not exported"


def test_version(femtc):
    assert femtc.load().femtc_version() >= 100


def test_supported_matrix(femtc):
    for P in range(1, 8):
        for op in (femtc.MASS, femtc.STIFFNESS):
            for dt in (femtc.F64, femtc.F32):
                assert femtc.supported(op, dt, femtc.REFERENCE, P, P + 1)
                for Q in (P + 1, P + 2):
                    assert femtc.supported(op, dt, femtc.EXACT, P, Q)
                assert not femtc.supported(op, dt, femtc.REFERENCE, P, P + 2)
    assert not femtc.supported(femtc.MASS, femtc.F64, femtc.EXACT, 30, 31)


@pytest.mark.parametrize("args,code", [
    (dict(degree=0), -1),            # degree < 1 (bench_mass.cpp:69-70 throws)
    (dict(nquad=0), -1),
    (dict(semantics=1, nquad=6), -1), # reference semantics needs Q == N
    (dict(degree=30, nquad=31), -2),  # not built
    (dict(dtype=9), -1),
])
def test_argument_errors(femtc, args, code):
    kw = dict(dtype=femtc.F64, semantics=femtc.EXACT, degree=3, nquad=4)
    kw.update(args)
    lib = femtc.load()
    buf = np.zeros(16)
    rc = lib.femtc_mass_apply(kw["dtype"], kw["semantics"], kw["degree"], kw["nquad"],
                              buf.ctypes.data, 16, 16, 16, 1, None)
    assert rc == code
    assert len(lib.femtc_last_error()) > 0


def test_null_pointer_rejected(femtc):
    lib = femtc.load()
    t = np.zeros(64)
    rc = lib.femtc_stiffness_apply(femtc.F64, femtc.EXACT, 3, 4, t.ctypes.data, None, 16, 16, 1, None)
    assert rc == -1


def test_tile_config_roundtrip(femtc, tmp_path):
    old = femtc.get_tile_config(femtc.MASS, femtc.F64, femtc.EXACT, 3, 5)
    femtc.set_tile_config(femtc.MASS, femtc.F64, femtc.EXACT, 3, 5, 8, 0, 128)
    assert femtc.get_tile_config(femtc.MASS, femtc.F64, femtc.EXACT, 3, 5) == (8, 0, 128, 1)
    with pytest.raises(femtc.FemtcError):
        femtc.set_tile_config(femtc.MASS, femtc.F64, femtc.EXACT, 3, 5, 6, 0)  # not a multiple of 4
    with pytest.raises(femtc.FemtcError):
        femtc.set_tile_config(femtc.MASS, femtc.F64, femtc.EXACT, 3, 5, 8, 0, 100)  # threads % 32
    db = str(tmp_path / "tiles.txt")
    femtc.tile_db_save(db)
    femtc.set_tile_config(femtc.MASS, femtc.F64, femtc.EXACT, 3, 5, 0, 0)  # back to default
    assert femtc.get_tile_config(femtc.MASS, femtc.F64, femtc.EXACT, 3, 5) == old
    assert femtc.tile_db_load(db) >= 1
    assert femtc.get_tile_config(femtc.MASS, femtc.F64, femtc.EXACT, 3, 5) == (8, 0, 128, 1)
    femtc.set_tile_config(femtc.MASS, femtc.F64, femtc.EXACT, 3, 5, 0, 0)


def test_geometry_modes_of_a_tile(femtc, tmp_path):
    """Geometry modes 0 (per-pencil L2 prefetch), 1 (TMA-staged) and 2
    (tile-start L2 prefetch) are accepted, stored and saved; others rejected."""
    key = (femtc.STIFFNESS, femtc.F32, femtc.EXACT, 4, 6)
    for mode in (0, 1, 2):
        femtc.set_tile_config(*key, 12, mode, 128, 2)
        assert femtc.get_tile_config(*key) == (12, mode, 128, 2)
    db = str(tmp_path / "tiles.txt")
    femtc.tile_db_save(db)
    femtc.set_tile_config(*key, 0, 0)
    assert femtc.tile_db_load(db) >= 1
    assert femtc.get_tile_config(*key) == (12, 2, 128, 2)
    for bad in (3, -1):
        with pytest.raises(femtc.FemtcError):
            femtc.set_tile_config(*key, 12, bad, 128, 2)
    femtc.set_tile_config(*key, 0, 0)


def test_fp32_lanes_choice_roundtrip(femtc):
    key = (femtc.STIFFNESS, femtc.F32, femtc.EXACT, 4, 6)
    for lanes in (1, 2):
        femtc.set_tile_config(*key, 12, 0, 128, lanes)
        assert femtc.get_tile_config(*key) == (12, 0, 128, lanes)
    femtc.set_tile_config(*key, 0, 0)
    assert femtc.get_tile_config(*key)[3] in (1, 2)


def test_helmholtz_supported_and_rejected(femtc):
    """The fused Helmholtz action: FP32 exact Q in N..N+2 built, other forms
    rejected before any device work."""
    lib = femtc.load()
    for P in range(1, 8):
        for Q in (P + 1, P + 2, P + 3):
            assert femtc.supported(femtc.HELMHOLTZ, femtc.F32, femtc.EXACT, P, Q)
        assert not femtc.supported(femtc.HELMHOLTZ, femtc.F64, femtc.EXACT, P, P + 1)
    t = np.zeros(128, dtype=np.float32)
    assert lib.femtc_helmholtz_apply(femtc.F64, 3, 4, t.ctypes.data, 16, 16, 16, 1, None) == -2
    assert lib.femtc_helmholtz_apply(femtc.F32, 3, 4, t.ctypes.data, None, 16, 16, 1, None) == -1
    assert lib.femtc_helmholtz_geometry(0, 1.0, 16, 1.0, 16, 16, 1, None) == -1
    assert lib.femtc_helmholtz_geometry(4, 1.0, 16, 1.0, 16, 24, 1, None) == -1  # misaligned


def test_affine_supported_and_rejected(femtc):
    """Affine forms: FP64 and FP32, exact semantics, degree 1..7 with Q in
    N..N+2; other forms and bad arguments rejected before any device work."""
    lib = femtc.load()
    for op in (femtc.MASS_AFFINE, femtc.STIFFNESS_AFFINE):
        for P in range(1, 8):
            for Q in (P + 1, P + 2, P + 3):
                for dt in (femtc.F64, femtc.F32):
                    assert femtc.supported(op, dt, femtc.EXACT, P, Q)
                assert femtc.supported(op, femtc.F64E, femtc.EXACT, P, Q) == (P <= 4)
            assert not femtc.supported(op, femtc.F64, femtc.REFERENCE, P, P + 1)
            assert not femtc.supported(op, femtc.F16X2, femtc.EXACT, P, P + 1)
    t = np.zeros(128)
    # the per-point operators are not affine forms
    assert lib.femtc_affine_apply(femtc.MASS, femtc.F64, 3, 4, t.ctypes.data, 16, 16, 16, 1,
                                  None) == -1
    assert lib.femtc_affine_apply_host(femtc.STIFFNESS, femtc.F64, 3, 4, t.ctypes.data, 16, 16,
                                       16, 1) == -1
    assert lib.femtc_affine_apply(femtc.MASS_AFFINE, femtc.F16X2, 3, 4, t.ctypes.data, 16, 16,
                                  16, 1, None) == -2
    assert lib.femtc_affine_apply(femtc.STIFFNESS_AFFINE, femtc.F64, 3, 4, t.ctypes.data, None,
                                  16, 16, 1, None) == -1
    with pytest.raises(ValueError):
        femtc.apply(femtc.MASS_AFFINE, femtc.F64, femtc.REFERENCE, 3, 4, t, 16, 16, 16, 1)


def test_affine_even_odd_selection(femtc):
    """Affine forms run the even-odd kernels when the tables and the
    weights are symmetric: tabulated tables with Gauss weights yes, with
    asymmetric weights no."""
    t, _, w, _ = femtc.tabulate(4, 6)
    at = femtc.affine_tables(t, w)
    for op in (femtc.MASS_AFFINE, femtc.STIFFNESS_AFFINE):
        for dt in (femtc.F64, femtc.F32):
            assert femtc.even_odd_used(op, dt, femtc.EXACT, 4, 6, at)
            skew = femtc.affine_tables(t, w * np.linspace(0.9, 1.1, w.size))
            assert not femtc.even_odd_used(op, dt, femtc.EXACT, 4, 6, skew)


def test_even_odd_selection(femtc):
    """Host-side choice of the even-odd kernels: FP64 exact with the
    tabulated (symmetric) tables, not with random tables, not for FP32 with
    two lanes, double-float with one or two lanes, not when switched off,
    not for stiffness N = 8 (the plain form there)."""
    t4 = femtc.tabulate(4, 6)[0]
    assert femtc.even_odd_used(femtc.STIFFNESS, femtc.F64, femtc.EXACT, 4, 6, t4)
    assert femtc.even_odd_used(femtc.MASS, femtc.F64, femtc.EXACT, 7, 9, femtc.tabulate(7, 9)[0])
    assert not femtc.even_odd_used(femtc.STIFFNESS, femtc.F64, femtc.EXACT, 7, 9,
                                   femtc.tabulate(7, 9)[0])
    assert not femtc.even_odd_used(femtc.STIFFNESS, femtc.F32, femtc.EXACT, 4, 6, t4)
    rnd = np.random.default_rng(0).uniform(-1, 1, t4.size)
    assert not femtc.even_odd_used(femtc.STIFFNESS, femtc.F64, femtc.EXACT, 4, 6, rnd)
    # double-float at degree 6 (Q = 8): the even-odd slab kernel for the
    # tabulated tables; the general-degree kernel (no even-odd form) for others
    t6 = femtc.tabulate(6, 8)[0]
    assert femtc.even_odd_used(femtc.STIFFNESS, femtc.F64E, femtc.EXACT, 6, 8, t6)
    rnd6 = np.random.default_rng(1).uniform(-1, 1, t6.size)
    assert not femtc.even_odd_used(femtc.STIFFNESS, femtc.F64E, femtc.EXACT, 6, 8, rnd6)
    # built with two lanes only: the built-in lane choice falls back to them
    femtc.set_tile_config(femtc.STIFFNESS, femtc.F64E, femtc.EXACT, 6, 8, 8, 0, 256)
    assert femtc.get_tile_config(femtc.STIFFNESS, femtc.F64E, femtc.EXACT, 6, 8)[3] == 2
    femtc.set_tile_config(femtc.STIFFNESS, femtc.F64E, femtc.EXACT, 6, 8, 0, 0)
    # double-float with two lanes per slab: the two-lane even-odd twin
    femtc.set_tile_config(femtc.STIFFNESS, femtc.F64E, femtc.EXACT, 4, 6, 12, 0, 256, 2)
    try:
        assert femtc.even_odd_used(femtc.STIFFNESS, femtc.F64E, femtc.EXACT, 4, 6, t4)
        assert not femtc.even_odd_used(femtc.STIFFNESS, femtc.F64E, femtc.EXACT, 4, 6, rnd)
    finally:
        femtc.set_tile_config(femtc.STIFFNESS, femtc.F64E, femtc.EXACT, 4, 6, 0, 0)
    femtc.set_even_odd(False)
    try:
        assert not femtc.even_odd_used(femtc.STIFFNESS, femtc.F64, femtc.EXACT, 4, 6, t4)
    finally:
        femtc.set_even_odd(True)


def test_bounded_wait_check_rejects_bad_limits(femtc):
    # checked before any launch (no GPU needed)
    lib = femtc.load()
    assert lib.femtc_bounded_wait_check(0, None) == -1
    assert lib.femtc_bounded_wait_check((1 << 22) + 1, None) == -1


def test_gemm_micro_rejects_bad_shapes_before_launch(femtc):
    lib = femtc.load()
    # lda < m
    assert lib.femtc_gemm_micro(0, 4, 4, 16, 3, 16, 16, 16, 16, 16, 1, 0, 0, 0, None) == -1
    # ldc < nc
    assert lib.femtc_gemm_micro(0, 4, 4, 16, 4, 16, 8, 16, 16, 16, 1, 0, 0, 0, None) == -1
    # overlapping C blocks
    assert lib.femtc_gemm_micro(0, 4, 4, 16, 4, 16, 16, 16, 16, 16, 2, 0, 0, 8, None) == -1


def test_supported_general_degrees(femtc):
    # the reference's ladder runs degrees 1..25 (src/mass.hpp:57-137)
    for P in range(8, 26):
        for op in (femtc.MASS, femtc.STIFFNESS):
            for dt in (femtc.F64, femtc.F32):
                assert femtc.supported(op, dt, femtc.REFERENCE, P, P + 1)
                assert femtc.supported(op, dt, femtc.EXACT, P, P + 2)
                assert not femtc.supported(op, dt, femtc.REFERENCE, P, P + 2)
        assert femtc.supported(femtc.MASS, femtc.F64E, femtc.EXACT, P, P + 2)
        assert not femtc.supported(femtc.MASS, femtc.F64E, femtc.REFERENCE, P, P + 1)
        assert not femtc.supported(femtc.STIFFNESS, femtc.BF16X3, femtc.EXACT, P, P + 2)
    assert not femtc.supported(femtc.MASS, femtc.F64, femtc.REFERENCE, 26, 27)
    assert not femtc.supported(femtc.MASS, femtc.F64, femtc.EXACT, 25, 29)


def test_general_kernel_tile_config_and_even_odd_query(femtc):
    # the general-degree kernel has one fixed shape and no even-odd form
    t = femtc.tabulate(12, 14)[0]
    assert femtc.get_tile_config(femtc.STIFFNESS, femtc.F64, femtc.EXACT, 12, 14) == (1, 0, 256, 1)
    assert femtc.even_odd_used(femtc.STIFFNESS, femtc.F64, femtc.EXACT, 12, 14, t) is False
