"""GPU parity: the CUDA kernels (through the C ABI) against the oracle.

Tolerances (normwise: max|y - y_ref| / max|y_ref|):
  FP64 path vs FP64 oracle ...................... 1e-12
  FP32 path vs FP64 oracle ...................... 2e-6
  reference semantics vs the reference's own outputs (golden vectors),
    FP64 1e-12, FP32 vs the reference's float build 2e-6
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
TOL = {0: 1e-12, 1: 2e-6}


def relerr(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def run_gpu(femtc, dev, op, dtype, sem, P, Q, tables, u, geo, host=False):
    import torch
    tdt = torch.float64 if dtype in femtc.FP64_STORAGE else torch.float32
    if host:
        uh = np.ascontiguousarray(u, dtype=np.float64 if dtype in femtc.FP64_STORAGE else np.float32)
        gh = np.ascontiguousarray(geo, dtype=uh.dtype)
        yh = np.empty_like(uh)
        femtc.apply_host(op, dtype, sem, P, Q, tables, uh, yh, gh, u.shape[0])
        return yh.astype(np.float64)
    ud = torch.from_numpy(np.ascontiguousarray(u)).to(dev, tdt)
    gd = torch.from_numpy(np.ascontiguousarray(geo)).to(dev, tdt)
    yd = torch.full_like(ud, float("nan"))
    femtc.apply(op, dtype, sem, P, Q, tables, ud, yd, gd, u.shape[0])
    torch.cuda.synchronize()
    assert femtc.device_status() == 0
    return yd.cpu().double().numpy()


def oracle_apply(orc, op, sem, P, Q, tables, u, geo):
    fn = orc.mass if op == 0 else orc.stiffness
    return fn(sem, P, Q, tables, u, geo)


@pytest.mark.parametrize("dtype", [0, 1])
@pytest.mark.parametrize("op", [0, 1])
@pytest.mark.parametrize("P", range(1, 8))
@pytest.mark.parametrize("dq", [0, 1, 2])
def test_exact_vs_oracle(femtc, orc, dev, dtype, op, P, dq):
    from femtc_gb300 import workloads as W
    Q = P + 1 + dq
    if not femtc.supported(op, dtype, femtc.EXACT, P, Q):
        pytest.skip("variant not built")
    for ncells in (37, 1001):  # ragged tails, many tiles and CTAs
        w = W.make_custom("t", op, P, Q, ncells, seed=10 * P + dq + 100 * op)
        y = run_gpu(femtc, dev, op, dtype, femtc.EXACT, P, Q, w.tables, w.u, w.geo)
        ref = oracle_apply(orc, op, orc.EXACT, P, Q, w.tables, w.u, w.geo)
        assert relerr(y, ref) <= TOL[dtype], (ncells, relerr(y, ref))


@pytest.mark.parametrize("dtype", [0, 1])
@pytest.mark.parametrize("op", ["mass", "stiffness"])
@pytest.mark.parametrize("P", range(1, 8))
def test_reference_semantics_vs_golden(femtc, dev, dtype, op, P):
    """Literal parity with the reference's own kernels (golden vectors)."""
    z = np.load(os.path.join(HERE, "golden", "reference_ops.npz"))
    t, u, g = z[f"{op}_P{P}_tables"], z[f"{op}_P{P}_u"], z[f"{op}_P{P}_geo"]
    opc = 0 if op == "mass" else 1
    y = run_gpu(femtc, dev, opc, dtype, femtc.REFERENCE, P, P + 1, t, u, g)
    yref = z[f"{op}_P{P}_{'f64' if dtype == 0 else 'f32'}_y"]
    assert relerr(y, yref) <= TOL[dtype]


@pytest.mark.parametrize("op", [0, 1])
@pytest.mark.parametrize("P", [1, 3, 5, 7])
def test_reference_semantics_vs_oracle_many_cells(femtc, orc, dev, op, P):
    from femtc_gb300 import workloads as W
    t, u, g = W.random_reference_inputs(op, P, 777, seed=P)
    y = run_gpu(femtc, dev, op, femtc.F64, femtc.REFERENCE, P, P + 1, t, u, g)
    assert relerr(y, oracle_apply(orc, op, orc.REFERENCE, P, P + 1, t, u, g)) <= 1e-12


@pytest.mark.parametrize("op", [0, 1])
def test_host_path_matches_device_path(femtc, dev, op):
    from femtc_gb300 import workloads as W
    w = W.make_custom("t", op, 3, 5, 333, seed=4)
    a = run_gpu(femtc, dev, op, femtc.F64, femtc.EXACT, 3, 5, w.tables, w.u, w.geo)
    b = run_gpu(femtc, dev, op, femtc.F64, femtc.EXACT, 3, 5, w.tables, w.u, w.geo, host=True)
    assert np.array_equal(a, b)


def test_zero_cells_is_a_noop(femtc, dev):
    import torch
    t, _, _, _ = femtc.tabulate(3, 5)
    u = torch.zeros(64, dtype=torch.float64, device=dev)
    femtc.apply(femtc.MASS, femtc.F64, femtc.EXACT, 3, 5, t, u, u, u, 0)
    torch.cuda.synchronize()


def test_in_place(femtc, orc, dev):
    import torch
    from femtc_gb300 import workloads as W
    w = W.make_custom("t", 1, 4, 6, 500, seed=9)
    ud = torch.from_numpy(w.u).to(dev)
    gd = torch.from_numpy(w.geo).to(dev)
    femtc.apply(femtc.STIFFNESS, femtc.F64, femtc.EXACT, 4, 6, w.tables, ud, ud, gd, 500)
    torch.cuda.synchronize()
    ref = orc.stiffness(orc.EXACT, 4, 6, w.tables, w.u, w.geo)
    assert relerr(ud.cpu().numpy(), ref) <= 1e-12


def test_misaligned_pointer_rejected(femtc, dev):
    import torch
    t, _, _, _ = femtc.tabulate(3, 5)
    u = torch.zeros(1000, dtype=torch.float64, device=dev)
    with pytest.raises(femtc.FemtcError):
        femtc.apply(femtc.MASS, femtc.F64, femtc.EXACT, 3, 5, t, u.data_ptr() + 8, u, u, 2)


@pytest.mark.parametrize("dtype,lanes", [(0, 1), (1, 1), (1, 2), (2, 1)])
@pytest.mark.parametrize("P", [3, 4])
@pytest.mark.parametrize("staged", [0, 1, 2])
@pytest.mark.parametrize("cb,nt", [(4, 64), (8, 256), (12, 128), (28, 96)])
def test_tile_configs_agree(femtc, orc, dev, dtype, lanes, P, staged, cb, nt):
    from femtc_gb300 import workloads as W
    Q = P + 1
    w = W.make_custom("t", 1, P, Q, 203, seed=2)
    try:
        femtc.set_tile_config(femtc.STIFFNESS, dtype, femtc.EXACT, P, Q, cb, staged, nt, lanes)
    except femtc.FemtcError:
        pytest.skip("tile does not fit in shared memory")
    try:
        y = run_gpu(femtc, dev, 1, dtype, femtc.EXACT, P, Q, w.tables, w.u, w.geo)
    finally:
        femtc.set_tile_config(femtc.STIFFNESS, dtype, femtc.EXACT, P, Q, 0, 0)
    tol = {0: 1e-12, 1: 2e-6, 2: 1e-6}[dtype]
    assert relerr(y, orc.stiffness(orc.EXACT, P, Q, w.tables, w.u, w.geo)) <= tol


@pytest.mark.parametrize("lanes", [1, 2])
@pytest.mark.parametrize("op", [0, 1])
@pytest.mark.parametrize("P", range(1, 8))
@pytest.mark.parametrize("dq", [0, 1, 2])
def test_fp32_pairs_every_lane_count_vs_oracle(femtc, orc, dev, lanes, op, P, dq):
    """The FP32 exact kernels (contractions on packed FP32 pairs where the
    tile allows) with one and two lanes per slab, tile-start geometry
    prefetch, tabulated and random (non-symmetric) tables."""
    from femtc_gb300 import workloads as W
    Q = P + 1 + dq
    if not femtc.supported(op, 1, femtc.EXACT, P, Q):
        pytest.skip("variant not built")
    try:
        femtc.set_tile_config(op, 1, femtc.EXACT, P, Q, 8, 2, 128, lanes)
    except femtc.FemtcError:
        pytest.skip("tile does not fit in shared memory")
    try:
        w = W.make_custom("t", op, P, Q, 203, seed=7 * P + dq + 50 * op + lanes)
        y = run_gpu(femtc, dev, op, 1, femtc.EXACT, P, Q, w.tables, w.u, w.geo)
        assert relerr(y, oracle_apply(orc, op, orc.EXACT, P, Q, w.tables, w.u, w.geo)) <= 2e-6
        rng = np.random.default_rng(P + 10 * dq)
        tabs = rng.uniform(-1.0, 1.0, size=w.tables.shape)
        y = run_gpu(femtc, dev, op, 1, femtc.EXACT, P, Q, tabs, w.u, w.geo)
        assert relerr(y, oracle_apply(orc, op, orc.EXACT, P, Q, tabs, w.u, w.geo)) <= 2e-6
    finally:
        femtc.set_tile_config(op, 1, femtc.EXACT, P, Q, 0, 0)


@pytest.mark.parametrize("dtype,op,P,lanes,ncells", [
    (1, 1, 4, 2, 20001), (1, 1, 4, 2, 33333), (1, 0, 3, 1, 20001), (1, 0, 3, 1, 33335),
    (1, 1, 6, 1, 9001), (0, 0, 3, 1, 20003), (0, 1, 3, 1, 33333), (1, 1, 2, 2, 47779)])
def test_several_rounds_and_ragged_tail_vs_oracle(femtc, orc, dev, dtype, op, P, lanes, ncells):
    """Meshes of several rounds of tiles over every CTA plus a ragged last
    tile (8-cell tiles, 64-thread CTAs, so that a round is a few thousand
    cells), through both TMA stage counts.  Every cell is checked against
    the oracle, and none is left unwritten (y starts as NaN)."""
    from femtc_gb300 import workloads as W
    Q = P + 2
    try:
        femtc.set_tile_config(op, dtype, femtc.EXACT, P, Q, 8, 0, 64, lanes)
    except femtc.FemtcError:
        pytest.skip("tile does not fit in shared memory")
    try:
        w = W.make_custom("t", op, P, Q, ncells, seed=ncells % 97 + P)
        y = run_gpu(femtc, dev, op, dtype, femtc.EXACT, P, Q, w.tables, w.u, w.geo)
    finally:
        femtc.set_tile_config(op, dtype, femtc.EXACT, P, Q, 0, 0)
    assert np.isfinite(y).all()
    ref = oracle_apply(orc, op, orc.EXACT, P, Q, w.tables, w.u, w.geo)
    assert relerr(y, ref) <= TOL[dtype]


@pytest.mark.parametrize("dtype", [0, 1, 3])
def test_autotune_then_parity(femtc, orc, dev, dtype):
    import torch
    from femtc_gb300 import workloads as W
    P, Q = 4, 6
    w = W.make_custom("t", 1, P, Q, 3000, seed=8)
    tdt = torch.float64 if dtype == 0 else torch.float32
    u = torch.from_numpy(w.u).to(dev, tdt)
    g = torch.from_numpy(w.geo).to(dev, tdt)
    y = torch.empty_like(u)
    cb, st, nt, ms = femtc.autotune(femtc.STIFFNESS, dtype, femtc.EXACT, P, Q, w.tables, u, y, g, 3000)
    assert ms > 0 and cb % 4 == 0 and nt % 32 == 0
    assert femtc.get_tile_config(femtc.STIFFNESS, dtype, femtc.EXACT, P, Q)[:3] == (cb, st, nt)
    femtc.apply(femtc.STIFFNESS, dtype, femtc.EXACT, P, Q, w.tables, u, y, g, 3000)
    torch.cuda.synchronize()
    femtc.set_tile_config(femtc.STIFFNESS, dtype, femtc.EXACT, P, Q, 0, 0)
    ref = orc.stiffness(orc.EXACT, P, Q, w.tables, w.u, w.geo)
    assert relerr(y.double().cpu().numpy(), ref) <= (1e-12 if dtype == 0 else 1e-6)


def test_oversized_tile_rejected(femtc):
    # 20 cells of P=3/Q=5 FP64 stiffness with staged geometry need 260 KB
    with pytest.raises(femtc.FemtcError):
        femtc.set_tile_config(femtc.STIFFNESS, femtc.F64, femtc.EXACT, 3, 5, 20, 1)


@pytest.mark.parametrize("dtype", [0, 1, 3])
@pytest.mark.parametrize("op,P,Q", [(0, 3, 5), (1, 4, 6), (1, 1, 3), (0, 7, 9)])
def test_zero_copy_host_path(femtc, orc, dev, dtype, op, P, Q):
    """Pinned host buffers: the kernel reads and writes host memory directly
    (no staging copies) and must give the device path's bits."""
    import torch
    from femtc_gb300 import workloads as W
    w = W.make_custom("t", op, P, Q, 333, seed=21)
    tdt = torch.float64 if dtype == 0 else torch.float32
    uh = torch.from_numpy(w.u).to(tdt).pin_memory()
    gh = torch.from_numpy(w.geo).to(tdt).pin_memory()
    yh = torch.full_like(uh, float("nan")).pin_memory()
    femtc.apply_host(op, dtype, femtc.EXACT, P, Q, w.tables, uh, yh, gh, 333)
    ud, gd = uh.to(dev), gh.to(dev)
    yd = torch.empty_like(ud)
    femtc.apply(op, dtype, femtc.EXACT, P, Q, w.tables, ud, yd, gd, 333)
    torch.cuda.synchronize()
    assert torch.equal(yh, yd.cpu())
    # staging-copy mode gives the same result; zero-copy-only mode rejects pageable buffers
    femtc.set_host_path(1)
    try:
        yh2 = torch.full_like(uh, float("nan")).pin_memory()
        femtc.apply_host(op, dtype, femtc.EXACT, P, Q, w.tables, uh, yh2, gh, 333)
        assert torch.equal(yh2, yh)
        femtc.set_host_path(2)
        with pytest.raises(femtc.FemtcError):
            up = w.u.astype(np.float64 if dtype == 0 else np.float32)
            femtc.apply_host(op, dtype, femtc.EXACT, P, Q, w.tables, up, np.empty_like(up),
                             w.geo.astype(up.dtype), 333)
    finally:
        femtc.set_host_path(0)


def test_autotune_host_then_parity(femtc, orc, dev):
    import torch
    from femtc_gb300 import workloads as W
    P, Q = 4, 6
    w = W.make_custom("t", 1, P, Q, 2000, seed=31)
    uh = torch.from_numpy(w.u).pin_memory()
    gh = torch.from_numpy(w.geo).pin_memory()
    yh = torch.empty_like(uh).pin_memory()
    cb, st, nt, ms = femtc.autotune_host(femtc.STIFFNESS, femtc.F64, femtc.EXACT, P, Q, w.tables,
                                         uh, yh, gh, 2000)
    assert ms > 0 and cb % 4 == 0 and nt % 32 == 0
    yh.fill_(float("nan"))
    femtc.apply_host(femtc.STIFFNESS, femtc.F64, femtc.EXACT, P, Q, w.tables, uh, yh, gh, 2000)
    ref = orc.stiffness(orc.EXACT, P, Q, w.tables, w.u, w.geo)
    assert np.abs(yh.numpy() - ref).max() / np.abs(ref).max() <= 1e-12


@pytest.mark.parametrize("op", [0, 1])
@pytest.mark.parametrize("P", [1, 2, 3, 4])
@pytest.mark.parametrize("dq", [0, 1, 2])
def test_double_float_form_vs_oracle(femtc, orc, dev, op, P, dq):
    """FEMTC_F64E: FP64 storage, FP32-pair arithmetic, FP64 accuracy (1e-12)."""
    from femtc_gb300 import workloads as W
    Q = P + 1 + dq
    for ncells in (37, 1001):
        w = W.make_custom("t", op, P, Q, ncells, seed=3 * P + dq + 50 * op)
        y = run_gpu(femtc, dev, op, femtc.F64E, femtc.EXACT, P, Q, w.tables, w.u, w.geo)
        ref = oracle_apply(orc, op, orc.EXACT, P, Q, w.tables, w.u, w.geo)
        assert relerr(y, ref) <= 1e-12, relerr(y, ref)


@pytest.mark.parametrize("dtype", ["f64", "f64e"])
@pytest.mark.parametrize("op", [0, 1])
@pytest.mark.parametrize("P", range(1, 8))
@pytest.mark.parametrize("dq", [0, 1, 2])
def test_fp64_even_odd_and_plain_vs_oracle(femtc, orc, dev, dtype, op, P, dq):
    """FP64 and double-float, exact semantics, tabulated (symmetric)
    tables: the even-odd kernels (default) and the plain kernels (switched
    off) both within 1e-12 of the oracle, and within 1e-13 of one another."""
    from femtc_gb300 import workloads as W
    dt = femtc.F64 if dtype == "f64" else femtc.F64E
    Q = P + 1 + dq
    if not femtc.supported(op, dt, femtc.EXACT, P, Q):
        pytest.skip("variant not built")
    w = W.make_custom("eo", op, P, Q, 1001, seed=31 * P + dq + 7 * op)
    ref = oracle_apply(orc, op, orc.EXACT, P, Q, w.tables, w.u, w.geo)
    y_eo = run_gpu(femtc, dev, op, dt, femtc.EXACT, P, Q, w.tables, w.u, w.geo)
    femtc.set_even_odd(False)
    try:
        y_plain = run_gpu(femtc, dev, op, dt, femtc.EXACT, P, Q, w.tables, w.u, w.geo)
    finally:
        femtc.set_even_odd(True)
    assert relerr(y_eo, ref) <= 1e-12
    assert relerr(y_plain, ref) <= 1e-12
    assert relerr(y_eo, y_plain) <= 1e-13


@pytest.mark.parametrize("lanes", [1, 2])
@pytest.mark.parametrize("op", [0, 1])
@pytest.mark.parametrize("P", [1, 2, 3, 4, 6])
@pytest.mark.parametrize("dq", [0, 1, 2])
def test_f64e_even_odd_lanes_vs_plain_and_oracle(femtc, orc, dev, lanes, op, P, dq):
    """Double-float with one or two lanes per slab: the even-odd kernels (the
    default for tabulated tables; with two lanes the column pairs are split
    between the lanes and their sums combined by shuffles, including the
    middle column of odd Q) against the plain kernels and the oracle, on a
    ragged cell count and on several tile shapes of both streaming loops.
    At degree 6 (stiffness, Q = 8, two lanes) the even-odd slab kernel runs
    against the general-degree kernel, which serves the switched-off case."""
    from femtc_gb300 import workloads as W
    if P == 6 and (op != 1 or dq != 1 or lanes != 2):
        pytest.skip("degree 6: the slab kernel is built for stiffness, Q = 8, two lanes")
    Q = P + 1 + dq
    w = W.make_custom("eo2", op, P, Q, 1001, seed=17 * P + dq + 3 * op)
    ref = oracle_apply(orc, op, orc.EXACT, P, Q, w.tables, w.u, w.geo)
    ran = 0
    for cb, nt in ((8, 256), (12, 128), (20, 64)):
        try:
            femtc.set_tile_config(op, femtc.F64E, femtc.EXACT, P, Q, cb, 0, nt, lanes)
        except femtc.FemtcError:
            continue
        try:
            assert femtc.even_odd_used(op, femtc.F64E, femtc.EXACT, P, Q, w.tables)
            y_eo = run_gpu(femtc, dev, op, femtc.F64E, femtc.EXACT, P, Q, w.tables, w.u, w.geo)
            femtc.set_even_odd(False)
            try:
                y_plain = run_gpu(femtc, dev, op, femtc.F64E, femtc.EXACT, P, Q, w.tables, w.u,
                                  w.geo)
            finally:
                femtc.set_even_odd(True)
        finally:
            femtc.set_tile_config(op, femtc.F64E, femtc.EXACT, P, Q, 0, 0)
        assert relerr(y_eo, ref) <= 1e-12
        assert relerr(y_plain, ref) <= 1e-12
        assert relerr(y_eo, y_plain) <= 1e-13
        ran += 1
    assert ran > 0


@pytest.mark.parametrize("op", [0, 1])
@pytest.mark.parametrize("P", range(1, 5))
@pytest.mark.parametrize("dq", [0, 1, 2])
def test_fp32_even_odd_vs_plain_and_oracle(femtc, orc, dev, op, P, dq):
    """FP32 with one lane per slab (the form that has even-odd twins): the
    even-odd kernels (the default for tabulated tables) against the plain
    kernels and the oracle, on a ragged cell count and on several tiles."""
    from femtc_gb300 import workloads as W
    Q = P + 1 + dq
    w = W.make_custom("eo1", op, P, Q, 1001, seed=13 * P + dq + 5 * op)
    ref = oracle_apply(orc, op, orc.EXACT, P, Q, w.tables, w.u, w.geo)
    t32 = w.tables.astype(np.float32)
    for cb, nt in ((8, 256), (12, 128), (20, 64)):
        try:
            femtc.set_tile_config(op, femtc.F32, femtc.EXACT, P, Q, cb, 0, nt, 1)
        except femtc.FemtcError:
            continue
        try:
            assert femtc.even_odd_used(op, femtc.F32, femtc.EXACT, P, Q, t32)
            y_eo = run_gpu(femtc, dev, op, femtc.F32, femtc.EXACT, P, Q, w.tables, w.u, w.geo)
            femtc.set_even_odd(False)
            try:
                y_plain = run_gpu(femtc, dev, op, femtc.F32, femtc.EXACT, P, Q, w.tables, w.u,
                                  w.geo)
            finally:
                femtc.set_even_odd(True)
        finally:
            femtc.set_tile_config(op, femtc.F32, femtc.EXACT, P, Q, 0, 0)
        assert relerr(y_eo, ref) <= 2e-6
        assert relerr(y_plain, ref) <= 2e-6
        assert relerr(y_eo, y_plain) <= 2e-6


@pytest.mark.parametrize("op", [0, 1])
@pytest.mark.parametrize("P", [2, 4, 6])
def test_fp64_exact_nonsymmetric_tables(femtc, orc, dev, op, P):
    """Tables without the symmetry (random) run the plain kernels: still
    within 1e-12 of the oracle."""
    from femtc_gb300 import workloads as W
    Q = P + 2
    w = W.make_custom("ns", op, P, Q, 333, seed=P + 50 * op)
    rng = np.random.default_rng(P)
    tables = rng.uniform(-1.0, 1.0, size=w.tables.shape)
    ref = oracle_apply(orc, op, orc.EXACT, P, Q, tables, w.u, w.geo)
    y = run_gpu(femtc, dev, op, femtc.F64, femtc.EXACT, P, Q, tables, w.u, w.geo)
    assert relerr(y, ref) <= 1e-12
