"""GPU parity of the assembled (global-DOF) action y = sum_c P_c^T A_c P_c x
(femtc_assembled_apply) on box meshes with shared DOFs, against the FP64
oracle's cell results scattered with numpy (np.add.at).

Tolerances (normwise): FP64 1e-12, FP32 2e-6, FP16x2 / BF16x3 1e-6.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {0: 1e-12, 1: 2e-6, 2: 1e-6, 3: 1e-6}


def relerr(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def setup(femtc, dev, op, dtype, P, shape, seed):
    import torch
    from femtc_gb300 import workloads as W
    Q = P + 2
    dm, nd = W.box_dofmap(*shape, P)
    ncells = dm.shape[0]
    w = W.make_custom("a", op, P, Q, ncells, seed=seed)
    x = np.random.default_rng(seed + 1).uniform(-1.0, 1.0, nd)
    offsets, entries = femtc.dofmap_transpose(dm, nd)
    tdt = torch.float64 if dtype in femtc.FP64_STORAGE else torch.float32
    dev_i = lambda a: torch.from_numpy(a).to(dev)
    bufs = dict(dm=dev_i(dm), off=dev_i(offsets), ent=dev_i(entries),
                x=torch.from_numpy(x).to(dev, tdt), g=torch.from_numpy(w.geo).to(dev, tdt),
                y=torch.full((nd,), float("nan"), device=dev, dtype=tdt),
                work=torch.empty(femtc.assembled_work_bytes(dtype, P, ncells), device=dev,
                                 dtype=torch.uint8))
    return w, dm, nd, x, bufs


def reference(orc, op, P, w, dm, nd, x):
    fn = orc.mass if op == 0 else orc.stiffness
    yl = fn(orc.EXACT, P, P + 2, w.tables, x[dm], w.geo)
    y = np.zeros(nd)
    np.add.at(y, dm.ravel(), yl.ravel())
    return y


def run(femtc, op, dtype, P, w, nd, b):
    import torch
    femtc.assembled_apply(op, dtype, femtc.EXACT, P, P + 2, w.tables, b["dm"], b["off"], b["ent"],
                          nd, b["x"], b["y"], b["g"], w.ncells, b["work"])
    torch.cuda.synchronize()
    assert femtc.device_status() == 0
    return b["y"].double().cpu().numpy()


@pytest.mark.parametrize("dtype", [0, 1, 2, 3])
@pytest.mark.parametrize("op", [0, 1])
@pytest.mark.parametrize("P", [1, 2, 3, 4])
def test_assembled_vs_oracle(femtc, orc, dev, dtype, op, P):
    w, dm, nd, x, b = setup(femtc, dev, op, dtype, P, (5, 4, 3), seed=P + 10 * op)
    y = run(femtc, op, dtype, P, w, nd, b)
    xs = x.astype(np.float32).astype(np.float64) if dtype != 0 else x
    ref = reference(orc, op, P, w, dm, nd, xs)
    assert relerr(y, ref) <= TOL[dtype]


def test_assembled_deterministic_and_symmetric(femtc, dev):
    """Same bits on every call (fixed summation order), and the exact
    stiffness operator is symmetric: <x2, A x1> = <x1, A x2>."""
    import torch
    op, dtype, P = 1, 0, 3
    w, dm, nd, x, b = setup(femtc, dev, op, dtype, P, (20, 16, 12), seed=7)
    y1 = run(femtc, op, dtype, P, w, nd, b)
    y1b = run(femtc, op, dtype, P, w, nd, b)
    assert np.array_equal(y1, y1b)
    x2 = np.random.default_rng(99).uniform(-1.0, 1.0, nd)
    b["x"].copy_(torch.from_numpy(x2).to(dev))
    y2 = run(femtc, op, dtype, P, w, nd, b)
    lhs, rhs = float(x2 @ y1), float(x @ y2)
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0) * 10


def test_assembled_bad_map_entry_gives_nan(femtc, dev):
    """A map entry outside [0, ndofs) is not dereferenced (the kernels check
    every index): the DOFs it touches come out NaN, the rest are unchanged."""
    import torch
    op, dtype, P = 0, 0, 2
    w, dm, nd, x, b = setup(femtc, dev, op, dtype, P, (3, 3, 3), seed=5)
    y_ok = run(femtc, op, dtype, P, w, nd, b)
    bad = dm.copy()
    bad[4, 0] = nd + 1000  # cell 4, local DOF 0
    b["dm"].copy_(torch.from_numpy(bad).to(dev))
    y = run(femtc, op, dtype, P, w, nd, b)
    hit = np.unique(dm[4])  # every DOF of cell 4 sees the NaN through its cell result
    assert np.isnan(y[hit]).all()
    rest = np.setdiff1d(np.arange(nd), hit)
    assert np.array_equal(y[rest], y_ok[rest])


def test_assembled_no_cells_gives_zero(femtc, dev):
    """With no cells every global DOF's sum is empty: y is written as zero."""
    import torch
    op, dtype, P = 0, 0, 2
    w, dm, nd, x, b = setup(femtc, dev, op, dtype, P, (2, 2, 2), seed=3)
    femtc.assembled_apply(op, dtype, femtc.EXACT, P, P + 2, w.tables, b["dm"], b["off"], b["ent"],
                          nd, b["x"], b["y"], b["g"], 0, b["work"])
    torch.cuda.synchronize()
    assert np.array_equal(b["y"].cpu().numpy(), np.zeros(nd))
