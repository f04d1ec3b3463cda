"""GPU: the tensor-core split forms against the FP64 oracle.

Target: max relative error <= 1e-6 (normwise, max|y - y64| / max|y64|) for
FEMTC_F16X2 (FP16 hi/lo, FP32 accumulate) and FEMTC_BF16X3 (BF16 three-term
split), FP32 storage, exact semantics; also checked on inputs spanning many
orders of magnitude (the FP16 form scales each MMA row by a power of two).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-6


def relerr(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def run(femtc, dev, op, dtype, P, Q, w, u=None):
    import torch
    u = w.u if u is None else u
    ud = torch.from_numpy(np.ascontiguousarray(u)).to(dev, torch.float32)
    gd = torch.from_numpy(w.geo).to(dev, torch.float32)
    yd = torch.full_like(ud, float("nan"))
    femtc.apply(op, dtype, femtc.EXACT, P, Q, w.tables, ud, yd, gd, u.shape[0])
    torch.cuda.synchronize()
    assert femtc.device_status() == 0
    return yd.cpu().double().numpy()


@pytest.mark.parametrize("dtype", [2, 3])
@pytest.mark.parametrize("op", [0, 1])
@pytest.mark.parametrize("P", range(1, 8))
@pytest.mark.parametrize("dq", [0, 1, 2])
def test_split_forms_vs_fp64_oracle(femtc, orc, dev, dtype, op, P, dq):
    from femtc_gb300 import workloads as W
    Q = P + 1 + dq
    if not femtc.supported(op, dtype, femtc.EXACT, P, Q):
        pytest.skip("variant not built")
    w = W.make_custom("t", op, P, Q, 203, seed=7 * P + dq)
    # the oracle sees the FP32-rounded inputs the GPU sees
    u32 = w.u.astype(np.float32).astype(np.float64)
    g32 = w.geo.astype(np.float32).astype(np.float64)
    t32 = w.tables.astype(np.float32).astype(np.float64)
    fn = orc.mass if op == 0 else orc.stiffness
    ref = fn(orc.EXACT, P, Q, t32, u32, g32)
    y = run(femtc, dev, op, dtype, P, Q, w)
    assert relerr(y, ref) <= MIXED_TOL, relerr(y, ref)


@pytest.mark.parametrize("dtype", [2, 3])
def test_split_wide_dynamic_range(femtc, orc, dev, dtype):
    from femtc_gb300 import workloads as W
    P, Q = 4, 6
    w = W.make_custom("t", 1, P, Q, 64, seed=3)
    rng = np.random.default_rng(0)
    # per-cell magnitudes from 1e-20 to 1e20 (FP16 alone would overflow)
    u = w.u * (10.0 ** rng.uniform(-20, 20, size=(64, 1)))
    ref = orc.stiffness(orc.EXACT, P, Q, w.tables.astype(np.float32).astype(np.float64),
                        u.astype(np.float32).astype(np.float64),
                        w.geo.astype(np.float32).astype(np.float64))
    y = run(femtc, dev, 1, dtype, P, Q, w, u=u)
    # per cell: each cell is independent, compare cell by cell
    for c in range(64):
        assert relerr(y[c], ref[c]) <= MIXED_TOL


def test_config3_error_report(femtc, orc, dev):
    """Stiffness P=6, Q=8 (the precision workload's degree) on a slice of its
    inputs: every form states its error against the FP64 oracle."""
    from femtc_gb300 import workloads as W
    w = W.make("stiffness_p6", ncells=4096)
    ref = orc.stiffness(orc.EXACT, 6, 8, w.tables, w.u, w.geo)
    errs = {}
    for dtype in (1, 2, 3):
        errs[dtype] = relerr(run(femtc, dev, 1, dtype, 6, 8, w), ref)
    print("max rel err vs FP64 oracle:", errs)
    assert all(e <= MIXED_TOL for e in errs.values()), errs
