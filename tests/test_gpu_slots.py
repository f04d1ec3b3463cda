"""GPU parity of the padded DOF/output slab slots of even N, which the
single-mesh kernels fill and drain with 2D tensor copies (one to three boxes
per tile): FP64, double-float and FP32, both streaming loops, tile sizes
whose slab rows need one, two or three boxes, ragged last tiles, in place.

Tolerances (normwise): FP64 1e-12, double-float 1e-13, FP32 2e-6.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {0: 1e-12, 1: 2e-6, 4: 1e-13}


def relerr(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("dtype", [0, 1, 4])
@pytest.mark.parametrize("op", [0, 1])
@pytest.mark.parametrize("P", [1, 3, 5, 7])
@pytest.mark.parametrize("cb", [4, 36, 44, 64])
def test_slot_tiles_vs_oracle(femtc, orc, dev, dtype, op, P, cb):
    import torch
    from femtc_gb300 import workloads as W
    Q = P + 1
    if not femtc.supported(op, dtype, femtc.EXACT, P, Q):
        pytest.skip("variant not built")
    try:
        femtc.set_tile_config(op, dtype, femtc.EXACT, P, Q, cb, 0, 256, 1)
    except femtc.FemtcError:
        pytest.skip("tile does not fit in shared memory")
    try:
        w = W.make_custom("s", op, P, Q, 3 * cb * 152 + 37, seed=P + 10 * op)
        tdt = torch.float64 if dtype in femtc.FP64_STORAGE else torch.float32
        u = torch.from_numpy(w.u).to(dev, tdt)
        g = torch.from_numpy(w.geo).to(dev, tdt)
        y = torch.full_like(u, float("nan"))
        femtc.apply(op, dtype, femtc.EXACT, P, Q, w.tables, u, y, g, w.ncells)
        # in place: y aliasing u
        femtc.apply(op, dtype, femtc.EXACT, P, Q, w.tables, u, u, g, w.ncells)
        torch.cuda.synchronize()
        assert femtc.device_status() == 0
    finally:
        femtc.set_tile_config(op, dtype, femtc.EXACT, P, Q, 0, 0)
    fn = orc.mass if op == 0 else orc.stiffness
    k = 4000  # the oracle on the first cells (every tile shape repeats across tiles)
    ref = fn(orc.EXACT, P, Q, w.tables, w.u[:k], w.geo[:k])
    tail = fn(orc.EXACT, P, Q, w.tables, w.u[-300:], w.geo[-300:])
    yy = y.double().cpu().numpy()
    assert relerr(yy[:k], ref) <= TOL[dtype]
    assert relerr(yy[-300:], tail) <= TOL[dtype]
    assert np.array_equal(u.double().cpu().numpy(), yy)
