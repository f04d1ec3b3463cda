"""GPU parity of the general-degree kernel (cell_general.cu) against the
oracle, exact semantics, tabulated GLL-to-Gauss tables.

It serves every (N, Q) of mass and stiffness that the slab kernels do not
cover: degrees 8..25, quadrature sizes outside N..N+2 at low degree, and
the double-float form (F64E) above degree 4.  Work buffers sit in shared
memory up to about N = 16 (FP64 stiffness) and in a stream-ordered device
workspace above; both are exercised.
Tolerances (normwise): FP64 and F64E 1e-12, FP32 2e-6 up to degree 12,
1e-5 above.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run(femtc, dev, op, dtype, P, Q, ncells, seed):
    import torch
    from femtc_gb300 import workloads as W
    w = W.make_custom("g", op, P, Q, ncells, seed=seed)
    tdt = torch.float64 if dtype in femtc.FP64_STORAGE else torch.float32
    u = torch.from_numpy(w.u).to(dev, tdt)
    g = torch.from_numpy(w.geo).to(dev, tdt)
    y = torch.full_like(u, float("nan"))
    femtc.apply(op, dtype, femtc.EXACT, P, Q, w.tables, u, y, g, ncells)
    torch.cuda.synchronize()
    assert femtc.device_status() == 0
    return w, y.double().cpu().numpy()


@pytest.mark.parametrize("dtype", [0, 1])
@pytest.mark.parametrize("op", [0, 1])
@pytest.mark.parametrize("P,Q", [(8, 10), (9, 9), (11, 13), (12, 14), (15, 16), (20, 21),
                                 (3, 7), (1, 1)])
def test_general_exact_vs_oracle(femtc, orc, dev, dtype, op, P, Q):
    ncells = 33 if P <= 12 else 9  # ragged against any CTA count
    w, y = run(femtc, dev, op, dtype, P, Q, ncells, seed=P * 31 + Q + op)
    fn = orc.mass if op == 0 else orc.stiffness
    u = w.u.astype(np.float32).astype(np.float64) if dtype == 1 else w.u
    ref = fn(orc.EXACT, P, Q, w.tables, u, w.geo)
    tol = 1e-12 if dtype == 0 else (2e-6 if P <= 12 else 1e-5)
    assert np.abs(y - ref).max() / np.abs(ref).max() <= tol


@pytest.mark.parametrize("op", [0, 1])
@pytest.mark.parametrize("P,Q", [(5, 7), (6, 8), (7, 9), (9, 11), (4, 7)])
def test_general_double_float_vs_oracle(femtc, orc, dev, op, P, Q):
    # FP64-accurate on the FP32 pipes: the FP64 tolerance
    assert femtc.supported(op, femtc.F64E, femtc.EXACT, P, Q)
    w, y = run(femtc, dev, op, femtc.F64E, P, Q, 41, seed=P * 7 + Q + op)
    fn = orc.mass if op == 0 else orc.stiffness
    ref = fn(orc.EXACT, P, Q, w.tables, w.u, w.geo)
    assert np.abs(y - ref).max() / np.abs(ref).max() <= 1e-12


def test_general_repeat_is_bit_identical(femtc, dev):
    # the work buffers carry nothing from one call to the next
    _, y1 = run(femtc, dev, 1, 0, 10, 12, 40, seed=9)
    _, y2 = run(femtc, dev, 1, 0, 10, 12, 40, seed=9)
    assert np.array_equal(y1, y2)


def test_general_host_path_matches_device_path(femtc, dev):
    # the host-buffer entry (the drop-in path) through the general kernel
    from femtc_gb300 import workloads as W
    P, Q, n = 9, 11, 21
    w = W.make_custom("h", 1, P, Q, n, seed=4)
    _, yd = run(femtc, dev, 1, 0, P, Q, n, seed=4)
    yh = np.empty_like(w.u)
    femtc.apply_host(1, femtc.F64, femtc.EXACT, P, Q, w.tables, w.u, yh, w.geo, n)
    assert np.array_equal(yh, yd)
