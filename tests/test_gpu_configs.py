"""GPU parity at the benchmark configurations' sizes and generators.

- stiffness P=4, Q=6 (the headline workload's generator) on 2048 cells and
  the precision workload (stiffness P=6, Q=8, u = N(0,1) plus a smooth
  component) on 4096 cells: every form against the FP64 oracle;
- the 64-mesh batch at its full cell counts (342 M DOFs: 1e3..1e5 cells per
  mesh, degrees 1..7, Q = P+2, half mass, half stiffness): every mesh's
  first and last cells (the ragged tail included) against the oracle, for
  the three batch forms, and for the tuned split plan in FP32.

Tolerances (normwise): FP64 and double-float 1e-12; FP32 2e-6; FP16 hi/lo
and BF16x3 1e-6.  The batch runs FP32 inputs: its reference is the oracle
on the FP32-rounded inputs and geometry.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {0: 1e-12, 1: 2e-6, 2: 1e-6, 3: 1e-6, 4: 1e-12}


def relerr(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize("name,ncells,dtypes", [
    ("stiffness_p4", 2048, [0, 1, 2, 3, 4]),
    ("stiffness_p6", 4096, [0, 1, 2, 3, 4]),
    ("mass_p3", 4096, [0, 1, 2, 3, 4]),
])
def test_workload_forms_vs_oracle(femtc, orc, dev, name, ncells, dtypes):
    import torch
    from femtc_gb300 import workloads as W
    w = W.make(name, ncells=ncells)
    fn = orc.mass if w.op == 0 else orc.stiffness
    ref = fn(orc.EXACT, w.degree, w.nquad, w.tables, w.u, w.geo)
    for dtype in dtypes:
        assert femtc.supported(w.op, dtype, femtc.EXACT, w.degree, w.nquad)
        tdt = torch.float64 if dtype in femtc.FP64_STORAGE else torch.float32
        u = torch.from_numpy(w.u).to(dev, tdt)
        g = torch.from_numpy(w.geo).to(dev, tdt)
        y = torch.full_like(u, float("nan"))
        femtc.apply(w.op, dtype, femtc.EXACT, w.degree, w.nquad, w.tables, u, y, g, ncells)
        torch.cuda.synchronize()
        assert femtc.device_status() == 0
        assert relerr(y.double().cpu().numpy(), ref) <= TOL[dtype], (name, dtype)


def _batch64(femtc, dev):
    import torch
    from femtc_gb300 import workloads as W
    spec = W.batch64_spec()
    rng = np.random.default_rng(1004)
    gen = torch.Generator(device=dev).manual_seed(1004)
    meshes, J64 = [], []
    for op, P, n in spec:
        Q = P + 2
        tables, _, wts, _ = femtc.tabulate(P, Q)
        J = torch.from_numpy(W.random_jacobians(rng, n).reshape(n, 9)).to(dev)
        u = torch.rand(n, (P + 1) ** 3, device=dev, generator=gen, dtype=torch.float32) * 2 - 1
        shape = (n, Q ** 3) if op == 0 else (n, Q ** 3, 6)
        geo = torch.empty(shape, device=dev, dtype=torch.float32)
        if op == 0:
            femtc.geometry(femtc.F32, Q, wts, J, geo, None, n)
        else:
            femtc.geometry(femtc.F32, Q, wts, J, None, geo, n)
        meshes.append((op, P, Q, tables.astype(np.float32), u, torch.empty_like(u), geo, n))
    torch.cuda.synchronize()
    return spec, meshes


def _sample(n, k=32):
    return np.unique(np.concatenate([np.arange(min(k, n)), np.arange(max(0, n - k), n)]))


@pytest.mark.parametrize("dtype,tune", [(1, False), (2, False), (3, False), (1, True)])
def test_batch64_full_size_vs_oracle(femtc, orc, dev, dtype, tune):
    import torch
    spec, meshes = _batch64(femtc, dev)
    b = femtc.Batch(dtype, meshes, tune=tune)
    for m in meshes:
        m[5].fill_(float("nan"))
    b.launch()
    torch.cuda.synchronize()
    assert femtc.device_status() == 0
    worst = 0.0
    for op, P, Q, tab, u, y, geo, n in meshes:
        idx = _sample(n)
        fn = orc.mass if op == 0 else orc.stiffness
        ref = fn(orc.EXACT, P, Q, tab.astype(np.float64), u[idx].double().cpu().numpy(),
                 geo[idx].double().cpu().numpy())
        err = relerr(y[idx].double().cpu().numpy(), ref)
        worst = max(worst, err)
        assert err <= TOL[dtype], (op, P, n, err)
    b.close()
    assert worst > 0.0  # the forms round: an exact match would mean no work
