"""GPU parity of the fused Helmholtz action y = alpha M u + beta K u
(femtc_helmholtz_apply, FP32, exact semantics) against the FP64 oracle
(oracle_helmholtz), and of its interleaved geometry (femtc_helmholtz_geometry).

Tolerance (normwise, max|y - y_ref| / max|y_ref|): 2e-6, the FP32 operators'.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_F32 = 2e-6


def relerr(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def pack_geo8(d, g, alpha, beta):
    """[beta G (6), alpha dw, 0] per point, as the kernel reads it."""
    nc, q3 = d.shape
    out = np.zeros((nc, q3, 8))
    out[:, :, :6] = beta * g.reshape(nc, q3, 6)
    out[:, :, 6] = alpha * d
    return out


def mesh(femtc, P, Q, ncells, seed):
    from femtc_gb300 import workloads as W
    rng = np.random.default_rng(seed)
    t, _, w, _ = femtc.tabulate(P, Q)
    J = W.random_jacobians(rng, ncells)
    w3 = W.tensor_weights(w)
    d = np.linalg.det(J)[:, None] * w3[None]
    g = W.geometry_from_jacobians(J, w3).reshape(ncells, -1)
    u = rng.uniform(-1.0, 1.0, (ncells, (P + 1) ** 3))
    return t, d, g, u


@pytest.mark.parametrize("P", range(1, 8))
@pytest.mark.parametrize("dq", [0, 1, 2])
def test_helmholtz_vs_oracle(femtc, orc, dev, P, dq):
    import torch
    Q = P + 1 + dq
    if not femtc.supported(femtc.HELMHOLTZ, femtc.F32, femtc.EXACT, P, Q):
        pytest.skip("variant not built")
    for ncells, alpha, beta in ((37, 1.0, 0.3), (1001, 2.5, 7.0)):
        t, d, g, u = mesh(femtc, P, Q, ncells, seed=P * 7 + dq)
        ref = orc.helmholtz(P, Q, t, u, d, g, alpha, beta)
        geo8 = torch.from_numpy(pack_geo8(d, g, alpha, beta)).to(dev, torch.float32)
        ud = torch.from_numpy(u).to(dev, torch.float32)
        yd = torch.full_like(ud, float("nan"))
        femtc.helmholtz_apply(femtc.F32, P, Q, t, ud, yd, geo8, ncells)
        torch.cuda.synchronize()
        assert femtc.device_status() == 0
        err = relerr(yd.cpu().double().numpy(), ref)
        assert err <= TOL_F32, (ncells, err)


def test_helmholtz_geometry_packing(femtc, dev):
    import torch
    P, Q, n = 3, 5, 211
    _, d, g, _ = mesh(femtc, P, Q, n, seed=5)
    dd = torch.from_numpy(d).to(dev, torch.float32)
    gd = torch.from_numpy(g).to(dev, torch.float32)
    out = torch.full((n, Q ** 3, 8), float("nan"), device=dev, dtype=torch.float32)
    femtc.helmholtz_geometry(Q, 0.75, dd, 3.0, gd, out, n)
    torch.cuda.synchronize()
    want = pack_geo8(d.astype(np.float32).astype(np.float64),
                     g.astype(np.float32).astype(np.float64), 0.75, 3.0)
    assert np.abs(out.cpu().double().numpy() - want).max() <= 1e-6 * np.abs(want).max()


def test_helmholtz_equals_mass_plus_stiffness(femtc, dev):
    """The fused pass against alpha * mass + beta * stiffness (two FP32
    launches of the library), on a full-size tile count."""
    import torch
    P, Q, n, alpha, beta = 4, 6, 5000, 1.5, 0.25
    t, d, g, u = mesh(femtc, P, Q, n, seed=11)
    f32 = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev, torch.float32)
    ud, dd, gd = f32(u), f32(d), f32(g)
    geo8 = torch.empty((n, Q ** 3, 8), device=dev, dtype=torch.float32)
    femtc.helmholtz_geometry(Q, alpha, dd, beta, gd, geo8, n)
    y = torch.empty_like(ud)
    femtc.helmholtz_apply(femtc.F32, P, Q, t, ud, y, geo8, n)
    ym, yk = torch.empty_like(ud), torch.empty_like(ud)
    femtc.apply(femtc.MASS, femtc.F32, femtc.EXACT, P, Q, t, ud, ym, dd, n)
    femtc.apply(femtc.STIFFNESS, femtc.F32, femtc.EXACT, P, Q, t, ud, yk, gd, n)
    torch.cuda.synchronize()
    two = (alpha * ym.double() + beta * yk.double()).cpu().numpy()
    assert relerr(y.cpu().double().numpy(), two) <= 2e-6


def test_helmholtz_rejects_other_forms(femtc, dev):
    import torch
    P, Q, n = 2, 3, 8
    t, d, g, u = mesh(femtc, P, Q, n, seed=1)
    ud = torch.from_numpy(u).to(dev)
    geo8 = torch.zeros((n, Q ** 3, 8), device=dev, dtype=torch.float64)
    with pytest.raises(femtc.FemtcError):
        femtc.helmholtz_apply(femtc.F64, P, Q, t, ud, torch.empty_like(ud), geo8, n)
