"""GPU parity of the affine forms (femtc_affine_apply: one detJ or one
detJ J^-1 J^-T per cell, the quadrature weights folded into the backward
tables) against the FP64 oracle run on the equivalent per-point factors
dw[c][q0][q1][q2] = w(q0) w(q1) w(q2) detJ[c] and
G[c][q0][q1][q2][k] = w(q0) w(q1) w(q2) Gc[c][k].

Tolerances (normwise, max|y - y_ref| / max|y_ref|): FP64 1e-12, FP32
2e-6 and double-float (F64E) 1e-13, the per-point operators' own.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {0: 1e-12, 1: 2e-6, 4: 1e-13}


def relerr(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def affine_mesh(femtc, op, P, Q, ncells, seed, weights=None):
    """(tables, weights, u, per-cell geometry, per-point geometry)."""
    from femtc_gb300 import workloads as W
    rng = np.random.default_rng(seed)
    t, _, w, _ = femtc.tabulate(P, Q)
    if weights is not None:
        w = weights
    J = W.random_jacobians(rng, ncells)
    w3 = W.tensor_weights(w)
    u = rng.uniform(-1.0, 1.0, (ncells, (P + 1) ** 3))
    if op == femtc.MASS_AFFINE:
        cg = np.linalg.det(J)
        pg = cg[:, None] * w3[None]
    else:
        cg = W.geometry_from_jacobians(J, np.ones(1)).reshape(ncells, 6)
        pg = cg[:, None, :] * w3[None, :, None]
    return t, w, u, np.ascontiguousarray(cg), np.ascontiguousarray(pg)


def oracle_ref(orc, femtc, op, P, Q, t, u, pg):
    fn = orc.mass if op == femtc.MASS_AFFINE else orc.stiffness
    return fn(orc.EXACT, P, Q, t, u, pg)


def run_affine(femtc, dev, op, dtype, P, Q, t, w, u, cg):
    import torch
    tdt = torch.float64 if dtype in femtc.FP64_STORAGE else torch.float32
    ud = torch.from_numpy(u).to(dev, tdt)
    gd = torch.from_numpy(cg).to(dev, tdt)
    yd = torch.full_like(ud, float("nan"))
    femtc.affine_apply(op, dtype, P, Q, t, w, ud, yd, gd, u.shape[0])
    torch.cuda.synchronize()
    assert femtc.device_status() == 0
    return yd.cpu().double().numpy()


@pytest.mark.parametrize("dtype", [0, 1, 4])
@pytest.mark.parametrize("op", [3, 4])
@pytest.mark.parametrize("P", range(1, 8))
@pytest.mark.parametrize("dq", [0, 1, 2])
def test_affine_vs_oracle(femtc, orc, dev, dtype, op, P, dq):
    Q = P + 1 + dq
    if dtype == 4 and P > 4:
        assert not femtc.supported(op, dtype, femtc.EXACT, P, Q)
        pytest.skip("double-float forms up to degree 4")
    assert femtc.supported(op, dtype, femtc.EXACT, P, Q)
    for ncells in (37, 1001):  # ragged tails, many tiles and CTAs
        t, w, u, cg, pg = affine_mesh(femtc, op, P, Q, ncells, seed=10 * P + dq + 100 * op)
        y = run_affine(femtc, dev, op, dtype, P, Q, t, w, u, cg)
        ref = oracle_ref(orc, femtc, op, P, Q, t, u, pg)
        assert relerr(y, ref) <= TOL[dtype], (ncells, relerr(y, ref))


@pytest.mark.parametrize("dtype", [0, 1, 4])
@pytest.mark.parametrize("op", [3, 4])
@pytest.mark.parametrize("P,Q", [(1, 3), (3, 5), (4, 6), (6, 8)])
def test_affine_plain_and_even_odd(femtc, orc, dev, dtype, op, P, Q):
    """Both kernel forms against the oracle: even-odd (symmetric tables and
    weights), plain (switched off), and plain with asymmetric weights (the
    even-odd split does not apply to them)."""
    if not femtc.supported(op, dtype, femtc.EXACT, P, Q):
        pytest.skip("variant not built")
    t, w, u, cg, pg = affine_mesh(femtc, op, P, Q, 555, seed=P + 7 * op)
    at = femtc.affine_tables(t, w)
    assert femtc.even_odd_used(op, dtype, femtc.EXACT, P, Q, at)
    y_eo = run_affine(femtc, dev, op, dtype, P, Q, t, w, u, cg)
    femtc.set_even_odd(False)
    try:
        assert not femtc.even_odd_used(op, dtype, femtc.EXACT, P, Q, at)
        y_plain = run_affine(femtc, dev, op, dtype, P, Q, t, w, u, cg)
    finally:
        femtc.set_even_odd(True)
    ref = oracle_ref(orc, femtc, op, P, Q, t, u, pg)
    assert relerr(y_eo, ref) <= TOL[dtype]
    assert relerr(y_plain, ref) <= TOL[dtype]
    skew = w * np.linspace(0.8, 1.2, Q)
    t, w2, u, cg, pg = affine_mesh(femtc, op, P, Q, 555, seed=P + 7 * op, weights=skew)
    assert not femtc.even_odd_used(op, dtype, femtc.EXACT, P, Q, femtc.affine_tables(t, w2))
    y = run_affine(femtc, dev, op, dtype, P, Q, t, w2, u, cg)
    assert relerr(y, oracle_ref(orc, femtc, op, P, Q, t, u, pg)) <= TOL[dtype]


@pytest.mark.parametrize("op", [3, 4])
def test_affine_matches_per_point_operator(femtc, dev, op):
    """Against the library's own per-point operator on a full-size tile
    count (FP64): same action, the weights applied in another order."""
    import torch
    P, Q, n = 4, 6, 20000
    t, w, u, cg, pg = affine_mesh(femtc, op, P, Q, n, seed=3)
    y = run_affine(femtc, dev, op, femtc.F64, P, Q, t, w, u, cg)
    ud = torch.from_numpy(u).to(dev)
    gd = torch.from_numpy(pg).to(dev)
    yp = torch.empty_like(ud)
    base = femtc.MASS if op == femtc.MASS_AFFINE else femtc.STIFFNESS
    femtc.apply(base, femtc.F64, femtc.EXACT, P, Q, t, ud, yp, gd, n)
    torch.cuda.synchronize()
    assert relerr(y, yp.cpu().numpy()) <= 1e-13


@pytest.mark.parametrize("dtype", [0, 1])
@pytest.mark.parametrize("op,P,Q", [(3, 3, 5), (4, 4, 6), (4, 1, 3)])
def test_affine_host_paths(femtc, dev, dtype, op, P, Q):
    """Host buffers: zero-copy (pinned), the staging pipeline and pageable
    buffers give the device path's bits."""
    import torch
    t, w, u, cg, _ = affine_mesh(femtc, op, P, Q, 333, seed=21)
    tdt = torch.float64 if dtype == 0 else torch.float32
    y_dev = run_affine(femtc, dev, op, dtype, P, Q, t, w, u, cg)
    at = femtc.affine_tables(t, w)
    uh = torch.from_numpy(u).to(tdt).pin_memory()
    gh = torch.from_numpy(cg).to(tdt).pin_memory()
    for mode in (0, 1):
        femtc.set_host_path(mode)
        try:
            yh = torch.full_like(uh, float("nan")).pin_memory()
            femtc.apply_host(op, dtype, femtc.EXACT, P, Q, at, uh, yh, gh, 333)
        finally:
            femtc.set_host_path(0)
        assert np.array_equal(yh.double().numpy(), y_dev), mode
    up, gp = uh.numpy().copy(), gh.numpy().copy()
    yp = np.empty_like(up)
    femtc.apply_host(op, dtype, femtc.EXACT, P, Q, at, up, yp, gp, 333)
    assert np.array_equal(yp.astype(np.float64), y_dev)


def test_affine_autotune_then_parity(femtc, orc, dev):
    """The autotuner on an affine form (no geometry staging candidates)
    keeps a shape that still matches the oracle."""
    import torch
    op, P, Q, n = femtc.STIFFNESS_AFFINE, 4, 6, 3000
    t, w, u, cg, pg = affine_mesh(femtc, op, P, Q, n, seed=9)
    at = femtc.affine_tables(t, w)
    ud = torch.from_numpy(u).to(dev)
    gd = torch.from_numpy(cg).to(dev)
    yd = torch.empty_like(ud)
    cb, staged, nt, ms = femtc.autotune(op, femtc.F64, femtc.EXACT, P, Q, at, ud, yd, gd, n)
    assert staged == 0 and cb % 4 == 0 and ms > 0
    assert femtc.get_tile_config(op, femtc.F64, femtc.EXACT, P, Q)[:3] == (cb, staged, nt)
    y = run_affine(femtc, dev, op, femtc.F64, P, Q, t, w, u, cg)
    assert relerr(y, oracle_ref(orc, femtc, op, P, Q, t, u, pg)) <= TOL[0]


def test_affine_geometry_from_jacobians(femtc, dev):
    """femtc_geometry with one point of weight 1 gives the affine forms'
    per-cell factors."""
    import torch
    from femtc_gb300 import workloads as W
    n = 257
    J = W.random_jacobians(np.random.default_rng(4), n)
    Jd = torch.from_numpy(np.ascontiguousarray(J.reshape(n, 9))).to(dev)
    dj = torch.empty(n, dtype=torch.float64, device=dev)
    G = torch.empty((n, 6), dtype=torch.float64, device=dev)
    femtc.geometry(femtc.F64, 1, np.ones(1), Jd, dj, G, n)
    torch.cuda.synchronize()
    assert np.allclose(dj.cpu().numpy(), np.linalg.det(J), rtol=1e-14, atol=0)
    want = W.geometry_from_jacobians(J, np.ones(1)).reshape(n, 6)
    assert relerr(G.cpu().numpy(), want) <= 1e-14


def test_affine_zero_cells_and_in_place(femtc, orc, dev):
    import torch
    op, P, Q = femtc.STIFFNESS_AFFINE, 3, 5
    t, w, u, cg, pg = affine_mesh(femtc, op, P, Q, 64, seed=2)
    ud = torch.from_numpy(u).to(dev)
    gd = torch.from_numpy(cg).to(dev)
    femtc.affine_apply(op, femtc.F64, P, Q, t, w, ud, ud, gd, 0)  # no-op
    torch.cuda.synchronize()
    assert np.array_equal(ud.cpu().numpy(), u)
    # y aliasing u: every tile reads its cells before it writes them
    femtc.affine_apply(op, femtc.F64, P, Q, t, w, ud, ud, gd, 64)
    torch.cuda.synchronize()
    assert relerr(ud.cpu().numpy(), oracle_ref(orc, femtc, op, P, Q, t, u, pg)) <= TOL[0]
