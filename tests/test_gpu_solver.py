"""GPU: matrix-free CG with the mixed-precision operator inside FP64
iterative refinement, and the continuous-batching server.

Checked against the oracle: the FP64 residual ||b - (alpha M + beta K) x||
computed on the CPU must be <= rtol ||b|| (1e-8), and x must match the
oracle's own FP64 CG solution; a solve gives the same bits alone and in a
mix of concurrent solves on the server."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def problem(femtc, P, Q, ncells, sigma, seed, inner_dtype=1, rtol=1e-8):
    from femtc_gb300 import workloads as W
    rng = np.random.default_rng(seed)
    J = W.random_jacobians(rng, ncells)
    b = rng.standard_normal((ncells, (P + 1) ** 3))
    return femtc.Problem(P, Q, J.reshape(-1, 9), b, alpha=1.0, beta=sigma, rtol=rtol,
                         inner_dtype=inner_dtype), J


def oracle_geo(femtc, P, Q, J):
    from femtc_gb300 import workloads as W
    _, _, w, _ = femtc.tabulate(P, Q)
    w3 = W.tensor_weights(w)
    d = np.linalg.det(J)[:, None] * w3[None]
    g = W.geometry_from_jacobians(J, w3)
    t, _, _, _ = femtc.tabulate(P, Q)
    return t, d, g


@pytest.mark.parametrize("inner_dtype", [1, 2, 3])
@pytest.mark.parametrize("P,Q,sigma", [(2, 4, 0.5), (3, 5, 5.0), (5, 7, 0.1)])
def test_solve_matches_oracle(femtc, orc, dev, inner_dtype, P, Q, sigma):
    pr, J = problem(femtc, P, Q, 60, sigma, seed=P * 10 + inner_dtype, inner_dtype=inner_dtype)
    res = femtc.solve(pr)
    assert res["rc"] == 0 and res["relres"] <= 1e-8, res
    t, d, g = oracle_geo(femtc, P, Q, J)
    r = pr.b - orc.helmholtz(P, Q, t, pr.x, d, g, 1.0, sigma)
    assert np.linalg.norm(r) <= 1.5e-8 * np.linalg.norm(pr.b)
    xo, it, rel = orc.cg(P, Q, t, d, g, 1.0, sigma, pr.b.reshape(-1), 1e-12, 5000)
    assert it > 0
    assert np.abs(pr.x.reshape(-1) - xo).max() <= 1e-6 * np.abs(xo).max()


def test_not_converged_is_reported(femtc, dev):
    pr, _ = problem(femtc, 3, 5, 40, 1.0, seed=1, rtol=1e-14)
    pr.req.max_outer = 1
    res = femtc.solve(pr)
    assert res["rc"] == femtc.NOT_CONVERGED and res["outer_iters"] == 1 and res["relres"] > 1e-14


def test_server_mix_equals_alone(femtc, dev):
    probs = [problem(femtc, P, P + 2, n, s, seed=i)[0]
             for i, (P, n, s) in enumerate([(2, 300, 0.3), (4, 120, 2.0), (3, 500, 7.0),
                                            (6, 40, 0.1), (5, 80, 1.0), (2, 50, 9.0)])]
    alone = []
    for p in probs:
        femtc.solve(p)
        alone.append(p.x.copy())
        p.x[:] = 0.0
    srv = femtc.Server(hbm_budget_bytes=8 << 30, max_active=3)
    try:
        tickets = [srv.submit(p) for p in probs]
        results = [srv.wait(t, 300.0) for t in tickets]
        st = srv.stats()
    finally:
        srv.close()
    assert all(r["rc"] == 0 for r in results)
    assert st["completed"] == len(probs) and st["max_concurrent"] >= 2
    for p, a in zip(probs, alone):
        assert np.array_equal(p.x, a)  # same bits alone and in the mix
    for r in results:
        assert r["t_submit_ms"] <= r["t_admit_ms"] <= r["t_done_ms"]


def test_server_applications_and_solves_mixed(femtc, orc, dev):
    """Operator applications served beside solves: each application's y is
    the same bits as the same application run alone through the host-buffer
    entry point, and matches the oracle; the solves are unchanged."""
    from femtc_gb300 import workloads as W
    probs = [problem(femtc, P, P + 2, n, s, seed=20 + i)[0]
             for i, (P, n, s) in enumerate([(3, 200, 1.0), (5, 60, 0.5), (2, 400, 4.0)])]
    alone_x = []
    for p in probs:
        femtc.solve(p)
        alone_x.append(p.x.copy())
        p.x[:] = 0.0
    apps, alone_y, refs = [], [], []
    for i, (op, dt, P, Q, n) in enumerate([(1, femtc.F64, 4, 6, 700), (0, femtc.F32, 3, 5, 900),
                                           (1, femtc.F64E, 3, 5, 300), (1, femtc.F32, 7, 9, 50),
                                           (0, femtc.F64, 9, 10, 20)]):
        w = W.make_custom("a", op, P, Q, n, seed=40 + i)
        # mass reads Phi only: its applications carry the Q x N Phi table alone
        tab = np.ravel(w.tables)[:Q * (P + 1)].copy() if op == 0 else w.tables
        a = femtc.Application(op, dt, femtc.EXACT, P, Q, tab, w.u, w.geo)
        y = np.empty_like(a.u)
        femtc.apply_host(op, dt, femtc.EXACT, P, Q, tab, a.u, y, a.geo, n)
        apps.append(a)
        alone_y.append(y)
        fn = orc.mass if op == 0 else orc.stiffness
        refs.append((fn(orc.EXACT, P, Q, w.tables, w.u, w.geo), 2e-6 if dt == femtc.F32 else 1e-12))
    srv = femtc.Server(hbm_budget_bytes=8 << 30, max_active=4)
    try:
        tickets = []
        for k in range(max(len(probs), len(apps))):
            if k < len(apps):
                tickets.append(srv.submit_apply(apps[k]))
            if k < len(probs):
                tickets.append(srv.submit(probs[k]))
        results = [srv.wait(t, 300.0) for t in tickets]
        st = srv.stats()
    finally:
        srv.close()
    assert all(r["rc"] == 0 for r in results)
    assert st["completed"] == len(tickets)
    for a, y, (ref, tol) in zip(apps, alone_y, refs):
        assert np.array_equal(a.y, y)  # same bits alone and in the mix
        err = np.abs(a.y - ref).max() / np.abs(ref).max()
        assert err <= tol, err
    for p, x in zip(probs, alone_x):
        assert np.array_equal(p.x, x)
    for r in results:
        assert r["t_submit_ms"] <= r["t_admit_ms"] <= r["t_done_ms"]


def test_server_budget_serialises(femtc, dev):
    p1 = problem(femtc, 3, 5, 400, 1.0, seed=1)[0]
    p2 = problem(femtc, 3, 5, 400, 1.0, seed=2)[0]
    need = femtc.solve_bytes(3, 5, 400)
    srv = femtc.Server(hbm_budget_bytes=int(need * 1.5), max_active=4)  # room for one at a time
    try:
        t1, t2 = srv.submit(p1), srv.submit(p2)
        r1, r2 = srv.wait(t1, 300.0), srv.wait(t2, 300.0)
        st = srv.stats()
    finally:
        srv.close()
    assert r1["rc"] == 0 and r2["rc"] == 0
    assert st["max_concurrent"] == 1 and st["peak_in_use_bytes"] <= need * 1.5
    assert r2["t_admit_ms"] >= r1["t_done_ms"] - 1.0


@pytest.mark.parametrize("policy", ["fifo", "shortest"])
def test_server_admission_order(femtc, dev, policy):
    """One worker: FIFO admits in arrival order; shortest-first admits the
    queued requests smallest first (equal waits, so the estimates decide)."""
    big = problem(femtc, 5, 7, 3000, 1.0, seed=11)[0]
    others = [problem(femtc, P, P + 2, n, 1.0, seed=20 + i)[0]
              for i, (P, n) in enumerate([(4, 800), (3, 300), (2, 50)])]
    pol = femtc.SERVE_FIFO if policy == "fifo" else femtc.SERVE_SHORTEST_FIRST
    srv = femtc.Server(hbm_budget_bytes=8 << 30, max_active=1, policy=pol)
    try:
        tickets = [srv.submit(big)] + [srv.submit(p) for p in others]
        res = [srv.wait(t, 300.0) for t in tickets]
    finally:
        srv.close()
    assert all(r["rc"] == 0 for r in res)
    admits = [r["t_admit_ms"] for r in res[1:]]
    if policy == "fifo":
        assert admits == sorted(admits)
    else:
        assert admits == sorted(admits, reverse=True)
