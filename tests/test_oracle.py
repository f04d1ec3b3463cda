"""CPU: pin the oracle against the reference's own outputs and the math.

1. reference-semantics oracle == the reference templates' golden vectors
   (tests/golden/reference_ops.npz, made by tests/golden/make_golden.py from
   oracle/_ref, i.e. the reference's own src/mass.hpp / src/stiffness.hpp);
2. when oracle/_ref is built here, the same against freshly run reference
   code on new seeds;
3. exact-semantics oracle == an independent dense einsum formulation of
   B^T D B and sum_d D_d^T G D_d (general Q);
4. gemm_blocked restatement == the reference's gemm_blocked golden vectors
   (the reference's own unit test, tests/test_gemm.cpp, at 1e-10 abs).
"""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


def dense(op, P, Q, t, u, g):
    N = P + 1
    Phi = t[: Q * N].reshape(N, Q).T
    Gam = t[Q * N: 2 * Q * N].reshape(N, Q).T
    U = u.reshape(-1, N, N, N)
    if op == 0:
        v = np.einsum("ai,bj,ck,nijk->nabc", Phi, Phi, Phi, U) * g.reshape(-1, Q, Q, Q)
        return np.einsum("ai,bj,ck,nabc->nijk", Phi, Phi, Phi, v).reshape(u.shape)
    gx = np.einsum("ai,bj,ck,nijk->nabc", Gam, Phi, Phi, U)
    gy = np.einsum("ai,bj,ck,nijk->nabc", Phi, Gam, Phi, U)
    gz = np.einsum("ai,bj,ck,nijk->nabc", Phi, Phi, Gam, U)
    G = g.reshape(-1, Q, Q, Q, 6)
    fx = G[..., 5] * gx + G[..., 4] * gy + G[..., 2] * gz
    fy = G[..., 4] * gx + G[..., 3] * gy + G[..., 1] * gz
    fz = G[..., 2] * gx + G[..., 1] * gy + G[..., 0] * gz
    y = (np.einsum("ai,bj,ck,nabc->nijk", Gam, Phi, Phi, fx)
         + np.einsum("ai,bj,ck,nabc->nijk", Phi, Gam, Phi, fy)
         + np.einsum("ai,bj,ck,nabc->nijk", Phi, Phi, Gam, fz))
    return y.reshape(u.shape)


def relerr(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("P", range(1, 8))
@pytest.mark.parametrize("op", ["mass", "stiffness"])
def test_oracle_reference_semantics_vs_golden(orc, P, op):
    z = np.load(os.path.join(GOLD, "reference_ops.npz"))
    t, u, g = z[f"{op}_P{P}_tables"], z[f"{op}_P{P}_u"], z[f"{op}_P{P}_geo"]
    fn = orc.mass if op == "mass" else orc.stiffness
    y = fn(orc.REFERENCE, P, P + 1, t, u, g)
    # the same products summed in the same order: bit for bit
    assert np.array_equal(y, z[f"{op}_P{P}_f64_y"])


@pytest.mark.skipif(not __import__("oracle").ref_available(), reason="oracle/_ref not built")
@pytest.mark.parametrize("P", [1, 2, 3, 5, 7])
def test_oracle_vs_reference_fresh(orc, P):
    from femtc_gb300 import workloads as W
    for op in (0, 1):
        t, u, g = W.random_reference_inputs(op, P, 11, seed=100 + P)
        if op == 0:
            yr = orc.ref_mass(P, t[: (P + 1) ** 2], u, g)
            yo = orc.mass(orc.REFERENCE, P, P + 1, t, u, g)
        else:
            yr = orc.ref_stiffness(P, t, u, g)
            yo = orc.stiffness(orc.REFERENCE, P, P + 1, t, u, g)
        assert np.array_equal(yo, yr)


@pytest.mark.parametrize("P", [1, 2, 3, 4, 6, 7])
@pytest.mark.parametrize("dq", [0, 1, 2])
def test_oracle_exact_vs_dense(orc, femtc, P, dq):
    from femtc_gb300 import workloads as W
    Q = P + 1 + dq
    for op in (0, 1):
        w = W.make_custom("t", op, P, Q, 5, seed=3 * P + dq)
        fn = orc.mass if op == 0 else orc.stiffness
        y = fn(orc.EXACT, P, Q, w.tables, w.u, w.geo)
        assert relerr(y, dense(op, P, Q, w.tables, w.u, w.geo)) <= 1e-13


def test_oracle_exact_mass_equals_reference_for_symmetric_table(orc):
    # with Phi symmetric (Phi == Phi^T) the reference's backward pass (Phi
    # reused) and the exact one (Phi^T) coincide
    P, n = 3, 4
    rng = np.random.default_rng(1)
    A = rng.uniform(size=(n, n))
    S = A + A.T
    t = np.concatenate([S.T.reshape(-1), np.zeros(n * n)])
    u = rng.uniform(size=(4, n ** 3))
    d = rng.uniform(size=(4, n ** 3))
    assert relerr(orc.mass(orc.EXACT, P, n, t, u, d), orc.mass(orc.REFERENCE, P, n, t, u, d)) <= 1e-14


@pytest.mark.parametrize("P", range(1, 9))
def test_gemm_blocked_vs_golden(orc, P):
    z = np.load(os.path.join(GOLD, "reference_gemm.npz"))
    n = P + 1
    c = orc.gemm_blocked(n, n, n * n, z[f"P{P}_a"], z[f"P{P}_b"])
    # tests/test_gemm.cpp:46,57 use 1e-10 absolute
    assert np.abs(c - z[f"P{P}_c_blocked"]).max() <= 1e-10
    assert np.abs(c - z[f"P{P}_c_plain"]).max() <= 1e-10


def test_apply_contractions_matches_dense(orc):
    # src/tmm.hpp:91-126: A = (I0 x I1 x I2) B, Tr flag selects I or I^T
    rng = np.random.default_rng(2)
    na, nb, nc = 5, 4, 3
    I0, I1, I2 = (rng.uniform(size=na * nb) for _ in range(3))
    B = rng.uniform(size=nc * nb ** 3)
    a_tr = orc.apply_contractions(na, nb, True, I0, I1, I2, B, nc)
    M = [I.reshape(na, nb) for I in (I0, I1, I2)]
    ref = np.einsum("ai,bj,ck,nijk->nabc", *M, B.reshape(nc, nb, nb, nb)).reshape(-1)
    assert relerr(a_tr, ref) <= 1e-14
    a_nt = orc.apply_contractions(na, nb, False, I0, I1, I2, B, nc)
    M = [I.reshape(nb, na).T for I in (I0, I1, I2)]
    ref = np.einsum("ai,bj,ck,nijk->nabc", *M, B.reshape(nc, nb, nb, nb)).reshape(-1)
    assert relerr(a_nt, ref) <= 1e-14


def test_oracle_tabulate_matches_library(femtc):
    # two independent restatements of the GLL-to-Gauss tables (numpy's
    # Legendre module vs the library's Newton iterations)
    import oracle
    for P in range(1, 26):
        for Q in (P + 1, P + 2, P + 3):
            for a, b in zip(oracle.tabulate(P, Q), femtc.tabulate(P, Q)):
                assert np.abs(a - b).max() <= 1e-12 * max(1.0, np.abs(b).max())


def test_fast_build_agrees_with_parity_build():
    # the timing build (-Ofast, native ISA) computes the same operators to
    # rounding
    import oracle
    from femtc_gb300 import workloads as W
    for op, P, Q in ((0, 3, 5), (1, 4, 6)):
        w = W.make_custom("t", op, P, Q, 17, seed=5, tabulate=oracle.tabulate)
        fn = oracle.mass if op == 0 else oracle.stiffness
        a = fn(oracle.EXACT, P, Q, w.tables, w.u, w.geo)
        b = fn(oracle.EXACT, P, Q, w.tables, w.u, w.geo, fast=True)
        assert relerr(b, a) <= 1e-13


def test_gemm_micro_oracle_matches_loop(orc):
    # src/linalg.hpp:45-94 at the reference's own test sizes
    # (tests/test_micro.cpp:24-29: k=26, m=4, n=16, lda=4, ldb=ldc=16)
    rng = np.random.default_rng(7)
    k, m, n, lda, ldb, ldc = 26, 4, 16, 4, 16, 16
    a, b, c0 = rng.uniform(size=lda * k), rng.uniform(size=k * ldb), rng.uniform(size=m * ldc)
    c = orc.gemm_micro(k, m, n, lda, ldb, ldc, a, b, c0)
    ref = c0.copy()
    for i in range(m):
        for j in range(n):
            for p in range(k):
                ref[i * ldc + j] += a[i + p * lda] * b[p * ldb + j]
    assert np.abs(c - ref).max() <= 1e-12


def test_cg_oracle_converges(orc, femtc):
    from femtc_gb300 import workloads as W
    P, Q = 2, 4
    wm = W.make_custom("m", 0, P, Q, 6, seed=1)
    ws = W.make_custom("s", 1, P, Q, 6, seed=1)
    b = np.random.default_rng(0).standard_normal(wm.u.shape).reshape(-1)
    x, it, rel = orc.cg(P, Q, wm.tables, wm.geo, ws.geo, 1.0, 0.5, b, 1e-10, 500)
    assert it > 0 and rel <= 1e-10
    r = b - orc.helmholtz(P, Q, wm.tables, x.reshape(wm.u.shape), wm.geo, ws.geo, 1.0, 0.5).reshape(-1)
    assert np.linalg.norm(r) <= 1e-9 * np.linalg.norm(b)
