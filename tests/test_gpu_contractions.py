"""GPU: the stand-alone contraction entries and the FP64 geometry kernel.

femtc_gemm_micro mirrors the reference's micro-kernel test
(tests/test_micro.cpp:12-53: k = 26, m = 4, n = 16, lda = 4, ldb = ldc = 16,
accumulating into C) against the oracle's restatement at 1e-12 absolute;
femtc_gemm_blocked mirrors the reference's own unit test
(tests/test_gemm.cpp: P = 1..25, A (P+1)x(P+1) column-major, B row-major,
1e-10 absolute) and the golden vectors of the reference's gemm_blocked;
femtc_apply_contractions is checked against the oracle's restatement of
src/tmm.hpp:91-126; femtc_geometry against numpy in FP64.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.parametrize("P", range(1, 26))
def test_gemm_blocked_like_reference_test(femtc, dev, P):
    import torch
    k = m = P + 1
    n = (P + 1) ** 2
    rng = np.random.default_rng(P)
    batch = 7
    A = rng.uniform(size=m * k)                     # column-major m x k
    B = rng.uniform(size=(batch, k * n))            # row-major k x n per cell
    Bd = torch.from_numpy(B).to(dev)
    Cd = torch.full((batch, m * n), float("nan"), dtype=torch.float64, device=dev)
    femtc.gemm_blocked(femtc.F64, k, m, n, A, Bd, Cd, batch)
    torch.cuda.synchronize()
    C = Cd.cpu().numpy()
    Am = A.reshape(k, m).T
    for c in range(batch):
        ref = (Am @ B[c].reshape(k, n)).T.reshape(-1)  # column-major m x n
        assert np.abs(C[c] - ref).max() <= 1e-10


def test_gemm_micro_like_reference_test(femtc, orc, dev):
    import torch
    k, m, n, lda, ldb, ldc = 26, 4, 16, 4, 16, 16
    rng = np.random.default_rng(26)
    A = rng.uniform(size=lda * k)   # column-major 4 x k
    B = rng.uniform(size=k * ldb)   # row-major k x 16
    C0 = np.zeros(m * ldc)          # row-major 4 x 16, accumulated into
    d = lambda x: torch.from_numpy(x).to(dev)
    Cd = d(C0)
    femtc.gemm_micro(femtc.F64, k, m, n, lda, ldb, ldc, d(A), d(B), Cd)
    torch.cuda.synchronize()
    ref = orc.gemm_micro(k, m, n, lda, ldb, ldc, A, B, C0)
    assert np.abs(Cd.cpu().numpy() - ref).max() <= 1e-12  # tests/test_micro.cpp:47


@pytest.mark.parametrize("dtype", [0, 1])
def test_gemm_micro_batched_accumulates_with_strides(femtc, orc, dev, dtype):
    # padded leading dimensions, a shared A, per-item B and C, C nonzero on
    # entry (+= semantics); padding columns of C are left untouched
    import torch
    k, m, n, lda, ldb, ldc, batch = 7, 5, 9, 6, 11, 10, 13
    rng = np.random.default_rng(5 + dtype)
    A = rng.uniform(-1, 1, size=lda * k)
    B = rng.uniform(-1, 1, size=(batch, k * ldb))
    C0 = rng.uniform(-1, 1, size=(batch, m * ldc))
    tdt = torch.float64 if dtype == 0 else torch.float32
    d = lambda x: torch.from_numpy(np.ascontiguousarray(x)).to(dev, tdt)
    Cd = d(C0)
    femtc.gemm_micro(dtype, k, m, n, lda, ldb, ldc, d(A), d(B), Cd, batch=batch,
                     strides=(0, k * ldb, m * ldc))
    torch.cuda.synchronize()
    C = Cd.double().cpu().numpy()
    tol = 1e-12 if dtype == 0 else 2e-6
    for c in range(batch):
        a, b, c0 = A, B[c], C0[c]
        if dtype == 1:
            a, b, c0 = (x.astype(np.float32).astype(np.float64) for x in (a, b, c0))
        ref = orc.gemm_micro(k, m, n, lda, ldb, ldc, a, b, c0)
        assert np.abs(C[c] - ref).max() <= tol * max(1.0, np.abs(ref).max())
        pad = np.ones(m * ldc, bool)
        pad.reshape(m, ldc)[:, :n] = False
        assert np.array_equal(C[c][pad], d(C0[c]).double().cpu().numpy()[pad])


def test_gemm_micro_rejects_overlapping_items(femtc, dev):
    import torch
    x = torch.zeros(64, dtype=torch.float64, device=dev)
    with pytest.raises(femtc.FemtcError):
        femtc.gemm_micro(femtc.F64, 2, 2, 2, 2, 2, 2, x, x, x, batch=2, strides=(0, 0, 0))


@pytest.mark.parametrize("P", range(1, 9))
def test_gemm_blocked_vs_reference_golden(femtc, dev, P):
    import torch
    z = np.load(os.path.join(HERE, "golden", "reference_gemm.npz"))
    n = P + 1
    Bd = torch.from_numpy(z[f"P{P}_b"]).to(dev).reshape(1, -1)
    Cd = torch.empty((1, n * n * n), dtype=torch.float64, device=dev)
    femtc.gemm_blocked(femtc.F64, n, n, n * n, z[f"P{P}_a"], Bd, Cd, 1)
    torch.cuda.synchronize()
    assert np.abs(Cd.cpu().numpy()[0] - z[f"P{P}_c_blocked"]).max() <= 1e-12


@pytest.mark.parametrize("tr", [True, False])
@pytest.mark.parametrize("na,nb", [(5, 4), (4, 4), (3, 6), (9, 8)])
@pytest.mark.parametrize("dtype", [0, 1])
def test_apply_contractions_vs_oracle(femtc, orc, dev, tr, na, nb, dtype):
    import torch
    rng = np.random.default_rng(na * 10 + nb)
    ncells = 300
    I = [rng.uniform(-1, 1, size=na * nb) for _ in range(3)]
    B = rng.uniform(-1, 1, size=ncells * nb ** 3)
    ref = orc.apply_contractions(na, nb, tr, *I, B, ncells)
    tdt = torch.float64 if dtype == 0 else torch.float32
    Bd = torch.from_numpy(B).to(dev, tdt)
    Ad = torch.empty(ncells * na ** 3, dtype=tdt, device=dev)
    femtc.apply_contractions(dtype, na, nb, tr, *I, Bd, Ad, ncells)
    torch.cuda.synchronize()
    err = np.abs(Ad.double().cpu().numpy() - ref).max() / np.abs(ref).max()
    assert err <= (1e-13 if dtype == 0 else 1e-6)


@pytest.mark.parametrize("per_point", [False, True])
@pytest.mark.parametrize("out_dtype", [0, 1])
def test_geometry_vs_numpy(femtc, dev, per_point, out_dtype):
    import torch
    from femtc_gb300 import workloads as W
    Q, ncells = 6, 257
    rng = np.random.default_rng(5)
    _, _, w, _ = femtc.tabulate(4, Q)
    w3 = W.tensor_weights(w)
    J = W.random_jacobians(rng, ncells)
    if per_point:
        Jp = np.repeat(J[:, None], Q ** 3, axis=1) * (1 + 0.01 * rng.standard_normal((ncells, Q ** 3, 1, 1)))
        Jin = Jp.reshape(-1, 9)
        Jinv = np.linalg.inv(Jp)
        K = np.einsum("cqij,cqkj->cqik", Jinv, Jinv)
        det = np.linalg.det(Jp)
        comps = np.stack([K[..., 2, 2], K[..., 1, 2], K[..., 0, 2], K[..., 1, 1], K[..., 0, 1],
                          K[..., 0, 0]], axis=-1) * (det * w3[None])[..., None]
        Gref, dref = comps, det * w3[None]
    else:
        Jin = J.reshape(-1, 9)
        Gref = W.geometry_from_jacobians(J, w3)
        dref = np.linalg.det(J)[:, None] * w3[None]
    tdt = torch.float64 if out_dtype == 0 else torch.float32
    Jd = torch.from_numpy(np.ascontiguousarray(Jin)).to(dev)
    Gd = torch.empty((ncells, Q ** 3, 6), dtype=tdt, device=dev)
    Dd = torch.empty((ncells, Q ** 3), dtype=tdt, device=dev)
    femtc.geometry(out_dtype, Q, w, Jd, Dd, Gd, ncells, per_point=per_point)
    torch.cuda.synchronize()
    tol = 1e-13 if out_dtype == 0 else 1e-6
    assert np.abs(Gd.double().cpu().numpy() - Gref).max() / np.abs(Gref).max() <= tol
    assert np.abs(Dd.double().cpu().numpy() - dref).max() / np.abs(dref).max() <= tol
