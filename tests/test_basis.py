"""CPU: the library's FP64 basis tabulation (femtc_tabulate) against
known answers and an independent numpy construction."""
import numpy as np
import pytest


@pytest.mark.parametrize("P", range(1, 9))
@pytest.mark.parametrize("dq", [0, 1, 2])
def test_tabulation_known_answers(femtc, P, dq):
    Q = P + 1 + dq
    N = P + 1
    t, x, w, z = femtc.tabulate(P, Q)
    Phi = t[: Q * N].reshape(N, Q).T
    Gam = t[Q * N:].reshape(N, Q).T
    # partition of unity and its derivative
    assert np.abs(Phi.sum(axis=1) - 1).max() < 1e-13
    assert np.abs(Gam.sum(axis=1)).max() < 1e-11
    # Gauss points / weights (numpy's Golub-Welsch-based leggauss)
    xg, wg = np.polynomial.legendre.leggauss(Q)
    assert np.abs((xg + 1) / 2 - x).max() < 1e-14
    assert np.abs(wg / 2 - w).max() < 1e-14
    # exact quadrature up to degree 2Q-1
    for k in range(2 * Q):
        assert abs((w * x ** k).sum() - 1.0 / (k + 1)) < 1e-14
    # GLL nodes: endpoints plus the roots of L_P'
    dl = np.polynomial.legendre.Legendre.basis(P).deriv().roots() if P > 1 else np.array([])
    ref = np.concatenate([[0.0], np.sort((dl.real + 1) / 2), [1.0]])
    assert np.abs(np.sort(z) - ref).max() < 1e-13
    # Lagrange property l_i(z_j) = delta_ij via the independent product formula
    # and the interpolation of x^P is exact
    f = z ** P
    assert np.abs(Phi @ f - x ** P).max() < 1e-12
    assert np.abs(Gam @ f - P * x ** (P - 1)).max() < 1e-10


def test_tabulation_bad_args(femtc):
    with pytest.raises(femtc.FemtcError):
        femtc.tabulate(0, 3)
