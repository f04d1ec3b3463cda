"""CPU: the serving loop's admission control and error paths, without a GPU.

Failure is injected on the host: malformed requests, a request larger than
the whole HBM budget, and a wait that runs out of time.  No solve runs."""
import numpy as np
import pytest


def test_solve_bytes_grows_with_size(femtc):
    a = femtc.solve_bytes(2, 4, 1000)
    b = femtc.solve_bytes(2, 4, 2000)
    c = femtc.solve_bytes(6, 8, 1000)
    assert 0 < a < b and a < c


def test_server_rejects_over_budget_and_malformed(femtc):
    s = femtc.Server(hbm_budget_bytes=1 << 20, max_active=2)  # 1 MiB budget
    try:
        n = 5000
        big = femtc.Problem(3, 5, np.tile(np.eye(3).reshape(1, 9), (n, 1)), np.ones((n, 64)))
        with pytest.raises(femtc.FemtcError) as e:
            s.submit(big)
        assert e.value.status == -4  # FEMTC_ERR_NOMEM: over the whole budget
        bad = femtc.Problem(3, 5, np.eye(3).reshape(1, 9), np.ones((1, 64)))
        bad.req.degree = 9
        with pytest.raises(femtc.FemtcError):
            s.submit(bad)
        st = s.stats()
        assert st["rejected"] == 1 and st["submitted"] == 0 and st["active"] == 0
        with pytest.raises(femtc.FemtcError) as e:
            s.wait(12345, timeout_s=0.01)  # never submitted: times out
        assert e.value.status == -7
    finally:
        s.close()


def test_server_rejects_bad_applications(femtc):
    s = femtc.Server(hbm_budget_bytes=1 << 20, max_active=1)  # 1 MiB budget
    try:
        t = np.zeros(2 * 4 * 5)
        big = femtc.Application(1, femtc.F64, femtc.EXACT, 3, 5, t, np.zeros((5000, 64)),
                                np.zeros((5000, 125 * 6)))
        with pytest.raises(femtc.FemtcError) as e:
            s.submit_apply(big)
        assert e.value.status == -4  # FEMTC_ERR_NOMEM: over the whole budget
        bad = femtc.Application(1, femtc.F64, femtc.EXACT, 3, 5, t, np.zeros((1, 64)),
                                np.zeros((1, 125 * 6)))
        bad.req.op = 7
        with pytest.raises(femtc.FemtcError) as e:
            s.submit_apply(bad)
        assert e.value.status == -1  # FEMTC_ERR_INVALID
        bad.req.ncells = 1 << 60  # its byte count would overflow size_t
        with pytest.raises(femtc.FemtcError) as e:
            s.submit_apply(bad)
        assert e.value.status == -1  # FEMTC_ERR_INVALID
        bad.req.ncells = 1
        bad.req.op = 1
        bad.req.dtype = femtc.F16X2
        bad.req.degree = 12
        with pytest.raises(femtc.FemtcError) as e:
            s.submit_apply(bad)  # the tensor-core forms stop at degree 7
        assert e.value.status == -2  # FEMTC_ERR_UNSUPPORTED
        st = s.stats()
        assert st["rejected"] == 1 and st["submitted"] == 0
    finally:
        s.close()


def test_server_policy_validation(femtc):
    s = femtc.Server(hbm_budget_bytes=1 << 20, max_active=1, policy=femtc.SERVE_FIFO)
    try:
        lib = femtc.load()
        assert lib.femtc_server_set_policy(s.handle, femtc.SERVE_SHORTEST_FIRST) == 0
        assert lib.femtc_server_set_policy(s.handle, 7) == -1
        assert lib.femtc_server_set_policy(None, 0) == -1
    finally:
        s.close()


def test_solve_argument_errors(femtc):
    p = femtc.Problem(3, 5, np.eye(3).reshape(1, 9), np.ones((1, 64)), alpha=0.0)
    with pytest.raises(femtc.FemtcError):
        femtc.solve(p)  # alpha must be > 0 (SPD)
    p = femtc.Problem(3, 5, np.eye(3).reshape(1, 9), np.ones((1, 64)), inner_dtype=femtc.F64)
    with pytest.raises(femtc.FemtcError):
        femtc.solve(p)  # inner operator must be a mixed-precision form
