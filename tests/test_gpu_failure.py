"""GPU: a bounded device wait that runs out ends as a status, not a hang.

femtc_bounded_wait_check launches one CTA whose mbarrier wait cannot
complete (armed for transaction bytes that no copy delivers) through the
same bounded wait every kernel of the library uses, with a short poll
limit.  The kernel must return, femtc_device_status() must report the
timeout bit (1) once and then read clean, and the GPU must stay usable: an
operator launch right after still matches the oracle.  No copy is issued
and no memory is touched; nothing here faults or hangs the GPU.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_reports(femtc, orc, dev):
    import torch
    from femtc_gb300 import workloads as W
    lib = femtc.load()
    assert femtc.device_status() == 0
    femtc.check(lib.femtc_bounded_wait_check(1000, None))
    torch.cuda.synchronize()
    assert femtc.device_status() == 1   # FAULT_MBAR_TIMEOUT, read and cleared
    assert femtc.device_status() == 0
    # the context is intact: a normal launch matches the oracle
    w = W.make_custom("f", femtc.STIFFNESS, 3, 5, 64, seed=4)
    u = torch.from_numpy(w.u).to(dev)
    g = torch.from_numpy(w.geo).to(dev)
    y = torch.empty_like(u)
    femtc.apply(femtc.STIFFNESS, femtc.F64, femtc.EXACT, 3, 5, w.tables, u, y, g, w.ncells)
    ref = orc.stiffness(orc.EXACT, 3, 5, w.tables, w.u, w.geo)
    err = np.abs(y.cpu().numpy() - ref).max() / np.abs(ref).max()
    assert err <= 1e-12
    assert femtc.device_status() == 0
