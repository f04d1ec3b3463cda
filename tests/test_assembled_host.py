"""CPU: the DOF-map transpose behind the assembled operator, and the
assembled entry point's argument checks (no device work)."""
import numpy as np
import pytest


def test_box_dofmap_shares_face_dofs(femtc):
    from femtc_gb300 import workloads as W
    dm, nd = W.box_dofmap(3, 2, 2, 2)
    assert dm.shape == (12, 27) and nd == 7 * 5 * 5
    assert np.array_equal(np.unique(dm), np.arange(nd))  # every grid point used
    counts = np.bincount(dm.ravel(), minlength=nd)
    assert counts.max() == 8 and counts.min() == 1  # interior vertices: 8 cells, corners: 1


@pytest.mark.parametrize("P", [1, 3])
def test_dofmap_transpose_matches_numpy(femtc, P):
    from femtc_gb300 import workloads as W
    dm, nd = W.box_dofmap(4, 3, 2, P)
    offsets, entries = femtc.dofmap_transpose(dm, nd)
    flat = dm.ravel()
    order = np.argsort(flat, kind="stable")  # by global index, then position
    assert np.array_equal(entries, order.astype(np.int32))
    assert np.array_equal(np.diff(offsets), np.bincount(flat, minlength=nd))
    assert offsets[0] == 0 and offsets[-1] == flat.size


def test_dofmap_transpose_rejects_out_of_range(femtc):
    dm = np.array([[0, 1], [2, 5]], dtype=np.int32)
    with pytest.raises(femtc.FemtcError):
        femtc.dofmap_transpose(dm, 5)


def test_assembled_apply_argument_errors(femtc):
    lib = femtc.load()
    t = np.zeros(64)
    # op, dtype, null pointers, misaligned work: rejected before any device work
    assert lib.femtc_assembled_apply(2, 0, 0, 2, 3, t.ctypes.data, 16, 16, 16, 8, 16, 16, 16, 1,
                                     256, None) == -1
    assert lib.femtc_assembled_apply(0, 9, 0, 2, 3, t.ctypes.data, 16, 16, 16, 8, 16, 16, 16, 1,
                                     256, None) == -1
    assert lib.femtc_assembled_apply(0, 0, 0, 2, 3, t.ctypes.data, None, 16, 16, 8, 16, 16, 16, 1,
                                     256, None) == -1
    assert lib.femtc_assembled_apply(0, 0, 0, 2, 3, t.ctypes.data, 16, 16, 16, 8, 16, 16, 16, 1,
                                     272, None) == -1
    assert lib.femtc_assembled_apply(0, 0, 1, 2, 4, t.ctypes.data, 16, 16, 16, 8, 16, 16, 16, 1,
                                     256, None) == -2  # reference semantics needs Q = N
    n = 7
    assert femtc.assembled_work_bytes(femtc.F64, 2, n) == 2 * ((n * 27 * 8 + 255) // 256 * 256)
