"""GPU: femtc_batch_apply_static, the batched launch for callers that cannot
allocate device memory (e.g. while another thread captures a CUDA graph in
global mode, or when their memory manager owns the device memory).

Its schedule lives in the library's fixed device array instead of memory
from cudaMalloc.  Two calls in a row, on different meshes, must give the
same results as femtc_batch_create + femtc_batch_launch on the same data,
within the tolerance the batch tests use for two launches of one mesh.
This file is collected last (its name), so a stop at the first failure has
run every other test already; it also passes alone in a fresh process."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def meshes(femtc, dev, seed, dtype):
    import torch
    from femtc_gb300 import workloads as W
    rng = np.random.default_rng(seed)
    out = []
    for P in range(1, 8):
        for op in (0, 1):
            n = int(rng.integers(1, 200)) + (seed % 7)
            w = W.make_custom("s", op, P, P + 2, n, seed=seed * 100 + P * 2 + op)
            u = torch.from_numpy(w.u).to(dev, torch.float32)
            g = torch.from_numpy(w.geo).to(dev, torch.float32)
            out.append([op, P, P + 2, w.tables.astype(np.float32), u, None, g, n])
    return out


@pytest.mark.parametrize("dtype", [1, 3])
def test_static_batch_matches_batch_launch(femtc, dev, dtype):
    import torch
    for seed in (11, 12):  # two calls in a row, different meshes
        ms = meshes(femtc, dev, seed, dtype)
        ref_meshes, st_meshes = [], []
        for m in ms:
            a, b = list(m), list(m)
            a[5] = torch.full_like(m[4], float("nan"))
            b[5] = torch.full_like(m[4], float("nan"))
            ref_meshes.append(tuple(a))
            st_meshes.append(tuple(b))
        batch = femtc.Batch(dtype, ref_meshes)
        batch.launch()
        femtc.batch_apply_static(dtype, st_meshes)
        torch.cuda.synchronize()
        assert femtc.device_status() == 0
        for r, s in zip(ref_meshes, st_meshes):
            yr = r[5].double().cpu().numpy()
            ys = s[5].double().cpu().numpy()
            assert np.isfinite(ys).all()
            assert np.abs(ys - yr).max() <= 1e-6 * np.abs(yr).max()
        batch.close()


def test_static_batch_leaves_free_memory_unchanged(femtc, dev):
    # the call allocates no device memory: after a first call (which may load
    # the kernel's module), the device's free bytes stay the same across calls
    import torch
    ms = meshes(femtc, dev, 13, 1)
    for m in ms:
        m[5] = torch.empty_like(m[4])
    ms = [tuple(m) for m in ms]
    femtc.batch_apply_static(1, ms)
    torch.cuda.synchronize()
    before = torch.cuda.mem_get_info(dev)[0]
    for _ in range(3):
        femtc.batch_apply_static(1, ms)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(dev)[0] == before
    assert femtc.device_status() == 0


def test_static_batch_rejects_a_capturing_stream(femtc, dev):
    # the schedule is copied from host memory freed on return: a copy
    # recorded into a graph would read freed memory at replay, so the call
    # refuses a capturing stream before doing any work
    import torch
    ms = meshes(femtc, dev, 14, 1)
    for m in ms:
        m[5] = torch.empty_like(m[4])
    ms = [tuple(m) for m in ms]
    femtc.batch_apply_static(1, ms)  # first call on the device, outside capture
    torch.cuda.synchronize()
    s = torch.cuda.Stream(device=dev)
    g = torch.cuda.CUDAGraph()
    err = None
    with torch.cuda.stream(s):
        g.capture_begin()
        try:
            femtc.batch_apply_static(1, ms, stream=s)
        except femtc.FemtcError as e:
            err = e
        g.capture_end()
    torch.cuda.synchronize()
    assert err is not None and err.status == -2  # FEMTC_ERR_UNSUPPORTED
    del g
    femtc.batch_apply_static(1, ms)  # still usable afterwards
    torch.cuda.synchronize()
    assert femtc.device_status() == 0


def test_static_batch_while_another_thread_captures(femtc, dev):
    """The case the entry exists for: another thread captures a CUDA graph in
    global mode (cudaMalloc is then refused everywhere in the process) while
    this thread calls the entry on its own stream.  The call succeeds, the
    capture ends cleanly, and the results match the graph-built batch."""
    import threading
    import torch
    ms = meshes(femtc, dev, 15, 1)
    ref_meshes, st_meshes = [], []
    for m in ms:
        a, b = list(m), list(m)
        a[5] = torch.full_like(m[4], float("nan"))
        b[5] = torch.full_like(m[4], float("nan"))
        ref_meshes.append(tuple(a))
        st_meshes.append(tuple(b))
    batch = femtc.Batch(1, ref_meshes)
    batch.launch()
    femtc.batch_apply_static(1, st_meshes)  # first call on the device, outside capture
    torch.cuda.synchronize()
    for m in st_meshes:
        m[5].fill_(float("nan"))
    st = torch.cuda.Stream(device=dev)
    x = torch.zeros(1024, device=dev)
    capturing, called = threading.Event(), threading.Event()
    errors = []

    def capturer():
        s = torch.cuda.Stream(device=dev)
        g = torch.cuda.CUDAGraph()
        try:
            with torch.cuda.graph(g, stream=s, capture_error_mode="global"):
                x.add_(1.0)
                capturing.set()
                called.wait(120)
                x.add_(1.0)
        except Exception as e:  # an unsafe call elsewhere invalidates the capture
            errors.append(e)
        finally:
            capturing.set()

    th = threading.Thread(target=capturer)
    th.start()
    capturing.wait(120)
    try:
        femtc.batch_apply_static(1, st_meshes, stream=st)
    finally:
        called.set()
        th.join(120)
    assert not errors, errors
    torch.cuda.synchronize()
    assert femtc.device_status() == 0
    for r, s_ in zip(ref_meshes, st_meshes):
        yr = r[5].double().cpu().numpy()
        ys = s_[5].double().cpu().numpy()
        assert np.isfinite(ys).all()
        assert np.abs(ys - yr).max() <= 1e-6 * np.abs(yr).max()
    batch.close()


def test_static_batch_rejects_oversize(femtc, dev):
    import torch
    # more meshes than the static mesh table holds
    u = torch.zeros(64, dtype=torch.float32, device=dev)
    t = np.zeros(2 * 5 * 4, dtype=np.float32)
    one = (0, 3, 5, t, u, u, u, 1)
    with pytest.raises(femtc.FemtcError):
        femtc.batch_apply_static(1, [one] * 5000)
