"""GPU: the batched persistent launch (femtc_batch_*, CUDA graph replay).

Every mesh of a mixed batch (degrees 1..7, Q = P+2, mass and stiffness,
ragged cell counts) must match the FP64 oracle within its form's tolerance,
and equal the single-mesh call on the same data ("alone and in the mix").
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {1: 2e-6, 2: 1e-6, 3: 1e-6}


def make_meshes(femtc, dev, dtype, seed=0, scale=1, random_tables=False):
    import torch
    from femtc_gb300 import workloads as W
    rng = np.random.default_rng(seed)
    meshes, hosts = [], []
    rtabs = {}
    for P in range(1, 8):
        for op in (0, 1):
            ncells = int(rng.integers(1, 300)) * scale + (P * 7 + op) % 5
            w = W.make_custom("b", op, P, P + 2, ncells, seed=100 * P + op + seed)
            if random_tables:  # no symmetry: the plain (not even-odd) kernels
                if P not in rtabs:
                    rtabs[P] = np.random.default_rng(P).uniform(-1.0, 1.0, w.tables.shape)
                w.tables = rtabs[P]
            u = torch.from_numpy(w.u).to(dev, torch.float32)
            g = torch.from_numpy(w.geo).to(dev, torch.float32)
            y = torch.full_like(u, float("nan"))
            meshes.append((op, P, P + 2, w.tables.astype(np.float32), u, y, g, ncells))
            hosts.append(w)
    return meshes, hosts


@pytest.mark.parametrize("dtype", [1, 2, 3])
@pytest.mark.parametrize("tune", [False, True])
def test_batch_matches_oracle_and_single_calls(femtc, orc, dev, dtype, tune):
    import torch
    meshes, hosts = make_meshes(femtc, dev, dtype)
    b = femtc.Batch(dtype, meshes, tune=tune)
    info = b.info()
    assert info["tiles"] >= len(meshes) and info["ctas"] >= 1
    b.launch()
    torch.cuda.synchronize()
    assert femtc.device_status() == 0
    for (op, P, Q, tab, u, y, g, n), w in zip(meshes, hosts):
        t32 = tab.astype(np.float64)
        u32 = w.u.astype(np.float32).astype(np.float64)
        g32 = w.geo.astype(np.float32).astype(np.float64)
        fn = orc.mass if op == 0 else orc.stiffness
        ref = fn(orc.EXACT, P, Q, t32, u32, g32)
        yb = y.double().cpu().numpy()
        err = np.abs(yb - ref).max() / np.abs(ref).max()
        assert err <= TOL[dtype], (op, P, err)
        # alone: the single-mesh entry point on the same data
        ys = torch.full_like(u, float("nan"))
        femtc.apply(op, dtype, femtc.EXACT, P, Q, tab, u, ys, g, n)
        torch.cuda.synchronize()
        alone = ys.double().cpu().numpy()
        assert np.abs(alone - yb).max() <= 1e-6 * np.abs(ref).max()
    b.close()


def test_batch_split_plan(femtc, orc, dev):
    """The split plan (per-variant batch kernels plus single-mesh launches,
    one graph) gives every mesh its oracle result and its single-call bits,
    and relaunches see new inputs."""
    import torch
    meshes, hosts = make_meshes(femtc, dev, 1, seed=5, scale=20)
    b = femtc.Batch(1, meshes, tune=True, split=True)
    info = b.info()
    assert info["batch_kernels"] + info["single_launches"] >= 2
    assert info["batch_kernels"] <= 14
    for rep in range(2):
        if rep:
            for (op, P, Q, tab, u, y, g, n), w in zip(meshes, hosts):
                w.u = -2.0 * w.u
                u.copy_(torch.from_numpy(w.u).to(dev, torch.float32))
        b.launch()
        torch.cuda.synchronize()
        assert femtc.device_status() == 0
        for (op, P, Q, tab, u, y, g, n), w in zip(meshes, hosts):
            fn = orc.mass if op == 0 else orc.stiffness
            ref = fn(orc.EXACT, P, Q, tab.astype(np.float64), w.u.astype(np.float32).astype(np.float64),
                     w.geo.astype(np.float32).astype(np.float64))
            yb = y.double().cpu().numpy()
            assert np.abs(yb - ref).max() <= TOL[1] * np.abs(ref).max(), (rep, op, P)
    for op in (0, 1):
        for P in range(1, 8):
            cb, staged = b.layout(op, P)
            assert cb == 0 or cb % 4 == 0
    b.close()


def test_batch_plain_family_nonsymmetric_tables(femtc, orc, dev):
    """FP32 meshes whose tables lack the GLL-to-Gauss symmetry run the plain
    CUDA-core family (the symmetric ones take the even-odd family): every
    mesh against the oracle.  Random tables of both signs cancel more than
    the tabulated ones, so the FP32 tolerance here is 2e-5."""
    import torch
    meshes, hosts = make_meshes(femtc, dev, 1, seed=7, random_tables=True)
    b = femtc.Batch(1, meshes)
    b.launch()
    torch.cuda.synchronize()
    assert femtc.device_status() == 0
    for (op, P, Q, tab, u, y, g, n), w in zip(meshes, hosts):
        fn = orc.mass if op == 0 else orc.stiffness
        ref = fn(orc.EXACT, P, Q, tab.astype(np.float64), w.u.astype(np.float32).astype(np.float64),
                 w.geo.astype(np.float32).astype(np.float64))
        err = np.abs(y.double().cpu().numpy() - ref).max() / np.abs(ref).max()
        assert err <= 2e-5, (op, P, err)
    b.close()


def test_batch_relaunch_sees_new_inputs(femtc, orc, dev):
    import torch
    meshes, hosts = make_meshes(femtc, dev, 1, seed=3)
    b = femtc.Batch(1, meshes)
    b.launch()
    for m in meshes:
        m[4].mul_(2.0)  # linear operator: doubling u doubles y
    y1 = [m[5].clone() for m in meshes]
    b.launch()
    torch.cuda.synchronize()
    for m, a in zip(meshes, y1):
        assert torch.allclose(m[5], 2 * a, rtol=1e-5, atol=1e-6 * float(a.abs().max()))
    b.close()


def test_batch_rejects_mismatched_tables(femtc, dev):
    meshes, _ = make_meshes(femtc, dev, 1)
    bad = list(meshes[2])
    bad[3] = bad[3] * 1.5  # same degree as another mesh, different tables
    with pytest.raises(femtc.FemtcError):
        femtc.Batch(1, meshes + [tuple(bad)])


def test_batch_rejects_bad_items(femtc, dev):
    meshes, _ = make_meshes(femtc, dev, 1)
    bad = list(meshes[0])
    bad[2] = bad[1] + 1  # nquad must be degree + 2
    with pytest.raises(femtc.FemtcError):
        femtc.Batch(1, [tuple(bad)])
    with pytest.raises(femtc.FemtcError):
        femtc.Batch(0, meshes)  # FP64 batches are not built
