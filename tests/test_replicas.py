"""CPU, world_size 2 over gloo: the replica aggregation used by bench.py for
N > 1 GPUs (max of step times, sum of work, no data-path collective)."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from femtc_gb300 import replicas
    step = [0.5, 0.75][rank]          # rank 1 is the slowest
    units = [100.0, 300.0][rank]
    out[rank] = (replicas.max_over_ranks(step), replicas.sum_over_ranks(units),
                 replicas.job_throughput(units, step))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_aggregation_gloo_world2():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        port = _free_port()
        procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        for r in range(2):
            mx, total, thr = out[r]
            assert mx == 0.75 and total == 400.0
            assert thr == pytest.approx(400.0 / 0.75)


def test_single_process_is_identity():
    from femtc_gb300 import replicas
    assert replicas.max_over_ranks(3.0) == 3.0
    assert replicas.job_throughput(10.0, 2.0) == 5.0
