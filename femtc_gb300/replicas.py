"""Multi-GPU = replicas: host-side aggregation of independent ranks.

The cell-local operator is block diagonal, so N ranks run N independent
replicas of a workload with no data exchange (the reference's MPI ranks do
the same: run.sh:20, bench_mass.cpp:135-137 only sum throughputs).  The only
cross-rank operations are a barrier around the timed region and these
reductions of scalars (any torch.distributed backend: NCCL on GPUs, gloo on
CPU).
"""
from __future__ import annotations


def _reduce(x: float, op_name: str, device=None) -> float:
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=getattr(dist.ReduceOp, op_name))
    return float(t.item())


def max_over_ranks(x: float, device=None) -> float:
    """Slowest rank's value (the step time of the whole job)."""
    return _reduce(x, "MAX", device)


def sum_over_ranks(x: float, device=None) -> float:
    return _reduce(x, "SUM", device)


def job_throughput(units_per_rank: float, seconds_per_rank: float, device=None) -> float:
    """Whole-job throughput of weak-scaled replicas: all ranks' units over
    the slowest rank's time."""
    total = sum_over_ranks(units_per_rank, device)
    slowest = max_over_ranks(seconds_per_rank, device)
    return total / slowest
