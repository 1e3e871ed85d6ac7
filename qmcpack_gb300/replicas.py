"""Multi-GPU runs are independent replicas: every rank owns one crowd on its own GPU
with its own random stream, and no data moves between ranks during a sweep.  The only
cross-rank steps are the ones a VMC driver needs at the end of a block: the slowest
rank's time, the total work, and FP64 sums of the energy estimators (the reference
reduces its estimator sums with an MPI allreduce, src/Estimators/EstimatorManagerNew.cpp:363).
"""
from __future__ import annotations

import numpy as np


def replica_seed(base: int, rank: int) -> int:
    """Per-rank 64-bit seed of the counter-based random stream (distinct, reproducible)."""
    x = (int(base) + 0x9E3779B97F4A7C15 * (int(rank) + 1)) & 0xFFFFFFFFFFFFFFFF
    x ^= x >> 31
    x = (x * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
    return x ^ (x >> 29)


def aggregate_timing(moves: float, ms: float, group=None):
    """(total moves over ranks, max time over ranks) with torch.distributed; one rank
    without an initialised process group returns its own values."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(moves), float(ms)
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.tensor([ms], dtype=torch.float64, device=dev)
    m = torch.tensor([moves], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    dist.all_reduce(m, op=dist.ReduceOp.SUM, group=group)
    return float(m.item()), float(t.item())


def reduce_estimators(e_local, group=None):
    """FP64 sums over ranks of (sum E_L, sum E_L^2, number of samples) for a block of
    local energies [sweeps][walkers]; returns (mean, variance, samples)."""
    import torch
    import torch.distributed as dist
    e = np.asarray(e_local, dtype=np.float64)
    v = torch.tensor([e.sum(), (e * e).sum(), float(e.size)], dtype=torch.float64)
    if dist.is_available() and dist.is_initialized():
        if dist.get_backend(group) == "nccl":
            v = v.cuda()
        dist.all_reduce(v, op=dist.ReduceOp.SUM, group=group)
    s, s2, n = (float(x) for x in v.cpu())
    mean = s / n
    return mean, s2 / n - mean * mean, int(n)
