"""Replica bookkeeping of multi-GPU runs on CPU ranks (gloo, world size 2): distinct
seeds, max-over-ranks time, summed work, FP64 estimator reduction."""
import os

import numpy as np
import torch.multiprocessing as mp

from qmcpack_gb300.replicas import aggregate_timing, reduce_estimators, replica_seed


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    moves, ms = aggregate_timing(1000.0 * (rank + 1), 10.0 + rank)
    rng = np.random.default_rng(rank)
    e = -5.0 + rng.normal(size=(20, 8))
    mean, var, n = reduce_estimators(e)
    out.put((rank, replica_seed(2024, rank), moves, ms, mean, var, n))
    dist.destroy_process_group()


def test_replicas_gloo_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    all_e = np.concatenate([-5.0 + np.random.default_rng(r).normal(size=(20, 8)).reshape(-1) for r in range(2)])
    for rank, seed, moves, ms, mean, var, n in res:
        assert moves == 3000.0 and ms == 11.0 and n == 320
        assert abs(mean - all_e.mean()) < 1e-12 and abs(var - all_e.var()) < 1e-10
    assert res[0][1] != res[1][1]


def test_single_rank_passthrough():
    assert aggregate_timing(5.0, 2.0) == (5.0, 2.0)
    assert len({replica_seed(1, r) for r in range(64)}) == 64
