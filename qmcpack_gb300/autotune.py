"""Per-system autotuning of the walker-resident move loop.

For a system and a walker count, every candidate delay rank k (the delayed-update
window, which sets how many electrons one resident launch moves and how often the
batched flush runs) and CTA size is timed over a few device-RNG sweeps of a fresh crowd,
and the fastest is kept.  The walker-resident design fixes one walker per CTA
and the spline work unit (one coefficient column x one x-plane: 16 rows of orbitals),
so those are reported, not searched; the threads per walker (128, 256, 512) are searched
with the delay rank.  Results are cached in a JSON file keyed by the
system shape, the walker count, the precision and the GPU name.
"""
from __future__ import annotations

import json
import os
import time

import numpy as np

from .system import System, make_walkers


def _cache_path() -> str:
    return os.environ.get("QMCG_TUNING_FILE",
                          os.path.join(os.path.expanduser("~"), ".cache", "qmcpack_gb300", "tuning.json"))


def _key(system: System, nw: int, flush: int) -> str:
    import torch
    gpu = torch.cuda.get_device_name(0) if torch.cuda.is_available() else "none"
    s = system.spec
    return (f"ne{system.n_elec}-norb{system.norb}-grid{int(system.grid[0])}-ions{len(system.ion_pos)}-"
            f"nw{nw}-p{s.precision}-flush{flush}-{gpu}")


def candidate_ranks(system: System):
    n = system.norb
    return [k for k in (1, 4, 8, 16, 32, 64) if k <= n and (k == 1 or k >= min(8, n))]


def tune(system: System, nw: int, dsys=None, flush: int = 3, sweeps: int = 3, candidates=None,
         use_cache: bool = True) -> dict:
    """{'delay': k, 'threads_per_walker': t, 'walkers_per_block': 1, 'ms_per_sweep': ms, 'table': {...}}"""
    from .crowd import Crowd, DeviceSystem
    path = _cache_path()
    key = _key(system, nw, flush)
    cache = {}
    if use_cache and os.path.exists(path):
        try:
            cache = json.load(open(path))
        except (OSError, ValueError):
            cache = {}
        if key in cache:
            return cache[key]
    dsys = dsys or DeviceSystem(system)
    R = make_walkers(system, nw, seed=5)
    table = {}
    threads = (128, 256, 512) if system.spec.precision == 4 else (128, 256)
    for k in candidates or candidate_ranks(system):
        g = Crowd(dsys, nw, k)
        g.load_walkers(R)
        g.mw_evaluateLog()
        for nt in threads:
            g.set_threads(nt)
            g.vmc_sweeps(2, system.spec.tau, 1, rng_mode=1, flush=flush)  # warm-up, builds the graph
            g.sync()
            t0 = time.perf_counter()
            g.vmc_sweeps_async(sweeps)
            g.sync()
            table[(k, nt)] = (time.perf_counter() - t0) / sweeps * 1e3
        del g
    best = min(table, key=table.get)
    res = {"delay": int(best[0]), "threads_per_walker": int(best[1]), "walkers_per_block": 1,
           "spline_unit": "one coefficient column x one x-plane (16 rows of orbitals)",
           "ms_per_sweep": float(table[best]),
           "table": {f"k{k}/t{nt}": float(v) for (k, nt), v in table.items()}}
    if use_cache:
        cache[key] = res
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as f:
            json.dump(cache, f, indent=1)
    return res
