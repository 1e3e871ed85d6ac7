"""Benchmark of the batched particle-by-particle Slater-Jastrow VMC move loop.

One step = one VMC sweep: every electron of every walker is proposed once
(drift-diffusion), tested and accepted or rejected, delayed updates are flushed,
and the FP64 recompute runs on its schedule (every 100 sweeps), all through the
captured CUDA graph of the library.  The workload is the production-shape system
(384 electrons, 512 walkers, delay rank 32, FP32 move loop).  Inputs are seeded
synthetic systems; the working set (~0.9 GB) is larger than L2.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

Multi-GPU runs are independent replicas (walkers are independent Markov chains):
every rank runs its own crowd with its own seed; value = all ranks' walker-moves
divided by the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from qmcpack_gb300.system import SPECS, make_system, make_walkers  # noqa: E402

DESCRIPTIONS = {
    "c1_384e": "384 electrons (192 up / 192 down) in a cubic cell a=15.8 bohr, 32 ions on a jittered lattice, "
               "192 real orbitals as tricubic B-splines on a 48^3 grid (FP32 coefficients N(0,0.1)), J1/J2 B-spline "
               "Jastrows with 10 parameters, 512 walkers, delay rank 32, tau 0.3, FP32 move loop, FP64 recompute "
               "every 100 sweeps",
    "c0_32e": "32 electrons, 16 orbitals on a 32^3 grid, 8 ions, a=10 bohr, 64 walkers, rank-1 updates, FP64",
    "c2_1536e": "1536 electrons, 768 orbitals on a 60^3 grid, 128 ions, a=25 bohr, 256 walkers, delay rank 64, FP32",
    "c3_mixed": "uneven crowd of 1024 walkers: 410 on the 32-electron system, 410 on the 384-electron system, "
                "204 on a 768-electron system (384 orbitals, 40^3 grid, 64 ions, a=20 bohr), FP32, one persistent "
                "launch per stage, delay rank autotuned per system",
}


def flush_bytes_per_launch(system, k: int, nw: int) -> int:
    """Algorithmic bytes of one batched flush of one spin: the inverse read and written,
    U, V (k x lda) and Binv (k x k) read, per walker."""
    s = 4 if system.spec.precision == 4 else 8
    lda, n = system.npad, system.norb
    return int(s * nw * (2 * n * lda + 2 * k * lda + k * k))


def bytes_per_walker_move(system, k: int, with_flush: bool = True) -> int:
    """Algorithmic bytes of one walker-move of the walker-resident sweep kernel.

    spline: 64 coefficient rows of lda orbitals; inverse row: lda; delayed-update rows
    U and V read for the inverse row: 2 x (k-1)/2 rows of lda on average; current-row
    orbital gradients and values: 4 x lda; delayed-update flush: the inverse read and
    written once every k moves, 2 x N x lda / k.  Positions and the two-body Jastrow
    state live in shared memory for the whole sweep and are not counted.
    """
    s = 4 if system.spec.precision == 4 else 8
    lda, n = system.npad, system.norb
    elems = 64 * lda + lda + (k - 1) * lda + 4 * lda
    if with_flush:
        elems += (2 * n * lda) / max(k, 1)
    return int(elems * s)


def launches_per_sweep(system, k: int) -> int:
    """Kernels per sweep on the walker-resident path: one resident launch and one batched
    flush per segment of up to k electrons of a spin group (one resident launch for the
    sweep with rank-1 updates), the masked repair (vgl_all, Gauss-Jordan, jastrow_full,
    finish_repair) and the counter bump."""
    if k > 1:
        segs = 2 * ((system.spec.n_up + k - 1) // k)
        return 2 * segs + 5
    return 1 + 5


def block_update_bytes_per_sweep(system, k: int, nw: int, acceptance: float) -> int:
    """Algorithmic bytes of the block-lazy updates of one sweep: per spin group, every row
    block but the first read and written before its segment and every block read and
    written by the completing pass; per (block, set) application the accepted U and V rows
    (acceptance x k of them), Binv restricted to them and the delay list."""
    s = 4 if system.spec.precision == 4 else 8
    lda, nspin = system.npad, system.spec.n_up
    nseg = (nspin + k - 1) // k
    rows = 2 * (nspin - min(k, nspin)) * lda + 2 * nspin * lda
    m = acceptance * k
    sets = nseg * nseg * (2 * m * lda + m * m + k)
    return int(2 * nw * s * (rows + sets))


def flush_kernel_name(n: int, k: int, flush: int, block_lazy: bool = False) -> str:
    """The flush kernel the library takes for n orbitals and delay rank k (flush_tc_variant:
    one pass while the whole product fits one MMA and 200 KB of shared memory, else column
    tiles; block-lazy updates where the crowd's segment rows are staged)."""
    if flush == 4 and block_lazy:
        return "block_update_kernel (block-lazy, SIMT FP32)"
    if flush == 0:
        return "flush_fused_kernel (SIMT)"
    terms = "TF32" if flush == 1 else "3xTF32"
    k1, npad = (k + 31) // 32 * 32, (n + 15) // 16 * 16
    al = lambda x: (x + 1023) & ~1023
    first = 2 * al(128 * 64 * 4) + 2 * al(k1 * 64 * 4)
    later = 2 * al(128 * k1 * 4) + 2 * al(npad * k1 * 4)
    o = max(first, later)
    tail = max(al(o + k * n * 4), al(al(o + k1 * k1 * 4) + k1 * k1 * 4))
    one_pass = k <= 32 and npad <= 256 and al(al(tail + k * 4) + 32) <= 200 * 1024
    name = "flush_tc_kernel" if one_pass else "flush_tc_tiled_kernel"
    return f"{name} (tcgen05 {terms})"


def read_traffic(workload: str):
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", f"sweep_kernel_{workload}.md")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return int(line.split(":")[1])
    except (OSError, ValueError):
        pass
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(workload: str, max_seconds: float = 15.0):
    """The oracle (CPU restatement of the reference math) on the host cores, bounded sample.

    Full VMC sweeps (VMCBatched::advanceWalkers semantics, mt19937 stream) of 4 walkers
    per host core, repeated until about max_seconds of work; OpenMP over walkers.
    """
    from oracle import oracle as orc
    spec = SPECS[workload]
    system = make_system(spec)
    cores = os.cpu_count() or 1
    nw = 4 * cores
    R = make_walkers(system, nw, seed=3)
    orc.set_threads(cores)
    c = orc.Crowd(system, nw, spec.delay, spec.precision)
    c.load_walkers(R)
    c.evaluate_log(nthreads=cores)
    rng = orc.Rng(11)
    sweeps = 0
    t0 = time.perf_counter()
    while True:
        c.vmc_sweeps(rng, 1, spec.tau, True)
        sweeps += 1
        if time.perf_counter() - t0 > max_seconds:
            break
    dt = time.perf_counter() - t0
    moves = sweeps * nw * system.n_elec
    return {"value": moves / dt, "unit": "walker-moves/s", "cores": cores, "kind": "port",
            "sample": f"{sweeps} sweep(s) x {nw} walkers x {system.n_elec} electrons of {workload} "
                      f"({'FP32' if spec.precision == 4 else 'FP64'} oracle, OpenMP over walkers), {dt:.1f} s"}


def _fp64_twin(system):
    """The same system in FP64 (the FP32 coefficient values, upcast)."""
    import dataclasses
    spec64 = dataclasses.replace(system.spec, precision=8)
    return dataclasses.replace(system, spec=spec64, coefs=system.coefs.astype(np.float64))


def ratio_error(system, dsys32, nw: int, k: int, nelec: int = 4, R=None):
    """Per-move ratio error of the FP32 move loop against FP64 on identical positions and
    coefficients: relative |ratio32 - ratio64| / |ratio64| over nelec electrons x nw walkers,
    both crowds freshly recomputed from the positions R (uniform random if None)."""
    from qmcpack_gb300.crowd import Crowd, DeviceSystem
    sys64 = _fp64_twin(system)
    ds64 = DeviceSystem(sys64)
    label = "uniform random" if R is None else "equilibrated configurations"
    R = make_walkers(system, nw, seed=77) if R is None else R
    g32, g64 = Crowd(dsys32, nw, k), Crowd(ds64, nw, k)
    errs = []
    for g in (g32, g64):
        g.load_walkers(R)
        g.mw_evaluateLog()
    rng = np.random.default_rng(5)
    for iat in range(nelec):
        d = rng.normal(size=(nw, 3)) * 0.3
        out = []
        for g in (g32, g64):
            g.mw_evalGrad(iat)
            g.mw_makeMove(iat, d)
            r, _ = g.mw_calcRatioGrad(iat)
            g.mw_accept_rejectMove(iat, np.zeros(nw, np.int32))
            out.append(r)
        errs.append(np.abs(out[0] - out[1]) / np.maximum(np.abs(out[1]), 1e-300))
    e = np.concatenate(errs)
    del g32, g64, ds64
    return {"median": float(np.median(e)), "p99": float(np.percentile(e, 99)), "max": float(e.max()),
            "moves": int(e.size), "against": "FP64 move loop, same positions and coefficients",
            "walkers": label}


def virtual_moves(crowd, system, peak: float, rcut: float = 2.0, seed: int = 5):
    """Non-local pseudopotential ratios at the crowd's current configurations: the 12-point
    quadrature points of every electron within rcut of an ion (qmcg_mw_evaluate_ratios).
    Device time of the ratio kernel alone (CUDA events, inputs resident) and end to end
    through the C ABI (host lists in, ratios out)."""
    from qmcpack_gb300.nlpp import quadrature_moves
    R = crowd.positions()
    w, e, pos, _ = quadrature_moves(system, R, rcut, np.random.default_rng(seed))
    n = len(w)
    ms = crowd.profile_ratios(w, e, pos, reps=10)
    t0 = time.perf_counter()
    reps = 5
    for _ in range(reps):
        crowd.mw_evaluateRatios(w, e, pos)
    e2e_s = (time.perf_counter() - t0) / reps
    sz = 4 if system.spec.precision == 4 else 8
    per = (65 * system.npad + 3 * system.n_elec) * sz
    achieved = per * n / (ms / 1e3) / 1e9
    return {"moves": int(n), "per_walker": n / crowd.nw, "cutoff_bohr": rcut, "rule": "12-point icosahedral",
            "kernel": "vp_ratio_kernel", "ms_per_launch": ms, "moves_per_s": n / (ms / 1e3),
            "e2e_moves_per_s": n / e2e_s, "algorithmic_bytes_per_move": per,
            "gathered_gbs": achieved,
            "bound": "L2: the points of one quadrature sphere and the spheres of nearby electrons share grid "
                     "cells, so most coefficient rows are L2 hits and the gathered bytes per second exceed the "
                     "HBM copy bandwidth; no HBM fraction is claimed"}


def dmc_rate(dsys, system, R, flush: int, steps: int = 20, warmup: int = 10, tau: float = 0.02):
    """Fixed-node DMC steps of the production crowd through the host driver (device step,
    comb population control, SFNBranch parameters): wall clock of `steps` steps after
    `warmup` warm-up steps."""
    from qmcpack_gb300.crowd import Crowd
    from qmcpack_gb300.dmc import DMCDriver
    spec = system.spec
    g = Crowd(dsys, spec.walkers, spec.delay)
    g.load_walkers(R)
    g.mw_evaluateLog()
    d = DMCDriver(g, tau=tau, seed=77, warmup_steps=warmup, flush=flush, recompute_every=spec.recompute_every)
    d.run(warmup)
    torch_sync()
    t0 = time.perf_counter()
    hist = d.run(steps)
    dt = time.perf_counter() - t0
    moves = steps * spec.walkers * system.n_elec
    acc = sum(h["accepted"] for h in hist) / max(sum(h["accepted"] + h["rejected"] for h in hist), 1)
    return {"tau": tau, "steps": steps, "warmup_steps": warmup, "ms_per_step": dt / steps * 1e3,
            "walker_moves_per_s": moves / dt, "acceptance": acc,
            "e_now_last": hist[-1]["e_now"], "e_trial_last": hist[-1]["e_trial"],
            "walkers_copied_per_step": float(np.mean([h["copied"] for h in hist])),
            "step": "fixed-node sweep + local energy + branch weights on the device, comb population control "
                    "and SFNBranch updates on the host"}


def monotonic(x) -> bool:
    d = np.diff(np.asarray(x, np.float64))
    return bool(np.all(d > 0) or np.all(d < 0))


def effective_samples(args, system, dsys32, seed: int):
    """Effective independent samples/s = walker-sweeps/s / kappa for
      plain_fp64:   drift-diffusion, FP64 move loop (the comparator the metric names)
      plain_fp32:   drift-diffusion, FP32 move loop, tcgen05 3xTF32 flush
      learned_fp32: the learned MH proposal, trained on the FP32 plain run's configurations
                    (staged kernels, BF16 network on the tensor cores, hand-written backward
                    and Adam), then run frozen on the walker-resident kernel.
    Protocol: one FP32 drift-diffusion crowd is equilibrated in blocks of args.eff_block
    sweeps, at least args.eff_min_blocks of them, until twice in a row the last block's
    mean energy agrees with the previous block's within 2 combined standard errors and the
    last four block means show no monotonic trend (at most args.eff_max_blocks blocks; the
    record says whether the test passed); the three methods then start from that configuration and
    run the same number of sweeps (args.eff_sweeps), so their kappa estimates see series
    of equal length.  Each method's kappa is its own: the autocorrelation function averaged
    over the walkers' own E_L series (independent chains, simstats truncation rule);
    kappa_resolved says whether it reached zero within the first quarter of the series
    (otherwise kappa is bounded by the series length and the effective samples are upper
    bounds).  Energies and variances of every method are compared with plain FP64 at 2
    sigma.  Wall clock around each whole call; the local energy is measured after every
    sweep in every method."""
    from qmcpack_gb300.crowd import Crowd, DeviceSystem
    from qmcpack_gb300.stats import agree_within, ensemble_statistics
    spec = system.spec
    nw, k, tau = spec.walkers, spec.delay, spec.tau
    rec = spec.recompute_every
    out = {}

    def timed(fn):
        torch_sync()
        t0 = time.perf_counter()
        res = fn()
        return res, time.perf_counter() - t0

    def summarize(name, el, dt, n, extra=None):
        st = ensemble_statistics(el)
        wsps = nw * n / dt
        h = el.mean(axis=1)
        d = dict(st)
        d.update({"energy_first_half": float(h[: n // 2].mean()), "energy_second_half": float(h[n // 2:].mean()),
                  "walker_sweeps_per_s": wsps, "effective_samples_per_s": wsps / st["kappa"],
                  "ms_per_sweep": dt / n * 1e3})
        if extra:
            d.update(extra)
        out[name] = d

    # equilibration until two consecutive block comparisons pass
    g = Crowd(dsys32, nw, k)
    g.load_walkers(make_walkers(system, nw, seed=300))
    g.mw_evaluateLog()
    blocks, passes, t_eq = [], 0, 0.0
    for _ in range(args.eff_max_blocks):
        (_, _, el, _), dt = timed(lambda: g.vmc_sweeps_measure(args.eff_block, tau, seed, recompute_every=rec,
                                                                flush=args.flush))
        t_eq += dt
        blocks.append(ensemble_statistics(el))
        if len(blocks) >= max(4, args.eff_min_blocks) and agree_within(blocks[-1], blocks[-2], "energy", "error") \
                and not monotonic([b["energy"] for b in blocks[-4:]]):
            passes += 1
            if passes >= 2:
                break
        else:
            passes = 0
    out["equilibration"] = {"method": "plain FP32 drift-diffusion", "block_sweeps": args.eff_block,
                            "blocks": len(blocks), "sweeps": len(blocks) * args.eff_block, "seconds": t_eq,
                            "stationary": passes >= 2,
                            "test": f"at least {args.eff_min_blocks} blocks, then twice in a row: the last block "
                                    "mean within 2 sigma of the previous block and the last four block means not "
                                    "monotonic (no trend)",
                            "block_energies": [b["energy"] for b in blocks],
                            "block_errors": [b["error"] for b in blocks]}
    Req = g.positions()
    n = args.eff_sweeps
    (a, r, el, _), dt = timed(lambda: g.vmc_sweeps_measure(n, tau, seed + 1, recompute_every=rec, flush=args.flush))
    summarize("plain_fp32", el, dt, n, {"acceptance": a / max(a + r, 1)})
    del g
    # FP64 drift-diffusion from the same configurations
    ds64 = DeviceSystem(_fp64_twin(system))
    g = Crowd(ds64, nw, k)
    g.load_walkers(Req)
    g.mw_evaluateLog()
    (a, r, el, _), dt = timed(lambda: g.vmc_sweeps_measure(n, tau, seed + 1, recompute_every=rec))
    summarize("plain_fp64", el, dt, n, {"acceptance": a / max(a + r, 1)})
    del g, ds64
    # learned proposal: trained on the plain run's configurations, then frozen
    g = Crowd(dsys32, nw, k)
    g.load_walkers(Req)
    g.mw_evaluateLog()
    g.proposal_init(seed=seed)
    (_, _, _, tr), t_train = timed(lambda: g.vmc_sweeps_learned(args.train_sweeps, tau, seed + 2, train=True,
                                                                 lr=args.lr, recompute_every=rec, flush=args.flush))
    params_finite = bool(np.isfinite(g.proposal_params()).all())
    (a, r, el, _), dt = timed(lambda: g.vmc_sweeps_learned(n, tau, seed + 4, measure=True, recompute_every=rec,
                                                           flush=args.flush))
    summarize("learned_fp32", el, dt, n, {
        "acceptance": a / max(a + r, 1),
        "training": {"sweeps": args.train_sweeps, "electron_moves": args.train_sweeps * nw * system.n_elec,
                     "seconds": t_train, "lr": args.lr, "final_mean_alpha_jump2": tr[0],
                     "final_mean_alpha": tr[1], "final_objective": tr[2], "parameters_finite": params_finite,
                     "data": "configurations of the equilibrated FP32 drift-diffusion run, continued on-policy "
                             "(one Adam step per electron move over the 512 walkers)"}})
    del g
    p64 = out["plain_fp64"]
    for name in ("plain_fp32", "learned_fp32"):
        o = out[name]
        o["speedup_vs_plain_fp64"] = o["effective_samples_per_s"] / p64["effective_samples_per_s"]
        o["energy_within_2sigma_of_plain_fp64"] = agree_within(o, p64, "energy", "error")
        o["variance_within_2sigma_of_plain_fp64"] = agree_within(o, p64, "variance", "variance_error")
    lf, pf = out["learned_fp32"], out["plain_fp32"]
    lf["speedup_vs_plain_fp32"] = lf["effective_samples_per_s"] / pf["effective_samples_per_s"]
    lf["energy_within_2sigma_of_plain_fp32"] = agree_within(lf, pf, "energy", "error")
    lf["variance_within_2sigma_of_plain_fp32"] = agree_within(lf, pf, "variance", "variance_error")
    out["unit"] = "effective samples/s (walker-sweeps/s / kappa, kappa per method from its own walker series)"
    return out


def torch_sync():
    try:
        import torch
        if torch.cuda.is_available():
            torch.cuda.synchronize()
    except ImportError:
        pass


def c3_systems():
    from qmcpack_gb300.system import scaled_spec
    return [make_system(scaled_spec("c0_32e", precision=4, walkers=410)),
            make_system(scaled_spec("c1_384e", walkers=410)),
            make_system(scaled_spec("c3_768e", walkers=204))]


def run_c3(args, rank: int, world: int):
    """Uneven crowd: the three systems swept together by qmcg_group_sweeps (one persistent
    launch per stage), against each crowd replaying its own sweep graph on its own stream
    (the three streams run concurrently)."""
    import torch
    from qmcpack_gb300.autotune import tune
    from qmcpack_gb300.crowd import Crowd, DeviceSystem, Group
    from qmcpack_gb300.replicas import aggregate_timing, replica_seed
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    seed = replica_seed(2024, rank)
    systems = c3_systems()
    dss = [DeviceSystem(s) for s in systems]
    tuned = [tune(s, s.spec.walkers, dsys=ds, flush=args.flush) for s, ds in zip(systems, dss)]
    crowds = []
    for i, (s, ds, t) in enumerate(zip(systems, dss, tuned)):
        g = Crowd(ds, s.spec.walkers, t["delay"])
        g.set_threads(t["threads_per_walker"])
        g.load_walkers(make_walkers(s, s.spec.walkers, seed=50 + i + 100 * rank))
        g.mw_evaluateLog()
        g.vmc_sweeps(max(args.equil // 2, 1), 0.3, seed + i, rng_mode=1, flush=args.flush)
        crowds.append(g)
    moves_per_sweep = sum(s.spec.walkers * s.n_elec for s in systems)
    # each crowd's own sweep graph on its own stream; launched back to back, the streams overlap
    for g in crowds:
        g.vmc_sweeps(args.warmup, 0.3, seed, rng_mode=1, flush=args.flush)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for g in crowds:
        g.vmc_sweeps_async(args.steps)
    for g in crowds:
        g.sync()
    seq_s = time.perf_counter() - t0
    grp = Group(crowds)
    grp.sweeps(args.warmup, 0.3, seed, flush=args.flush)
    stream = torch.cuda.ExternalStream(crowds[0].stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(dev)
    clocks.start()
    time.sleep(0.3)
    torch.cuda.synchronize()
    e0.record(stream)
    stats = grp.sweeps(args.steps, 0.3, seed + 1, flush=args.flush)
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    moves, ms = aggregate_timing(args.steps * moves_per_sweep, ms)
    value = moves / (ms / 1e3)
    # end to end through the C ABI with host buffers (positions in and out of every crowd)
    hosts = [g.positions() for g in crowds]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for g, h in zip(crowds, hosts):
            g.load_walkers(h)
        grp.sweeps(1, 0.3, seed + 2, flush=args.flush)
        for i, g in enumerate(crowds):
            hosts[i] = g.positions()
    e2e_s = time.perf_counter() - t0
    _, e2e_s = aggregate_timing(0.0, e2e_s)
    h2d = sum(h.nbytes for h in hosts)
    algo = sum(bytes_per_walker_move(s, t["delay"]) * s.spec.walkers * s.n_elec for s, t in zip(systems, tuned))
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = peaks.get("hbm_gbs") or 6800.0
    achieved = algo / (ms / args.steps / 1e3) / 1e9
    info = grp.info()
    if rank != 0:
        return
    acc = sum(x[0] for x in stats)
    rej = sum(x[1] for x in stats)
    line = {
        "metric": "walker-moves/s", "value": value, "unit": "walker-moves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"c3_mixed: {DESCRIPTIONS['c3_mixed']}",
                   "step": "one VMC sweep of every crowd (group graph: one persistent launch per stage + flushes)",
                   "crowds": [{"electrons": s.n_elec, "orbitals": s.norb, "walkers": s.spec.walkers,
                               "delay_rank": t["delay"], "threads_per_walker": t["threads_per_walker"],
                               "autotune_ms_per_sweep": t["table"]}
                              for s, t in zip(systems, tuned)],
                   "group": info, "l2": "inputs larger than L2", "parallelism": f"replicas x{world}"},
        "roofline": {"bound": "hbm", "kernel": "whole group sweep (sweep_multi_kernel stages + flushes + repair)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if peaks.get("hbm_gbs")
                     else "fallback 6.8 TB/s", "traffic": None, "algorithmic_bytes_per_sweep": algo},
        "cpu_baseline": None,
        "e2e": {"value": moves / e2e_s, "unit": "walker-moves/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": h2d},
        "gpu_launches": (2 * info["stages"] + 6) * args.steps,
        "clocks": clk,
        "acceptance": acc / max(acc + rej, 1),
        "concurrent_crowds": {"value": args.steps * moves_per_sweep / seq_s, "unit": "walker-moves/s",
                              "what": "the same crowds, each replaying its own sweep graph on its own stream "
                                      "(launched back to back, so the three streams run concurrently)"},
    }
    print(json.dumps(line), flush=True)


def run_reference(args, rank: int, world: int):
    """The reference's CPU implementation of the path (the oracle port of its algorithms,
    mt19937 stream of StdRandom) on the full workload: all walkers of the config, one
    sweep per step, W untimed warm-up sweeps, K timed sweeps, OpenMP over walkers on all
    host cores; the periodic FP64 recompute is timed once and added pro rata."""
    if rank != 0:
        return
    if args.workload not in SPECS:
        print(json.dumps({"impl": "reference", "unavailable": "the CPU restatement is timed on single-system "
                          "workloads only (c0_32e, c1_384e, c2_1536e, c3_768e)"}), flush=True)
        return
    from oracle import oracle as orc
    spec = SPECS[args.workload]
    system = make_system(spec)
    cores = os.cpu_count() or 1
    nw, ne = spec.walkers, system.n_elec
    orc.set_threads(cores)
    c = orc.Crowd(system, nw, spec.delay, spec.precision)
    c.load_walkers(make_walkers(system, nw, seed=100))
    t0 = time.perf_counter()
    c.evaluate_log(nthreads=cores)
    rec_s = time.perf_counter() - t0
    rng = orc.Rng(11)
    # the same untimed sweeps before the timed ones as the GPU arm (equilibration + warm-up)
    c.vmc_sweeps(rng, args.equil + args.warmup, spec.tau, True)
    t0 = time.perf_counter()
    na, nr, _ = c.vmc_sweeps(rng, args.steps, spec.tau, True)
    sweep_s = time.perf_counter() - t0
    n_rec = args.steps / spec.recompute_every if spec.recompute_every else 0.0
    total_s = sweep_s + n_rec * rec_s
    moves = args.steps * nw * ne
    value = moves / total_s
    sample = (f"{args.steps} timed sweeps (after {args.equil} + {args.warmup} untimed) x {nw} walkers x {ne} electrons of "
              f"{args.workload}, {'FP32' if spec.precision == 4 else 'FP64'} move loop, mt19937 stream, "
              f"{sweep_s:.1f} s; FP64 recompute of all walkers {rec_s * 1e3:.0f} ms, added {n_rec:g} times")
    base = {"value": value, "unit": "walker-moves/s", "cores": cores, "kind": "port", "sample": sample}
    line = {
        "impl": "reference", "metric": "walker-moves/s", "value": value, "unit": "walker-moves/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_s / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if spec.precision == 4 else "f64", "data": "synthetic",
        "config": {"workload": f"{args.workload}: {DESCRIPTIONS.get(args.workload, '')}",
                   "step": "one VMC sweep (every electron of every walker moved once)",
                   "walkers": nw, "electrons": ne, "delay_rank": spec.delay,
                   "recompute": f"FP64 recompute every {spec.recompute_every} sweeps, measured once and added "
                                f"pro rata" if spec.recompute_every else "none",
                   "what_runs": "the CPU restatement of the reference algorithms (oracle/), OpenMP over walkers "
                                "on all host cores; the reference's own build needs LAPACK/HDF5/libxml2/Boost "
                                "and an offload compiler that this image lacks, and its sources are not on the "
                                "GPU host"},
        "acceptance": na / max(na + nr, 1),
        "cpu_baseline": base,
        "e2e": {"value": value, "unit": "walker-moves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, rank: int, world: int):
    import torch
    from qmcpack_gb300.crowd import Crowd, DeviceSystem

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    spec = SPECS[args.workload]
    if args.walkers:
        import dataclasses
        spec = dataclasses.replace(spec, walkers=args.walkers)
    system = make_system(spec)
    nw, k = spec.walkers, spec.delay
    dsys = DeviceSystem(system)
    crowd = Crowd(dsys, nw, k)
    R = make_walkers(system, nw, seed=100 + rank)
    crowd.load_walkers(R)
    crowd.mw_evaluateLog()
    from qmcpack_gb300.replicas import aggregate_timing, replica_seed
    seed = replica_seed(2024, rank)
    recompute_every = spec.recompute_every
    # equilibration from the uniform start (untimed), then warm-up (also captures the sweep graph).
    # The timed loops run the sweep graph alone; the periodic FP64 recompute (every
    # recompute_every sweeps) is measured once and added pro rata: steps / recompute_every of it.
    if args.equil > 0:
        crowd.vmc_sweeps(args.equil, spec.tau, seed, rng_mode=1, recompute_every=recompute_every, flush=args.flush)
    crowd.vmc_sweeps(args.warmup, spec.tau, seed, rng_mode=1, recompute_every=0, flush=args.flush)
    # every measurement below starts from this configuration: the chain is still relaxing
    # (acceptance, and with it the cost of a sweep, keeps falling), so measurements taken one
    # after the other would see different amounts of work
    R_start = crowd.positions()

    def restart():
        crowd.load_walkers(R_start)
        crowd.mw_evaluateLog()

    stream = torch.cuda.ExternalStream(crowd.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(dev)
    clocks.start()
    time.sleep(0.3)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    crowd.vmc_sweeps_async(args.steps)
    e1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    acc, rej = crowd.sync()
    repaired = crowd.last_repaired
    rec_ms = crowd.profile_recompute() if recompute_every else 0.0
    n_rec = args.steps / recompute_every if recompute_every else 0.0
    sweep_ms = ms
    ms = ms + n_rec * rec_ms
    moves, ms = aggregate_timing(args.steps * nw * system.n_elec, ms)
    value = moves / (ms / 1e3)

    # end to end through the C ABI with host buffers: one qmcg_vmc_sweeps_host call per step copies
    # the positions in, sweeps, and copies the positions and log|psi| out (the caller's buffers are
    # pinned and reused every step, as a driver's walker buffers are)
    restart()
    Rnp = torch.from_numpy(crowd.positions()).pin_memory().numpy()
    lp = torch.from_numpy(np.zeros(nw)).pin_memory().numpy()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        crowd.vmc_sweeps_host(1, spec.tau, seed, R_in=Rnp, R_out=Rnp, log_out=lp, recompute_every=0,
                              flush=args.flush)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0 + n_rec * rec_ms / 1e3
    _, e2e_s = aggregate_timing(0.0, e2e_s)
    e2e_value = moves / e2e_s
    h2d = Rnp.nbytes
    d2h = Rnp.nbytes + lp.nbytes

    # dominant kernel: per-launch CUDA-event time of the walker-resident kernel (one
    # launch = one segment of up to k electrons of every walker); the batched flush
    # is timed alongside
    restart()
    seg_ms, flush_ms, seg_per_sweep, flush_per_sweep = crowd.profile_sweep(3)
    algo = bytes_per_walker_move(system, k, with_flush=False) * nw * system.n_elec // seg_per_sweep
    block_lazy = crowd.sweep_info(args.flush)["block_lazy"]
    if block_lazy:
        flush_bytes = block_update_bytes_per_sweep(system, k, nw, acc / max(acc + rej, 1)) // flush_per_sweep
    else:
        flush_bytes = flush_bytes_per_launch(system, k, nw)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = peaks.get("hbm_gbs")
    peak_src = "measured" if peak else "fallback"
    peak = peak or 6800.0
    achieved = algo / (seg_ms / 1e3) / 1e9
    traffic = read_traffic(args.workload)
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    base = cpu_baseline(args.workload) if world == 1 and not args.no_cpu_baseline else None
    eff = None
    rerr = None
    extras = {}
    if world == 1 and not args.no_extras:
        extras["virtual_moves"] = virtual_moves(crowd, system, peak)
        # DMC's small time step accepts ~3/4 of the moves: the block-lazy updates then carry
        # most slots of every set and the tensor-core flush after every segment is faster
        extras["dmc"] = dmc_rate(dsys, system, crowd.positions(), 3 if args.flush == 4 else args.flush)
    if world == 1 and not args.no_effective and args.workload == "c1_384e":
        Req = crowd.positions()[:64]
        rerr = {"uniform_start": ratio_error(system, dsys, 64, k),
                "equilibrated": ratio_error(system, dsys, 64, k, R=Req)}
        eff = effective_samples(args, system, dsys, seed + 11)
    line = {
        "metric": "walker-moves/s", "value": value, "unit": "walker-moves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if spec.precision == 4 else "f64", "data": "synthetic",
        "config": {"workload": f"{args.workload}: {DESCRIPTIONS.get(args.workload, '')}",
                   "step": "one VMC sweep (every electron of every walker moved once), CUDA graph replay",
                   "walkers_per_gpu": nw, "electrons": system.n_elec, "delay_rank": k,
                   "flush": {0: "SIMT FP32", 1: "tcgen05 TF32", 3: "tcgen05 3xTF32",
                             4: "block-lazy updates, SIMT FP32" if block_lazy else "tcgen05 3xTF32"}[args.flush],
                   "l2": "inputs larger than L2 (spline table 102 MB + inverses/gradients ~0.8 GB per sweep)",
                   "recompute": ({"every_sweeps": recompute_every, "measured_ms": rec_ms, "added": n_rec,
                                  "how": "the FP64 recompute of all walkers, timed once with CUDA events, added "
                                         "steps/recompute_every times to the device and e2e totals"}
                                 if recompute_every else None),
                   "sweep_graph_ms_per_step": sweep_ms / args.steps,
                   "parallelism": f"replicas x{world}"},
        "roofline": {"bound": "hbm", "kernel": "sweep_kernel (walker-resident; one launch = up to k electrons "
                                                 "of every walker)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)" if peak_src == "measured"
                     else "fallback 6.8 TB/s", "traffic": traffic, "ms_per_launch": seg_ms,
                     "algorithmic_bytes_per_launch": algo, "launches_per_sweep": seg_per_sweep,
                     "flush": {"kernel": flush_kernel_name(system.spec.n_up, k, args.flush, block_lazy),
                               "ms_per_launch": flush_ms,
                               "launches_per_sweep": flush_per_sweep, "algorithmic_bytes_per_launch": flush_bytes,
                               "achieved_gbs": flush_bytes / (flush_ms / 1e3) / 1e9 if flush_ms else None}},
        "cpu_baseline": base,
        "e2e": {"value": e2e_value, "unit": "walker-moves/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches_per_sweep(system, k) * args.steps,
        "clocks": clk,
        "acceptance": acc / max(acc + rej, 1),
        "walkers_repaired_in_timed_sweeps": repaired,
        "equilibration_sweeps": args.equil,
        "walker_sweeps_per_s": value / system.n_elec,
        "effective_samples": eff,
        "ratio_error_fp32": rerr,
        **extras,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c1_384e", choices=sorted(SPECS) + ["c3_mixed"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--equil", type=int, default=20, help="untimed equilibration sweeps before the warm-up")
    ap.add_argument("--flush", type=int, default=4, choices=[0, 1, 3, 4],
                    help="delayed-update flush: 0 SIMT, 1 tensor cores TF32, 3 tensor cores 3xTF32, 4 block-lazy "
                         "updates where the segment rows are staged (else as 3)")
    ap.add_argument("--no-effective", action="store_true", help="skip the effective-samples comparison")
    ap.add_argument("--no-extras", action="store_true", help="skip the virtual-move and DMC measurements")
    ap.add_argument("--walkers", type=int, default=0, help="walkers of the crowd (0: the workload's own count; "
                                                           "smaller counts size profiler captures)")
    ap.add_argument("--eff-sweeps", type=int, default=500, help="measured sweeps per method in the comparison")
    ap.add_argument("--eff-block", type=int, default=250, help="sweeps per equilibration block")
    ap.add_argument("--eff-min-blocks", type=int, default=8, help="fewest equilibration blocks")
    ap.add_argument("--eff-max-blocks", type=int, default=16, help="most equilibration blocks")
    ap.add_argument("--train-sweeps", type=int, default=10)
    ap.add_argument("--lr", type=float, default=1e-3)
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.workload == "c3_mixed":
        run_c3(args, rank, world)
    else:
        run_ours(args, rank, world)


if __name__ == "__main__":
    main()
