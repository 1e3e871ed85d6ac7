"""The walker-resident sweep kernel (the benchmarked path) against the CPU oracle.

Both sides draw from the same counter-based stream (Philox4x32-10 with counter
(walker, electron, sweep, j)).  Two FP64 checks:

* step by step: the oracle follows the GPU's recorded trajectory and, at every
  move, forms on that shared state its own gradient, its own proposal from the
  stream's Gaussians, the ratio and gradient at the proposed position, and its own
  decision with the stream's uniform.  Proposals agree to 1e-10 bohr; ratios to
  1e-10 of max(|ratio|, 1) (next to a node of psi the ratio is a sum of O(1) terms
  cancelling to a small value, so its rounding is absolute); gradients at R to 1e-10
  relative in the vector norm, gradients at R' to 1e-10 max(1, 1/|ratio|) (they are
  divided by the ratio, whose error is absolute); decisions are identical (a differing decision
  is allowed only at a tie, |u - P| <= 1e-9 P, and none is expected); the final
  inverses, log|psi|, Jastrow state and G/L agree to 1e-10.
* as independent chains: the oracle runs its own chain from the same start.  The
  drift-diffusion chain amplifies last-bit differences (GPU and host transcendentals,
  fused multiply-adds) by about ten every 15-25 moves, so two correct FP64 chains
  part after a few hundred moves per walker.  Every decision taken while the two
  trajectories are within 1e-6 bohr must be identical.

In FP32 the GPU's moves are replayed by the FP64 oracle on identical positions and
coefficients, and the errors of ratios, gradients, Laplacians, inverses and the
decisions are measured and bounded.

Workloads: the 32-electron system exactly as configured (64 walkers, 32^3 grid,
rank-1 updates, FP64, 100 sweeps); the 384-electron system (48^3 grid, 192
orbitals, delay rank 32) in FP64 and FP32; the 1536-electron system (60^3 grid,
768 orbitals, delay rank 64) in FP32.  Walker counts are reduced where the scalar
oracle would take minutes.

Set QMCG_ERROR_TABLE to a file path to append the measured error statistics
(one JSON object per workload).
"""
import dataclasses
import json
import os

import numpy as np
import pytest

from oracle import oracle as orc
from qmcpack_gb300.system import make_system, make_walkers

pytestmark = pytest.mark.gpu

TAU = 0.3
TIE = 1e-9


def _gpu():
    from qmcpack_gb300.crowd import Crowd, DeviceSystem
    return Crowd, DeviceSystem


def fp64_twin(system):
    spec64 = dataclasses.replace(system.spec, precision=8)
    return dataclasses.replace(system, spec=spec64, coefs=system.coefs.astype(np.float64))


def rel_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def stats(x):
    x = np.asarray(x).ravel()
    if x.size == 0:
        return {"median": 0.0, "p99": 0.0, "max": 0.0, "n": 0}
    return {"median": float(np.median(x)), "p99": float(np.percentile(x, 99)), "max": float(x.max()),
            "n": int(x.size)}


def report(name, table):
    print(name, json.dumps(table))
    path = os.environ.get("QMCG_ERROR_TABLE")
    if path:
        with open(path, "a") as f:
            f.write(json.dumps({"workload": name, **table}) + "\n")


def ratio_errors(a, b, tol=1e-10):
    """|a - b| / max(|b|, 1) <= tol for every move; returns the plain relative errors' statistics too."""
    e = np.abs(a - b) / np.maximum(np.abs(b), 1.0)
    assert np.all(e <= tol), (np.max(e), np.argwhere(e > tol)[:5])
    return {"scaled": stats(e), "relative": stats(np.abs(a - b) / np.maximum(np.abs(b), 1e-300))}


def grad_errors(a, b, scale, tol=1e-10):
    """Norm-wise relative errors |a - b| / |b| of gradient vectors [..., 3], at most tol * scale
    per move; statistics where scale is 1 and where it is larger."""
    e = np.linalg.norm(a - b, axis=-1) / np.maximum(np.linalg.norm(b, axis=-1), 1e-300)
    assert np.all(e <= tol * scale), (np.max(e / scale), np.argwhere(e > tol * scale)[:5])
    near = scale > 1
    return {"away_from_nodes": stats(e[~near]), "near_nodes": stats(e[near])}


def oracle_crowd(system, nw, k, R):
    orc.set_threads(os.cpu_count() or 1)
    o = orc.Crowd(system, nw, k, 8)
    o.load_walkers(R)
    o.evaluate_log(nthreads=os.cpu_count() or 1)
    return o


def fp64_parity(name, system, nw, k, nsweeps, seed, walker_seed, flush=0):
    Crowd, DeviceSystem = _gpu()
    R = make_walkers(system, nw, seed=walker_seed)
    g = Crowd(DeviceSystem(system), nw, k)
    assert g.sweep_info(flush)["block_lazy"] == (flush == 4)
    g.load_walkers(R)
    g.mw_evaluateLog()
    ag, _, tg = g.vmc_sweeps_trace(nsweeps, TAU, seed, flush=flush)
    # ---- step by step on the GPU's trajectory
    o = oracle_crowd(system, nw, k, R)
    to, margin = o.replay_philox(tg, seed, TAU)
    np.testing.assert_allclose(to[..., 0:3], tg[..., 0:3], rtol=0, atol=1e-10)
    r_err = ratio_errors(tg[..., 3], to[..., 3])
    gn_err = grad_errors(tg[..., 4:7], to[..., 4:7], np.maximum(1.0, 1.0 / np.abs(to[..., 3])))
    gw_err = grad_errors(tg[..., 7:10], to[..., 7:10], np.ones(to.shape[:-1]))
    differ = tg[..., 10] != to[..., 10]
    assert np.all(np.abs(margin[differ]) <= TIE), np.argwhere(differ)[:5]
    np.testing.assert_array_equal(g.positions(), o.positions())
    lg, sg, _ = g.get_log()
    lo, so, _ = o.get_log()
    assert rel_err(lg, lo) < 1e-10 and (sg == so).all()
    for spin in (0, 1):
        assert rel_err(g.inverse(spin), o.ainv(spin)) < 1e-10
    j2g, j1g = g.jastrow_state()
    j2o, j1o = o.jastrow_state()
    assert rel_err(j2g, j2o) < 1e-10 and rel_err(j1g, j1o) < 1e-10
    _, Gg, Lg = g.mw_evaluateGL()
    _, glo = o.kinetic(with_gl=True)
    assert rel_err(Gg, glo[..., 0:3]) < 1e-10 and rel_err(Lg, glo[..., 3]) < 1e-10
    # ---- independent chains from the same start
    oi = oracle_crowd(system, nw, k, R)
    _, _, ti = oi.vmc_sweeps_philox(seed, nsweeps, TAU, trace=True)
    ne = system.n_elec
    dpos = np.abs(tg[..., 0:3] - ti[..., 0:3]).max(axis=-1).reshape(nsweeps * ne, nw)
    same = (tg[..., 10] == ti[..., 10]).reshape(nsweeps * ne, nw)
    close = np.maximum.accumulate(dpos, axis=0) < 1e-6
    assert np.all(same[close]), np.argwhere(close & ~same)[:5]
    horizon = np.where(close.all(axis=0), nsweeps * ne, np.argmin(close, axis=0))
    report(name, {
        "moves": int(tg[..., 10].size), "walkers": nw, "sweeps": nsweeps, "accepted": int(ag),
        "step_by_step": {"proposal_abs": stats(np.abs(to[..., 0:3] - tg[..., 0:3])),
                         "ratio_rel": r_err, "grad_new_rel": gn_err, "grad_now_rel": gw_err,
                         "differing_decisions": int(differ.sum()),
                         "closest_tie": float(np.min(np.abs(margin)))},
        "independent_chains": {"decisions_compared_within_1e-6_bohr": int(close.sum()),
                               "moves_to_divergence_per_walker": stats(horizon),
                               "walkers_never_diverged": int(close.all(axis=0).sum())},
    })


def test_c0_exact_parity():
    """The 32-electron workload as configured: 64 walkers, rank-1 updates, FP64, 100 sweeps."""
    s = make_system("c0_32e")
    assert s.spec.walkers == 64 and s.spec.delay == 1 and s.spec.precision == 8 and s.spec.steps == 100
    fp64_parity("c0_32e_fp64", s, s.spec.walkers, s.spec.delay, s.spec.steps, seed=20241, walker_seed=31)


@pytest.mark.parametrize("flush", [0, 4])
def test_c1_system_fp64_parity(flush):
    """The 384-electron system (FP32 coefficient values upcast to FP64) with delay rank 32,
    flushing after every segment (0) or with block-lazy updates (4)."""
    s = fp64_twin(make_system("c1_384e"))
    name = "c1_384e_fp64" + ("_block_lazy" if flush == 4 else "")
    fp64_parity(name, s, 4, s.spec.delay, 2, seed=777, walker_seed=41, flush=flush)


def fp32_errors(system, nw, k, equil, nsweeps, seed, flush, walker_seed):
    """FP32 resident sweeps recorded on the GPU, replayed by the FP64 oracle on the same
    positions and decisions; errors of every move and of the final state."""
    Crowd, DeviceSystem = _gpu()
    assert system.spec.precision == 4
    g = Crowd(DeviceSystem(system), nw, k)
    g.load_walkers(make_walkers(system, nw, seed=walker_seed))
    g.mw_evaluateLog()
    if equil:
        g.vmc_sweeps(equil, TAU, seed, rng_mode=1, flush=flush)
    R = g.positions()
    g.load_walkers(R)
    g.mw_evaluateLog()
    o = orc.Crowd(system, nw, k, 8)
    o.load_walkers(R)
    orc.set_threads(os.cpu_count() or 1)
    o.evaluate_log(nthreads=os.cpu_count() or 1)
    _, _, tg = g.vmc_sweeps_trace(nsweeps, TAU, seed + 1, flush=flush)
    # the traced sweeps follow the equilibration sweeps on the crowd's sweep counter
    to, margin = o.replay_philox(tg, seed + 1, TAU, sweep0=equil)
    differ = tg[..., 10] != to[..., 10]
    r32, r64 = tg[..., 3], to[..., 3]
    rat = np.abs(r32 - r64) / np.maximum(np.abs(r64), 1e-300)
    away = np.abs(r64) > 1e-2
    gn32, gn64 = tg[..., 4:7], to[..., 4:7]
    gw32, gw64 = tg[..., 7:10], to[..., 7:10]
    gn = np.linalg.norm(gn32 - gn64, axis=-1) / np.maximum(np.linalg.norm(gn64, axis=-1), 1e-300)
    gw = np.linalg.norm(gw32 - gw64, axis=-1) / np.maximum(np.linalg.norm(gw64, axis=-1), 1e-300)
    inv = []
    for spin in (0, 1):
        A32, A64 = g.inverse(spin), o.ainv(spin)
        inv.append(np.max(np.abs(A32 - A64), axis=(1, 2)) / np.max(np.abs(A64), axis=(1, 2)))
    inv = np.concatenate(inv)
    lg, _, _ = g.get_log()
    lo, _, _ = o.get_log()
    _, G32, L32 = g.mw_evaluateGL()
    _, glo = o.kinetic(with_gl=True)
    G64, L64 = glo[..., 0:3], glo[..., 3]
    Ge = np.linalg.norm(G32 - G64, axis=-1) / np.maximum(np.linalg.norm(G64, axis=-1), 1e-300)
    Le = np.abs(L32 - L64) / np.maximum(np.abs(L64), 1e-300)
    self_dev = np.abs(tg[..., 11] - 1.0)
    table = {
        "moves": int(r32.size), "walkers": nw, "sweeps": nsweeps, "equilibration_sweeps": equil,
        "flush": {0: "SIMT FP32", 1: "tcgen05 TF32", 3: "tcgen05 3xTF32", 4: "block-lazy SIMT FP32"}[flush],
        "ratio_rel": stats(rat), "ratio_rel_away_from_nodes": stats(rat[away]),
        "grad_new_rel": stats(gn), "grad_now_rel": stats(gw),
        "inverse_rel_to_max": stats(inv), "laplacian_rel": stats(Le), "gradient_G_rel": stats(Ge),
        "log_psi_abs": stats(np.abs(lg - lo)), "self_ratio_deviation": stats(self_dev),
        "proposal_abs": stats(np.abs(tg[..., 0:3] - to[..., 0:3])),
        "decisions_differing_from_fp64": int(differ.sum()),
        "differing_decision_margin": stats(np.abs(margin[differ])),
        "decisions_accepted": int(tg[..., 10].sum()), "walkers_repaired": int(g.last_repaired),
    }
    return table


@pytest.mark.parametrize("flush", [3, 4])
def test_c1_fp32_against_fp64_oracle(flush):
    """The 384-electron production shape in FP32 (tensor-core 3xTF32 flush after every
    segment, or block-lazy updates) against the FP64 oracle: per-move ratio and gradient
    errors, then inverse, G, L and log|psi|."""
    s = make_system("c1_384e")
    t = fp32_errors(s, 8, s.spec.delay, equil=20, nsweeps=2, seed=4242, flush=flush, walker_seed=51)
    report("c1_384e" + ("_block_lazy" if flush == 4 else ""), t)
    assert t["ratio_rel"]["median"] < 1e-4 and t["ratio_rel_away_from_nodes"]["p99"] < 1e-2
    assert t["grad_new_rel"]["median"] < 1e-4 and t["grad_now_rel"]["median"] < 1e-4
    assert t["inverse_rel_to_max"]["max"] < 2e-2
    assert t["gradient_G_rel"]["median"] < 1e-3 and t["laplacian_rel"]["median"] < 1e-3
    assert t["log_psi_abs"]["max"] < 1e-2


def test_c2_fp32_against_fp64_oracle():
    """The 1536-electron precision form (768 orbitals, delay rank 64, 3xTF32 flush)."""
    s = make_system("c2_1536e")
    t = fp32_errors(s, 2, s.spec.delay, equil=2, nsweeps=1, seed=99, flush=3, walker_seed=61)
    report("c2_1536e", t)
    assert t["ratio_rel"]["median"] < 1e-3 and t["ratio_rel_away_from_nodes"]["p99"] < 5e-2
    assert t["grad_new_rel"]["median"] < 1e-3
    assert t["inverse_rel_to_max"]["max"] < 5e-2
    assert t["gradient_G_rel"]["median"] < 1e-2 and t["laplacian_rel"]["median"] < 1e-2


@pytest.mark.parametrize("flush", [3, 4])
def test_plain_sweeps_match_traced_sweeps(flush):
    """The benchmarked FP32 sweep (the kernel form compiled without move records or DMC
    rules) gives bit-identical results to the traced sweep the oracle replays above."""
    Crowd, DeviceSystem = _gpu()
    s = make_system("c1_384e")
    ds = DeviceSystem(s)
    R = make_walkers(s, 8, seed=71)
    out = []
    for traced in (False, True):
        g = Crowd(ds, 8, s.spec.delay)
        g.load_walkers(R)
        g.mw_evaluateLog()
        if traced:
            a, r, _ = g.vmc_sweeps_trace(2, TAU, 505, flush=flush)
        else:
            a, r, _ = g.vmc_sweeps(2, TAU, 505, rng_mode=1, flush=flush)
        out.append((a, r, g.positions(), g.get_log()[0], g.inverse(0), g.inverse(1), *g.jastrow_state()))
    (a0, r0, *x0), (a1, r1, *x1) = out
    assert (a0, r0) == (a1, r1)
    for u, v in zip(x0, x1):
        np.testing.assert_array_equal(u, v)
