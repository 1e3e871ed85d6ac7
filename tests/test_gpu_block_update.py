"""Block-lazy delayed updates (flush kind 4) of the walker-resident sweep.

A row block of the inverse receives the pending rank-k updates of its spin group right
before the segment that reads it, and one pass completes the inverse after the spin
group.  The same updates reach every row in the same order as with a flush after every
segment, so in FP64:
  * against the CPU oracle, step by step on the GPU's trajectory: ratios and gradients to
    1e-10, identical decisions, final inverses, log|psi| and Jastrow state to 1e-10;
  * against the flush after every segment (kind 0): identical decisions and states within
    1e-10 (only the summation order differs), at both ends of the acceptance range (every
    slot of a set accepted, or nearly none) and on ragged spin groups whose last segment
    is shorter than the delay rank;
  * DMC steps (the local energy reads the completed inverse) agree likewise.
Crowds whose segment rows are not staged keep one delayed-update set and fall back to
the flush after every segment.
"""
import numpy as np
import pytest

from oracle import oracle as orc
from qmcpack_gb300.system import make_system, make_walkers, scaled_spec

pytestmark = pytest.mark.gpu

TAU = 0.3


def _gpu():
    from qmcpack_gb300.crowd import Crowd, DeviceSystem
    return Crowd, DeviceSystem


def rel_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def ragged(prec=8, n=13, grid=14, nw=6, delay=4, seed=5):
    spec = scaled_spec("c0_32e", n_up=n, n_dn=n, grid=grid, walkers=nw, delay=delay, precision=prec)
    return make_system(spec, seed=seed)


def run(system, nw, delay, R, flush, nsweeps, tau, seed):
    Crowd, DeviceSystem = _gpu()
    g = Crowd(DeviceSystem(system), nw, delay)
    g.load_walkers(R)
    g.mw_evaluateLog()
    a, r, tr = g.vmc_sweeps_trace(nsweeps, tau, seed, flush=flush)
    state = (g.positions(), g.get_log()[0], g.inverse(0), g.inverse(1), *g.jastrow_state())
    return g, a, r, tr, state


def test_sweep_info():
    """Sets per spin = segments of the larger spin group where the rows are staged."""
    Crowd, DeviceSystem = _gpu()
    s = ragged()
    g = Crowd(DeviceSystem(s), 6, 4)
    i4, i3 = g.sweep_info(4), g.sweep_info(3)
    assert i4["rows_staged"] and i4["sets"] == 4 and i4["block_lazy"]
    assert not i3["block_lazy"] and i3["sets"] == 4
    g1 = Crowd(DeviceSystem(ragged(delay=1)), 6, 1)
    assert not g1.sweep_info(4)["block_lazy"] and g1.sweep_info(4)["sets"] == 1


def test_ragged_fp64_against_oracle():
    """13 + 13 electrons, delay rank 4: segments of 4, 4, 4 and 1 in each spin group."""
    s = ragged()
    nw, k, seed = 6, 4, 901
    R = make_walkers(s, nw, seed=7)
    g, a, _, tg, _ = run(s, nw, k, R, 4, 3, TAU, seed)
    assert g.sweep_info(4)["block_lazy"]
    o = orc.Crowd(s, nw, k, 8)
    o.load_walkers(R)
    o.evaluate_log()
    to, margin = o.replay_philox(tg, seed, TAU)
    np.testing.assert_allclose(to[..., 0:3], tg[..., 0:3], rtol=0, atol=1e-10)
    e = np.abs(tg[..., 3] - to[..., 3]) / np.maximum(np.abs(to[..., 3]), 1.0)
    assert e.max() < 1e-10
    differ = tg[..., 10] != to[..., 10]
    assert np.all(np.abs(margin[differ]) <= 1e-9)
    assert 0 < a < tg[..., 10].size
    lg, sg, _ = g.get_log()
    lo, so, _ = o.get_log()
    assert rel_err(lg, lo) < 1e-10 and (sg == so).all()
    for spin in (0, 1):
        assert rel_err(g.inverse(spin), o.ainv(spin)) < 1e-10
    j2g, j1g = g.jastrow_state()
    j2o, j1o = o.jastrow_state()
    assert rel_err(j2g, j2o) < 1e-10 and rel_err(j1g, j1o) < 1e-10


def replay_errors(system, nw, k, R, tg, seed, tau):
    """The FP64 oracle on a recorded trajectory: scaled ratio errors, tie margins of the
    differing decisions, and the oracle crowd (its final state)."""
    o = orc.Crowd(system, nw, k, 8)
    o.load_walkers(R)
    o.evaluate_log()
    to, margin = o.replay_philox(tg, seed, tau)
    e = np.abs(tg[..., 3] - to[..., 3]) / np.maximum(np.abs(to[..., 3]), 1.0)
    differ = tg[..., 10] != to[..., 10]
    return e, margin[differ], o


@pytest.mark.parametrize("tau,accept_range", [(1e-4, (0.97, 1.0)), (0.3, (0.05, 0.95)), (40.0, (0.0, 0.5))])
def test_acceptance_range_against_oracle(tau, accept_range):
    """Every slot of a set accepted, a mixture, or steps across the cell (many sets with
    no accepted slot at all): the flush after every segment and the block-lazy updates
    each replayed by the FP64 oracle.  (The two runs are not compared with each other
    move by move: the drift amplifies their last-bit differences along the chain.)"""
    s = ragged()
    R = make_walkers(s, 6, seed=8)
    lo, hi = accept_range
    for flush in (0, 4):
        g, a, r, tg, _ = run(s, 6, 4, R, flush, 3, tau, 77)
        assert lo <= a / (a + r) <= hi
        e, margins, o = replay_errors(s, 6, 4, R, tg, 77, tau)
        assert e.max() < 1e-10, (flush, e.max())
        assert np.all(np.abs(margins) <= 1e-9)
        for spin in (0, 1):
            assert rel_err(g.inverse(spin), o.ainv(spin)) < 1e-10


@pytest.mark.parametrize("flush", [3, 4])
def test_fp32_against_fp64_oracle(flush):
    """FP32 sweeps (tensor-core flush after every segment, or block-lazy updates) replayed by
    the FP64 oracle on the same positions: ratios away from nodes and the final inverses
    within FP32 rounding."""
    s = ragged(prec=4)
    nw, k, seed = 6, 4, 55
    R = make_walkers(s, nw, seed=9)
    g, _, _, tg, _ = run(s, nw, k, R, flush, 2, TAU, seed)
    o = orc.Crowd(s, nw, k, 8)
    o.load_walkers(R)
    o.evaluate_log()
    to, _ = o.replay_philox(tg, seed, TAU)
    r32, r64 = tg[..., 3], to[..., 3]
    away = np.abs(r64) > 1e-2
    rel = np.abs(r32 - r64) / np.abs(r64)
    # the tail belongs to an ill-conditioned walker, with either flush
    assert np.median(rel[away]) < 1e-4 and np.percentile(rel[away], 90) < 1e-3, np.percentile(rel[away], [50, 90])
    for spin in (0, 1):
        e = np.max(np.abs(g.inverse(spin) - o.ainv(spin)), axis=(1, 2)) / np.max(np.abs(o.ainv(spin)), axis=(1, 2))
        assert np.median(e) < 1e-4, e


def test_unstaged_crowd_falls_back():
    """Delay rank 64 on 64 orbitals: the segment rows are not staged, one set per spin is
    kept and flush kind 4 runs the flush after every segment (identical to kind 0 in FP64)."""
    s = make_system(scaled_spec("c0_32e", n_up=64, n_dn=64, grid=12, walkers=3, delay=64, precision=8), seed=3)
    Crowd, DeviceSystem = _gpu()
    info = Crowd(DeviceSystem(s), 3, 64).sweep_info(4)
    assert not info["rows_staged"] and info["sets"] == 1 and not info["block_lazy"]
    R = make_walkers(s, 3, seed=4)
    (_, a0, _, t0, st0), (_, a4, _, t4, st4) = [run(s, 3, 64, R, flush, 1, TAU, 66) for flush in (0, 4)]
    assert a0 == a4
    np.testing.assert_array_equal(t0, t4)
    for x0, x4 in zip(st0, st4):
        np.testing.assert_array_equal(x0, x4)


def test_dmc_steps_match():
    """Fixed-node DMC steps: the local energies read the completed inverse."""
    s = ragged()
    R = make_walkers(s, 6, seed=10)
    Crowd, DeviceSystem = _gpu()
    res = []
    for flush in (0, 4):
        g = Crowd(DeviceSystem(s), 6, 4)
        g.load_walkers(R)
        g.mw_evaluateLog()
        el0 = g.dmc_init()
        e_t, sd = float(np.mean(el0)), float(np.std(el0))
        steps = []
        for it in range(3):
            out = g.dmc_step(0.02, 31 + it, e_trial=e_t, e_ref=e_t, tau_eff=0.02, branch_cutoff=0.5 * sd,
                             branch_max=1.0 * sd, flush=flush)
            steps.append((out["weights"].copy(), out["e_local"].copy(), out["accepted"]))
        res.append((steps, g.inverse(0), g.inverse(1)))
    (s0, A0, B0), (s4, A4, B4) = res
    for (w0, e0, n0), (w4, e4, n4) in zip(s0, s4):
        assert n0 == n4
        assert rel_err(w4, w0) < 1e-10 and rel_err(e4, e0) < 1e-10
    assert rel_err(A4, A0) < 1e-10 and rel_err(B4, B0) < 1e-10
