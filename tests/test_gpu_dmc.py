"""Diffusion Monte Carlo on the GPU against the oracle (FP64, step by step).

Per DMC step the oracle follows the GPU's recorded moves on the shared state and forms
its own fixed-node decisions (a move that changes the sign of psi is rejected), the
tau |xi|^2 sums of proposed and accepted moves, the local energies and the branch
weights of SFNBranch::branchWeight (oracle/dmc_oracle.py); population control is the
comb of WalkerReconfiguration on both sides.  Tolerances: decisions identical (a tie
|u - P| <= 1e-9 P excepted), r^2 sums 1e-12, local energies 1e-9, weights 1e-9
relative, walker copies exact, final inverses and log|psi| 1e-10.
"""
import numpy as np
import pytest

from oracle import dmc_oracle as dmo
from oracle import oracle as orc
from qmcpack_gb300.system import make_system, make_walkers, scaled_spec

pytestmark = pytest.mark.gpu


def _gpu():
    from qmcpack_gb300.crowd import Crowd, DeviceSystem
    return Crowd, DeviceSystem


def rel_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def small(prec=8, n=8, nw=32, delay=4, seed=41):
    spec = scaled_spec("c0_32e", n_up=n, n_dn=n, grid=12, walkers=nw, delay=delay, precision=prec)
    return make_system(spec, seed=seed)


def test_dmc_steps_match_oracle():
    Crowd, DeviceSystem = _gpu()
    nw, k, tau, seed = 32, 4, 0.05, 515
    s = small(nw=nw, delay=k)
    R = make_walkers(s, nw, seed=42)
    g = Crowd(DeviceSystem(s), nw, k)
    g.load_walkers(R)
    g.mw_evaluateLog()
    o = orc.Crowd(s, nw, k, 8)
    o.load_walkers(R)
    o.evaluate_log()
    el_g = g.dmc_init()
    e_old, _, _ = o.local_energy()
    assert rel_err(el_g, e_old) < 1e-9
    sd = float(np.std(e_old))
    # a window narrow enough that some walkers are filtered and some are cut off
    params = dict(e_trial=float(np.mean(e_old)), e_ref=float(np.mean(e_old)), tau_eff=tau,
                  branch_cutoff=0.5 * sd, branch_max=1.0 * sd)
    w_prev = np.ones(nw)
    rng = np.random.default_rng(3)
    rejected_sign = 0
    for step in range(4):
        out = g.dmc_step(tau, seed, **params, trace=True)
        tr = out["trace"]
        to, margin = o.replay_philox(tr, seed, tau, sweep0=step, dmc=True)
        np.testing.assert_allclose(to[..., 0:3], tr[..., 0:3], rtol=0, atol=1e-10)
        differ = tr[..., 10] != to[..., 10]
        assert np.all(np.abs(margin[differ]) <= 1e-9), np.argwhere(differ)[:5]
        sign_change = to[..., 3] <= 0
        assert not np.any(tr[..., 10][sign_change])
        rejected_sign += int(sign_change.sum())
        r2 = to[0, ..., 11]
        np.testing.assert_allclose(out["sums"][4], r2.sum(), rtol=1e-12)
        np.testing.assert_allclose(out["sums"][3], (r2 * tr[0, ..., 10]).sum(), rtol=1e-12)
        assert np.all(out["age"] == 0)
        e_new, _, _ = o.local_energy()
        assert rel_err(out["e_local"], e_new) < 1e-9
        w_exp = w_prev * dmo.branch_weight(e_new, e_old, **params)
        np.testing.assert_allclose(out["weights"], w_exp, rtol=1e-9)
        w, e = out["weights"], out["e_local"]
        np.testing.assert_allclose(out["sums"][0:3], [w.sum(), (w * e).sum(), (w * e * e).sum()], rtol=1e-12)
        u = rng.random()
        src_g = g.dmc_reconfigure(u)
        src_o, _ = dmo.comb(w, u)
        np.testing.assert_array_equal(src_g, src_o)
        o.copy_walkers(src_o)
        e_old = e_new[src_o]
        w_prev = np.ones(nw)
    assert rejected_sign > 0, "no move crossed a node: the fixed-node rejection was not exercised"
    np.testing.assert_array_equal(g.positions(), o.positions())
    assert rel_err(g.get_log()[0], o.get_log()[0]) < 1e-10
    for spin in (0, 1):
        assert rel_err(g.inverse(spin), o.ainv(spin)) < 1e-10


def test_copy_walkers_is_exact():
    Crowd, DeviceSystem = _gpu()
    nw = 12
    s = small(prec=4, nw=nw, delay=4, seed=43)
    g = Crowd(DeviceSystem(s), nw, 4)
    g.load_walkers(make_walkers(s, nw, seed=44))
    g.mw_evaluateLog()
    g.dmc_init()
    g.vmc_sweeps(2, 0.3, 7, rng_mode=1)
    before = (g.positions(), g.inverse(0), g.inverse(1), g.jastrow_state(), g.get_log())
    src = np.arange(nw)
    src[[1, 4, 7]] = [0, 0, 9]
    g.dmc_copy_walkers(src)
    after = (g.positions(), g.inverse(0), g.inverse(1), g.jastrow_state(), g.get_log())
    np.testing.assert_array_equal(after[0], before[0][src])
    np.testing.assert_array_equal(after[1], before[1][src])
    np.testing.assert_array_equal(after[2], before[2][src])
    for a, b in zip(after[3], before[3]):
        np.testing.assert_array_equal(a, b[src])
    for a, b in zip(after[4], before[4]):
        np.testing.assert_array_equal(a, b[src])
    # a slot that is copied elsewhere must keep its own walker
    bad = np.arange(nw)
    bad[0], bad[1] = 1, 2
    from qmcpack_gb300._lib import QmcgError
    with pytest.raises(QmcgError):
        g.dmc_copy_walkers(bad)


def test_dmc_driver_fp32():
    """The host driver over the device steps: finite energies, the population weight kept
    near the target by E_trial, the reference energy following the step energies."""
    from qmcpack_gb300.dmc import DMCDriver
    Crowd, DeviceSystem = _gpu()
    nw = 256
    s = small(prec=4, n=16, nw=nw, delay=8, seed=45)
    g = Crowd(DeviceSystem(s), nw, 8)
    g.load_walkers(make_walkers(s, nw, seed=46))
    g.mw_evaluateLog()
    g.vmc_sweeps(50, 0.3, 9, rng_mode=1)
    d = DMCDriver(g, tau=0.02, seed=10, warmup_steps=10, flush=3)
    hist = d.run(60)
    e = np.array([h["e_now"] for h in hist])
    w = np.array([h["weight"] for h in hist])
    assert np.all(np.isfinite(e)) and np.all(w > 0)
    assert abs(np.mean(w[20:]) / nw - 1) < 0.2
    assert abs(d.engine.e_ref - np.mean(e[10:])) < 5 * np.std(e[10:]) / np.sqrt(10)
    assert sum(h["copied"] for h in hist) > 0
