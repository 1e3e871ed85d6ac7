"""Self-consistency of the oracle's batched crowd (FP64).

After particle-by-particle sweeps with rank-1 and delayed updates the tracked
state must equal a from-scratch recompute (the reference's debug check
checkLogAndGL, src/QMCDrivers/QMCDriverNew.cpp:492-560), and the drift
gradient must be the gradient of log|psi|.
"""
import numpy as np
import pytest

from oracle import oracle as orc
from qmcpack_gb300.system import make_system, make_walkers, scaled_spec


def small_system(delay=1, n=8, grid=12, prec=8):
    spec = scaled_spec("c0_32e", n_up=n, n_dn=n, grid=grid, walkers=3, delay=delay, precision=prec)
    return make_system(spec, seed=11)


@pytest.mark.parametrize("delay", [1, 3])
def test_sweep_state_matches_recompute(delay):
    s = small_system(delay)
    R = make_walkers(s, 3, seed=1)
    c = orc.Crowd(s, 3, delay, 8)
    c.load_walkers(R)
    c.evaluate_log()
    rng = orc.Rng(17)
    na, nr, _ = c.vmc_sweeps(rng, 3, 0.3, True)
    assert na > 0 and nr >= 0
    lp_tracked, sg_tracked, _ = c.get_log()
    A0 = c.ainv(0)
    j2_tracked, j1_tracked = c.jastrow_state()
    lp_fresh, sg_fresh = c.evaluate_log()
    np.testing.assert_allclose(lp_tracked, lp_fresh, rtol=1e-10, atol=1e-10)
    assert (sg_tracked == sg_fresh).all()
    np.testing.assert_allclose(A0, c.ainv(0), rtol=1e-8, atol=1e-9)
    j2_fresh, j1_fresh = c.jastrow_state()
    np.testing.assert_allclose(j2_tracked, j2_fresh, rtol=1e-9, atol=1e-11)
    np.testing.assert_allclose(j1_tracked, j1_fresh, rtol=1e-9, atol=1e-11)


def test_grad_is_grad_log_psi():
    s = small_system(1)
    R = make_walkers(s, 3, seed=2)
    c = orc.Crowd(s, 3, 1, 8)
    c.load_walkers(R)
    lp0, _ = c.evaluate_log()
    iat = 5
    g = c.eval_grad(iat)
    h = 1e-5
    num = np.zeros_like(g)
    for d in range(3):
        Rp = R.copy()
        Rp[:, iat, d] += h
        Rm = R.copy()
        Rm[:, iat, d] -= h
        c.load_walkers(Rp)
        lpp, _ = c.evaluate_log()
        c.load_walkers(Rm)
        lpm, _ = c.evaluate_log()
        num[:, d] = (lpp - lpm) / (2 * h)
    np.testing.assert_allclose(g, num, rtol=1e-5, atol=1e-6)


def test_ratio_is_psi_ratio():
    s = small_system(3)
    R = make_walkers(s, 3, seed=4)
    c = orc.Crowd(s, 3, 3, 8)
    c.load_walkers(R)
    lp0, sg0 = c.evaluate_log()
    iat = 9
    c.eval_grad(iat)
    d = np.random.default_rng(0).normal(size=(3, 3)) * 0.3
    c.make_move(iat, d)
    ratio, _ = c.ratio_grad(iat)
    R2 = R.copy()
    R2[:, iat] += d
    c2 = orc.Crowd(s, 3, 3, 8)
    c2.load_walkers(R2)
    lp1, sg1 = c2.evaluate_log()
    np.testing.assert_allclose(np.abs(ratio), np.exp(lp1 - lp0), rtol=1e-9)
    assert (np.sign(ratio) == sg0 * sg1).all()


def test_fp32_crowd_tracks_fp64():
    s = small_system(3, prec=4)
    R = make_walkers(s, 3, seed=6)
    c8 = orc.Crowd(s, 3, 3, 8)
    c4 = orc.Crowd(s, 3, 3, 4)
    for c in (c8, c4):
        c.load_walkers(R)
        c.evaluate_log()
    for iat in range(4):
        g8 = c8.eval_grad(iat)
        g4 = c4.eval_grad(iat)
        np.testing.assert_allclose(g4, g8, rtol=2e-3, atol=2e-3)
        d = np.full((3, 3), 0.1)
        c8.make_move(iat, d)
        c4.make_move(iat, d)
        r8, _ = c8.ratio_grad(iat)
        r4, _ = c4.ratio_grad(iat)
        np.testing.assert_allclose(r4, r8, rtol=1e-3)
        c8.accept_reject(iat, [1, 0, 1])
        c4.accept_reject(iat, [1, 0, 1])
