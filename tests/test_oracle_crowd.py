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


@pytest.mark.parametrize("delay,drift", [(1, True), (3, True), (3, False)])
def test_philox_sweep_state_matches_recompute(delay, drift):
    """Sweeps on the counter-based stream keep the tracked state equal to a recompute."""
    s = small_system(delay)
    R = make_walkers(s, 3, seed=4)
    c = orc.Crowd(s, 3, delay, 8)
    c.load_walkers(R)
    c.evaluate_log()
    na, nr, tr = c.vmc_sweeps_philox(seed=77, nsteps=3, tau=0.3, use_drift=drift, trace=True)
    assert na > 0 and nr > 0 and na + nr == 3 * s.n_elec * 3
    assert int(tr[..., 10].sum()) == na
    lp_tracked, _, _ = c.get_log()
    j2_tracked, _ = c.jastrow_state()
    lp_fresh, _ = c.evaluate_log()
    np.testing.assert_allclose(lp_tracked, lp_fresh, rtol=1e-10, atol=1e-10)
    j2_fresh, _ = c.jastrow_state()
    np.testing.assert_allclose(j2_tracked, j2_fresh, rtol=1e-9, atol=1e-11)


def test_philox_sweeps_deterministic_and_sweep_indexed():
    """The stream depends only on (seed, walker, electron, sweep): two sweeps in one call
    equal one sweep at sweep index 0 followed by one at sweep index 1."""
    s = small_system(3)
    R = make_walkers(s, 3, seed=5)
    a, b = orc.Crowd(s, 3, 3, 8), orc.Crowd(s, 3, 3, 8)
    for c in (a, b):
        c.load_walkers(R)
        c.evaluate_log()
    _, _, ta = a.vmc_sweeps_philox(seed=9, nsteps=2, tau=0.3, trace=True)
    _, _, t0 = b.vmc_sweeps_philox(seed=9, nsteps=1, tau=0.3, sweep0=0, trace=True)
    _, _, t1 = b.vmc_sweeps_philox(seed=9, nsteps=1, tau=0.3, sweep0=1, trace=True)
    np.testing.assert_array_equal(ta, np.concatenate([t0, t1]))
    np.testing.assert_array_equal(a.positions(), b.positions())


def test_replay_reproduces_trajectory():
    """Replaying a recorded trajectory on a fresh crowd gives the same ratios, gradients
    and final state as the run that recorded it."""
    s = small_system(3)
    R = make_walkers(s, 3, seed=6)
    a, b = orc.Crowd(s, 3, 3, 8), orc.Crowd(s, 3, 3, 8)
    for c in (a, b):
        c.load_walkers(R)
        c.evaluate_log()
    _, _, ta = a.vmc_sweeps_philox(seed=21, nsteps=2, tau=0.3, trace=True)
    tb = b.replay(ta)
    np.testing.assert_allclose(tb, ta, rtol=1e-12, atol=1e-12)
    np.testing.assert_array_equal(a.positions(), b.positions())
    np.testing.assert_allclose(a.get_log()[0], b.get_log()[0], rtol=1e-13)


def test_philox_proposals_are_unit_gaussians():
    """Proposal displacements without drift are sqrt(tau) times unit Gaussians: first
    moves of many walkers have mean 0 and variance tau per axis."""
    spec = scaled_spec("c0_32e", n_up=2, n_dn=2, grid=8, walkers=4000, delay=1, precision=8)
    s = make_system(spec, seed=3)
    nw = 4000
    R = make_walkers(s, nw, seed=8)
    c = orc.Crowd(s, nw, 1, 8)
    c.load_walkers(R)
    c.evaluate_log()
    tau = 0.3
    _, _, tr = c.vmc_sweeps_philox(seed=5, nsteps=1, tau=tau, use_drift=False, trace=True)
    d = tr[0, 0, :, 0:3] - R[:, 0, :]
    d -= s.lattice * np.round(d / s.lattice)
    z = d.ravel() / np.sqrt(tau)
    assert abs(z.mean()) < 4 / np.sqrt(z.size)
    assert abs(z.var() - 1) < 5 * np.sqrt(2 / z.size)


@pytest.mark.parametrize("delay", [1, 3])
def test_replay_philox_reproduces_own_chain(delay):
    """Following its own recorded chain, the step-by-step check forms the same proposals
    and the same decisions (every decision away from a tie)."""
    s = small_system(delay)
    R = make_walkers(s, 3, seed=9)
    a, b = orc.Crowd(s, 3, delay, 8), orc.Crowd(s, 3, delay, 8)
    for c in (a, b):
        c.load_walkers(R)
        c.evaluate_log()
    _, _, ta = a.vmc_sweeps_philox(seed=31, nsteps=2, tau=0.3, trace=True)
    tb, margin = b.replay_philox(ta, seed=31, tau=0.3)
    np.testing.assert_allclose(tb[..., 0:3], ta[..., 0:3], rtol=0, atol=1e-12)
    np.testing.assert_allclose(tb[..., 3:10], ta[..., 3:10], rtol=1e-12, atol=1e-12)
    np.testing.assert_array_equal(tb[..., 10], ta[..., 10])
    assert np.all(np.abs(margin) > 0)
    # a decision that differs from the recorded one is caught
    tc = ta.copy()
    tc[0, 2, 1, 10] = 1 - tc[0, 2, 1, 10]
    d = orc.Crowd(s, 3, delay, 8)
    d.load_walkers(R)
    d.evaluate_log()
    td, _ = d.replay_philox(tc, seed=31, tau=0.3)
    assert td[0, 2, 1, 10] != tc[0, 2, 1, 10]


def test_virtual_move_ratio_equals_real_move():
    """The ratio of a virtual move equals mw_calcRatioGrad's ratio of the same move, and a
    virtual move onto the electron's own position has ratio 1."""
    s = small_system(3)
    R = make_walkers(s, 3, seed=12)
    c = orc.Crowd(s, 3, 3, 8)
    c.load_walkers(R)
    c.evaluate_log()
    c.vmc_sweeps_philox(seed=5, nsteps=1, tau=0.3)
    Rn = c.positions()
    iat = 6
    rng = np.random.default_rng(1)
    target = Rn[:, iat, :] + rng.normal(size=(3, 3)) * 0.4
    vr = c.evaluate_ratios(np.arange(3), np.full(3, iat), target)
    same = c.evaluate_ratios(np.arange(3), np.full(3, iat), Rn[:, iat, :])
    np.testing.assert_allclose(same, 1.0, rtol=1e-10)
    c.eval_grad(iat)
    c.make_move(iat, target - Rn[:, iat, :])
    r, _ = c.ratio_grad(iat)
    np.testing.assert_allclose(vr, r, rtol=1e-10)


def test_quadrature_moves_geometry():
    from qmcpack_gb300.nlpp import icosahedron, quadrature_moves
    u = icosahedron()
    assert u.shape == (12, 3)
    np.testing.assert_allclose(np.linalg.norm(u, axis=1), 1.0)
    np.testing.assert_allclose(u.sum(axis=0), 0.0, atol=1e-12)
    s = small_system(1)
    R = make_walkers(s, 2, seed=3)
    w, e, pos, ion = quadrature_moves(s, R, 3.0, np.random.default_rng(0))
    assert len(w) % 12 == 0 and len(w) > 0
    # every point lies on the sphere through its electron around its ion
    L = s.lattice
    d_e = R[w, e] - s.ion_pos[ion]
    d_e -= L * np.round(d_e / L)
    d_p = pos - s.ion_pos[ion]
    d_p -= L * np.round(d_p / L)
    np.testing.assert_allclose(np.linalg.norm(d_p, axis=1), np.linalg.norm(d_e, axis=1), rtol=1e-12)
