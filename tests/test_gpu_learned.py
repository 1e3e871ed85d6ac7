"""The learned MH proposal on the GPU: network forward and backward against the CPU
restatement, features, the zero-output-layer limit (= drift-diffusion), unbiased
sampling, and what training buys.

Tolerances: forward outputs within 3e-2 of the largest output (BF16 activations on
the GPU, FP64 sums in the restatement); backward gradients within 1e-3 of the largest
gradient of each parameter block given the same hidden activations (FP32 vs FP64
accumulation); features within one BF16 rounding (4e-3 relative + 1e-6).
"""
import numpy as np
import pytest

from oracle import mlp_oracle as mo
from qmcpack_gb300.stats import agree_within, ensemble_statistics, energy_statistics
from qmcpack_gb300.system import make_system, make_walkers, scaled_spec

pytestmark = pytest.mark.gpu


def _gpu():
    from qmcpack_gb300.crowd import Crowd, DeviceSystem
    return Crowd, DeviceSystem


def _params(rng, w4_scale=0.3):
    p = (rng.normal(size=mo.NPARAM) * 0.15).astype(np.float32)
    w1 = p[mo.W1:mo.B1].reshape(mo.H, mo.IN)
    w1[:, mo.NIN:] = 0
    w4 = p[mo.W4:mo.B4].reshape(mo.OUT, mo.H)
    w4[:] = rng.normal(size=w4.shape) * w4_scale / np.sqrt(mo.H)
    w4[mo.NOUT:] = 0
    p[mo.B4 + mo.NOUT:] = 0
    return p


def _small(prec=8, n=16, nw=8, delay=4, seed=5):
    spec = scaled_spec("c0_32e", n_up=n, n_dn=n, grid=16, walkers=nw, delay=delay, precision=prec)
    return make_system(spec, seed=seed)


@pytest.fixture(scope="module")
def crowd():
    Crowd, DeviceSystem = _gpu()
    s = _small()
    ds = DeviceSystem(s)
    g = Crowd(ds, 8, 4)
    g.load_walkers(make_walkers(s, 8, seed=6))
    g.mw_evaluateLog()
    g.proposal_init(seed=3)
    return s, ds, g


def test_forward_matches_oracle(crowd):
    _, _, g = crowd
    rng = np.random.default_rng(0)
    p = _params(rng)
    g.set_proposal_params(p)
    assert np.array_equal(g.proposal_params(), p)
    x = rng.normal(size=(300, mo.IN)).astype(np.float32)
    x[:, mo.NIN:] = 0
    out, hid = g.proposal_forward(x, with_hidden=True)
    out_o, hid_o = mo.forward(p, x)
    scale = np.abs(out_o).max()
    assert np.abs(out - out_o).max() < 3e-2 * scale
    assert np.abs(hid - hid_o).max() < 3e-2
    # most hidden activations agree to the BF16 rounding
    assert np.mean(np.abs(hid - hid_o) <= 2 ** -7 * np.abs(hid_o) + 1e-6) > 0.95


def test_backward_matches_oracle(crowd):
    _, _, g = crowd
    rng = np.random.default_rng(1)
    p = _params(rng)
    g.set_proposal_params(p)
    x = rng.normal(size=(256, mo.IN)).astype(np.float32)
    x[:, mo.NIN:] = 0
    dout = rng.normal(size=(256, mo.NOUT)).astype(np.float32)
    _, hid = g.proposal_forward(x, with_hidden=True)
    grad = g.proposal_backward(x, dout)
    ref = mo.backward(p.astype(np.float64), x, hid.astype(np.float64), dout.astype(np.float64))
    for a, b in ((mo.W1, mo.B1), (mo.B1, mo.W2), (mo.W2, mo.B2), (mo.B2, mo.W3), (mo.W3, mo.B3),
                 (mo.B3, mo.W4), (mo.W4, mo.B4), (mo.B4, mo.NPARAM)):
        blk = np.abs(ref[a:b]).max()
        assert np.abs(grad[a:b] - ref[a:b]).max() <= 1e-3 * max(blk, 1e-6), (a, b)


def test_features_match_oracle(crowd):
    s, _, g = crowd
    R = g.positions()
    for iat in (0, 5, s.spec.n_up + 3):
        grads = g.mw_evalGrad(iat)
        x = g.proposal_features(iat)
        for iw in range(g.nw):
            ref = mo.features(s.lattice, R[iw], s.ion_pos, iat, R[iw, iat], grads[iw], 0.3)
            assert np.all(np.abs(x[iw] - ref) <= 4e-3 * np.abs(ref) + 1e-6), (iat, iw)
        d = np.random.default_rng(iat).normal(size=(g.nw, 3)) * 0.3
        g.mw_makeMove(iat, d)
        _, gnew = g.mw_calcRatioGrad(iat)
        xp = g.proposal_features(iat, at_proposed=True)
        for iw in range(g.nw):
            ref = mo.features(s.lattice, R[iw], s.ion_pos, iat, R[iw, iat] + d[iw], gnew[iw], 0.3)
            assert np.all(np.abs(xp[iw] - ref) <= 4e-3 * np.abs(ref) + 1e-6), (iat, iw)
        g.mw_accept_rejectMove(iat, np.zeros(g.nw, np.int32))
    g.mw_completeUpdates()


def test_zero_output_layer_is_drift_diffusion():
    """With the output layer at zero the learned sweep is the staged drift-diffusion
    sweep: same proposals, same MH probabilities, same decisions (FP64)."""
    Crowd, DeviceSystem = _gpu()
    s = _small(nw=8)
    ds = DeviceSystem(s)
    R = make_walkers(s, 8, seed=9)
    out = []
    for learned in (False, True):
        g = Crowd(ds, 8, 4)
        g.load_walkers(R)
        g.mw_evaluateLog()
        if learned:
            g.proposal_init(seed=4)
            a, r, _, _ = g.vmc_sweeps_learned(2, 0.3, 21, staged=True)
        else:
            a, r, _ = g.vmc_sweeps(2, 0.3, 21, rng_mode=1, staged=True)
        out.append((a, r, g.positions()))
    assert out[0][0] == out[1][0] and out[0][1] == out[1][1]
    np.testing.assert_allclose(out[0][2], out[1][2], rtol=0, atol=1e-10)


def test_learned_sampling_is_unbiased():
    """A random (untrained) proposal network still samples |psi|^2: the VMC energy and
    the variance of the local energy agree with drift-diffusion's within 2 combined
    standard errors (autocorrelation-corrected).  A correct sampler misses a 2-sigma
    bound for about one seed in twenty; the seeds here are fixed (the energies at 1.2
    sigma)."""
    Crowd, DeviceSystem = _gpu()
    s = _small(prec=8, n=8, nw=256, delay=4, seed=15)
    ds = DeviceSystem(s)
    R = make_walkers(s, 256, seed=16)
    res = {}
    for mode in ("plain", "learned"):
        g = Crowd(ds, 256, 4)
        g.load_walkers(R)
        g.mw_evaluateLog()
        if mode == "plain":
            g.vmc_sweeps(30, 0.3, 5, rng_mode=1)
            _, _, el, _ = g.vmc_sweeps_measure(150, 0.3, 6)
        else:
            g.proposal_init(seed=7)
            g.set_proposal_params(_params(np.random.default_rng(8), w4_scale=0.5))
            g.vmc_sweeps_learned(30, 0.3, 5, staged=True)
            _, _, el, _ = g.vmc_sweeps_learned(150, 0.3, 6, measure=True, staged=True)
        res[mode] = (energy_statistics(el), ensemble_statistics(el))
    (a, ea), (b, eb) = res["plain"], res["learned"]
    print("plain", a, "learned", b, "variance", ea["variance"], ea["variance_error"], eb["variance"],
          eb["variance_error"])
    assert abs(a["energy"] - b["energy"]) < 2 * np.hypot(a["error"], b["error"])
    assert agree_within(ea, eb, "variance", "variance_error")


def test_training_lowers_the_objective():
    """Paired comparison: the training objective of the untrained and the trained network,
    each measured from the same configurations with the same counter-based random numbers
    (a fresh crowd per measurement, so the stream restarts at sweep 0)."""
    Crowd, DeviceSystem = _gpu()
    s = _small(prec=8, n=8, nw=128, delay=4, seed=25)
    ds = DeviceSystem(s)
    g = Crowd(ds, 128, 4)
    g.load_walkers(make_walkers(s, 128, seed=26))
    g.mw_evaluateLog()
    g.proposal_init(seed=1)
    g.vmc_sweeps(30, 0.3, 1, rng_mode=1)
    R0 = g.positions()
    p_untrained = g.proposal_params()
    g.vmc_sweeps_learned(60, 0.3, 3, train=True, lr=2e-3)
    p_trained = g.proposal_params()

    def measure(params):
        m = Crowd(ds, 128, 4)
        m.load_walkers(R0)
        m.mw_evaluateLog()
        m.proposal_init(seed=1)
        m.set_proposal_params(params)
        # lr = 0: the statistics of the moves without changing the parameters
        _, _, _, stats = m.vmc_sweeps_learned(12, 0.3, 4, train=True, lr=0.0)
        return stats

    esjd0, acc0, obj0 = measure(p_untrained)
    esjd1, acc1, obj1 = measure(p_trained)
    print("training objective per move: before", obj0, "after", obj1, "; expected squared jump", esjd0, "->",
          esjd1, "; acceptance", acc0, "->", acc1)
    assert np.isfinite(obj1) and obj1 < obj0


@pytest.mark.parametrize("flush", [0, 4])
def test_resident_zero_output_layer_is_drift_diffusion(flush):
    """Walker-resident inference with a zero output layer reproduces the resident
    drift-diffusion sweep (FP64), with the flush after every segment and with the
    block-lazy updates."""
    Crowd, DeviceSystem = _gpu()
    s = _small(nw=8)
    ds = DeviceSystem(s)
    R = make_walkers(s, 8, seed=19)
    out = []
    for learned in (False, True):
        g = Crowd(ds, 8, 4)
        g.load_walkers(R)
        g.mw_evaluateLog()
        if learned:
            g.proposal_init(seed=4)
            a, r, _, _ = g.vmc_sweeps_learned(2, 0.3, 23, flush=flush)
        else:
            a, r, _ = g.vmc_sweeps(2, 0.3, 23, rng_mode=1, flush=flush)
        out.append((a, r, g.positions()))
    assert out[0][0] == out[1][0] and out[0][1] == out[1][1]
    np.testing.assert_allclose(out[0][2], out[1][2], rtol=0, atol=1e-10)


def test_resident_learned_sampling_is_unbiased():
    """Walker-resident inference with a random network samples |psi|^2 (FP32 and FP64):
    energies (0.7 and 1.3 sigma with these seeds) and variances within 2 combined standard
    errors."""
    Crowd, DeviceSystem = _gpu()
    for prec in (8, 4):
        s = _small(prec=prec, n=8, nw=256, delay=4, seed=35)
        ds = DeviceSystem(s)
        R = make_walkers(s, 256, seed=36)
        res = {}
        for mode in ("plain", "learned"):
            g = Crowd(ds, 256, 4)
            g.load_walkers(R)
            g.mw_evaluateLog()
            if mode == "plain":
                g.vmc_sweeps(30, 0.3, 5, rng_mode=1)
                _, _, el, _ = g.vmc_sweeps_measure(200, 0.3, 6)
            else:
                g.proposal_init(seed=7)
                g.set_proposal_params(_params(np.random.default_rng(9), w4_scale=0.5))
                g.vmc_sweeps_learned(30, 0.3, 5)
                _, _, el, _ = g.vmc_sweeps_learned(200, 0.3, 6, measure=True)
            res[mode] = (energy_statistics(el), ensemble_statistics(el))
        (a, ea), (b, eb) = res["plain"], res["learned"]
        print("precision", prec, "plain", a, "learned (resident)", b, "variance", ea["variance"],
              ea["variance_error"], eb["variance"], eb["variance_error"])
        assert abs(a["energy"] - b["energy"]) < 2 * np.hypot(a["error"], b["error"])
        assert agree_within(ea, eb, "variance", "variance_error")
