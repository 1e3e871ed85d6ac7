"""The proposal network's CPU restatement: backward pass against finite differences
(FP64, no BF16 rounding), and BF16 rounding of the emulation."""
import numpy as np

from oracle import mlp_oracle as mo


def _params(rng, w4_scale=0.3):
    p = rng.normal(size=mo.NPARAM) * 0.2
    w1 = p[mo.W1:mo.B1].reshape(mo.H, mo.IN)
    w1[:, mo.NIN:] = 0
    w4 = p[mo.W4:mo.B4].reshape(mo.OUT, mo.H)
    w4[mo.NOUT:] = 0
    w4 *= w4_scale / 0.2
    p[mo.B4 + mo.NOUT:] = 0
    return p


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = _params(rng)
    x = rng.normal(size=(5, mo.IN))
    x[:, mo.NIN:] = 0
    dout = rng.normal(size=(5, mo.NOUT))
    out, hid = mo.forward(p, x, emulate_bf16=False)
    g = mo.backward(p, x, hid, dout, emulate_bf16=False)
    idx = np.concatenate([rng.integers(mo.W1, mo.B1, 20), rng.integers(mo.W2, mo.B2, 20),
                          rng.integers(mo.W3, mo.B3, 20), np.arange(mo.W4, mo.W4 + 10), [mo.B1, mo.B2, mo.B4]])
    h = 1e-6
    for i in idx:
        if (i < mo.B1 and (i - mo.W1) % mo.IN >= mo.NIN):
            continue
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = ((mo.forward(pp, x, False)[0] - mo.forward(pm, x, False)[0]) * dout).sum() / (2 * h)
        assert abs(fd - g[i]) < 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_bf16_rounding():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -3.14159, 0.0])
    r = mo.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -7 and r[4] == 0.0
    assert abs(r[3] + 3.14159) < 2 ** -7 * 4
