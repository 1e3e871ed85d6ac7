"""CPU restatement of the learned MH proposal's network, features and training
backward pass (test infrastructure only: tests/ and the bench's CPU legs use it).

The proposal has no counterpart in the reference; this file restates the
definitions the CUDA kernels implement so their outputs and gradients can be
checked: features (8 nearest electrons and ions, drift), the 51-128-128-128-6 tanh
MLP with BF16 weights/activations and FP32 accumulation, and the backward pass
(FP32 master weights, BF16 activations) for a given output gradient.
"""
from __future__ import annotations

import numpy as np

NIN, IN, H, OUT, NOUT = 51, 64, 128, 16, 6
LSCALE = 2.0
# flat FP32 parameter layout
W1, B1 = 0, H * IN
W2 = B1 + H
B2 = W2 + H * H
W3 = B2 + H
B3 = W3 + H * H
W4 = B3 + H
B4 = W4 + OUT * H
NPARAM = B4 + OUT


def bf16(a):
    """Round to BF16 (nearest even) and return float64."""
    a32 = np.ascontiguousarray(a, dtype=np.float32)
    u = a32.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[W1:B1].reshape(H, IN), p[B1:W2], p[W2:B2].reshape(H, H), p[B2:W3],
            p[W3:B3].reshape(H, H), p[B3:W4], p[W4:B4].reshape(OUT, H), p[B4:NPARAM])


def forward(params, x, emulate_bf16: bool = True):
    """x [rows][64] -> (out [rows][6], hidden [3][rows][128])."""
    w1, b1, w2, b2, w3, b3, w4, b4 = unpack(params)
    r = bf16 if emulate_bf16 else (lambda a: np.asarray(a, np.float64))
    h = r(x)
    hs = []
    for w, b in ((w1, b1), (w2, b2), (w3, b3)):
        h = r(np.tanh(h @ r(w).T + b))
        hs.append(h)
    out = h @ r(w4).T + b4
    return out[:, :NOUT], np.stack(hs)


def backward(params, x, hidden, dout, emulate_bf16: bool = True):
    """Gradient of sum(dout * out) w.r.t. the flat parameters, given the forward's
    hidden activations (as the GPU does: FP32 master weights in the delta products)."""
    w1, b1, w2, b2, w3, b3, w4, b4 = unpack(params)
    xb = bf16(x) if emulate_bf16 else np.asarray(x, np.float64)
    h1, h2, h3 = hidden
    g = np.zeros(NPARAM)
    d4 = np.zeros((x.shape[0], OUT))
    d4[:, :NOUT] = dout
    g[W4:B4] = (d4.T @ h3).reshape(-1)
    g[B4:NPARAM] = d4.sum(0)
    d3 = (d4 @ w4) * (1 - h3 ** 2)
    g[W3:B3] = (d3.T @ h2).reshape(-1)
    g[B3:W4] = d3.sum(0)
    d2 = (d3 @ w3) * (1 - h2 ** 2)
    g[W2:B2] = (d2.T @ h1).reshape(-1)
    g[B2:W3] = d2.sum(0)
    d1 = (d2 @ w2) * (1 - h1 ** 2)
    gw1 = d1.T @ xb
    gw1[:, NIN:] = 0
    g[W1:B1] = gw1.reshape(-1)
    g[B1:W2] = d1.sum(0)
    return g


def unr_drift(tau, g):
    g = np.asarray(g, np.float64)
    vsq = float(g @ g)
    sc = tau if vsq < np.finfo(np.float64).eps else (-1.0 + np.sqrt(1.0 + 2.0 * tau * vsq)) / vsq
    return g * sc


def features(lattice, R, ions, iat, pos, grad, tau):
    """Features of electron iat at position pos of one walker (R: [ne][3] other electrons'
    positions; iat's own entry is skipped)."""
    L = np.asarray(lattice, np.float64)

    def disp(q):
        d = q - pos
        return d - L * np.rint(d / L)

    de = np.array([disp(R[j]) for j in range(len(R)) if j != iat])
    order = np.argsort((de ** 2).sum(1), kind="stable")[:8]
    di = np.array([disp(q) for q in ions])
    oi = np.argsort((di ** 2).sum(1), kind="stable")[:8]
    x = np.zeros(IN)
    x[:3 * len(order)] = (de[order] / LSCALE).reshape(-1)
    x[24:24 + 3 * len(oi)] = (di[oi] / LSCALE).reshape(-1)
    x[48:51] = unr_drift(tau, grad) / np.sqrt(tau)
    return x
