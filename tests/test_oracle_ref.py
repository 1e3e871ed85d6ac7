"""The oracle's spline restatement against the reference's own evaluator compiled in
place (oracle/build_ref.sh -> oracle/_ref/libref.so): identical VGH to rounding on
random tables and points.  Skipped where the reference sources were not available
to build it (or the library was built for another architecture)."""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "..", "oracle", "_ref", "libref.so")


def _ref():
    if not os.path.exists(LIB):
        pytest.skip("oracle/_ref not built (reference sources absent)")
    try:
        return C.CDLL(LIB)
    except OSError as e:
        pytest.skip(f"oracle/_ref not loadable here: {e}")


@pytest.mark.parametrize("grid,norb,npad", [((5, 5, 5), 1, 16), ((12, 10, 8), 20, 32), ((16, 16, 16), 48, 48)])
def test_spline_vgh_matches_reference_build(grid, norb, npad):
    L = _ref()
    dp = C.POINTER(C.c_double)
    rng = np.random.default_rng(sum(grid) + norb)
    coefs = rng.uniform(-0.5, 0.5, size=(grid[0] + 3, grid[1] + 3, grid[2] + 3, npad))
    gi = np.array(grid, np.int32)
    for _ in range(20):
        u = rng.uniform(0, 1, 3)
        v, g, h = np.zeros(norb), np.zeros(3 * norb), np.zeros(6 * norb)
        L.ref_spline_vgh(gi.ctypes.data_as(C.POINTER(C.c_int)), npad, coefs.ctypes.data_as(dp), norb,
                         u.ctypes.data_as(dp), v.ctypes.data_as(dp), g.ctypes.data_as(dp), h.ctypes.data_as(dp))
        vo, go, ho = orc.spline_vgh(coefs, norb, u)
        scale = max(1.0, np.abs(v).max())
        assert np.abs(v - vo).max() < 1e-12 * scale
        assert np.abs(g.reshape(3, norb) - go).max() < 1e-10 * max(1.0, np.abs(go).max())
        assert np.abs(h.reshape(6, norb) - ho).max() < 1e-9 * max(1.0, np.abs(ho).max())


def _ref_delayed():
    lib = os.path.join(HERE, "..", "oracle", "_ref", "libref_delayed.so")
    if not os.path.exists(lib):
        pytest.skip("oracle/_ref delayed-update engine not built")
    try:
        return C.CDLL(lib)
    except OSError as e:
        pytest.skip(f"oracle/_ref not loadable here: {e}")


@pytest.mark.parametrize("n,k", [(8, 1), (16, 4), (32, 8), (40, 16)])
def test_delayed_update_matches_reference_build(n, k):
    """The oracle's delayed-update engine (batched form: pseudo-accepted rejected moves)
    against the reference's CPU DelayedUpdate on the same move sequence."""
    L = _ref_delayed()
    dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
    rng = np.random.default_rng(n * 100 + k)
    M = rng.normal(size=(n, n)) + 3 * np.eye(n)
    d = orc.Det(n, k)
    d.recompute(M)
    a0 = np.ascontiguousarray(d.ainv())
    nm = 3 * n
    # electron-by-electron sweeps: a row changes at most once per delay window
    rows = np.tile(np.arange(n), 3).astype(np.int32)
    phis = rng.normal(size=(nm, n)) * 0.3 + M[rows]
    acc = (rng.random(nm) < 0.6).astype(np.int32)
    ratios = np.zeros(nm)
    out = np.zeros((n, n))
    L.ref_delayed_run(n, k, a0.ctypes.data_as(dp), nm, rows.ctypes.data_as(ip), phis.ctypes.data_as(dp),
                      acc.ctypes.data_as(ip), ratios.ctypes.data_as(dp), out.ctypes.data_as(dp))
    mine = []
    for m in range(nm):
        r = d.ratio(int(rows[m]), phis[m])
        mine.append(r)
        d.accept_reject(int(rows[m]), phis[m], r, bool(acc[m]))
    d.complete()
    np.testing.assert_allclose(mine, ratios, rtol=1e-10, atol=1e-12)
    assert np.abs(d.ainv() - out).max() < 1e-10 * np.abs(out).max()
