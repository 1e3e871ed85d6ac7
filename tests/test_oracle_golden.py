"""Pin the CPU oracle against the reference's own golden vectors.

Every number compared here is copied (by tests/golden/extract_reference_golden.py)
from QMCPACK's unit tests: src/spline2/tests/test_multi_spline.cpp,
src/QMCWaveFunctions/tests/test_J2_bspline.cpp,
src/Particle/tests/test_distance_table.cpp and
src/QMCWaveFunctions/tests/test_DiracDeterminantBatched.cpp.

Tolerance: the reference checks with Catch's Approx (relative 100 * FLT_EPSILON);
the same relative tolerance is used here, plus an absolute 1e-9 for golden values
that are zero to print precision (|x| < 1e-6).
"""
import numpy as np
import pytest

from oracle import oracle as orc

REL = 100 * np.finfo(np.float32).eps


def approx(a, b, rel=REL, abs_small=1e-9):
    if abs(b) < 1e-6:
        return abs(a - b) <= abs_small
    return abs(a - b) <= rel * abs(b)


def periodic_coefs(data):
    """Interpolating periodic cubic B-spline coefficients of a 3D grid function.

    Restates einspline's periodic solve (src/einspline/bspline_create.c:991-1036):
    (c[m-1] + 4 c[m] + c[m+1]) / 6 = data[m] per axis, solved here exactly in
    Fourier space (the system is circulant), then ghost-wrapped.
    """
    from qmcpack_gb300.system import ghost_wrap
    c = np.fft.fftn(data)
    for ax, m in enumerate(data.shape):
        k = np.arange(m)
        lam = (4.0 + 2.0 * np.cos(2 * np.pi * k / m)) / 6.0
        shape = [1, 1, 1]
        shape[ax] = m
        c = c / lam.reshape(shape)
    c = np.real(np.fft.ifftn(c))
    return ghost_wrap(c[..., None])


def test_prefactors(golden):
    g = golden["prefactors"]
    names = {"a": 0, "da": 1, "d2a": 2}
    # first tx: only a[0..3] checked; second tx: a, da, d2a
    res0 = orc.prefactors(g["tx"][0])
    res1 = orc.prefactors(g["tx"][1])
    chk = g["checks"]
    for name, val in chk[:4]:
        arr, idx = name.split("[")
        assert approx(res0[names[arr]][int(idx[0])], val)
    for name, val in chk[4:]:
        arr, idx = name.split("[")
        assert approx(res1[names[arr]][int(idx[0])], val), (name, val)


def test_spline_vgh(golden):
    g = golden["spline_vgh"]
    n = g["grid"]
    x = np.arange(n) / n
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    data = np.sin(2 * np.pi * X) + np.sin(3 * 2 * np.pi * Y) + np.sin(4 * 2 * np.pi * Z)
    coefs = periodic_coefs(data)
    v0, g0, h0 = orc.spline_vgh(coefs, 1, g["pos0"])
    v1, g1, h1 = orc.spline_vgh(coefs, 1, g["pos1"])
    chk = g["checks"]
    # order in the reference: v(pos0); dv(pos0) x3; then v, v (pos1); dv x3; hess x6; v; dv x3; lap; ...
    assert approx(v0[0], chk[0][1])
    for d in range(3):
        assert approx(g0[d, 0], chk[1 + d][1])
    assert approx(v1[0], chk[4][1])
    for d in range(3):
        assert approx(g1[d, 0], chk[6 + d][1])
    for d in range(6):
        assert approx(h1[d, 0], chk[9 + d][1], abs_small=1e-8), (d, h1[d, 0], chk[9 + d])
    lap = [c for c in chk if c[0] == "lap[0][0]"][0][1]
    assert approx(h1[0, 0] + h1[3, 0] + h1[5, 0], lap)


def test_j2_functor_table(golden):
    g = golden["j2_functor"]
    tab = np.array(g["table_r_u_du_ddu"])
    u, du, d2u = orc.functor_eval(g["params"], g["rcut"], g["cusp_ud"], tab[:, 0])
    for i in range(len(tab)):
        assert approx(u[i], tab[i, 1]), i
        assert approx(du[i], tab[i, 2]), i
        assert approx(d2u[i], tab[i, 3]), i


def test_j2_log_ratio_ke(golden):
    g = golden["j2_functor"]
    f = lambda r: orc.functor_eval(g["params"], g["rcut"], g["cusp_ud"], r)
    e0, e1 = np.array(g["elec"])
    r01 = np.linalg.norm(e0 - e1)
    u, du, d2u = f(r01)
    assert approx(-u[0], g["logpsi_r1"])
    # G_i = sum_j (du/r) (R_j - R_i), L_i = -(d2u + 2 du/r)
    G0 = du[0] / r01 * (e1 - e0)
    G1 = du[0] / r01 * (e0 - e1)
    L = -(d2u[0] + 2 * du[0] / r01)
    ke = -0.5 * (G0 @ G0 + G1 @ G1 + 2 * L)
    assert approx(ke, g["KE"])
    newpos = np.array(g["newpos"])
    un, _, _ = f(np.linalg.norm(newpos - e1))
    assert approx(np.exp(u[0] - un[0]), g["ratio_0"])
    un1, _, _ = f(np.linalg.norm(newpos - e0))
    assert approx(np.exp(u[0] - un1[0]), g["ratio_1"])
    assert approx(-un1[0], g["log_after_accept_1"])


def test_distance_pbc(golden):
    g = golden["distance_pbc"]
    R = np.array(g["elec"])
    R[0] += g["shift0"]
    R[0] += g["disp"]          # electron 0 accepted, electron 1 rejected
    lat = [g["cell"]] * 3
    dist, dr = orc.distance_row(lat, R, R[1])
    chk = g["checks"]
    assert approx(dist[0], chk[0][1])
    for d in range(3):
        assert approx(dr[d, 0], chk[1 + d][1])


def test_det_sm1_fakespo(golden):
    g = golden["det_fakespo"]
    a = np.array(g["a"])
    v = np.array(g["v"])
    det = orc.Det(3, 1)
    log0, sign0 = det.recompute(a.T)            # psiM[e][o] = a[o][e]
    np.testing.assert_allclose(det.ainv(), np.array(g["b_initial"]), rtol=REL)
    r0 = det.ratio(0, v)
    assert approx(r0, g["det_ratio_0"])
    det.accept_reject(0, v, r0, True)
    np.testing.assert_allclose(det.ainv(), np.array(g["b_after_accept0"]), rtol=REL)
    r1 = det.ratio(1, a[1])
    assert approx(r1, g["ratio_1"])
    det.accept_reject(1, a[1], r1, True)
    log = log0 + np.log(abs(r0)) + np.log(abs(r1))
    assert approx(log, g["log_after_accept_1"])


@pytest.mark.parametrize("k", [2, 3])
def test_det_delayed_fakespo(golden, k):
    """test_DiracDeterminantBatched.cpp:274-470: delayed ratios equal fresh-inverse ratios."""
    g = golden["det_fakespo"]
    a2 = np.array(g["a2"])
    v2 = np.array(g["v2"])
    det = orc.Det(4, k)
    det.recompute(a2.T)
    cur = a2.copy()
    for row in range(3):
        r = det.ratio(row, v2[row])
        nxt = cur.copy()
        nxt[:, row] = v2[row]
        assert approx(r, np.linalg.det(nxt) / np.linalg.det(cur), rel=1e-12)
        det.accept_reject(row, v2[row], r, True)
        if row == 0:
            det.complete()
            np.testing.assert_allclose(det.ainv(), np.linalg.inv(nxt), rtol=1e-12, atol=1e-14)
        cur = nxt
    det.complete()
    np.testing.assert_allclose(det.ainv(), np.linalg.inv(cur), rtol=1e-12, atol=1e-14)


def test_det_delayed_pseudo_accept():
    """Rejected moves inside a delay window (pseudo accept) leave the inverse exact."""
    rng = np.random.default_rng(3)
    n, k = 12, 5
    M = rng.normal(size=(n, n)) + 3 * np.eye(n)
    det = orc.Det(n, k)
    det.recompute(M)
    cur = M.copy()
    for step in range(17):
        row = step % n
        phi = cur[row] + 0.3 * rng.normal(size=n)
        r = det.ratio(row, phi)
        nxt = cur.copy()
        nxt[row] = phi
        assert abs(r - np.linalg.det(nxt) / np.linalg.det(cur)) < 1e-10 * max(1, abs(r))
        acc = bool(rng.integers(0, 2))
        det.accept_reject(row, phi, r, acc)
        if acc:
            cur = nxt
    det.complete()
    np.testing.assert_allclose(det.ainv(), np.linalg.inv(cur).T, rtol=1e-10, atol=1e-12)


def test_inverse_logdet():
    rng = np.random.default_rng(5)
    for n in (1, 3, 17, 64):
        A = rng.normal(size=(n, n))
        inv, la, sg = orc.invert(A)
        np.testing.assert_allclose(inv, np.linalg.inv(A), rtol=1e-9, atol=1e-12)
        s, l = np.linalg.slogdet(A)
        assert abs(la - l) < 1e-10 * max(1, abs(l)) and sg == int(s)
