"""The plane-wave orbital restatement (oracle/orbitals_oracle.py), pinned on the CPU:
  * its periodic B-spline solve against the reference's own set_multi_UBspline_3d_d compiled
    in place (oracle/build_ref.sh -> oracle/_ref/libref_bspline.so) on random data: equal to
    rounding (skipped where the reference sources were not there to build it);
  * the interpolation property: the spline's values at the grid points are the data, and the
    ghost coefficients repeat the periodic ones;
  * the backward transform of a single plane wave is exp(+2 pi i G.r / n), and unpack drops the
    Miller indices outside the mesh's range as unpack4fftw does;
  * the phase rotation of fix_phase_rotate_c2r makes a rotated real orbital real again (up to
    the scale the rotation leaves)."""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import orbitals_oracle as oo
from qmcpack_gb300.orbitals import synthetic_planewaves

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "..", "oracle", "_ref", "libref_bspline.so")


def _ref():
    if not os.path.exists(LIB):
        pytest.skip("oracle/_ref not built (reference sources absent)")
    try:
        return C.CDLL(LIB)
    except OSError as e:
        pytest.skip(f"oracle/_ref not loadable here: {e}")


@pytest.mark.parametrize("mesh,norb", [((5, 6, 7), 1), ((12, 10, 8), 3), ((16, 16, 16), 5)])
def test_spline_solve_matches_reference_build(mesh, norb):
    L = _ref()
    rng = np.random.default_rng(sum(mesh) + norb)
    data = np.ascontiguousarray(rng.normal(size=(norb,) + mesh))
    N = (mesh[0] + 3) * (mesh[1] + 3) * (mesh[2] + 3)
    buf = np.zeros(N * (norb + 64))
    padded = C.c_int(0)
    n = np.array(mesh, np.int32)
    rc = L.ref_multi_spline_3d_d(n.ctypes.data_as(C.POINTER(C.c_int)), norb,
                                 data.ctypes.data_as(C.POINTER(C.c_double)),
                                 buf.ctypes.data_as(C.POINTER(C.c_double)), C.byref(padded))
    assert rc == 0 and padded.value >= norb
    ref = buf[:N * padded.value].reshape(mesh[0] + 3, mesh[1] + 3, mesh[2] + 3, padded.value)[..., :norb]
    ours = np.moveaxis(oo.spline_coefs_3d(data), 0, -1)
    assert np.abs(ours - ref).max() <= 1e-13 * np.abs(ref).max()


@pytest.mark.parametrize("mesh", [(4, 5, 6), (12, 12, 12), (9, 14, 11)])
def test_interpolation_property_and_ghosts(mesh):
    rng = np.random.default_rng(1)
    data = rng.normal(size=(3,) + mesh)
    c = oo.spline_coefs_3d(data)
    table = np.moveaxis(c, 0, -1)
    np.testing.assert_allclose(oo.values_at_grid_points(table, 3), data, rtol=0, atol=1e-12)
    for ax, m in zip((1, 2, 3), mesh):
        take = lambda i: np.take(c, i, axis=ax)
        np.testing.assert_array_equal(take(0), take(m))
        np.testing.assert_array_equal(take(m + 1), take(1))
        np.testing.assert_array_equal(take(m + 2), take(2))


def test_transform_of_one_plane_wave_and_unpack_bounds():
    mesh = (8, 6, 5)
    g = np.array([[1, -2, 2], [4, 0, 0], [0, 3, 0], [0, 0, -3]], np.int32)  # x upper 3, y upper 2, z lower -2
    cg = np.zeros((1, 4), complex)
    cg[0, 0] = 1.0
    cg[0, 1:] = 5.0  # outside [lower, upper] on some axis: dropped
    box = oo.unpack(g, cg, mesh)
    assert np.count_nonzero(box) == 1
    psi = oo.backward_transform(box)[0]
    ix, iy, iz = np.meshgrid(*[np.arange(m) for m in mesh], indexing="ij")
    expect = np.exp(2j * np.pi * (1 * ix / 8 - 2 * iy / 6 + 2 * iz / 5))
    np.testing.assert_allclose(psi, expect, rtol=0, atol=1e-12)


def test_phase_rotation_recovers_a_real_orbital():
    gv, cg = synthetic_planewaves(2, (10, 10, 10), 3.0, seed=4, real_orbitals=True)
    psi = oo.backward_transform(oo.unpack(gv, cg, (10, 10, 10)))
    assert np.abs(psi.imag).max() < 1e-10 * np.abs(psi.real).max()
    rot = psi * np.exp(0.7j)
    real, ph = oo.phase_rotate(rot)
    # the rotated orbital is phase_r Re - phase_i Im = |.| cos(theta + 0.7 + phi): proportional to psi
    for o in range(2):
        ratio = real[o] / psi[o].real
        mask = np.abs(psi[o].real) > 1e-3 * np.abs(psi[o].real).max()
        assert np.ptp(ratio[mask]) < 1e-8 * np.abs(ratio[mask]).max()
    np.testing.assert_allclose(ph[:, 0] ** 2 + ph[:, 1] ** 2, 1.0, rtol=1e-12)
