"""qmcg_spline_from_planewaves (the numeric part of the ESHDF orbital input) against the
CPU restatement oracle/orbitals_oracle.py on seeded synthetic bands: the FP64 coefficient
table and the phases within 1e-11 relative of the largest coefficient (the GPU sums its
transforms directly instead of by FFT and fuses multiply-adds), the FP32 table the FP64 one
rounded; the spline's values at the grid points are the phase-rotated orbitals (the
interpolation property); Miller indices outside the mesh are dropped; and a C1-sized set of
192 bands on a 48^3 mesh is timed."""
import time

import numpy as np
import pytest

from oracle import orbitals_oracle as oo
from qmcpack_gb300.orbitals import spline_from_planewaves, synthetic_planewaves

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mesh,norb,gmax,real", [((12, 10, 8), 3, 3.5, False), ((16, 16, 16), 5, 5.0, True),
                                                 ((9, 14, 11), 2, 8.0, False)])
def test_planewave_splines_match_oracle(mesh, norb, gmax, real):
    gv, cg = synthetic_planewaves(norb, mesh, gmax, seed=norb, real_orbitals=real)
    lda = (norb + 15) // 16 * 16
    table, ph = spline_from_planewaves(gv, cg, mesh, precision=8, num_orbitals_padded=lda, with_phases=True)
    ref, ph_o, real_o = oo.spline_from_planewaves(gv, cg, mesh, lda)
    scale = np.abs(ref).max()
    assert np.abs(table - ref).max() <= 1e-11 * scale
    if real:
        # Im psi is rounding only: the sign of sum(Re Im), and with it that of phase_i, is the
        # rounding's (as in the reference); it multiplies Im psi and leaves the table unchanged
        np.testing.assert_allclose(np.abs(ph), np.abs(ph_o), rtol=0, atol=1e-11)
    else:
        np.testing.assert_allclose(ph, ph_o, rtol=0, atol=1e-11)
    assert np.all(table[..., norb:] == 0)
    np.testing.assert_allclose(oo.values_at_grid_points(table, norb), real_o, rtol=0, atol=1e-10 * scale)
    t32 = spline_from_planewaves(gv, cg, mesh, precision=4, num_orbitals_padded=lda)
    assert t32.dtype == np.float32
    np.testing.assert_allclose(t32, ref.astype(np.float32), rtol=2e-6, atol=1e-6 * scale)


def test_c1_sized_orbitals_timed():
    mesh, norb = (48, 48, 48), 192
    gv, cg = synthetic_planewaves(norb, mesh, 12.0, seed=11)
    spline_from_planewaves(gv[:10], cg[:2, :10], (8, 8, 8))  # first call: context and module load
    t0 = time.perf_counter()
    table = spline_from_planewaves(gv, cg, mesh, precision=4, num_orbitals_padded=192)
    dt = time.perf_counter() - t0
    print(f"192 bands, {len(gv)} plane waves, 48^3 mesh: {dt * 1e3:.1f} ms (host-timed, copies included)")
    assert table.shape == (51, 51, 51, 192) and np.isfinite(table).all()
    # spot check three bands against the oracle
    ref, _, _ = oo.spline_from_planewaves(gv, cg[:3], mesh, 16)
    assert np.abs(table[..., :3] - ref[..., :3]).max() <= 2e-6 * np.abs(ref).max()


def test_system_from_planewave_orbitals():
    """The table drives the move loop: a system whose orbitals come from plane waves gives
    the FP64 oracle's log|psi| and inverse after mw_evaluateLog."""
    import dataclasses

    from oracle import oracle as orc
    from qmcpack_gb300.crowd import Crowd, DeviceSystem
    from qmcpack_gb300.system import make_system, make_walkers, scaled_spec
    spec = scaled_spec("c0_32e", n_up=8, n_dn=8, grid=16, walkers=4, delay=1, precision=8)
    s = make_system(spec, seed=3)
    gv, cg = synthetic_planewaves(s.norb, (16, 16, 16), 5.0, seed=9)
    table = spline_from_planewaves(gv, cg, (16, 16, 16), precision=8, num_orbitals_padded=s.npad)
    s = dataclasses.replace(s, coefs=np.ascontiguousarray(table / np.abs(table).max()))
    R = make_walkers(s, 4, seed=5)
    g = Crowd(DeviceSystem(s), 4, 1)
    g.load_walkers(R)
    lg, _ = g.mw_evaluateLog()
    o = orc.Crowd(s, 4, 1, 8)
    o.load_walkers(R)
    lo, _ = o.evaluate_log()
    np.testing.assert_allclose(lg, lo, rtol=1e-10)
    ai = o.ainv(0)
    np.testing.assert_allclose(g.inverse(0), ai, rtol=0, atol=1e-10 * np.abs(ai).max())
