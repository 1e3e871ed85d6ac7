"""The masked recompute the resident sweeps use to repair a walker whose tracked inverse
lost accuracy (qmcg_mw_recompute_walkers; TrialWaveFunction::mw_recompute with its
recompute mask, TrialWaveFunction.cpp:225-240).

FP32 crowds eliminate in FP32 with the matrix in registers: one CTA up to 192 x 192, a
cluster of 8 CTAs up to 384 x 384, 16 CTAs up to 768 x 768; FP64 crowds in FP64.  Against the FP64 recompute of mw_evaluateLog:
FP64 inverse within 1e-10 of the largest element, log|det| within 1e-9; FP32 inverse in
the relative Frobenius norm and log|det| within max(2e-4, 5e-7 c), c the matrix's
condition number (an FP32 elimination carries about c * 6e-8); walkers without a flag
keep their state bit for bit.
"""
import numpy as np
import pytest

from qmcpack_gb300.system import make_system, make_walkers, scaled_spec

pytestmark = pytest.mark.gpu


def _crowd(spec, nw, delay, seed):
    from qmcpack_gb300.crowd import Crowd, DeviceSystem
    s = make_system(spec, seed=seed)
    ds = DeviceSystem(s)
    g = Crowd(ds, nw, delay)
    g.load_walkers(make_walkers(s, nw, seed=seed + 1))
    return s, ds, g


@pytest.mark.parametrize("name,prec", [
    ("c0_32e", 4),    # 16 x 16: one CTA, registers, FP32
    ("c1_384e", 4),   # 192 x 192: one CTA, registers, FP32
    ("c3_768e", 4),   # 384 x 384: 8-CTA cluster, registers, FP32
    ("c2_1536e", 4),  # 768 x 768: 16-CTA cluster, registers, FP32
    ("c1_384e", 8),   # 192 x 192: 8-CTA cluster, FP64
])
def test_repair_matches_fp64_recompute(name, prec):
    spec = scaled_spec(name, walkers=4, precision=prec)
    n = spec.n_up
    s, ds, g = _crowd(spec, 4, 4, seed=61)
    g.mw_evaluateLog()
    # a few sweeps so that the tracked state is not the one just computed
    g.vmc_sweeps(2, 0.3, 3, rng_mode=1)
    before = [g.inverse(sp) for sp in (0, 1)]
    lp_before, _, parts_before = g.get_log()
    flags = np.array([1, 0, 1, 0], np.int32)
    g.mw_recompute_walkers(flags)
    rep = [g.inverse(sp) for sp in (0, 1)]
    _, _, parts_rep = g.get_log()
    g.mw_evaluateLog()
    ref = [g.inverse(sp) for sp in (0, 1)]
    _, _, parts_ref = g.get_log()
    for iw in range(4):
        for sp in (0, 1):
            if flags[iw]:
                a, b = rep[sp][iw], ref[sp][iw]
                if prec == 8:
                    tol_inv, tol_log = 1e-10, 1e-9
                    err = np.abs(a - b).max() / np.abs(b).max()
                else:
                    # an FP32 elimination carries about cond * 6e-8; the floor covers
                    # well-conditioned matrices
                    cond = np.linalg.cond(b)
                    tol_inv = tol_log = max(2e-4, 5e-7 * cond)
                    err = np.linalg.norm(a - b) / np.linalg.norm(b)
                dlog = abs(parts_rep[iw, sp] - parts_ref[iw, sp])
                print(f"n={n} prec={prec} walker {iw} spin {sp}: inverse error {err:.2e}, log|det| error {dlog:.2e}, "
                      f"tolerance {tol_inv:.1e}")
                assert err < tol_inv
                assert dlog < tol_log
            else:
                assert np.array_equal(rep[sp][iw], before[sp][iw])
                assert parts_rep[iw, sp] == parts_before[iw, sp]


def test_repair_needs_completed_updates():
    from qmcpack_gb300._lib import QmcgError
    spec = scaled_spec("c0_32e", n_up=16, n_dn=16, grid=16, walkers=4, precision=4)
    s, ds, g = _crowd(spec, 4, 4, seed=71)
    g.mw_evaluateLog()
    g.mw_evalGrad(0)
    g.mw_makeMove(0, np.full((4, 3), 0.05))
    g.mw_calcRatioGrad(0)
    g.mw_accept_rejectMove(0, np.ones(4, np.int32))
    with pytest.raises(QmcgError):
        g.mw_recompute_walkers(np.ones(4, np.int32))
    g.mw_completeUpdates()
    g.mw_recompute_walkers(np.ones(4, np.int32))
