"""Host side of DMC (no GPU): the library's comb population control against its
restatement (WalkerReconfiguration::getIndexPermutation), its invariants, and the
branching-parameter updates of SFNBranch."""
import numpy as np
import pytest

from oracle import dmc_oracle as dmo
from qmcpack_gb300.crowd import dmc_comb
from qmcpack_gb300.dmc import BranchEngine


@pytest.mark.parametrize("nw,spread", [(1, 0.1), (7, 0.5), (64, 0.3), (512, 1.5)])
def test_comb_matches_restatement(nw, spread):
    rng = np.random.default_rng(nw)
    for _ in range(20):
        w = np.exp(rng.normal(size=nw) * spread)
        u = rng.random()
        src, kept = dmc_comb(w, u)
        src_o, kept_o = dmo.comb(w, u)
        np.testing.assert_array_equal(src, src_o)
        assert kept == kept_o
        # every source keeps its own slot; copies of a walker are at most ceil(nw w / W) + 1
        assert np.all(src[src] == src)
        counts = np.bincount(src, minlength=nw)
        assert counts.sum() == nw
        assert np.all(counts <= np.ceil(nw * w / w.sum()) + 1)


def test_comb_is_unbiased():
    """Averaged over the comb's offset, walker i gets nw w_i / W copies."""
    rng = np.random.default_rng(2)
    nw = 16
    w = rng.random(nw) * 2
    mean = np.zeros(nw)
    us = (np.arange(2000) + 0.5) / 2000
    for u in us:
        src, _ = dmc_comb(w, u)
        mean += np.bincount(src, minlength=nw)
    mean /= len(us)
    np.testing.assert_allclose(mean, nw * w / w.sum(), atol=2e-3)


def test_comb_rejects_bad_input():
    from qmcpack_gb300._lib import QmcgError
    with pytest.raises(QmcgError):
        dmc_comb(np.array([1.0, np.nan]), 0.5)
    with pytest.raises(QmcgError):
        dmc_comb(np.array([1.0, 2.0]), 1.0)


def test_branch_weight_window():
    """Inside the window the bare weight; beyond branch_max no branching; linear between."""
    p = dict(e_trial=-10.0, e_ref=-10.0, tau_eff=0.02, branch_cutoff=1.0, branch_max=1.5)
    assert np.isclose(dmo.branch_weight(-10.2, -10.1, **p), np.exp(0.01 * (-20 + 20.3)))
    assert dmo.branch_weight(-12.0, -10.0, **p) == 1.0
    w = dmo.branch_weight(-11.25, -10.0, **p)
    assert np.isclose(w, np.exp(0.01 * 0.5 * (-20 + 21.25)))


def test_branch_engine_updates():
    eng = BranchEngine(tau=0.01, num_electrons=32, target_walkers=100, warmup_steps=2)
    eng.start(np.array([-10.0, -10.2, -9.8]))
    assert np.isclose(eng.e_trial, -10.0) and np.isclose(eng.tau_eff, 0.01)
    assert np.isclose(eng.branch_cutoff, min(max(eng.sigma2 * 10, 50), 2.5 / 0.01))
    # warm-up: E_ref = E_now, E_trial corrected by the population weight
    eng.update([90.0, 90.0 * -10.5, 90.0 * 110.5, 0.5, 1.0])
    assert np.isclose(eng.e_ref, -10.5)
    assert np.isclose(eng.e_trial, -10.5 + (np.log(100) - np.log(90)) / 0.01)
    assert np.isclose(eng.tau_eff, 0.005)
    eng.update([100.0, 100.0 * -10.4, 100.0 * 108.4, 0.5, 1.0])
    assert eng.warmup_left == 0 and np.isclose(eng.branch_cutoff, min(max(eng.sigma2 * 10, 10), 250))
    # after warm-up: E_ref is the weighted average of the step energies
    eng.update([100.0, 100.0 * -10.2, 100.0 * 104.2, 0.5, 1.0])
    eng.update([300.0, 300.0 * -10.6, 300.0 * 112.5, 0.5, 1.0])
    assert np.isclose(eng.e_ref, (100 * -10.2 + 300 * -10.6) / 400)
    assert np.isclose(eng.e_trial, eng.e_ref + (np.log(100) - np.log(300)))
