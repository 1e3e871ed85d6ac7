"""qmcg_vmc_sweeps_host: positions in from a host buffer, sweeps, positions and log|psi|
out to host buffers with one synchronisation.  Identical bit for bit to the sequence of
separate calls (qmcg_load_walkers, qmcg_vmc_sweeps, qmcg_get_positions, qmcg_get_log),
with pinned and pageable buffers, the input and output buffer the same array, and
either side left out."""
import numpy as np
import pytest

from qmcpack_gb300.system import make_system, make_walkers, scaled_spec

pytestmark = pytest.mark.gpu

TAU = 0.3


def _crowd(system, nw, k, R):
    from qmcpack_gb300.crowd import Crowd, DeviceSystem
    g = Crowd(DeviceSystem(system), nw, k)
    g.load_walkers(R)
    g.mw_evaluateLog()
    return g


@pytest.mark.parametrize("prec,k,flush", [(8, 4, 0), (4, 8, 4), (4, 1, 0)])
def test_sweeps_host_matches_separate_calls(prec, k, flush):
    import torch
    s = make_system(scaled_spec("c0_32e", n_up=24, n_dn=24, grid=16, walkers=12, delay=k, precision=prec), seed=4)
    nw = 12
    R = make_walkers(s, nw, seed=5)
    a = _crowd(s, nw, k, R)
    b = _crowd(s, nw, k, R)
    for step in range(3):
        Rin = a.positions()
        a.load_walkers(Rin)
        acc_a = a.vmc_sweeps(2, TAU, 99, rng_mode=1, flush=flush)[:2]
        Ra = a.positions()
        la = a.get_log()[0]
        # pinned in/out buffers, the same array for both
        Rb = torch.from_numpy(Rin.copy()).pin_memory().numpy()
        lb = torch.from_numpy(np.zeros(nw)).pin_memory().numpy()
        acc_b = b.vmc_sweeps_host(2, TAU, 99, R_in=Rb, R_out=Rb, log_out=lb, flush=flush)
        assert acc_a == acc_b
        np.testing.assert_array_equal(Ra, Rb)
        np.testing.assert_array_equal(la, lb)
    # pageable buffers; no input (the device keeps its positions); no outputs
    Rout = np.zeros_like(R)
    acc_a = a.vmc_sweeps(1, TAU, 7, rng_mode=1, flush=flush)[:2]
    acc_b = b.vmc_sweeps_host(1, TAU, 7, R_out=Rout, flush=flush)
    assert acc_a == acc_b
    np.testing.assert_array_equal(a.positions(), Rout)
    a.vmc_sweeps(1, TAU, 8, rng_mode=1, flush=flush)
    b.vmc_sweeps_host(1, TAU, 8, flush=flush)
    np.testing.assert_array_equal(a.positions(), b.positions())
    np.testing.assert_array_equal(a.get_log()[0], b.get_log()[0])
