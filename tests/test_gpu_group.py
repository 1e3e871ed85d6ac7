"""Uneven crowds swept together (one persistent launch per stage): every crowd's
result is bit-identical to sweeping it alone with its group seed, with the flush after
every segment (kind 0) and with the block-lazy updates (kind 4: the crowds whose segment
rows are staged sequence them per stage of the group)."""
import numpy as np
import pytest

from qmcpack_gb300.system import make_system, make_walkers, scaled_spec

pytestmark = pytest.mark.gpu


def _systems(prec):
    a = make_system(scaled_spec("c0_32e", n_up=8, n_dn=8, grid=12, walkers=20, delay=1, precision=prec), seed=1)
    b = make_system(scaled_spec("c0_32e", n_up=24, n_dn=24, grid=16, walkers=12, delay=8, precision=prec), seed=2)
    c = make_system(scaled_spec("c3_768e", n_up=40, n_dn=40, grid=12, walkers=6, delay=16, precision=prec), seed=3)
    return [a, b, c]


@pytest.mark.parametrize("prec,flush", [(8, 0), (4, 0), (8, 4), (4, 4)])
def test_group_matches_separate_crowds(prec, flush):
    from qmcpack_gb300.crowd import Crowd, DeviceSystem, Group, group_seed
    systems = _systems(prec)
    dss = [DeviceSystem(s) for s in systems]
    Rs = [make_walkers(s, s.spec.walkers, seed=10 + i) for i, s in enumerate(systems)]

    def crowds():
        out = []
        for s, ds, R in zip(systems, dss, Rs):
            g = Crowd(ds, s.spec.walkers, s.spec.delay)
            g.load_walkers(R)
            g.mw_evaluateLog()
            out.append(g)
        return out

    together = crowds()
    grp = Group(together)
    print("group", grp.info())
    if flush == 4:
        assert any(g.sweep_info(4)["block_lazy"] for g in together)
    stats = grp.sweeps(2, 0.3, 1234, flush=flush)
    alone = crowds()
    for i, g in enumerate(alone):
        a, r, _ = g.vmc_sweeps(2, 0.3, group_seed(1234, i), rng_mode=1, flush=flush)
        assert (a, r) == stats[i][:2]
        np.testing.assert_array_equal(g.positions(), together[i].positions())
        np.testing.assert_array_equal(g.get_log()[0], together[i].get_log()[0])
