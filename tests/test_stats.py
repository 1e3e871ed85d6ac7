"""Estimator statistics against the reference's simstats (nexus/nexus/numerics.py:894-997)
on the committed golden series (tests/golden/make_simstats_golden.py)."""
import json
import os

import numpy as np

from qmcpack_gb300.stats import energy_statistics, simstats

HERE = os.path.dirname(os.path.abspath(__file__))


def test_simstats_matches_reference_golden():
    g = json.load(open(os.path.join(HERE, "golden", "simstats_golden.json")))
    for c in g["cases"]:
        s = simstats(np.array(c["series"]))
        assert abs(s.mean - c["mean"]) < 1e-12 * abs(c["mean"])
        assert abs(s.var - c["var"]) < 1e-12 * c["var"]
        assert abs(s.error - c["error"]) < 1e-10 * c["error"]
        assert abs(s.kappa - c["kappa"]) < 1e-10 * c["kappa"]


def test_simstats_edge_cases():
    assert simstats(np.full(10, 3.0)).kappa == 1.0
    s = simstats(np.array([1.0, -1.0] * 50))
    assert s.kappa == 1.0 and abs(s.mean) < 1e-15


def test_energy_statistics_shapes():
    rng = np.random.default_rng(0)
    e = -10 + rng.normal(size=(200, 16))
    st = energy_statistics(e, equilibration=20)
    assert st["sweeps"] == 180 and st["walkers"] == 16
    assert abs(st["energy"] + 10) < 5 * st["error"] + 1e-12
    assert 0.5 < st["kappa"] < 2.0


def test_walker_kappa_matches_ar1():
    """Independent AR(1) chains x_t = a x_{t-1} + noise have kappa = (1 + a) / (1 - a)."""
    from qmcpack_gb300.stats import ensemble_statistics, walker_kappa
    rng = np.random.default_rng(4)
    a, n, nw = 0.8, 2000, 256
    x = np.zeros((n, nw))
    x[0] = rng.normal(size=nw) / np.sqrt(1 - a * a)
    for t in range(1, n):
        x[t] = a * x[t - 1] + rng.normal(size=nw)
    k = walker_kappa(x)
    assert abs(k - (1 + a) / (1 - a)) < 0.5
    st = ensemble_statistics(x + 3.0)
    assert abs(st["energy"] - 3.0) < 4 * st["error"]
    assert abs(st["variance"] - 1 / (1 - a * a)) < 4 * st["variance_error"]
