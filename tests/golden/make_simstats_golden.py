"""Golden values of the reference's autocorrelation statistics for the estimator code.

Runs nexus.numerics.simstats (nexus/nexus/numerics.py:894-997 of the reference; the
statistics qmca reports) on seeded AR(1) series and writes tests/golden/simstats_golden.json
with the series and the reference's (mean, var, error, kappa).

usage: python tests/golden/make_simstats_golden.py [REFERENCE_ROOT]
"""
import json
import os
import sys

import numpy as np


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("QMCPACK_REFERENCE_DIR", "/root/reference")
    sys.path.insert(0, os.path.join(root, "nexus"))
    from nexus.numerics import simstats

    rng = np.random.Generator(np.random.PCG64(20261204))
    cases = []
    for phi, n in [(0.0, 800), (0.6, 1000), (0.9, 1200), (0.97, 1500)]:
        x = np.zeros(n)
        e = rng.normal(size=n)
        for i in range(1, n):
            x[i] = phi * x[i - 1] + e[i]
        x = -12.5 + 0.3 * x
        mean, var, error, kappa = simstats(x)
        cases.append({"phi": phi, "series": [float(v) for v in x], "mean": float(mean), "var": float(var),
                      "error": float(error), "kappa": float(kappa)})
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "simstats_golden.json")
    with open(out, "w") as f:
        json.dump({"source": "nexus/nexus/numerics.py simstats (reference)", "cases": cases}, f)
    print("wrote", out, [(c["phi"], round(c["kappa"], 3)) for c in cases])


if __name__ == "__main__":
    main()
