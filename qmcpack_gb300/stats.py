"""Estimator statistics of a VMC run: mean, variance, error bar and integrated
autocorrelation time of a scalar series (the local energy per sweep).

The autocorrelation estimate is the one QMCPACK's analysis tools report
(nexus/nexus/numerics.py:894-997, simstats): kappa = 1 + 2 sum_{i>=1} C(i), with
C(i) = sum_t (x_t - m)(x_{t+i} - m) / ((N - i) var) summed until the first C(i) <= 0;
error = sqrt(var / (N / kappa)).  Effective samples = N / kappa.
"""
from __future__ import annotations

import dataclasses

import numpy as np


@dataclasses.dataclass
class SeriesStats:
    mean: float
    var: float
    error: float
    kappa: float

    @property
    def n_eff_per_sample(self) -> float:
        return 1.0 / self.kappa


def _autocov(x: np.ndarray) -> np.ndarray:
    """sum_t (x_t - m)(x_{t+i} - m) for i = 0..N-1 by FFT."""
    n = len(x)
    y = x - x.mean()
    m = 1 << int(np.ceil(np.log2(2 * n)))
    f = np.fft.rfft(y, m)
    return np.fft.irfft(f * np.conj(f), m)[:n]


def simstats(x) -> SeriesStats:
    """mean, variance (1/N), error bar and autocorrelation time kappa of a 1-D series."""
    x = np.asarray(x, dtype=np.float64)
    n = len(x)
    mean = float(x.mean())
    var = float(x.var())
    if abs(var) < 1e-15 or n < 2:
        kappa = 1.0
    else:
        ac = _autocov(x)
        kappa = 1.0
        # lags 1 .. N-2: the reference's loop stops once the lag reaches N-1
        for i in range(1, n - 1):
            c = ac[i] / ((n - i) * var)
            if c <= 0:
                break
            kappa += 2.0 * c
    neff = n / kappa if kappa != 0 else 1.0
    return SeriesStats(mean, var, float(np.sqrt(var / neff)), float(kappa))


def energy_statistics(e_local: np.ndarray, equilibration: int = 0) -> dict:
    """Statistics of a [sweeps][walkers] local-energy history: the series is the
    walker-averaged energy per sweep (one scalar per step, as scalar.dat holds);
    the variance of the local energy is over all walkers and sweeps."""
    e = np.asarray(e_local, dtype=np.float64)[equilibration:]
    st = simstats(e.mean(axis=1))
    return {
        "energy": st.mean,
        "error": st.error,
        "kappa": st.kappa,
        "variance": float(e.var()),
        "sweeps": int(e.shape[0]),
        "walkers": int(e.shape[1]),
    }
