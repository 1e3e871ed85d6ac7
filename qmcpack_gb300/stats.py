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


def walker_kappa(e_local: np.ndarray, with_lag: bool = False):
    """Integrated autocorrelation time of independent, identically distributed chains:
    the autocorrelation function of every walker's own series (around the common mean,
    normalised by the common variance) averaged over the walkers, summed with the
    simstats rule (kappa = 1 + 2 sum C(i) up to the first C(i) <= 0).  It estimates the
    same kappa as simstats of the walker-averaged series, from num_walkers times the data.
    e_local: [sweeps][walkers].  with_lag: also return the lag at which the sum stopped
    (n - 1 when the autocorrelation never reached zero inside the series)."""
    e = np.asarray(e_local, dtype=np.float64)
    n, nw = e.shape
    var = float(e.var())
    if n < 3 or var < 1e-300:
        return (1.0, 0) if with_lag else 1.0
    y = e - e.mean()
    m = 1 << int(np.ceil(np.log2(2 * n)))
    f = np.fft.rfft(y, m, axis=0)
    ac = np.fft.irfft(f * np.conj(f), m, axis=0)[:n].sum(axis=1)
    kappa = 1.0
    lag = n - 1
    for i in range(1, n - 1):
        c = ac[i] / ((n - i) * nw * var)
        if c <= 0:
            lag = i
            break
        kappa += 2.0 * c
    return (float(kappa), lag) if with_lag else float(kappa)


def ensemble_statistics(e_local: np.ndarray) -> dict:
    """Energy, variance and their error bars from a [sweeps][walkers] history of
    independent walkers, with kappa from walker_kappa: error(E) = sqrt(var kappa /
    (sweeps walkers)); the variance's error from the series of E_L^2 the same way.
    kappa_resolved: the autocorrelation reached zero within the first quarter of the
    series; otherwise kappa (and the error bars) are bounded by the series length."""
    e = np.asarray(e_local, dtype=np.float64)
    n, nw = e.shape
    kappa, lag = walker_kappa(e, with_lag=True)
    mean = float(e.mean())
    var = float(e.var())
    err = float(np.sqrt(var * kappa / (n * nw)))
    e2 = e * e
    k2 = walker_kappa(e2)
    err_e2 = float(np.sqrt(e2.var() * k2 / (n * nw)))
    err_var = float(np.hypot(err_e2, 2 * abs(mean) * err))
    crowd = simstats(e.mean(axis=1))
    return {"energy": mean, "error": err, "variance": var, "variance_error": err_var, "kappa": kappa,
            "kappa_cut_lag": int(lag), "kappa_resolved": bool(lag < n // 4),
            "kappa_crowd_series": crowd.kappa, "error_crowd_series": crowd.error, "sweeps": int(n),
            "walkers": int(nw)}


def agree_within(a: dict, b: dict, key: str, err_key: str, nsigma: float = 2.0) -> bool:
    """|a - b| <= nsigma * combined error"""
    return bool(abs(a[key] - b[key]) <= nsigma * np.hypot(a[err_key], b[err_key]))
