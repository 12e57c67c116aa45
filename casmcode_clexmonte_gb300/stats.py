"""Autocorrelation and error estimates for sampled Monte Carlo series."""

from __future__ import annotations

import numpy as np


def tau_int(x, c: float = 5.0) -> float:
    """Integrated autocorrelation time with Sokal's automatic window
    (smallest M with M >= c * tau(M)); tau = 1/2 + sum_{t=1..M} rho(t)."""
    x = np.asarray(x, dtype=np.float64)
    n = x.size
    if n < 8:
        return float("nan")
    y = x - x.mean()
    var = float(np.dot(y, y) / n)
    if var == 0.0:
        return 0.5
    f = np.fft.rfft(y, 2 * n)
    acf = np.fft.irfft(f * np.conj(f))[:n] / (n * var)
    tau = 0.5
    for m in range(1, n):
        tau += acf[m]
        if m >= c * tau:
            break
    return float(max(tau, 0.5))


def mean_error(x) -> tuple:
    """(mean, standard error corrected by 2 tau_int, tau_int)."""
    x = np.asarray(x, dtype=np.float64)
    t = tau_int(x)
    var = float(x.var())
    return float(x.mean()), float(np.sqrt(2.0 * t * var / x.size)), t


def batch_means(x, n_batches: int = 20) -> tuple:
    x = np.asarray(x, dtype=np.float64)
    m = x.size // n_batches
    b = x[: m * n_batches].reshape(n_batches, m).mean(axis=1)
    return float(b.mean()), float(b.std(ddof=1) / np.sqrt(n_batches))
