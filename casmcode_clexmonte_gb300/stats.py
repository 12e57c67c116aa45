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


def jackknife_chains(estimator, chains) -> tuple:
    """(estimate, standard error) of ``estimator`` over independent chains.

    ``chains`` is a list of per-chain sample arrays (first axis = samples);
    the estimate is ``estimator`` of all chains' samples pooled, the error the
    delete-one-chain jackknife (Efron 1982). Each chain is an independent
    unit, so the error carries every chain's autocorrelation without a tau_int
    model."""
    pooled = np.concatenate(chains, axis=0)
    est = estimator(pooled)
    r = len(chains)
    if r < 2:
        return est, float("nan")
    loo = np.array([estimator(np.concatenate(chains[:k] + chains[k + 1:], axis=0))
                    for k in range(r)])
    se = np.sqrt((r - 1) / r * np.sum((loo - loo.mean(axis=0)) ** 2, axis=0))
    return est, se


def family_2sigma(z, alpha: float = 0.01) -> tuple:
    """Two-sigma test of a family of m independent z-scores: each comparison
    is judged at |z| <= 2; the family passes when at most k of them exceed 2,
    k the smallest count that exact sampling exceeds with probability below
    alpha (binomial, p = P(|Z| > 2) = 0.0455), and no |z| exceeds the
    Bonferroni bound z(1 - alpha / (2 m)). Each condition alone falsely fails
    with probability below alpha, so the family's false-alarm level is below
    2 alpha (for alpha = 0.01 and 2 to 18 comparisons: 1.1-1.8 % by
    simulation). Returns (passed, k, bonferroni_bound, n_beyond_2sigma)."""
    from scipy import stats as st

    z = np.abs(np.asarray(z, dtype=np.float64)).ravel()
    m = z.size
    p2 = 2.0 * st.norm.sf(2.0)
    k = 0
    while st.binom.sf(k, m, p2) >= alpha:
        k += 1
    bound = float(st.norm.isf(alpha / (2.0 * m)))
    n2 = int(np.sum(z > 2.0))
    return bool(n2 <= k and np.all(z <= bound)), k, bound, n2
