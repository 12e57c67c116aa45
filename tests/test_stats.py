"""Unit tests of the error estimates and the two-sigma family test that the
equilibrium comparisons between the CUDA chains and the oracle's rest on."""

import numpy as np
import pytest

from casmcode_clexmonte_gb300 import stats


def _ar1(rng, rho, n, chains=1):
    """AR(1) series x_t = rho x_{t-1} + sqrt(1 - rho^2) e_t, unit variance,
    started in equilibrium; tau_int = (1 + rho) / (2 (1 - rho))."""
    e = rng.standard_normal((chains, n))
    x = np.empty((chains, n))
    x[:, 0] = e[:, 0]
    s = np.sqrt(1.0 - rho * rho)
    for t in range(1, n):
        x[:, t] = rho * x[:, t - 1] + s * e[:, t]
    return x


def test_tau_int_of_ar1():
    rng = np.random.default_rng(11)
    x = _ar1(rng, 0.8, 200_000)[0]
    assert abs(stats.tau_int(x) - 4.5) < 0.4
    assert abs(stats.tau_int(rng.standard_normal(100_000)) - 0.5) < 0.05
    assert stats.tau_int(np.ones(100)) == 0.5
    assert np.isnan(stats.tau_int(np.arange(4.0)))


def test_mean_error_covers_correlated_series():
    rng = np.random.default_rng(12)
    x = _ar1(rng, 0.8, 100_000)[0]
    m, err, t = stats.mean_error(x)
    expect = np.sqrt(2 * 4.5 / x.size)
    assert abs(err / expect - 1.0) < 0.1
    assert abs(m) < 4 * expect


def test_jackknife_of_the_mean_is_the_spread_of_chain_means():
    """For equal-length chains and the mean estimator, the delete-one-chain
    jackknife error equals the sample standard deviation of the chain means
    over sqrt(r) (an identity, not a statistical statement)."""
    rng = np.random.default_rng(13)
    chains = [rng.standard_normal(500) for _ in range(40)]
    est, se = stats.jackknife_chains(np.mean, chains)
    means = np.array([c.mean() for c in chains])
    assert est == pytest.approx(np.concatenate(chains).mean(), rel=1e-12)
    assert se == pytest.approx(means.std(ddof=1) / np.sqrt(len(chains)), rel=1e-10)
    assert abs(se * np.sqrt(20_000) - 1.0) < 0.3
    _, se1 = stats.jackknife_chains(np.mean, chains[:1])
    assert np.isnan(se1)


def test_jackknife_carries_the_autocorrelation():
    rng = np.random.default_rng(14)
    x = _ar1(rng, 0.8, 2_000, chains=48)
    _, se = stats.jackknife_chains(np.mean, list(x))
    expect = np.sqrt(2 * 4.5 / x.size)
    assert 0.7 < se / expect < 1.3


def test_jackknife_of_a_fluctuation_estimator():
    """Variance (a heat-capacity-like estimator) with a vector result."""
    rng = np.random.default_rng(15)
    chains = [rng.standard_normal((400, 2)) * [1.0, 3.0] for _ in range(32)]
    est, se = stats.jackknife_chains(lambda a: a.var(axis=0), chains)
    assert est.shape == se.shape == (2,)
    assert abs(est[0] - 1.0) < 4 * se[0] and abs(est[1] - 9.0) < 4 * se[1]
    # var of N(0, s^2) from n samples has standard error s^2 sqrt(2 / n)
    n = 32 * 400
    assert 0.7 < se[0] / np.sqrt(2.0 / n) < 1.3
    assert 0.7 < se[1] / (9.0 * np.sqrt(2.0 / n)) < 1.3


@pytest.mark.parametrize("m,k,bound", [(1, 1, 2.576), (2, 1, 2.807), (4, 2, 3.023),
                                       (6, 2, 3.144), (12, 3, 3.341), (18, 3, 3.452)])
def test_family_2sigma_thresholds(m, k, bound):
    ok, kk, bb, n2 = stats.family_2sigma(np.zeros(m))
    assert ok and n2 == 0
    assert kk == k
    assert bb == pytest.approx(bound, abs=1e-3)


def test_family_2sigma_decisions():
    ok, k, bound, n2 = stats.family_2sigma([2.5, 0.1, -0.3, 1.0])
    assert ok and n2 == 1 and k == 2
    assert not stats.family_2sigma([2.5, 2.1, -2.2, 1.0])[0]  # three beyond 2 sigma
    assert not stats.family_2sigma([3.1, 0.0, 0.0, 0.0])[0]  # beyond the Bonferroni bound
    assert stats.family_2sigma([-2.7, 0.0])[0]
    assert not stats.family_2sigma([-2.9, 0.0])[0]


@pytest.mark.parametrize("m", [2, 4, 6, 12, 18])
def test_family_2sigma_false_alarm_rate(m):
    """Under the null (independent standard normal z-scores) a family falsely
    fails with probability below 2 alpha = 2 %; the binomial condition alone
    holds it below alpha."""
    from scipy import stats as st

    _, k, bound, _ = stats.family_2sigma(np.zeros(m))
    rng = np.random.default_rng(100 + m)
    trials = 200_000
    z = np.abs(rng.standard_normal((trials, m)))
    fail = ((z > 2.0).sum(axis=1) > k) | (z > bound).any(axis=1)
    rate = fail.mean()
    assert rate < 0.02
    assert st.binom.sf(k, m, 2.0 * st.norm.sf(2.0)) < 0.01
    # the simulated rate is of the size the analytic union bound allows
    assert rate > 0.005
