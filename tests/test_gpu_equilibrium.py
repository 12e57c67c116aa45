"""Equilibrium averages of the parallel GPU sweep against the oracle's
sequential chain (the reference's occupation_metropolis_v2 loop restated,
include/casm/clexmonte/methods/occupation_metropolis.hh:72-123).

Observables, as the reference's samplers and analyses define them
(monte_calculator/sampling_functions.cc:274-283, :37-87;
monte_calculator/analysis_functions.cc:43-173; run/io/convariance_functions.cc:29-146):
potential energy per unit cell <E>; heat capacity C = var(E) N_uc / (k_B T^2);
in the semi-grand canonical ensemble also <x> (param composition), the
susceptibility chi = cov(x, x) N_uc / (k_B T) and the thermo-chemical
susceptibility cov(E, x) N_uc / (k_B T).

Both samplers run several independent chains per condition (same
conditions, different seeds and initial states). An observable is estimated
from the pooled post-equilibration samples of all chains; its standard error
is the delete-one-chain jackknife, so it carries each chain's autocorrelation.
Every chain holds at least 50 integrated autocorrelation times (Sokal window)
of each sampled series after its equilibration tail is dropped.

Criterion: each comparison |GPU - oracle| is judged at 2 combined standard
errors. A test of m comparisons passes when at most k exceed 2 sigma, k the
smallest count that correct sampling exceeds with probability below 1 %
(binomial, p = 0.0455 per comparison), and none exceeds the Bonferroni bound
z(1 - 0.01 / (2m)). Each condition alone falsely fails with probability
below 1 %, together below 2 % (1.1-1.8 % by simulation for 2-18 comparisons).
"""

import os

import numpy as np
import pytest

from casmcode_clexmonte_gb300 import workloads
from tests.stat_checks import compare as _compare

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


@pytest.fixture(scope="module")
def cm():
    from casmcode_clexmonte_gb300 import build

    build.build()
    from casmcode_clexmonte_gb300 import calculator

    return calculator


@pytest.fixture(scope="module")
def oracle_mod():
    from oracle import oracle

    oracle.build_oracle()
    return oracle


def _gpu_chains(cm, ce, ens, L, conds, mus, xs, n_rep, n_passes, n_equil, seed):
    """Per condition: a list of n_rep arrays [n_samples, 1 + nc] (E, x...)."""
    sysd = cm.System(ce)
    nc = ce.prim.n_occ - 1
    n_sites = int(np.prod(L)) * ce.prim.n_basis
    b = cm.ReplicaBatch(sysd, ens, [L] * (len(conds) * n_rep))
    rng = np.random.default_rng(seed)
    for c, (T, mu, x) in enumerate(zip(conds, mus, xs)):
        for r in range(n_rep):
            i = c * n_rep + r
            b.set_conditions(i, T, mu if ens == "semigrand_canonical" else None)
            b.set_seed(i, seed * 1000 + i)
            if ens == "canonical":
                b.set_occupation(i, workloads.fixed_composition(rng, n_sites, x))
            else:
                b.set_occupation(i, workloads.random_occupation(rng, n_sites, ce.prim.n_occ))
    n_s = n_passes - n_equil
    b.run(n_passes, n_equil, record_samples=True)
    out = []
    for c in range(len(conds)):
        chains = []
        for r in range(n_rep):
            pot, comp = b.samples(c * n_rep + r, n_s)
            assert pot.size == n_s
            chains.append(np.column_stack([pot, comp.reshape(n_s, nc)]))
        out.append(chains)
    return out, b


def _oracle_chains(oracle_mod, ce, ens, L, conds, mus, xs, n_rep, n_passes, n_equil, seed):
    o = oracle_mod.OracleSystem(ce, L)
    nc = ce.prim.n_occ - 1
    rng = np.random.default_rng(seed)
    occ, temps, mu_all = [], [], []
    for T, mu, x in zip(conds, mus, xs):
        for _ in range(n_rep):
            if ens == "canonical":
                occ.append(workloads.fixed_composition(rng, o.n_sites, x))
            else:
                occ.append(workloads.random_occupation(rng, o.n_sites, ce.prim.n_occ))
            temps.append(T)
            mu_all.append(np.zeros(nc) if mu is None else mu)
    occ = np.ascontiguousarray(np.concatenate(occ), dtype=np.int8)
    pot, comp, _ = o.run_chains(occ, 0 if ens == "semigrand_canonical" else 1, np.array(temps),
                                np.array(mu_all), seed, n_passes, THREADS)
    out = []
    for c in range(len(conds)):
        chains = []
        for r in range(n_rep):
            i = c * n_rep + r
            chains.append(np.column_stack([pot[i, n_equil:], comp[i, n_equil:]]))
        out.append(chains)
    return out


def test_canonical_bench_conditions_match_oracle(cm, oracle_mod):
    """The benchmark workload's own conditions: 24^3 FCC A/B (its cluster
    expansion), canonical, x_B in {0.25, 0.5} at T = 200, 700, 1200 K."""
    w = workloads.config(1, scale=1.0 / 64)
    ce, L = w.ce, (24, 24, 24)
    grid = [(T, x) for T in (200.0, 700.0, 1200.0) for x in (0.25, 0.5)]
    temps = [T for T, _ in grid]
    xs = [x for _, x in grid]
    mus = [None] * len(grid)
    labels = [(f"T={T:.0f} x_B={x}", T) for T, x in grid]
    g, _ = _gpu_chains(cm, ce, "canonical", L, temps, mus, xs, 32, 3000, 500, 71)
    o = _oracle_chains(oracle_mod, ce, "canonical", L, temps, mus, xs, 16, 560, 60, 73)
    print(_compare(labels, g, o, int(np.prod(L)), sgc=False))


def test_semigrand_fcc_matches_oracle(cm, oracle_mod):
    """Semi-grand canonical FCC A/B (configuration 0's cluster expansion),
    10^3 cells: <E>, <x>, C, chi, thermo-chemical chi."""
    w = workloads.config(0)
    ce, L = w.ce, (10, 10, 10)
    conds = [(1000.0, 0.0), (600.0, 0.05), (1500.0, -0.08)]
    temps = [T for T, _ in conds]
    mus = [np.array([m]) for _, m in conds]
    labels = [(f"T={T:.0f} mu={m:+.2f}", T) for T, m in conds]
    g, _ = _gpu_chains(cm, ce, "semigrand_canonical", L, temps, mus, [None] * 3, 32, 4000, 500, 81)
    o = _oracle_chains(oracle_mod, ce, "semigrand_canonical", L, temps, mus, [None] * 3, 16, 1200,
                       200, 83)
    print(_compare(labels, g, o, int(np.prod(L)), sgc=True))


def test_semigrand_bcc_ternary_matches_oracle(cm, oracle_mod):
    """Semi-grand canonical BCC A/B/C (configuration 2's cluster expansion,
    two site functions), 8^3 conventional cells: <E>, <x_1>, <x_2>, C, the
    2 x 2 susceptibility and both thermo-chemical susceptibilities."""
    w = workloads.config(2, scale=1.0 / 128)
    ce, L = w.ce, (8, 8, 8)
    conds = [(1200.0, np.array([0.1, -0.1])), (700.0, np.array([-0.05, 0.05]))]
    temps = [T for T, _ in conds]
    mus = [m for _, m in conds]
    labels = [(f"T={T:.0f} mu=({m[0]:+.2f},{m[1]:+.2f})", T) for T, m in conds]
    g, _ = _gpu_chains(cm, ce, "semigrand_canonical", L, temps, mus, [None] * 2, 32, 4000, 500, 91)
    o = _oracle_chains(oracle_mod, ce, "semigrand_canonical", L, temps, mus, [None] * 2, 16, 1200,
                       200, 93)
    print(_compare(labels, g, o, int(np.prod(L)), sgc=True))


def test_canonical_bcc_ternary_matches_oracle(cm, oracle_mod):
    """Canonical ternary BCC A/B/C (configuration 2's cluster expansion, two
    sublattices, two site functions), 8^3 conventional cells at fixed
    composition (A 0.5, B 0.3, C 0.2): <E> and C at 1200 and 700 K. The GPU
    swaps pairs of different species inside colour classes and with
    neighbours; the oracle draws the reference's swap types."""
    w = workloads.config(2, scale=1.0 / 128)
    ce, L = w.ce, (8, 8, 8)
    n_sites = int(np.prod(L)) * ce.prim.n_basis
    counts = (n_sites // 2, (3 * n_sites) // 10)
    temps = [1200.0, 700.0]

    def initial(rng):
        occ = np.zeros(n_sites, dtype=np.int8)
        perm = rng.permutation(n_sites)
        occ[perm[:counts[1]]] = 1
        occ[perm[counts[1]:n_sites - counts[0]]] = 2
        return occ

    rng = np.random.default_rng(95)
    n_rep, n_o_rep = 32, 16
    sysd = cm.System(ce)
    b = cm.ReplicaBatch(sysd, "canonical", [L] * (len(temps) * n_rep))
    for c, T in enumerate(temps):
        for r in range(n_rep):
            i = c * n_rep + r
            b.set_conditions(i, T)
            b.set_seed(i, 9500 + i)
            b.set_occupation(i, initial(rng))
    n_pass, n_eq = 3000, 500
    b.run(n_pass, n_eq, record_samples=True)
    g = [[b.samples(c * n_rep + r, n_pass - n_eq)[0][:, None] for r in range(n_rep)]
         for c in range(len(temps))]
    o = oracle_mod.OracleSystem(ce, L)
    occ = np.ascontiguousarray(np.concatenate([initial(rng) for _ in range(len(temps) * n_o_rep)]),
                               dtype=np.int8)
    n_o, eq_o = 1200, 200
    pot, _, _ = o.run_chains(occ, 1, np.repeat(temps, n_o_rep), np.zeros((len(temps) * n_o_rep, 2)),
                             97, n_o, THREADS)
    ora = [[pot[c * n_o_rep + r, eq_o:, None] for r in range(n_o_rep)] for c in range(len(temps))]
    labels = [(f"BCC ternary canonical T={T:.0f}", T) for T in temps]
    print(_compare(labels, g, ora, int(np.prod(L)), sgc=False))
