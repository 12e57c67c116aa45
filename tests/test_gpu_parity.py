"""GPU path (through the C ABI) against the CPU FP64 oracle.

Tolerances: integer delta correlations and counts, replayed site and accept
sequences, occupations: bit-exact. Energies and dE: 1e-10 relative (the ECI
dot runs in float-float), with an absolute floor of 1e-12 eV."""

import os

import numpy as np
import pytest

from casmcode_clexmonte_gb300 import workloads
from casmcode_clexmonte_gb300.system import ClusterExpansion, fcc_prim

pytestmark = pytest.mark.gpu

RTOL = 1e-10
ATOL = 1e-12


@pytest.fixture(scope="module")
def cm():
    from casmcode_clexmonte_gb300 import build

    build.build()
    from casmcode_clexmonte_gb300 import calculator

    return calculator


def _close(a, b):
    a, b = np.asarray(a), np.asarray(b)
    assert np.all(np.abs(a - b) <= RTOL * np.abs(b) + ATOL), np.max(np.abs(a - b))


def _systems():
    t = ClusterExpansion(fcc_prim(4.0, ("A", "B", "Va")), {2: 4.1, 3: 4.01})
    t.eci = np.random.default_rng(11).normal(0, 0.05, t.n_funcs)
    return [
        ("fcc_binary", workloads.fcc_binary_ce(1), (10, 10, 10)),
        ("fcc_binary_odd", workloads.fcc_binary_ce(2), (7, 9, 11)),
        ("fcc_ternary", t, (6, 6, 6)),
        ("bcc_ternary", workloads.bcc_ternary_ce(3), (6, 5, 7)),
    ]


@pytest.mark.parametrize("name,ce,L", _systems())
def test_energy_and_delta_match_oracle(name, ce, L, cm, oracle_mod):
    sysd = cm.System(ce)
    ens = "semigrand_canonical"
    b = cm.ReplicaBatch(sysd, ens, [L])
    o = oracle_mod.OracleSystem(ce, L)
    rng = np.random.default_rng(5)
    nocc = ce.prim.n_occ
    mu = rng.uniform(-0.3, 0.3, nocc - 1)
    b.set_conditions(0, 800.0, mu)
    for trial in range(3):
        occ = rng.integers(0, nocc, o.n_sites).astype(np.int8)
        b.set_occupation(0, occ)
        e, counts = b.energy(0)
        oc = o.counts(occ)
        np.testing.assert_array_equal(counts[1:], oc[1:])
        _close(e, o.energy(occ))
        # single-site changes and two-site sequential events (incl. neighbours)
        n_ev = 400
        s1 = rng.integers(0, o.n_sites, n_ev)
        f1 = (occ[s1] + rng.integers(1, nocc, n_ev)) % nocc
        dE, dc = b.delta(0, s1[:, None], f1[:, None])
        dEp, _ = b.delta(0, s1[:, None], f1[:, None], potential=True)
        nb = np.array([o.n_sites])
        part_sites = []
        for k in range(n_ev):
            de_o, dc_o = o.delta(occ, [s1[k]], [f1[k]])
            np.testing.assert_array_equal(dc[k], dc_o)
            _close(dE[k], de_o)
            dep_o, _ = o.delta(occ, [s1[k]], [f1[k]], mu=mu)
            _close(dEp[k], dep_o)
        # swaps: random pairs and close pairs (second site sees the first change)
        s2 = np.where(rng.random(n_ev) < 0.5, rng.integers(0, o.n_sites, n_ev), (s1 + 1) % nb[0])
        ev_s = np.stack([s1, s2], 1)
        ev_f = np.stack([occ[s2], occ[s1]], 1)
        dE2, dc2 = b.delta(0, ev_s, ev_f)
        for k in range(n_ev):
            de_o, dc_o = o.delta(occ, ev_s[k], ev_f[k])
            np.testing.assert_array_equal(dc2[k], dc_o)
            _close(dE2[k], de_o)


@pytest.mark.parametrize("kind", ["sgc_config0", "canonical_fcc", "sgc_bcc_ternary"])
def test_replay_matches_oracle_exactly(kind, cm, oracle_mod):
    rng = np.random.default_rng(17)
    if kind == "sgc_config0":
        w = workloads.config(0)
        ce, L, ens, T, mu = w.ce, w.L[0], "semigrand_canonical", 1000.0, np.zeros(1)
        occ = w.occupation[0].copy()
        n_passes = 60
    elif kind == "canonical_fcc":
        ce, L, ens, T, mu = workloads.fcc_binary_ce(4), (8, 8, 8), "canonical", 600.0, np.zeros(1)
        occ = workloads.fixed_composition(rng, 512, 0.5)
        n_passes = 60
    else:
        ce, L, ens, T = workloads.bcc_ternary_ce(6), (5, 5, 5), "semigrand_canonical", 900.0
        mu = np.array([0.05, -0.1])
        occ = rng.integers(0, 3, 250).astype(np.int8)
        n_passes = 80
    o = oracle_mod.OracleSystem(ce, L)
    n = o.n_sites
    steps = n_passes * n
    seed = 987654321
    occ_o = occ.copy()
    ref = o.run(occ_o, 0 if ens == "semigrand_canonical" else 1, T, mu, seed, n_passes,
                record_steps=steps)
    sysd = cm.System(ce)
    b = cm.ReplicaBatch(sysd, ens, [L])
    b.set_conditions(0, T, mu if ens == "semigrand_canonical" else None)
    b.set_occupation(0, occ)
    got = b.replay(0, seed, steps)
    np.testing.assert_array_equal(got["sites"][:, 0], ref["site0"])
    np.testing.assert_array_equal(got["sites"][:, 1], ref["site1"])
    np.testing.assert_array_equal(got["accept"], ref["accept"])
    _close(got["dE"], ref["dE"])
    assert got["n_accept"] == ref["n_accept"]
    assert got["draws"] == ref["draws"]
    np.testing.assert_array_equal(b.get_occupation(0), occ_o)


@pytest.mark.parametrize("ens", ["semigrand_canonical", "canonical"])
def test_parallel_running_energy_and_invariants(ens, cm):
    ce = workloads.bcc_ternary_ce(8) if ens == "semigrand_canonical" else workloads.fcc_binary_ce(8)
    L = [(6, 6, 6), (7, 7, 7), (9, 9, 9)] if ens == "semigrand_canonical" else [(8, 8, 8), (10, 10, 10), (12, 12, 12)]
    sysd = cm.System(ce)
    b = cm.ReplicaBatch(sysd, ens, L)
    rng = np.random.default_rng(9)
    occs = []
    for i, l in enumerate(L):
        n = int(b.n_sites[i])
        if ens == "canonical":
            occ = workloads.fixed_composition(rng, n, 0.3 + 0.1 * i)
            b.set_conditions(i, 500.0 + 300 * i)
        else:
            occ = rng.integers(0, 3, n).astype(np.int8)
            b.set_conditions(i, 700.0 + 200 * i, rng.uniform(-0.2, 0.2, 2))
        b.set_seed(i, 1000 + i)
        b.set_occupation(i, occ)
        occs.append(occ)
    b.run(40, 10)
    for i in range(len(L)):
        st = b.stats(i)
        e, _ = b.energy(i)
        assert abs(st["energy"] - e) <= 1e-9 * max(1.0, abs(e))
        assert st["n_samples"] == 30
        assert st["n_accepted"] > 0
        new = b.get_occupation(i)
        assert new.min() >= 0 and new.max() < ce.prim.n_occ
        if ens == "canonical":
            assert np.bincount(new, minlength=2).tolist() == np.bincount(occs[i], minlength=2).tolist()


def test_parallel_deterministic_for_fixed_seed(cm):
    ce = workloads.fcc_binary_ce(1)
    sysd = cm.System(ce)
    outs = []
    for _ in range(2):
        b = cm.ReplicaBatch(sysd, "canonical", [(12, 12, 12)])
        b.set_conditions(0, 700.0)
        b.set_seed(0, 77)
        b.set_occupation(0, workloads.fixed_composition(np.random.default_rng(1), 1728, 0.5))
        b.run(20, 0)
        outs.append(b.get_occupation(0))
    np.testing.assert_array_equal(outs[0], outs[1])


@pytest.mark.parametrize("ens,edge", [("semigrand_canonical", 8), ("canonical", 8),
                                      ("semigrand_canonical", 9), ("canonical", 9)])
def test_parallel_equilibrium_matches_oracle(ens, edge, cm, oracle_mod):
    """Equilibrium averages of the parallel GPU sampler against the oracle's
    sequential chains, 8^3 and 9^3 FCC (configuration 0's expansion; an odd
    edge takes colour blocks of unequal sizes) at 900 K: <E> and C, and
    semi-grand canonical also <x>, chi and the thermo-chemical chi.
    Independent chains on each side (GPU 16, oracle 16), pooled, jackknife
    errors, >= 50 tau_int per chain, 2 sigma per comparison under the
    family-wise contract of tests/test_gpu_equilibrium.py."""
    from tests.stat_checks import compare

    ce = workloads.fcc_binary_ce(0)
    L = (edge, edge, edge)
    n, nrep = edge ** 3, 16
    T = 900.0
    mu = np.array([0.05])
    sgc = ens == "semigrand_canonical"
    rng = np.random.default_rng(21)
    inits = [workloads.fixed_composition(rng, n, 0.4) for _ in range(2 * nrep)]
    o = oracle_mod.OracleSystem(ce, L)
    n_o, eq_o = 1500, 300
    occ = np.ascontiguousarray(np.concatenate(inits[:nrep]), dtype=np.int8)
    pot, comp, _ = o.run_chains(occ, 0 if sgc else 1, np.full(nrep, T), np.tile(mu, (nrep, 1)), 5,
                                n_o, os.cpu_count() or 1)
    ora = [np.column_stack([pot[i, eq_o:], comp[i, eq_o:]]) for i in range(nrep)]
    sysd = cm.System(ce)
    b = cm.ReplicaBatch(sysd, ens, [L] * nrep)
    for i in range(nrep):
        b.set_conditions(i, T, mu if sgc else None)
        b.set_seed(i, 100 + i)
        b.set_occupation(i, inits[nrep + i])
    n_pass, n_eq = 3000, 500
    b.run(n_pass, n_eq, record_samples=True)
    gpu = []
    for i in range(nrep):
        p_i, c_i = b.samples(i, n_pass - n_eq)
        gpu.append(np.column_stack([p_i, c_i.reshape(n_pass - n_eq, -1)]))
    print(compare([(f"{edge}^3 {ens} T={T:.0f}", T)], [gpu], [ora], n, sgc=sgc))


@pytest.mark.parametrize("ens,L", [("canonical", (24, 24, 24)), ("semigrand_canonical", (10, 10, 10)),
                                   ("canonical", (30, 30, 30))])
def test_generated_evaluator_matches_runtime_tables(ens, L, cm):
    """The generated binary FCC evaluator and the run-time table walk make
    the same decisions: identical occupations and statistics."""
    ce = workloads.fcc_binary_ce(2)
    sysd = cm.System(ce)
    rng = np.random.default_rng(4)
    n = L[0] * L[1] * L[2]
    occ0 = workloads.fixed_composition(rng, n, 0.35)
    out = []
    for generic in (False, True):
        b = cm.ReplicaBatch(sysd, ens, [L, L])
        if generic:
            b.set_option("generic_evaluator", 1)
            assert b.get_option("pitch") == 0
        else:
            assert b.get_option("pitch") == {24: 28, 10: 14, 30: 64}[L[0]]
        for i in range(2):
            b.set_conditions(i, 500.0 + 400 * i, np.array([0.02]) if ens != "canonical" else None)
            b.set_seed(i, 31 + i)
            b.set_occupation(i, occ0)
        b.run(25, 5)
        out.append([(b.get_occupation(i), b.stats(i)) for i in range(2)])
    for (oa, sa), (ob, sb) in zip(*out):
        np.testing.assert_array_equal(oa, ob)
        assert sa["n_accepted"] == sb["n_accepted"] and sa["n_proposed"] == sb["n_proposed"]
        assert abs(sa["energy"] - sb["energy"]) <= 1e-9 * abs(sb["energy"]) + 1e-9


def test_order_parameter_samples_match_final_state(cm):
    """The per-pass L1_2 order parameter of the plain sweep equals the one
    recomputed from the final occupation."""
    ce = workloads.fcc_binary_ce(3, nn1=0.08)
    sysd = cm.System(ce)
    L = (24, 24, 24)
    b = cm.ReplicaBatch(sysd, "canonical", [L])
    rng = np.random.default_rng(8)
    b.set_conditions(0, 250.0)
    b.set_seed(0, 3)
    b.set_occupation(0, workloads.fixed_composition(rng, 24 ** 3, 0.25))
    b.run(30, 0, record_samples=True)
    op = b.order_samples(0, 30)
    assert op.size == 30
    occ = b.get_occupation(0).reshape(24, 24, 24)  # [z][y][x]
    z, y, x = np.meshgrid(np.arange(24), np.arange(24), np.arange(24), indexing="ij")
    lab = ((y + z) & 1) | (((x + z) & 1) << 1)
    xb = occ.mean()
    c = np.array([occ[lab == k].mean() for k in range(4)])
    assert abs(op[-1] - np.sqrt(((c - xb) ** 2).sum())) < 1e-12


@pytest.mark.parametrize("ens", ["canonical", "semigrand_canonical"])
def test_streamed_sweep_matches_shared_memory_sweep(ens, cm):
    """The HBM-streamed path (one kernel per colour sub-step, CUDA graph per
    pass) runs the same chain as the shared-memory sweep: identical
    occupations, counts, energies and samples."""
    ce = workloads.fcc_binary_ce(5, nn1=0.08)
    sysd = cm.System(ce)
    L = (24, 24, 24)
    rng = np.random.default_rng(2)
    occs = [workloads.fixed_composition(rng, 24 ** 3, x) for x in (0.25, 0.5)]
    out = []
    for streamed in (False, True):
        b = cm.ReplicaBatch(sysd, ens, [L, L])
        if streamed:
            b.set_option("streamed", 1)
        assert b.get_option("streamed") == int(streamed)
        for i in range(2):
            b.set_conditions(i, 300.0 + 400 * i, np.array([0.01]) if ens != "canonical" else None)
            b.set_seed(i, 17 + i)
            b.set_occupation(i, occs[i])
        b.run(12, 2, record_samples=True)
        b.run(8, 0, record_samples=True)
        res = []
        for i in range(2):
            pot, comp = b.samples(i, 8)
            res.append((b.get_occupation(i), b.stats(i), pot, b.order_samples(i, 8)))
        out.append(res)
    for (oa, sa, pa, qa), (ob, sb, pb, qb) in zip(*out):
        np.testing.assert_array_equal(oa, ob)
        assert sa["n_accepted"] == sb["n_accepted"] and sa["n_proposed"] == sb["n_proposed"]
        assert sa["energy"] == sb["energy"]
        np.testing.assert_array_equal(pa, pb)
        np.testing.assert_array_equal(qa, qb)
