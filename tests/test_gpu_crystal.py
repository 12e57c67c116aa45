"""General crystals on the GPU, through the C ABI: the reference's
Clex_ZrO_Occ system (hcp Zr, O/Va on the octahedral sites; 73 orbits, 1591
clusters per site, a real CASM basis set) against the oracle, and the
orbit-at-a-time sweep kernel that such systems use against the register
accumulator sweep.

Tolerances as in test_gpu_parity: integer counts and delta correlations,
replayed sequences and occupations bit-exact; energies 1e-10 relative."""

import os

import numpy as np
import pytest

from casmcode_clexmonte_gb300 import workloads
from tests.stat_checks import compare
from tests.zro_fixture import zro_ce

pytestmark = pytest.mark.gpu

RTOL = 1e-10
ATOL = 1e-12
L = (8, 8, 8)


@pytest.fixture(scope="module")
def cm():
    from casmcode_clexmonte_gb300 import build

    build.build()
    from casmcode_clexmonte_gb300 import calculator

    return calculator


@pytest.fixture(scope="module")
def ce():
    return zro_ce()


def _close(a, b):
    a, b = np.asarray(a), np.asarray(b)
    assert np.all(np.abs(a - b) <= RTOL * np.abs(b) + ATOL), np.max(np.abs(a - b))


def test_zro_energy_and_delta_match_oracle(ce, cm, oracle_mod):
    sysd = cm.System(ce)
    b = cm.ReplicaBatch(sysd, "semigrand_canonical", [L])
    assert b.get_option("pitch") == -2  # binary: one warp per site change
    o = oracle_mod.OracleSystem(ce, L)
    rng = np.random.default_rng(3)
    mu = np.array([-0.4])
    b.set_conditions(0, 1500.0, mu)
    for x in (0.2, 0.6):
        occ = (rng.random(o.n_sites) < x).astype(np.int8)
        b.set_occupation(0, occ)
        e, counts = b.energy(0)
        np.testing.assert_array_equal(counts[1:], o.counts(occ)[1:])
        _close(e, o.energy(occ))
        n_ev = 200
        s1 = rng.integers(0, o.n_sites, n_ev)
        f1 = 1 - occ[s1]
        dE, dc = b.delta(0, s1[:, None], f1[:, None])
        dEp, _ = b.delta(0, s1[:, None], f1[:, None], potential=True)
        for k in range(n_ev):
            de_o, dc_o = o.delta(occ, [s1[k]], [f1[k]])
            np.testing.assert_array_equal(dc[k], dc_o)
            _close(dE[k], de_o)
            dep_o, _ = o.delta(occ, [s1[k]], [f1[k]], mu=mu)
            _close(dEp[k], dep_o)
        # swaps: random pairs and pairs inside one cluster (c-axis neighbours,
        # site l of sublattice 0 and site l + n_uc of sublattice 1)
        n_uc = o.n_uc
        s2 = np.where(rng.random(n_ev) < 0.5, rng.integers(0, o.n_sites, n_ev),
                      (s1 % n_uc) + n_uc * (1 - s1 // n_uc))
        ev_s = np.stack([s1, s2], 1)
        ev_f = np.stack([occ[s2], occ[s1]], 1)
        dE2, dc2 = b.delta(0, ev_s, ev_f)
        for k in range(n_ev):
            de_o, dc_o = o.delta(occ, ev_s[k], ev_f[k])
            np.testing.assert_array_equal(dc2[k], dc_o)
            _close(dE2[k], de_o)


@pytest.mark.parametrize("ens", ["semigrand_canonical", "canonical"])
def test_zro_replay_matches_oracle_exactly(ens, ce, cm, oracle_mod):
    rng = np.random.default_rng(23)
    o = oracle_mod.OracleSystem(ce, L)
    n = o.n_sites
    occ = (rng.random(n) < 0.5).astype(np.int8)
    T, mu = 3000.0, np.array([-0.3])
    n_passes = 4
    steps = n_passes * n
    seed = 24681357
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
    assert got["n_accept"] == ref["n_accept"] > 0
    np.testing.assert_array_equal(b.get_occupation(0), occ_o)


@pytest.mark.parametrize("ens", ["semigrand_canonical", "canonical"])
def test_orbit_walk_matches_register_sweep_ternary(ens, cm):
    """For three occupants both kernels fold the same float-float terms in
    the same order: identical chains."""
    ce = workloads.bcc_ternary_ce(4)
    sysd = cm.System(ce)
    Ls = [(6, 6, 6), (7, 7, 7)]
    rng = np.random.default_rng(12)
    occ0 = [rng.integers(0, 3, 2 * int(np.prod(x))).astype(np.int8) for x in Ls]
    mus = [rng.uniform(-0.2, 0.2, 2) if ens != "canonical" else None for _ in Ls]
    out = []
    for walk in (False, True):
        b = cm.ReplicaBatch(sysd, ens, Ls)
        if walk:
            b.set_option("orbit_walk", 1)
            assert b.get_option("pitch") == -1
        for i in range(2):
            b.set_conditions(i, 800.0 + 300 * i, mus[i])
            b.set_seed(i, 71 + i)
            b.set_occupation(i, occ0[i])
        b.run(20, 5)
        out.append([(b.get_occupation(i), b.stats(i)) for i in range(2)])
    for (oa, sa), (ob, sb) in zip(*out):
        np.testing.assert_array_equal(oa, ob)
        assert sa["n_accepted"] == sb["n_accepted"] and sa["n_proposed"] == sb["n_proposed"]
        assert abs(sa["energy"] - sb["energy"]) <= 1e-9 * abs(sb["energy"]) + 1e-9


@pytest.mark.parametrize("walk", [1, 2])
def test_orbit_walk_binary_running_energy(walk, cm):
    """Binary FCC through the large-expansion kernels (1: one thread per site,
    orbit by orbit; 2: one warp per site change): the FP64 running energy
    equals a fresh recompute; canonical composition is kept."""
    ce = workloads.fcc_binary_ce(5)
    sysd = cm.System(ce)
    b = cm.ReplicaBatch(sysd, "canonical", [(12, 12, 12)] * 3)
    b.set_option("orbit_walk", walk)
    assert b.get_option("pitch") == -walk
    rng = np.random.default_rng(2)
    occs = []
    for i in range(3):
        occ = workloads.fixed_composition(rng, 1728, 0.3 + 0.1 * i)
        occs.append(occ)
        b.set_conditions(i, 400.0 + 300 * i)
        b.set_seed(i, 5 + i)
        b.set_occupation(i, occ)
    b.run(30, 5)
    for i in range(3):
        st = b.stats(i)
        e, _ = b.energy(i)
        assert abs(st["energy"] - e) <= 1e-9 * max(1.0, abs(e))
        assert st["n_accepted"] > 0
        assert int(b.get_occupation(i).sum()) == int(occs[i].sum())


@pytest.mark.parametrize("walk", [0, 1])
@pytest.mark.parametrize("ens", ["semigrand_canonical", "canonical"])
def test_zro_sweep_running_energy_and_invariants(ens, walk, ce, cm):
    sysd = cm.System(ce)
    Ls = [(8, 8, 8), (9, 9, 8), (12, 12, 8)]
    b = cm.ReplicaBatch(sysd, ens, Ls)
    if walk:
        b.set_option("orbit_walk", walk)
    rng = np.random.default_rng(31)
    occs = []
    for i, x in enumerate(Ls):
        n = int(b.n_sites[i])
        occ = (rng.random(n) < 0.3 + 0.2 * i).astype(np.int8)
        occs.append(occ)
        b.set_conditions(i, 1200.0 + 400 * i, np.array([-0.5 + 0.2 * i]) if ens != "canonical" else None)
        b.set_seed(i, 900 + i)
        b.set_occupation(i, occ)
    b.run(20, 5)
    for i in range(len(Ls)):
        st = b.stats(i)
        e, _ = b.energy(i)
        assert abs(st["energy"] - e) <= 1e-9 * max(1.0, abs(e))
        assert st["n_samples"] == 15 and st["n_accepted"] > 0
        new = b.get_occupation(i)
        assert set(np.unique(new)) <= {0, 1}
        if ens == "canonical":
            assert int(new.sum()) == int(occs[i].sum())


@pytest.mark.parametrize("ens,walk", [("semigrand_canonical", 0), ("semigrand_canonical", 1),
                                      ("canonical", 0)])
def test_zro_equilibrium_matches_oracle(ens, walk, ce, cm, oracle_mod):
    """Equilibrium averages of the parallel sampler on the reference's ZrO
    basis set (default: one warp per site change or swap; 1: one thread per
    site, orbit by orbit) against the oracle's sequential chains, 8^3 cells at
    2500 K: <E> and C, and semi-grand canonical also <x>, chi and the
    thermo-chemical chi. Independent chains on each side (GPU 16, oracle 16),
    pooled, jackknife errors, >= 50 tau_int per chain, 2 sigma per comparison
    under the family-wise contract (tests/test_gpu_equilibrium.py)."""
    T, mu = 2500.0, np.array([-0.6])
    sgc = ens == "semigrand_canonical"
    o = oracle_mod.OracleSystem(ce, L)
    n, nrep = o.n_sites, 16
    rng = np.random.default_rng(41)

    def initial():
        if sgc:
            return (rng.random(n) < 0.5).astype(np.int8)
        return workloads.fixed_composition(rng, n, 0.5)

    n_o, eq_o = 800, 150
    occ = np.ascontiguousarray(np.concatenate([initial() for _ in range(nrep)]), dtype=np.int8)
    pot, comp, _ = o.run_chains(occ, 0 if sgc else 1, np.full(nrep, T), np.tile(mu, (nrep, 1)), 11,
                                n_o, os.cpu_count() or 1)
    ora = [np.column_stack([pot[i, eq_o:], comp[i, eq_o:]]) for i in range(nrep)]
    sysd = cm.System(ce)
    b = cm.ReplicaBatch(sysd, ens, [L] * nrep)
    if walk:
        b.set_option("orbit_walk", walk)
    for i in range(nrep):
        b.set_conditions(i, T, mu if sgc else None)
        b.set_seed(i, 300 + i)
        b.set_occupation(i, initial())
    n_pass, n_eq = 1000, 200
    b.run(n_pass, n_eq, record_samples=True)
    gpu = []
    for i in range(nrep):
        p_i, c_i = b.samples(i, n_pass - n_eq)
        gpu.append(np.column_stack([p_i, c_i.reshape(n_pass - n_eq, -1)]))
    label = f"ZrO {ens} walk={walk} T={T:.0f}"
    print(compare([(label, T)], [gpu], [ora], int(np.prod(L)), sgc=sgc))


def test_zro_nfold_matches_oracle_event_for_event(ce, cm, oracle_mod):
    """The n-fold way on the ZrO basis set (run-time tables walked one orbit
    at a time): event sequence, residence weights and final occupation equal
    the oracle's, which recomputes every rate after every event."""
    rng = np.random.default_rng(29)
    Ls = (7, 7, 7)
    sysd = cm.System(ce)
    b = cm.ReplicaBatch(sysd, "semigrand_canonical", [Ls])
    T, mu = 1800.0, np.array([-0.5])
    b.set_conditions(0, T, mu)
    seed = 0x5EED0F2
    b.set_seed(0, seed)
    occ = (rng.random(2 * 343) < 0.4).astype(np.int8)
    b.set_occupation(0, occ)
    n_events, n_equil = 120, 20
    rec = b.nfold_run(n_events, n_equil, record=n_events + n_equil)
    o = oracle_mod.OracleSystem(ce, Ls)
    occ_o = occ.copy()
    ref = o.nfold(occ_o, T, mu, sysd.arrays["weights"], seed, n_events, n_equil,
                  record=n_events + n_equil)
    np.testing.assert_array_equal(rec["site"][0], ref["site"])
    np.testing.assert_array_equal(rec["occ"][0], ref["occ"])
    np.testing.assert_array_equal(rec["dt"][0], ref["dt"])
    np.testing.assert_array_equal(b.get_occupation(0), occ_o)
    e_now, _ = b.energy(0)
    assert b.stats(0)["energy"] == pytest.approx(e_now, rel=1e-9, abs=1e-9)


def test_zro_enforce_matches_oracle(ce, cm, oracle_mod):
    """Composition enforcement on the O/Va sublattices: same flips as the
    oracle's restatement of clexmonte::enforce_composition."""
    Ls = [(8, 8, 8), (12, 12, 8)]
    sysd = cm.System(ce)
    b = cm.ReplicaBatch(sysd, "canonical", Ls)
    rng = np.random.default_rng(4)
    occs, targets = [], []
    for i, L in enumerate(Ls):
        n = 2 * L[0] * L[1] * L[2]
        occ = (rng.random(n) < 0.2).astype(np.int8)
        b.set_occupation(i, occ)
        occs.append(occ)
        x = 0.3 + 0.4 * i  # O per O/Va site
        targets.append(np.array([2 * (1 - x), 2 * x]))  # Va, O per unit cell
    seed = 0xBEEF
    flips = b.enforce_composition(np.array(targets), seed)
    for i, L in enumerate(Ls):
        o = oracle_mod.OracleSystem(ce, L)
        ref = occs[i].copy()
        nf, _ = o.enforce_composition(ref, targets[i], seed + i)
        assert flips[i] == nf > 0
        np.testing.assert_array_equal(b.get_occupation(i), ref)


@pytest.mark.parametrize("ens", ["semigrand_canonical", "canonical"])
def test_zro_16bit_records_match_32bit(ens, ce, cm):
    """The cooperative sweep's 16-bit cluster records (offsets and integer
    weights packed two per word) give the same sums as the 32-bit records:
    identical chains."""
    sysd = cm.System(ce)
    Ls = [(8, 8, 8), (10, 10, 8)]
    rng = np.random.default_rng(8)
    occs = [(rng.random(2 * int(np.prod(x))) < 0.45).astype(np.int8) for x in Ls]
    out = []
    for wide in (0, 1):
        b = cm.ReplicaBatch(sysd, ens, Ls)
        b.set_option("wide_records", wide)
        for i in range(len(Ls)):
            b.set_conditions(i, 1500.0 + 500 * i, np.array([-0.4]) if ens != "canonical" else None)
            b.set_seed(i, 61 + i)
            b.set_occupation(i, occs[i])
        b.run(12, 2)
        out.append([(b.get_occupation(i), b.stats(i)) for i in range(len(Ls))])
    for (oa, sa), (ob, sb) in zip(*out):
        np.testing.assert_array_equal(oa, ob)
        assert sa["n_accepted"] == sb["n_accepted"] and sa["energy"] == sb["energy"]
