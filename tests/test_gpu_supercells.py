"""Non-diagonal supercells (transformation_matrix_to_super,
include/casm/clexmonte/state/Configuration.hh:29-50) on the GPU through the C
ABI: against the oracle on the same supercell, and against a diagonal
supercell that tiles it (the diagonal path is the pinned one).

Tolerances as in tests/test_gpu_parity.py: cluster counts, delta counts,
replayed sites, accept sequences and occupations bit-exact; energies and dE
1e-10 relative with a 1e-12 eV floor."""

import numpy as np
import pytest

from casmcode_clexmonte_gb300 import workloads

pytestmark = pytest.mark.gpu

RTOL = 1e-10
ATOL = 1e-12
FCC_CONV = np.array([[-1, 1, 1], [1, -1, 1], [1, 1, -1]])
GENERAL = np.array([[6, 0, 0], [3, 6, 0], [3, 3, 6]]) @ np.array([[1, 1, 0], [0, 1, 1], [1, 1, 1]])
SUPERCELLS = {
    "fcc_conventional_2": 2 * FCC_CONV,
    "fcc_conventional_5": 5 * FCC_CONV,
    "sheared": np.array([[6, 0, 0], [3, 6, 0], [0, 0, 6]]),
    "general": GENERAL,
}


@pytest.fixture(scope="module")
def cm():
    from casmcode_clexmonte_gb300 import build

    build.build()
    from casmcode_clexmonte_gb300 import calculator

    return calculator


def _close(a, b):
    a, b = np.asarray(a), np.asarray(b)
    assert np.all(np.abs(a - b) <= RTOL * np.abs(b) + ATOL), np.max(np.abs(a - b))


def _ce(system):
    return workloads.fcc_binary_ce(1) if system == "fcc_binary" else workloads.bcc_ternary_ce(3)


@pytest.mark.parametrize("name", list(SUPERCELLS))
@pytest.mark.parametrize("system", ["fcc_binary", "bcc_ternary"])
def test_energy_and_delta_match_oracle(system, name, cm, oracle_mod):
    ce, T = _ce(system), SUPERCELLS[name]
    nocc = ce.prim.n_occ
    b = cm.ReplicaBatch(cm.System(ce), "semigrand_canonical", [T])
    o = oracle_mod.OracleSystem(ce, T)
    assert b.n_sites[0] == o.n_sites
    rng = np.random.default_rng(7)
    mu = rng.uniform(-0.3, 0.3, nocc - 1)
    b.set_conditions(0, 800.0, mu)
    for _ in range(2):
        occ = rng.integers(0, nocc, o.n_sites).astype(np.int8)
        b.set_occupation(0, occ)
        e, counts = b.energy(0)
        np.testing.assert_array_equal(counts[1:], o.counts(occ)[1:])
        _close(e, o.energy(occ))
        n_ev = 200
        s1 = rng.integers(0, o.n_sites, n_ev)
        f1 = (occ[s1] + rng.integers(1, nocc, n_ev)) % nocc
        dE, dc = b.delta(0, s1[:, None], f1[:, None])
        dEp, _ = b.delta(0, s1[:, None], f1[:, None], potential=True)
        for k in range(n_ev):
            de_o, dc_o = o.delta(occ, [s1[k]], [f1[k]])
            np.testing.assert_array_equal(dc[k], dc_o)
            _close(dE[k], de_o)
            _close(dEp[k], o.delta(occ, [s1[k]], [f1[k]], mu=mu)[0])
        # swaps with random partners and with the next unit cell's site (the
        # second site sees the first change)
        s2 = np.where(rng.random(n_ev) < 0.5, rng.integers(0, o.n_sites, n_ev),
                      (s1 + 1) % o.n_sites)
        ev_s, ev_f = np.stack([s1, s2], 1), np.stack([occ[s2], occ[s1]], 1)
        dE2, dc2 = b.delta(0, ev_s, ev_f)
        for k in range(n_ev):
            de_o, dc_o = o.delta(occ, ev_s[k], ev_f[k])
            np.testing.assert_array_equal(dc2[k], dc_o)
            _close(dE2[k], de_o)


@pytest.mark.parametrize("kind", ["canonical_fcc_conventional_5", "sgc_bcc_general"])
def test_replay_matches_oracle_exactly(kind, cm, oracle_mod):
    rng = np.random.default_rng(19)
    if kind == "canonical_fcc_conventional_5":
        ce, T, ens, temp, mu = workloads.fcc_binary_ce(4), SUPERCELLS["fcc_conventional_5"], "canonical", 600.0, np.zeros(1)
    else:
        ce, T, ens, temp, mu = workloads.bcc_ternary_ce(6), GENERAL, "semigrand_canonical", 900.0, np.array([0.05, -0.1])
    o = oracle_mod.OracleSystem(ce, T)
    n = o.n_sites
    occ = (workloads.fixed_composition(rng, n, 0.5) if ens == "canonical"
           else rng.integers(0, 3, n).astype(np.int8))
    n_passes, seed = 30, 1234567
    occ_o = occ.copy()
    ref = o.run(occ_o, 0 if ens == "semigrand_canonical" else 1, temp, mu, seed, n_passes,
                record_steps=n_passes * n)
    b = cm.ReplicaBatch(cm.System(ce), ens, [T])
    b.set_conditions(0, temp, mu if ens == "semigrand_canonical" else None)
    b.set_occupation(0, occ)
    got = b.replay(0, seed, n_passes * n)
    np.testing.assert_array_equal(got["sites"][:, 0], ref["site0"])
    np.testing.assert_array_equal(got["sites"][:, 1], ref["site1"])
    np.testing.assert_array_equal(got["accept"], ref["accept"])
    _close(got["dE"], ref["dE"])
    assert got["n_accept"] == ref["n_accept"] and got["draws"] == ref["draws"]
    np.testing.assert_array_equal(b.get_occupation(0), occ_o)


def _cell_index(H, i, j, k):
    L0, L1, L2 = int(H[0, 0]), int(H[1, 1]), int(H[2, 2])
    q = i // L0
    i, j, k = i - q * L0, j - q * int(H[1, 0]), k - q * int(H[2, 0])
    q = j // L1
    j, k = j - q * L1, k - q * int(H[2, 1])
    return i + L0 * (j + L1 * (k % L2))


@pytest.mark.parametrize("name", ["fcc_conventional_5", "sheared"])
def test_gpu_supercell_matches_its_diagonal_tiling(name, cm, oracle_mod):
    """The non-diagonal replica and the diagonal supercell D that tiles it, in
    one batch: D's counts are m times T's (m = 2 images per site), and one
    site change on T changes them by 1/m of the change of all its images."""
    ce, T = workloads.fcc_binary_ce(2), SUPERCELLS[name]
    H = oracle_mod.hermite_lower(T)
    d = tuple(next(x for x in range(1, 1000) if _cell_index(H, *(x * e)) == 0)
              for e in np.eye(3, dtype=int))
    k, j, i = np.meshgrid(np.arange(d[2]), np.arange(d[1]), np.arange(d[0]), indexing="ij")
    img = _cell_index(H, i.ravel(), j.ravel(), k.ravel())
    b = cm.ReplicaBatch(cm.System(ce), "canonical", [T, np.diag(d)])
    n_t, n_d = int(b.n_sites[0]), int(b.n_sites[1])
    m = n_d // n_t
    assert m == 2
    rng = np.random.default_rng(23)
    occ_t = workloads.fixed_composition(rng, n_t, 0.4)
    occ_d = occ_t[img]  # one sublattice
    b.set_occupation(0, occ_t)
    b.set_occupation(1, occ_d)
    e_t, c_t = b.energy(0)
    e_d, c_d = b.energy(1)
    np.testing.assert_array_equal(c_d[1:], m * c_t[1:])
    s = rng.integers(0, n_t, 100)
    f = 1 - occ_t[s]
    _, dc_t = b.delta(0, s[:, None], f[:, None])
    images = np.array([np.nonzero(img == x)[0] for x in s])
    _, dc_d = b.delta(1, images, np.repeat(f[:, None], m, 1))
    np.testing.assert_array_equal(dc_d[:, 1:], m * dc_t[:, 1:])


def test_parallel_runs_refuse_and_exact_paths_work(cm, oracle_mod):
    ce = workloads.fcc_binary_ce(2)
    T = SUPERCELLS["fcc_conventional_5"]
    b = cm.ReplicaBatch(cm.System(ce), "canonical", [(8, 8, 8), T])
    with pytest.raises(RuntimeError, match="parallel runs need diagonal supercells"):
        b.run(1, 0)
    with pytest.raises(RuntimeError, match="parallel runs need diagonal supercells"):
        b.autotune(1)
    # composition enforcement and state transfer work on every replica
    rng = np.random.default_rng(3)
    occs = [np.zeros(int(n), np.int8) for n in b.n_sites]
    for i, occ in enumerate(occs):
        b.set_occupation(i, occ)
    target = np.array([0.7, 0.3])
    seed = 77
    flips = b.enforce_composition(target, seed)
    o = oracle_mod.OracleSystem(ce, T)
    ref = occs[1].copy()
    nf, _ = o.enforce_composition(ref, target, seed + 1)
    assert flips[1] == nf
    np.testing.assert_array_equal(b.get_occupation(1), ref)
    occ, st = b.get_state(1)
    c = cm.ReplicaBatch(cm.System(ce), "canonical", [T])
    c.set_state(0, occ, st)
    np.testing.assert_array_equal(c.get_occupation(0), ref)
    assert c.energy(0)[0] == pytest.approx(o.energy(ref), rel=1e-10)


def test_cluster_on_two_images_is_refused(cm):
    """The conventional FCC cell: a second-neighbour pair joins a site and its
    own image."""
    sysd = cm.System(workloads.fcc_binary_ce(2))
    with pytest.raises(RuntimeError, match="supercell too small"):
        cm.ReplicaBatch(sysd, "canonical", [FCC_CONV])
    with pytest.raises(RuntimeError, match="singular"):
        cm.ReplicaBatch(sysd, "canonical", [np.array([[1, 2, 3], [2, 4, 6], [0, 0, 1]])])


def test_python_calculator_with_a_supercell_matrix(cm, oracle_mod):
    """The libcasm.clexmonte-style mirror on a non-diagonal state: the
    potential and the replay work, a parallel run says why it cannot."""
    ce, T = workloads.fcc_binary_ce(5), SUPERCELLS["sheared"]
    o = oracle_mod.OracleSystem(ce, T)
    rng = np.random.default_rng(29)
    occ = workloads.fixed_composition(rng, o.n_sites, 0.5)
    state = cm.MonteCarloState(occupation=occ.copy(), L=T, conditions={"temperature": 700.0})
    calc = cm.MonteCalculator("canonical", cm.System(ce))
    pot = calc.set_state_and_potential(state)
    _close(pot.per_supercell(), o.energy(occ))
    _close(pot.per_unitcell(), o.energy(occ) / 216)
    for s in rng.integers(0, o.n_sites, 20):
        _close(pot.occ_delta_per_supercell([s], [1 - occ[s]]), o.delta(occ, [s], [1 - occ[s]])[0])
    occ_o = occ.copy()
    ref = o.run(occ_o, 1, 700.0, np.zeros(1), 42, 5, record_steps=5 * o.n_sites)
    got = calc.replay(state, 42, 5 * o.n_sites)
    np.testing.assert_array_equal(got["accept"], ref["accept"])
    np.testing.assert_array_equal(state.occupation, occ_o)
    with pytest.raises(RuntimeError, match="parallel runs need diagonal supercells"):
        calc.run_fixture(state, cm.SamplingFixtureParams(n_passes=10, n_equil=0))


@pytest.mark.parametrize("T", [None, "fcc_conventional"])
def test_make_canonical_initial_state(T, cm, oracle_mod):
    """Default motif (pure A) in the scaled supercell, composition enforced to
    x_B = 0.25 with the oracle's flips, composition conditions matched."""
    ce = workloads.fcc_binary_ce(2)
    calc = cm.MonteCalculator("canonical", cm.System(ce))
    Tm = None if T is None else FCC_CONV
    state, motif = cm.make_canonical_initial_state(
        calc, {"temperature": 600.0, "param_composition": [0.25]}, min_volume=1000,
        transformation_matrix_to_super=Tm, seed=11)
    n_uc = 1000 if T is None else 1372
    assert state.occupation.size == n_uc
    if T is None:
        assert tuple(state.L) == (10, 10, 10)
    ref = np.zeros(n_uc, dtype=np.int8)
    o = oracle_mod.OracleSystem(ce, (10, 10, 10) if T is None else 7 * FCC_CONV)
    o.enforce_composition(ref, cm.mol_composition(calc.system, [0.25]), 11)
    np.testing.assert_array_equal(state.occupation, ref)
    assert abs(state.occupation.sum() - 0.25 * n_uc) <= 1
    np.testing.assert_allclose(state.conditions["param_composition"], [state.occupation.sum() / n_uc])
    np.testing.assert_allclose(state.conditions["mol_composition"],
                               [1 - state.occupation.sum() / n_uc, state.occupation.sum() / n_uc])
    pot = calc.set_state_and_potential(state)
    assert pot.per_supercell() == pytest.approx(o.energy(state.occupation), rel=1e-10)


@pytest.mark.parametrize("kind", ["fcc_sheared_10", "fcc_conventional_2", "bcc_ternary_general"])
def test_nfold_matches_oracle_event_for_event(kind, cm, oracle_mod):
    """The n-fold way on non-diagonal supercells (twisted halo images): the
    event sequence, residence times and final occupation equal the oracle's.
    fcc_sheared_10: box 10 x 10 x 10 with one twist, the generated evaluator;
    fcc_conventional_2: box 2 x 4 x 4, thinner than the cluster reach along x."""
    rng = np.random.default_rng(41)
    if kind == "fcc_sheared_10":
        ce, T, temp, mu = workloads.fcc_binary_ce(3), np.array([[10, 0, 0], [5, 10, 0], [0, 0, 10]]), 600.0, np.array([0.02])
    elif kind == "fcc_conventional_2":
        ce, T, temp, mu = workloads.fcc_binary_ce(2), SUPERCELLS["fcc_conventional_2"], 700.0, np.array([0.0])
    else:
        ce, T, temp, mu = workloads.bcc_ternary_ce(6), GENERAL, 900.0, np.array([0.05, -0.1])
    nocc = ce.prim.n_occ
    o = oracle_mod.OracleSystem(ce, T)
    occ = rng.integers(0, nocc, o.n_sites).astype(np.int8)
    sysd = cm.System(ce)
    b = cm.ReplicaBatch(sysd, "semigrand_canonical", [T])
    b.set_conditions(0, temp, mu)
    seed = 0x5EEDF00D
    b.set_seed(0, seed)
    b.set_occupation(0, occ)
    n_events, n_equil = 300, 40
    rec = b.nfold_run(n_events, n_equil, record=n_events + n_equil)
    occ_o = occ.copy()
    ref = o.nfold(occ_o, temp, mu, sysd.arrays["weights"], seed, n_events, n_equil,
                  record=n_events + n_equil)
    assert ref["n"] == n_events + n_equil
    np.testing.assert_array_equal(rec["site"][0], ref["site"])
    np.testing.assert_array_equal(rec["occ"][0], ref["occ"])
    np.testing.assert_array_equal(rec["dt"][0], ref["dt"])
    np.testing.assert_array_equal(b.get_occupation(0), occ_o)
    e_now, _ = b.energy(0)
    assert b.stats(0)["energy"] == pytest.approx(e_now, rel=1e-9, abs=1e-9)


@pytest.mark.parametrize("name", ["sheared", "general"])
def test_semigrand_parallel_sweep_on_a_supercell_matrix(name, cm, oracle_mod):
    """The parallel semi-grand sweep on a non-diagonal supercell (colour
    classes checked through the twisted periodicity; halo cells are twisted
    images): <E>, <x>, heat capacity and susceptibilities of 16 GPU chains
    against 16 oracle chains on the same supercell at 900 K, 2 sigma per
    comparison under the family-wise contract of
    tests/test_gpu_equilibrium.py; the running energy equals a recompute."""
    import os

    from tests.stat_checks import compare

    ce, T = workloads.fcc_binary_ce(0), SUPERCELLS[name]
    temp, mu, nrep = 900.0, np.array([0.05]), 16
    o = oracle_mod.OracleSystem(ce, T)
    n = o.n_sites
    rng = np.random.default_rng(33)
    inits = [workloads.fixed_composition(rng, n, 0.4) for _ in range(2 * nrep)]
    n_o, eq_o = 1500, 300
    occ = np.ascontiguousarray(np.concatenate(inits[:nrep]), dtype=np.int8)
    pot, comp, _ = o.run_chains(occ, 0, np.full(nrep, temp), np.tile(mu, (nrep, 1)), 5, n_o,
                                os.cpu_count() or 1)
    ora = [np.column_stack([pot[i, eq_o:], comp[i, eq_o:]]) for i in range(nrep)]
    b = cm.ReplicaBatch(cm.System(ce), "semigrand_canonical", [T] * nrep)
    for i in range(nrep):
        b.set_conditions(i, temp, mu)
        b.set_seed(i, 300 + i)
        b.set_occupation(i, inits[nrep + i])
    n_pass, n_eq = 3000, 500
    b.run(n_pass, n_eq, record_samples=True)
    gpu = []
    for i in range(nrep):
        p_i, c_i = b.samples(i, n_pass - n_eq)
        gpu.append(np.column_stack([p_i, c_i.reshape(n_pass - n_eq, -1)]))
        e_now, _ = b.energy(i)
        assert b.stats(i)["energy"] == pytest.approx(e_now, rel=1e-9, abs=1e-9)
    print(compare([(f"{name} sgc T={temp:.0f}", temp)], [gpu], [ora], n, sgc=True))
