"""Learned proposal: network kernels against an FP64 reference, training,
and exactness of the Metropolis-Hastings sampler against the oracle."""

import os

import numpy as np
import pytest

from casmcode_clexmonte_gb300 import workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cm():
    from casmcode_clexmonte_gb300 import build

    build.build()
    from casmcode_clexmonte_gb300 import calculator

    return calculator


def _snapshot_features(cm, L=10, n_rep=8, T=800.0, passes=50):
    ce = workloads.fcc_binary_ce(3, nn1=0.08)
    sysd = cm.System(ce)
    b = cm.ReplicaBatch(sysd, "canonical", [(L, L, L)] * n_rep)
    rng = np.random.default_rng(0)
    for i in range(n_rep):
        b.set_conditions(i, T)
        b.set_seed(i, 5 + i)
        b.set_occupation(i, workloads.fixed_composition(rng, L ** 3, 0.25))
    b.run(passes, 0)
    Xs, ts = zip(*[b.learned_features(i) for i in range(n_rep)])
    return ce, sysd, b, np.concatenate(Xs), np.concatenate(ts)


def test_forward_and_gradient_match_fp64_reference(cm):
    from tests import mlp_reference as ref

    _, _, _, X, t = _snapshot_features(cm)
    net = cm.LearnedProposal(seed=3)
    p = ref.bf16_round(net.get_params())
    z = net.forward(X[:4000])
    z_ref, _ = ref.forward(p, X[:4000].astype(np.float64))
    assert np.max(np.abs(z - z_ref)) <= 1e-4 * (1.0 + np.max(np.abs(z_ref)))
    g, loss = net.gradient(X[:2000], t[:2000])
    g_ref, loss_ref = ref.gradient(p, X[:2000], t[:2000].astype(np.float64))
    assert abs(loss - loss_ref) <= 1e-5 * max(1.0, loss_ref)
    scale = np.max(np.abs(g_ref))
    assert np.max(np.abs(g - g_ref)) <= 1e-4 * scale, np.max(np.abs(g - g_ref)) / scale


def test_features_and_targets(cm):
    ce, sysd, b, X, t = _snapshot_features(cm, n_rep=1)
    occ = b.get_occupation(0)
    assert X.shape[1] == 42
    # target = clamp(-beta dE_AB / 2): dE_AB is the exact energy change of
    # putting B on the site (the flip's dE for an A site, minus it for a B site)
    sites = np.arange(200)[:, None]
    dE, _ = b.delta(0, sites, 1 - occ[sites])
    dE_ab = np.where(occ[:200] == 0, dE, -dE)
    beta = 1.0 / (8.617333262e-5 * 800.0)
    want = np.clip(-0.5 * beta * dE_ab, -10, 10)
    np.testing.assert_allclose(t[:200], want, rtol=1e-5, atol=1e-5)


def test_training_reduces_loss(cm):
    _, _, _, X, t = _snapshot_features(cm)
    net = cm.LearnedProposal(seed=1)
    _, before = net.gradient(X, t)
    losses = net.train(X, t, epochs=8, batch=512, lr=3e-3, seed=2)
    _, after = net.gradient(X, t)
    assert after < 0.2 * before, (before, after, losses)


@pytest.mark.parametrize("T", [900.0, 90.0])
def test_learned_sampler_equilibrium_matches_oracle(T, cm, oracle_mod):
    """The global learned sampler (per-species sum trees over the replica,
    exact Metropolis-Hastings correction) against the oracle's sequential
    chains with uniform swaps, 10^3 cells, x_B = 0.25: with uniform weights
    and with the trained network at 900 K (disordered; random initial
    states), with the network at 90 K (0.9 T_c of this expansion,
    L1_2-ordered initial states, where the trained weights are far from
    uniform). <E> and C of pooled independent chains (GPU 16, oracle 16),
    jackknife errors, >= 50 tau_int per chain, 2 sigma per comparison at a
    family-wise contract (tests/test_gpu_equilibrium.py)."""
    from tests.stat_checks import compare

    L, nrep = 10, 16
    n = L ** 3
    ce = workloads.fcc_binary_ce(3, nn1=0.08)
    ordered = T < 100.0
    rng = np.random.default_rng(int(T) + 12)

    def initial(i):
        return _l12(L, i % 4) if ordered else workloads.fixed_composition(rng, n, 0.25)

    o = oracle_mod.OracleSystem(ce, (L, L, L))
    # the oracle's uniform swaps decorrelate slowly in the ordered phase
    # (tau_int ~ 130 passes at 90 K on 10^3)
    n_o, eq_o = (12000, 1000) if ordered else (1500, 300)
    occ = np.ascontiguousarray(np.concatenate([initial(i) for i in range(16)]), dtype=np.int8)
    pot, _, _ = o.run_chains(occ, 1, np.full(16, T), np.zeros((16, 1)), 77, n_o, os.cpu_count() or 1)
    ora = [pot[i, eq_o:, None] for i in range(16)]
    sysd = cm.System(ce)
    _, _, _, X, t = _snapshot_features(cm, T=T, passes=300 if ordered else 50)
    net = cm.LearnedProposal(seed=4)
    net.train(X, t, epochs=8, batch=512, lr=3e-3, seed=1)
    modes = (("network", net),) if ordered else (("uniform", None), ("network", net))
    n_pass, n_eq = (600, 100) if ordered else (400, 100)
    conds, gpus, oras = [], [], []
    for name, prop in modes:
        b = cm.ReplicaBatch(sysd, "canonical", [(L, L, L)] * nrep)
        for i in range(nrep):
            b.set_conditions(i, T)
            b.set_seed(i, 900 + i)
            b.set_occupation(i, initial(i))
        b.learned_run(prop, n_pass, n_eq, record_samples=True)
        gpus.append([b.learned_samples(i, n_pass - n_eq)[0][:, None] for i in range(nrep)])
        oras.append(ora)
        conds.append((f"global {name} T={T:.0f}", T))
        # bookkeeping: one proposal per site and pass, exact running energy,
        # conserved composition
        st = b.stats(0)
        assert st["n_proposed"] == n_pass * n
        e_now, _ = b.energy(0)
        assert abs(st["energy"] - e_now) <= 1e-9 * max(1.0, abs(e_now))
        assert b.get_occupation(0).sum() == initial(0).sum()
    print(compare(conds, gpus, oras, n, sgc=False))


def test_trained_network_raises_acceptance(cm):
    """What the network gains over the uniform proposal: a higher acceptance
    rate per proposal at the same conditions (and, reported, tau_int)."""
    L, T, nrep = 10, 400.0, 8
    ce, sysd, _, X, t = _snapshot_features(cm, T=T)
    net = cm.LearnedProposal(seed=7)
    net.train(X, t, epochs=8, batch=512, lr=3e-3, seed=3)
    rates = {}
    for name, prop in (("uniform", None), ("learned", net)):
        b = cm.ReplicaBatch(sysd, "canonical", [(L, L, L)] * nrep)
        rng = np.random.default_rng(1)
        for i in range(nrep):
            b.set_conditions(i, T)
            b.set_seed(i, 40 + i)
            b.set_occupation(i, workloads.fixed_composition(rng, L ** 3, 0.25))
        b.learned_run(prop, 150, 50)
        acc = sum(b.stats(i)["n_accepted"] for i in range(nrep))
        prop_n = sum(b.stats(i)["n_proposed"] for i in range(nrep))
        rates[name] = acc / prop_n
    print("acceptance per proposal", rates)
    assert rates["learned"] > 1.2 * rates["uniform"], rates


def test_tensor_core_forward_matches_fp64_reference(cm):
    """The group sweep's inference path (tcgen05.mma, bf16 operands in shared
    memory, fp32 accumulators in tensor memory, layer-1 activations rounded to
    bf16) against an FP64 evaluation of the same arithmetic: fp32
    accumulation order is the only difference, except where an activation
    sits on a bf16 rounding boundary."""
    from tests import mlp_reference as ref

    _, _, _, X, t = _snapshot_features(cm)
    net = cm.LearnedProposal(seed=5)
    net.train(X, t, epochs=2, batch=512, lr=3e-3, seed=4)
    p = ref.bf16_round(net.get_params())
    n = 5003  # not a multiple of 128: the last warpgroup's batch is partial
    z = net.forward_tc(X[:n])
    z_ref = ref.forward_bf16_hidden(p, X[:n].astype(np.float64))
    err = np.abs(z - z_ref)
    scale = 1.0 + np.max(np.abs(z_ref))
    assert np.median(err) <= 1e-5 * scale, np.median(err)
    assert np.quantile(err, 0.99) <= 1e-3 * scale, np.quantile(err, 0.99)
    assert np.max(err) <= 2e-2 * scale, np.max(err)
    # and close to the fp32-activation path that training uses
    z32 = net.forward(X[:n])
    assert np.quantile(np.abs(z - z32), 0.99) <= 2e-2 * scale


def _l12(L, k):
    """Perfect L1_2 order: B on the simple-cubic sublattice k of FCC."""
    x, y, z = np.meshgrid(np.arange(L), np.arange(L), np.arange(L), indexing="ij")
    x, y, z = (a.transpose(2, 1, 0).ravel() for a in (x, y, z))
    sub = ((y + z) & 1) | (((x + z) & 1) << 1)
    return (sub == k).astype(np.int8)


@pytest.mark.parametrize("T", [900.0, 90.0])
def test_learned_group_sweep_equilibrium_matches_oracle(T, cm, oracle_mod):
    """<E> and the heat capacity of the learned group sweep, with uniform,
    network and exact locally balanced weights, against the oracle's
    sequential chain (uniform global swaps), 12^3 cells, x_B = 0.25, at 900 K
    (disordered; random initial states) and 90 K (0.9 T_c of this expansion,
    L1_2-ordered; ordered initial states). Pooled chains, jackknife errors,
    >= 50 tau_int per chain, 2 sigma per comparison under the family-wise
    contract (tests/test_gpu_equilibrium.py)."""
    from casmcode_clexmonte_gb300.stats import family_2sigma, jackknife_chains
    from tests.stat_checks import check_chain_lengths as _check_chain_lengths

    L, KB = 12, 8.617333262e-5
    n = L ** 3
    ce = workloads.fcc_binary_ce(3, nn1=0.08)
    ordered = T < 100.0
    nrep = 64 if ordered else 32
    rng = np.random.default_rng(int(T))

    def initial(i):
        return _l12(L, i % 4) if ordered else workloads.fixed_composition(rng, n, 0.25)

    # oracle: 16 chains (32 in the ordered phase, whose single chains
    # decorrelate slowly: its estimate enters every comparison of the test)
    o = oracle_mod.OracleSystem(ce, (L, L, L))
    n_ch, n_o, eq_o = (32, 12000, 1000) if ordered else (16, 1500, 300)
    occ = np.ascontiguousarray(np.concatenate([initial(i) for i in range(n_ch)]), dtype=np.int8)
    pot, _, _ = o.run_chains(occ, 1, np.full(n_ch, T), np.zeros((n_ch, 1)), 5, n_o,
                             os.cpu_count() or 1)
    ora = [pot[i, eq_o:, None] for i in range(n_ch)]
    _check_chain_lengths(ora, False, f"oracle {T:.0f} K")
    sysd = cm.System(ce)
    # the network, trained on plain-sweep snapshots at this temperature
    snap = cm.ReplicaBatch(sysd, "canonical", [(L, L, L)] * 8)
    for i in range(8):
        snap.set_conditions(i, T)
        snap.set_seed(i, 50 + i)
        snap.set_occupation(i, initial(i))
    snap.run(300, 0)
    Xs, ts = zip(*[snap.learned_features(i) for i in range(8)])
    net = cm.LearnedProposal(seed=8)
    net.train(np.concatenate(Xs), np.concatenate(ts), epochs=8, batch=512, lr=3e-3, seed=3)
    rows, zs = [], []
    # uniform swaps inside groups decorrelate as slowly as the plain sweep in
    # the ordered phase (tau_int ~ 200 passes at 90 K); they are checked in the
    # disordered phase, where runs of 2500 samples hold >= 50 tau_int
    modes = ("network", "exact") if ordered else ("uniform", "network", "exact")
    # on 12^3 in the ordered phase single chains reach tau_int ~ 130-290
    # passes (two groups per class, few neighbour swaps per pass on so small a
    # box): 64 chains of 40 000 passes
    n_pass, n_eq = (40000, 2000) if ordered else (3000, 500)
    for weights in modes:
        b = cm.ReplicaBatch(sysd, "canonical", [(L, L, L)] * nrep)
        for i in range(nrep):
            b.set_conditions(i, T)
            b.set_seed(i, 700 + i)
            b.set_occupation(i, initial(i))
        b.learned_group_run(net if weights == "network" else None, n_pass, n_eq,
                            record_samples=True, weights=weights)
        gpu = [b.learned_samples(i, n_pass - n_eq)[0][:, None] for i in range(nrep)]
        _check_chain_lengths(gpu, False, f"group sweep {weights} {T:.0f} K")
        for name, f in (("<E>", lambda a: a[:, 0].mean()),
                        ("C", lambda a: a[:, 0].var() * n / (KB * T * T))):
            eg, sg = jackknife_chains(f, gpu)
            eo, so = jackknife_chains(f, ora)
            zs.append((eg - eo) / np.hypot(sg, so))
            rows.append(f"{weights:>8s} {name:>4s} gpu {eg:+.6e} +- {sg:.1e} oracle {eo:+.6e} "
                        f"+- {so:.1e} z {zs[-1]:+.2f}")
        # bookkeeping: exact running energy, conserved composition
        st = b.stats(0)
        e_now, _ = b.energy(0)
        assert abs(st["energy"] - e_now) <= 1e-9 * max(1.0, abs(e_now))
        assert b.get_occupation(0).sum() == initial(0).sum()
        assert st["n_proposed"] > 0
    ok, k, bound, n2 = family_2sigma(zs)
    msg = "\n".join(rows) + f"\n{n2} of {len(zs)} beyond 2 sigma (allowed {k}); bound {bound:.2f}"
    print(msg)
    assert ok, msg


def test_learned_group_chain_does_not_depend_on_cluster_size(cm):
    """A group's draws depend only on (pass, sub-step, group, round) and every
    accepted change reaches every CTA's copy of the replica, so 1, 2 and 4
    CTAs per replica run the same chain: identical occupations, running
    energies and acceptance counts."""
    L, T, nrep = 24, 150.0, 3
    ce = workloads.fcc_binary_ce(3, nn1=0.08)
    sysd = cm.System(ce)
    rng = np.random.default_rng(4)
    occ0 = [workloads.fixed_composition(rng, L ** 3, 0.25) for _ in range(nrep)]
    _, _, _, X, t = _snapshot_features(cm, T=T)
    net = cm.LearnedProposal(seed=2)
    net.train(X, t, epochs=2, batch=512, lr=3e-3, seed=1)
    results = []
    for cl in (1, 2, 4):
        b = cm.ReplicaBatch(sysd, "canonical", [(L, L, L)] * nrep)
        b.set_option("group_cluster", cl)
        for i in range(nrep):
            b.set_conditions(i, T)
            b.set_seed(i, 60 + i)
            b.set_occupation(i, occ0[i])
        b.learned_group_run(net, 40, 10, record_samples=True, rounds=8, local_substeps=4)
        assert b.get_option("group_cluster") == cl
        results.append(([b.get_occupation(i) for i in range(nrep)],
                        [(b.stats(i)["energy"], b.stats(i)["n_accepted"], b.stats(i)["n_proposed"])
                         for i in range(nrep)],
                        [b.learned_samples(i, 30)[0] for i in range(nrep)]))
    for occ, st, smp in results[1:]:
        for i in range(nrep):
            assert np.array_equal(occ[i], results[0][0][i])
            assert st[i] == results[0][1][i]
            assert np.array_equal(smp[i], results[0][2][i])



def test_trained_network_cuts_autocorrelation_of_the_group_sweep(cm):
    """What the trained network gains over the same sweep without it: in the
    L1_2-ordered phase (90 K, 24^3, x_B = 0.25, from an equilibrated ordered
    state) network-weighted group swaps decorrelate the energy several times
    faster per pass than uniform swaps in the same groups, and much faster
    than the plain sweep."""
    from casmcode_clexmonte_gb300.stats import tau_int

    L, T, nrep = 24, 90.0, 16
    ce = workloads.config(3).ce
    sysd = cm.System(ce)

    def batch():
        b = cm.ReplicaBatch(sysd, "canonical", [(L, L, L)] * nrep)
        for i in range(nrep):
            b.set_conditions(i, T)
            b.set_seed(i, 300 + i)
        return b

    plain = batch()
    for i in range(nrep):
        plain.set_occupation(i, _l12(L, i % 4))
    plain.run(3000, 0)
    state = plain.get_occupation_all()
    X, t = zip(*[plain.learned_features(i) for i in range(nrep)])
    net = cm.LearnedProposal(seed=9)
    net.train(np.concatenate(X), np.concatenate(t), epochs=4, batch=2048, lr=2e-3, seed=7)
    n = 4000
    plain.run(n, 0, record_samples=True)
    tau = {"plain": np.median([tau_int(plain.samples(i, n)[0]) for i in range(nrep)])}
    for weights in ("uniform", "network"):
        b = batch()
        b.set_occupation_all(state)
        b.learned_group_run(net if weights == "network" else None, n, 0, record_samples=True,
                            weights=weights, rounds=4, local_substeps=8)
        tau[weights] = np.median([tau_int(b.learned_samples(i, n)[0]) for i in range(nrep)])
    print("median tau_int(E) per pass", tau)
    assert tau["network"] * 3.0 < tau["uniform"], tau
    assert tau["network"] * 5.0 < tau["plain"], tau
