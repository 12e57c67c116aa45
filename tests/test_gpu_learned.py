"""Learned proposal: network kernels against an FP64 reference, training,
and exactness of the Metropolis-Hastings sampler against the oracle."""

import numpy as np
import pytest

from casmcode_clexmonte_gb300 import workloads
from casmcode_clexmonte_gb300.stats import batch_means

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
    assert np.array_equal(X[:, 42], occ)
    # target = clamp(-beta dE_flip / 2) with dE_flip from the exact delta API
    sites = np.arange(200)[:, None]
    dE, _ = b.delta(0, sites, 1 - occ[sites])
    beta = 1.0 / (8.617333262e-5 * 800.0)
    want = np.clip(-0.5 * beta * dE, -12, 8)
    np.testing.assert_allclose(t[:200], want, rtol=1e-5, atol=1e-5)


def test_training_reduces_loss(cm):
    _, _, _, X, t = _snapshot_features(cm)
    net = cm.LearnedProposal(seed=1)
    _, before = net.gradient(X, t)
    losses = net.train(X, t, epochs=8, batch=512, lr=3e-3, seed=2)
    _, after = net.gradient(X, t)
    assert after < 0.2 * before, (before, after, losses)


@pytest.mark.parametrize("trained", [False, True])
def test_learned_sampler_equilibrium_matches_oracle(trained, cm, oracle_mod):
    """<E> of the learned-proposal chain (exact MH correction) against the
    sequential oracle chain with uniform swaps, within 4 standard errors."""
    L, T, nrep = 10, 900.0, 16
    ce = workloads.fcc_binary_ce(3, nn1=0.08)
    rng = np.random.default_rng(12)
    occ0 = workloads.fixed_composition(rng, L ** 3, 0.25)
    o = oracle_mod.OracleSystem(ce, (L, L, L))
    ref = o.run(occ0.copy(), 1, T, np.zeros(1), 77, 4000)
    e_o, se_o = batch_means(ref["energy"][500:])
    sysd = cm.System(ce)
    net = None
    if trained:
        _, _, _, X, t = _snapshot_features(cm, T=T)
        net = cm.LearnedProposal(seed=4)
        net.train(X, t, epochs=8, batch=512, lr=3e-3, seed=1)
    b = cm.ReplicaBatch(sysd, "canonical", [(L, L, L)] * nrep)
    for i in range(nrep):
        b.set_conditions(i, T)
        b.set_seed(i, 900 + i)
        b.set_occupation(i, occ0)
    b.learned_run(net, 400, 100, record_samples=True)
    means = np.array([b.learned_samples(i, 300)[0].mean() for i in range(nrep)])
    e_g, se_g = means.mean(), means.std(ddof=1) / np.sqrt(nrep)
    assert abs(e_g - e_o) < 4.0 * np.hypot(se_g, se_o), (e_g, se_g, e_o, se_o)
    st = b.stats(0)
    assert st["n_proposed"] == 400 * L ** 3
    e_now, _ = b.energy(0)
    assert abs(st["energy"] - e_now) <= 1e-9 * max(1.0, abs(e_now))
    occ = b.get_occupation(0)
    assert occ.sum() == occ0.sum()


def test_learned_sampler_ordered_phase_matches_oracle(cm, oracle_mod):
    """The same check in the L1_2-ordered phase (90 K, 0.9 T_c of this
    expansion), where the trained weights are far from uniform: <E> of the
    learned chain against the oracle's uniform-swap chain within 4 standard
    errors."""
    L, T, nrep = 10, 90.0, 16
    ce = workloads.fcc_binary_ce(3, nn1=0.08)
    rng = np.random.default_rng(19)
    occ0 = workloads.fixed_composition(rng, L ** 3, 0.25)
    o = oracle_mod.OracleSystem(ce, (L, L, L))
    ref = o.run(occ0.copy(), 1, T, np.zeros(1), 91, 6000)
    e_o, se_o = batch_means(ref["energy"][1500:])
    sysd = cm.System(ce)
    _, _, _, X, t = _snapshot_features(cm, T=T, passes=300)
    net = cm.LearnedProposal(seed=6)
    net.train(X, t, epochs=8, batch=512, lr=3e-3, seed=2)
    b = cm.ReplicaBatch(sysd, "canonical", [(L, L, L)] * nrep)
    for i in range(nrep):
        b.set_conditions(i, T)
        b.set_seed(i, 1900 + i)
        b.set_occupation(i, occ0)
    b.learned_run(net, 500, 150, record_samples=True)
    means = np.array([b.learned_samples(i, 350)[0].mean() for i in range(nrep)])
    e_g, se_g = means.mean(), means.std(ddof=1) / np.sqrt(nrep)
    assert abs(e_g - e_o) < 4.0 * np.hypot(se_g, se_o), (e_g, se_g, e_o, se_o)


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
