"""n-fold way (rejection-free semi-grand canonical Monte Carlo) on the GPU
against the oracle's sequential restatement: same rates (FP64, explicitly
rounded), same sum tree, same Philox draws, so the event sequence, the
residence weights and the final occupation agree exactly; the weighted
moments agree to 1e-10 relative (the initial energies come from two
different summations)."""

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


def _case(kind, rng):
    if kind == "fcc_binary_generated":  # 10^3: pitch 14, generated evaluator
        ce, L, T, mu = workloads.fcc_binary_ce(2), (10, 10, 10), 700.0, np.array([0.03])
        occ = rng.integers(0, 2, 1000).astype(np.int8)
    elif kind == "fcc_binary_tables":  # odd sizes: run-time tables
        ce, L, T, mu = workloads.fcc_binary_ce(3), (7, 9, 11), 500.0, np.array([-0.02])
        occ = rng.integers(0, 2, 693).astype(np.int8)
    else:
        ce, L, T, mu = workloads.bcc_ternary_ce(6), (5, 5, 5), 900.0, np.array([0.05, -0.1])
        occ = rng.integers(0, 3, 250).astype(np.int8)
    return ce, L, T, mu, occ


@pytest.mark.parametrize("kind", ["fcc_binary_generated", "fcc_binary_tables", "bcc_ternary"])
def test_nfold_matches_oracle_event_for_event(kind, cm, oracle_mod):
    rng = np.random.default_rng(17)
    ce, L, T, mu, occ = _case(kind, rng)
    sysd = cm.System(ce)
    b = cm.ReplicaBatch(sysd, "semigrand_canonical", [L])
    b.set_conditions(0, T, mu)
    seed = 0x1234ABCD5678
    b.set_seed(0, seed)
    b.set_occupation(0, occ)
    n_events, n_equil = 400, 50
    rec = b.nfold_run(n_events, n_equil, record=n_events + n_equil)
    st = b.stats(0)

    o = oracle_mod.OracleSystem(ce, L)
    occ_o = occ.copy()
    ref = o.nfold(occ_o, T, mu, sysd.arrays["weights"], seed, n_events, n_equil,
                  record=n_events + n_equil)
    assert ref["n"] == n_events + n_equil
    np.testing.assert_array_equal(rec["site"][0], ref["site"])
    np.testing.assert_array_equal(rec["occ"][0], ref["occ"])
    np.testing.assert_array_equal(rec["dt"][0], ref["dt"])
    np.testing.assert_array_equal(b.get_occupation(0), occ_o)
    so = ref["stats"]
    W = so[0]
    assert st["n_samples"] == pytest.approx(W, rel=1e-12)
    assert st["mean_potential"] == pytest.approx(so[1] / W, rel=1e-10, abs=1e-12)
    assert st["mean_formation"] == pytest.approx(so[3] / W, rel=1e-10, abs=1e-12)
    nc = ce.prim.n_occ - 1
    np.testing.assert_allclose(st["mean_comp"], so[4:4 + nc] / W, rtol=1e-10, atol=1e-12)
    # the running energy equals a fresh recompute of the final state
    e_now, _ = b.energy(0)
    assert st["energy"] == pytest.approx(e_now, rel=1e-9, abs=1e-9)


def test_nfold_runs_continue_the_stream(cm):
    ce = workloads.fcc_binary_ce(5)
    sysd = cm.System(ce)
    occ = np.random.default_rng(2).integers(0, 2, 1000).astype(np.int8)

    def fresh():
        b = cm.ReplicaBatch(sysd, "semigrand_canonical", [(10, 10, 10)])
        b.set_conditions(0, 650.0, np.array([0.0]))
        b.set_seed(0, 77)
        b.set_occupation(0, occ)
        return b

    a = fresh()
    r_all = a.nfold_run(300, 0, record=300)
    b = fresh()
    r1 = b.nfold_run(120, 0, record=120)
    r2 = b.nfold_run(180, 0, record=180)
    np.testing.assert_array_equal(np.concatenate([r1["site"][0], r2["site"][0]]), r_all["site"][0])
    np.testing.assert_array_equal(np.concatenate([r1["dt"][0], r2["dt"][0]]), r_all["dt"][0])
    np.testing.assert_array_equal(b.get_occupation(0), a.get_occupation(0))


def test_nfold_agrees_with_metropolis_sweep(cm):
    """Residence-weighted n-fold averages reproduce the parallel Metropolis
    sweep's <x> and <E>: 16 independent replicas per sampler (each replica's
    run average one independent sample, standard errors from the replica
    spread), 2 sigma per comparison under the family-wise contract of
    tests/test_gpu_equilibrium.py."""
    from casmcode_clexmonte_gb300.stats import family_2sigma

    ce = workloads.fcc_binary_ce(7)
    sysd = cm.System(ce)
    L, T, mu, n = (10, 10, 10), 900.0, np.array([0.02]), 16
    rng = np.random.default_rng(4)
    occ = [rng.integers(0, 2, 1000).astype(np.int8) for _ in range(n)]

    def batch():
        b = cm.ReplicaBatch(sysd, "semigrand_canonical", [L] * n)
        for i in range(n):
            b.set_conditions(i, T, mu)
            b.set_seed(i, 1000 + i)
            b.set_occupation(i, occ[i])
        return b

    nf = batch()
    nf.nfold_run(40000, 20000)
    sw = batch()
    sw.run(400, 100)
    xs_n = np.array([nf.stats(i)["mean_comp"][0] for i in range(n)])
    xs_s = np.array([sw.stats(i)["mean_comp"][0] for i in range(n)])
    es_n = np.array([nf.stats(i)["mean_potential"] for i in range(n)])
    es_s = np.array([sw.stats(i)["mean_potential"] for i in range(n)])
    zs, rows = [], []
    for name, a, c in (("<x>", xs_n, xs_s), ("<E>", es_n, es_s)):
        se = np.sqrt(a.var(ddof=1) / n + c.var(ddof=1) / n)
        zs.append((a.mean() - c.mean()) / se)
        rows.append(f"{name} n-fold {a.mean():+.6e} sweep {c.mean():+.6e} +- {se:.1e} z {zs[-1]:+.2f}")
    ok, k, bound, n2 = family_2sigma(zs)
    msg = "\n".join(rows) + f"\n{n2} of {len(zs)} beyond 2 sigma (allowed {k}); bound {bound:.2f}"
    print(msg)
    assert ok, msg


def test_nfold_errors(cm):
    ce = workloads.fcc_binary_ce(1)
    sysd = cm.System(ce)
    b = cm.ReplicaBatch(sysd, "canonical", [(8, 8, 8)])
    with pytest.raises(RuntimeError, match="semi-grand canonical"):
        b.nfold_run(10)
    # zero temperature, every flip raises the potential: no event has a rate
    g = cm.ReplicaBatch(sysd, "semigrand_canonical", [(8, 8, 8)])
    g.set_conditions(0, 0.0, np.array([-5.0]))
    g.set_occupation(0, np.zeros(512, np.int8))
    with pytest.raises(RuntimeError, match="non-zero rate"):
        g.nfold_run(10)
