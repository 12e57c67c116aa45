"""Size-independent properties at the benchmark sizes (too large for the
oracle): composition conservation of canonical chains, the running energy
against a fresh full recompute, determinism, schedule invariance, and
degenerate compositions."""

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


def _batch(cm, sysd, w, streamed=False):
    b = cm.ReplicaBatch(sysd, w.ensemble, w.L)
    if streamed:
        b.set_option("streamed", 1)
    for i in range(w.n_replicas):
        mu = w.param_chem_pot[i] if w.ensemble == "semigrand_canonical" else None
        b.set_conditions(i, float(w.temperature[i]), mu)
        b.set_seed(i, int(w.seeds[i]))
    b.set_occupation_all(np.concatenate(w.occupation).astype(np.int8))
    return b


def test_benchmark_batch_invariants(cm):
    """128 x 24^3 canonical: composition kept per replica, running energy equal
    to a fresh recompute, a rerun from the same state and seeds identical."""
    w = workloads.config(1)
    sysd = cm.System(w.ce)
    a = _batch(cm, sysd, w)
    a.run(60, 10, record_samples=True)
    occ_a = a.get_occupation_all()
    for i in range(w.n_replicas):
        o0 = w.occupation[i]
        seg = occ_a[a.offsets[i]:a.offsets[i + 1]]
        assert int(seg.sum()) == int(o0.sum())
        st = a.stats(i)
        e, _ = a.energy(i)
        assert st["energy"] == pytest.approx(e, rel=1e-12, abs=1e-12)
        assert 0 < st["n_accepted"] <= st["n_proposed"]
        assert np.isfinite(st["mean_potential"]) and st["var_potential"] >= 0.0
    b = _batch(cm, sysd, w)
    b.set_option("threads", 256)
    b.set_option("cta_order", 1)
    b.run(60, 10, record_samples=True)
    np.testing.assert_array_equal(b.get_occupation_all(), occ_a)
    for i in range(0, w.n_replicas, 17):
        assert b.stats(i)["mean_potential"] == a.stats(i)["mean_potential"]


def test_streamed_96_invariants(cm):
    """4 x 96^3 HBM-streamed: composition kept, running energy consistent."""
    w = workloads.config(4)
    keep = [i for i, L in enumerate(w.L) if L[0] == 96]
    import copy

    v = copy.copy(w)
    v.L = [w.L[i] for i in keep]
    v.temperature = w.temperature[keep]
    v.param_chem_pot = w.param_chem_pot[keep]
    v.occupation = [w.occupation[i] for i in keep]
    v.seeds = w.seeds[keep]
    sysd = cm.System(w.ce)
    b = _batch(cm, sysd, v)
    assert b.get_option("streamed") == 1
    b.run(4, 0)
    occ = b.get_occupation_all()
    for i in range(len(keep)):
        seg = occ[b.offsets[i]:b.offsets[i + 1]]
        assert int(seg.sum()) == int(v.occupation[i].sum())
        e, _ = b.energy(i)
        assert b.stats(i)["energy"] == pytest.approx(e, rel=1e-12, abs=1e-12)


@pytest.mark.parametrize("x", [0.0, 1.0])
def test_single_species_canonical_has_no_proposals(x, cm):
    ce = workloads.fcc_binary_ce(2)
    sysd = cm.System(ce)
    b = cm.ReplicaBatch(sysd, "canonical", [(24, 24, 24)])
    b.set_conditions(0, 700.0)
    occ = np.full(24 ** 3, int(x), np.int8)
    b.set_occupation(0, occ)
    b.run(5, 0)
    st = b.stats(0)
    assert st["n_proposed"] == 0
    np.testing.assert_array_equal(b.get_occupation(0), occ)
    e, _ = b.energy(0)
    assert st["energy"] == pytest.approx(e, rel=1e-12, abs=1e-12)
