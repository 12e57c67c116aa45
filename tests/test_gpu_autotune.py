"""Launch schedules of the shared-memory sweep (threads per replica, replica
-> CTA order) and the autotuner that picks one: the chain must not depend on
the schedule (bit for bit for binary systems), and tuning must leave the
state as it found it."""

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


def _batch(cm, sysd, ens, Ls, occs, threads=None, order=None):
    b = cm.ReplicaBatch(sysd, ens, Ls)
    for i in range(len(Ls)):
        b.set_conditions(i, 500.0 + 40.0 * i, np.array([0.01]) if ens != "canonical" else None)
        b.set_seed(i, 31 + i)
        b.set_occupation(i, occs[i])
    if threads:
        b.set_option("threads", threads)
    if order is not None:
        b.set_option("cta_order", order)
    return b


@pytest.mark.parametrize("ens", ["canonical", "semigrand_canonical"])
def test_schedule_does_not_change_the_chain(ens, cm):
    ce = workloads.fcc_binary_ce(9)
    sysd = cm.System(ce)
    Ls = [(8, 8, 8), (12, 12, 12), (10, 10, 10), (24, 24, 24), (8, 10, 12)]
    rng = np.random.default_rng(8)
    occs = [workloads.fixed_composition(rng, int(np.prod(L)), 0.4) for L in Ls]
    runs = []
    for threads, order in ((512, 0), (256, 1), (256, 0), (512, 1)):
        b = _batch(cm, sysd, ens, Ls, occs, threads, order)
        b.run(30, 5)
        runs.append(([b.get_occupation(i) for i in range(len(Ls))],
                     [b.stats(i) for i in range(len(Ls))]))
    ref_occ, ref_st = runs[0]
    for occ, st in runs[1:]:
        for i in range(len(Ls)):
            np.testing.assert_array_equal(occ[i], ref_occ[i])
            assert st[i]["energy"] == ref_st[i]["energy"]
            assert st[i]["n_proposed"] == ref_st[i]["n_proposed"]
            assert st[i]["mean_potential"] == ref_st[i]["mean_potential"]


def test_autotune_restores_state_and_keeps_results(cm):
    ce = workloads.fcc_binary_ce(10)
    sysd = cm.System(ce)
    Ls = [(8, 8, 8)] * 3 + [(16, 16, 16)] * 2
    rng = np.random.default_rng(9)
    occs = [workloads.fixed_composition(rng, int(np.prod(L)), 0.5) for L in Ls]
    a = _batch(cm, sysd, "canonical", Ls, occs)
    a.run(10, 0)
    before = [a.get_occupation(i) for i in range(len(Ls))]
    st_before = [a.stats(i) for i in range(len(Ls))]
    choice = a.autotune(5)
    assert choice["threads"] in (256, 512) and choice["cta_order"] in (0, 1)
    assert choice["trial_ms"] > 0
    for i in range(len(Ls)):
        np.testing.assert_array_equal(a.get_occupation(i), before[i])
        assert a.stats(i)["energy"] == st_before[i]["energy"]
        assert a.stats(i)["n_proposed"] == st_before[i]["n_proposed"]
    a.run(20, 0)
    b = _batch(cm, sysd, "canonical", Ls, occs)
    b.run(10, 0)
    b.run(20, 0)
    for i in range(len(Ls)):
        np.testing.assert_array_equal(a.get_occupation(i), b.get_occupation(i))
        assert a.stats(i)["energy"] == b.stats(i)["energy"]
    with pytest.raises(RuntimeError, match="threads must be"):
        a.set_option("threads", 384)
