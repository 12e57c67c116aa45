"""Checkpoint/restart and failure paths of the C ABI (errors are raised on
the host; no test faults the GPU)."""

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


@pytest.mark.parametrize("ens,streamed", [("canonical", False), ("semigrand_canonical", False),
                                          ("canonical", True)])
def test_restart_continues_bit_for_bit(ens, streamed, cm):
    ce = workloads.fcc_binary_ce(6)
    sysd = cm.System(ce)
    L = (24, 24, 24)
    occ0 = workloads.fixed_composition(np.random.default_rng(3), 24 ** 3, 0.4)

    def fresh():
        b = cm.ReplicaBatch(sysd, ens, [L])
        if streamed:
            b.set_option("streamed", 1)
        b.set_conditions(0, 500.0, np.array([0.02]) if ens != "canonical" else None)
        b.set_seed(0, 99)
        return b

    a = fresh()
    a.set_occupation(0, occ0)
    a.run(20, 0)
    straight = a.get_occupation(0), a.stats(0)
    b = fresh()
    b.set_occupation(0, occ0)
    b.run(9, 0)
    occ, st = b.get_state(0)
    c = fresh()
    c.set_state(0, occ, st)
    c.run(11, 0)
    np.testing.assert_array_equal(c.get_occupation(0), straight[0])
    s1, s2 = c.stats(0), straight[1]
    assert s1["passes"] == s2["passes"] == 20
    assert s1["energy"] == s2["energy"]


def test_invalid_inputs_raise(cm):
    ce = workloads.fcc_binary_ce(0)
    sysd = cm.System(ce)
    with pytest.raises(RuntimeError, match="supercell too small"):
        cm.ReplicaBatch(sysd, "canonical", [(4, 4, 4)])
    b = cm.ReplicaBatch(sysd, "canonical", [(8, 8, 8)])
    bad = np.zeros(512, dtype=np.int8)
    bad[3] = 2
    with pytest.raises(RuntimeError, match="occupant index out of range"):
        b.set_occupation(0, bad)
    with pytest.raises(RuntimeError, match="site index out of range"):
        b.delta(0, np.array([[600]]), np.array([[1]]))
    with pytest.raises(RuntimeError, match="temperature"):
        b.set_conditions(0, -5.0)
    with pytest.raises(RuntimeError, match="semi-grand potential"):
        b.delta(0, np.array([[1]]), np.array([[1]]), potential=True)
    with pytest.raises(RuntimeError, match="local_sweeps must be >= 1"):
        b.set_option("local_sweeps", 0)
    with pytest.raises(RuntimeError, match="unknown option"):
        b.set_option("warp_drive", 1)
    sg = cm.ReplicaBatch(sysd, "semigrand_canonical", [(8, 8, 8)])
    with pytest.raises(RuntimeError, match="need param_chem_pot"):
        sg.set_conditions(0, 300.0, None)
    # no proposal possible: canonical replay on a pure-A state stops with an error
    b.set_occupation(0, np.zeros(512, dtype=np.int8))
    with pytest.raises(RuntimeError, match="no event can be proposed"):
        b.replay(0, 1, 10)
    e, counts = b.energy(0)  # the batch stays usable after the error
    assert counts[1] == 0


def test_nonfinite_eci_rejected(cm):
    ce = workloads.fcc_binary_ce(0)
    ce.eci[3] = float("nan")
    with pytest.raises(RuntimeError, match="non-finite weight"):
        cm.System(ce)


def test_zero_temperature_accepts_only_downhill(cm, oracle_mod):
    """T = 0: beta is infinite; dE > 0 and dE == 0 are both rejected in
    replay, as the reference's exp(-dE * inf) comparison does."""
    ce = workloads.fcc_binary_ce(1)
    L = (8, 8, 8)
    occ = workloads.fixed_composition(np.random.default_rng(4), 512, 0.5)
    o = oracle_mod.OracleSystem(ce, L)
    ref_occ = occ.copy()
    ref = o.run(ref_occ, 1, 0.0, np.zeros(1), 5, 3, record_steps=3 * 512)
    sysd = cm.System(ce)
    b = cm.ReplicaBatch(sysd, "canonical", [L])
    b.set_conditions(0, 0.0)
    b.set_occupation(0, occ)
    got = b.replay(0, 5, 3 * 512)
    np.testing.assert_array_equal(got["accept"], ref["accept"])
    assert np.all(got["dE"][got["accept"] == 1] < 0)


@pytest.mark.parametrize("kernel", ["sweep", "sweep_cluster", "group"])
def test_host_stop_request_ends_a_long_run_at_a_pass_boundary(kernel, cm):
    """A run of a million passes, stopped from the host after a fraction of a
    second: cem_synchronize reports CEM_STOPPED, the replicas hold a
    consistent state (running energy equals a fresh recompute, composition
    conserved), and the next run starts normally. sweep_cluster: each replica
    on a cluster of 4 CTAs (rank 0 broadcasts the stop decision)."""
    import time

    ce = workloads.fcc_binary_ce(0)
    edge = 24 if kernel == "sweep_cluster" else 12
    L = (edge, edge, edge)
    n = 4
    sysd = cm.System(ce)
    b = cm.ReplicaBatch(sysd, "canonical", [L] * n)
    if kernel == "sweep_cluster":
        b.set_option("sweep_cluster", 4)
    rng = np.random.default_rng(8)
    occ0 = [workloads.fixed_composition(rng, edge ** 3, 0.4) for _ in range(n)]
    for i in range(n):
        b.set_conditions(i, 700.0)
        b.set_seed(i, 31 + i)
        b.set_occupation(i, occ0[i])
    big = 1_000_000
    t0 = time.perf_counter()
    if kernel != "group":
        b.run(big, 0)
    else:
        b.learned_group_run(None, big, 0, weights="uniform", rounds=8, local_substeps=2)
    time.sleep(0.3)
    b.request_stop()
    assert b.synchronize() is True
    assert time.perf_counter() - t0 < 10.0
    for i in range(n):
        st = b.stats(i)
        assert 0 < st["passes"] < big
        e, _ = b.energy(i)
        assert abs(st["energy"] - e) <= 1e-9 * max(1.0, abs(e))
        assert b.get_occupation(i).sum() == occ0[i].sum()
    # the flag is cleared by the next run
    p0 = b.stats(0)["passes"]
    if kernel != "group":
        b.run(5, 0)
    else:
        b.learned_group_run(None, 5, 0, weights="uniform", rounds=8, local_substeps=2)
    assert b.synchronize() is False
    assert b.stats(0)["passes"] == p0 + 5


def test_canonical_batch_needs_connecting_local_swaps(cm):
    """The C ABI refuses canonical batches whose local-swap displacements do
    not connect every site (the chain would conserve the occupant count of a
    set of colour classes): here the hcp Zr-O system with only its O-O pairs
    along c. Semi-grand canonical batches need no swaps and are accepted."""
    from tests.zro_fixture import zro_ce

    ce = zro_ce()
    shortest = min((o for o in ce.orbits if o.size == 2), key=lambda o: o.max_length).index
    ce._local_swap_orbits = frozenset({shortest})  # the pre-fix choice: one column per swap set
    sysd = cm.System(ce)
    with pytest.raises(RuntimeError, match="do not connect every site"):
        cm.ReplicaBatch(sysd, "canonical", [(8, 8, 8)])
    b = cm.ReplicaBatch(sysd, "semigrand_canonical", [(8, 8, 8)])
    assert b.n == 1
    ce2 = zro_ce()
    cm.ReplicaBatch(cm.System(ce2), "canonical", [(8, 8, 8)])
