"""The plain sweep on thread-block clusters: a replica shared by 1, 2, 4 or
8 CTAs (each with a whole copy, candidates of every sub-step split between
them, accepted changes written into every copy) runs the same chain bit for
bit, because every proposal depends only on its own counter and on sites no
other proposal of the sub-step changes."""

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


@pytest.mark.parametrize("ens,edge", [("canonical", 24), ("semigrand_canonical", 24),
                                      ("canonical", 48), ("semigrand_canonical", 10)])
def test_sweep_chain_does_not_depend_on_cluster_size(ens, edge, cm):
    ce = workloads.fcc_binary_ce(3, nn1=0.08)
    sysd = cm.System(ce)
    L = (edge, edge, edge)
    n_rep = 3
    rng = np.random.default_rng(edge)
    occ0 = [workloads.fixed_composition(rng, edge ** 3, 0.3) for _ in range(n_rep)]
    temps = [150.0, 600.0, 2000.0]
    mu = np.array([0.02])
    results = []
    for cl in (1, 2, 4, 8):
        b = cm.ReplicaBatch(sysd, ens, [L] * n_rep)
        b.set_option("sweep_cluster", cl)
        for i in range(n_rep):
            b.set_conditions(i, temps[i], mu if ens == "semigrand_canonical" else None)
            b.set_seed(i, 40 + i)
            b.set_occupation(i, occ0[i])
        b.run(30, 10, record_samples=True)
        b.run(7, 0, record_samples=True)  # a second launch continues the chain
        assert b.get_option("sweep_cluster") == cl
        results.append(([b.get_occupation(i) for i in range(n_rep)],
                        [(b.stats(i)["energy"], b.stats(i)["n_accepted"], b.stats(i)["n_proposed"],
                          b.stats(i)["mean_potential"]) for i in range(n_rep)],
                        [b.samples(i, 7)[0] for i in range(n_rep)]))
    for occ, st, smp in results[1:]:
        for i in range(n_rep):
            assert np.array_equal(occ[i], results[0][0][i])
            assert st[i] == results[0][1][i]
            assert np.array_equal(smp[i], results[0][2][i])
    # the running energy is the exact energy of the final state
    b_e, _ = b.energy(0)
    assert abs(results[-1][1][0][0] - b_e) <= 1e-9 * max(1.0, abs(b_e))
