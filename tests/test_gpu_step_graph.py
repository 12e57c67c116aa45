"""The end-to-end step graph (copy in, passes, copy out) gives the same chain
as the separate calls it replaces."""

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


@pytest.mark.parametrize("kind", ["fcc_canonical", "bcc_sgc", "fcc_cluster"])
def test_step_graph_matches_separate_calls(kind, cm):
    """fcc_cluster: the step graph launches the sweep on clusters of 4 CTAs
    per replica, the separate calls on one CTA per replica."""
    if kind == "fcc_canonical":
        ce, ens, Ls, mu = workloads.fcc_binary_ce(3), "canonical", [(8, 8, 8), (12, 12, 12)], None
    elif kind == "fcc_cluster":
        ce, ens, Ls, mu = workloads.fcc_binary_ce(3), "canonical", [(48, 48, 48)] * 2, None
    else:
        ce, ens, Ls, mu = workloads.bcc_ternary_ce(3), "semigrand_canonical", [(6, 6, 6), (7, 7, 7)], \
            np.array([0.05, -0.02])
    sysd = cm.System(ce)
    rng = np.random.default_rng(6)
    n_sites = [ce.prim.n_basis * int(np.prod(L)) for L in Ls]
    occ = np.concatenate([rng.integers(0, ce.prim.n_occ, n).astype(np.int8) for n in n_sites])

    def batch():
        b = cm.ReplicaBatch(sysd, ens, Ls)
        for i in range(len(Ls)):
            b.set_conditions(i, 700.0, mu)
            b.set_seed(i, 50 + i)
        return b

    a = batch()
    if kind == "fcc_cluster":
        a.set_option("sweep_cluster", 4)
    h = a.pinned_buffer()
    h[:] = occ
    for _ in range(3):
        a.step_async(h, h, 2)
    a.synchronize()
    b = batch()
    if kind == "fcc_cluster":
        b.set_option("sweep_cluster", 1)
    cur = occ.copy()
    for _ in range(3):
        b.set_occupation_all(cur)
        b.run(2, 0)
        b.get_occupation_all(cur)
    np.testing.assert_array_equal(h, cur)
    for i in range(len(Ls)):
        assert a.stats(i)["energy"] == pytest.approx(b.stats(i)["energy"], rel=1e-12, abs=1e-12)
        assert a.stats(i)["n_proposed"] == b.stats(i)["n_proposed"]


def test_step_graph_needs_pinned_buffers(cm):
    sysd = cm.System(workloads.fcc_binary_ce(1))
    b = cm.ReplicaBatch(sysd, "canonical", [(8, 8, 8)])
    pageable = np.zeros(512, np.int8)
    with pytest.raises(RuntimeError, match="page-locked"):
        b.step_async(pageable, pageable, 1)
