"""The oracle's restatement of clexmonte::enforce_composition
(state/enforce_composition.hh:56-210) on the CPU: greedy flips end at the
closest reachable composition, a second call does nothing, and the draws
follow the documented pattern (one random_real and one random_int per flip,
the latter with rejection only for ranges that are not powers of two)."""

import numpy as np
import pytest

from casmcode_clexmonte_gb300 import workloads


@pytest.mark.parametrize("ternary", [False, True])
def test_enforce_closest_and_idempotent(ternary, oracle_mod):
    ce = workloads.bcc_ternary_ce(1) if ternary else workloads.fcc_binary_ce(1)
    L = (6, 6, 6)
    o = oracle_mod.OracleSystem(ce, L)
    nb, no = ce.prim.n_basis, ce.prim.n_occ
    rng = np.random.default_rng(2)
    n_uc = 216
    for trial in range(5):
        occ = rng.integers(0, no, o.n_sites).astype(np.int8)
        x = rng.uniform(0.0, 1.0 / (no - 1), no - 1)
        target = np.concatenate([[nb * (1 - x.sum())], nb * x])
        before = np.bincount(occ, minlength=no)
        n, draws = o.enforce_composition(occ, target, 100 + trial)
        after = np.bincount(occ, minlength=no)
        assert np.all(np.abs(after / n_uc - target) <= 1.002 / n_uc)
        # each flip moves one site; the count change bounds the flips from below
        assert n >= np.abs(after - before).sum() // 2
        assert draws >= 2 * n
        n2, d2 = o.enforce_composition(occ, target, 7)
        assert n2 == 0 and d2 == 0


def test_enforce_reproducible(oracle_mod):
    ce = workloads.fcc_binary_ce(1)
    o = oracle_mod.OracleSystem(ce, (8, 8, 8))
    a = np.zeros(512, np.int8)
    b = np.zeros(512, np.int8)
    o.enforce_composition(a, [0.5, 0.5], 42)
    o.enforce_composition(b, [0.5, 0.5], 42)
    np.testing.assert_array_equal(a, b)
    c = np.zeros(512, np.int8)
    o.enforce_composition(c, [0.5, 0.5], 43)
    assert (a != c).any() and a.sum() == c.sum() == 256
