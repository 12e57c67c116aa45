"""Composition enforcement on the GPU against the oracle's restatement of
clexmonte::enforce_composition (state/enforce_composition.hh:56-210): same
std::mt19937_64 draws, same greedy flip types, same occupant-list updates,
so the final occupations must be identical site for site."""

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


def _case(name):
    if name == "fcc_binary":
        return workloads.fcc_binary_ce(2), [(8, 8, 8), (10, 10, 10), (24, 24, 24)]
    return workloads.bcc_ternary_ce(2), [(8, 8, 8), (10, 10, 10)]


@pytest.mark.parametrize("name", ["fcc_binary", "bcc_ternary"])
@pytest.mark.parametrize("start", ["pure", "random"])
def test_enforce_matches_oracle(name, start, cm, oracle_mod):
    ce, Ls = _case(name)
    sysd = cm.System(ce)
    b = cm.ReplicaBatch(sysd, "canonical", Ls)
    nb, no = ce.prim.n_basis, ce.prim.n_occ
    rng = np.random.default_rng(11)
    occs, targets = [], []
    for i, L in enumerate(Ls):
        n = nb * L[0] * L[1] * L[2]
        occ = (np.zeros(n, np.int8) if start == "pure"
               else rng.integers(0, no, n).astype(np.int8))
        b.set_occupation(i, occ)
        occs.append(occ)
        x = rng.uniform(0.05, 0.9 / (no - 1), no - 1)
        targets.append(np.concatenate([[nb * (1 - x.sum())], nb * x]))
    seed = 0xC0FFEE
    flips = b.enforce_composition(np.array(targets), seed)
    for i, L in enumerate(Ls):
        o = oracle_mod.OracleSystem(ce, L)
        ref = occs[i].copy()
        nf, _ = o.enforce_composition(ref, targets[i], seed + i)
        got = b.get_occupation(i)
        assert flips[i] == nf
        np.testing.assert_array_equal(got, ref)
        # the result is the closest reachable composition
        n_uc = L[0] * L[1] * L[2]
        counts = np.bincount(got, minlength=no)
        assert np.all(np.abs(counts / n_uc - targets[i]) <= 1.002 / n_uc)


def test_enforce_is_idempotent_and_energy_consistent(cm, oracle_mod):
    ce = workloads.fcc_binary_ce(4)
    sysd = cm.System(ce)
    L = (12, 12, 12)
    b = cm.ReplicaBatch(sysd, "canonical", [L])
    b.set_occupation(0, np.zeros(12 ** 3, np.int8))
    target = np.array([0.25, 0.75])
    f1 = b.enforce_composition(target, 5)
    f2 = b.enforce_composition(target, 6)
    assert f1[0] == 1296 and f2[0] == 0
    occ = b.get_occupation(0)
    e, _ = b.energy(0)
    assert e == pytest.approx(oracle_mod.OracleSystem(ce, L).energy(occ), abs=1e-9)
    # a run afterwards starts from the enforced state (statistics re-initialised)
    b.set_conditions(0, 600.0)
    b.set_seed(0, 1)
    b.run(4, 0)
    assert np.bincount(b.get_occupation(0), minlength=2).tolist() == [432, 1296]


def test_enforce_function_and_errors(cm):
    ce = workloads.fcc_binary_ce(4)
    sysd = cm.System(ce)
    st = cm.MonteCarloState(occupation=np.zeros(8 ** 3, np.int8), L=(8, 8, 8),
                            conditions={"temperature": 300.0})
    n = cm.enforce_composition(st, cm.mol_composition(sysd, [0.5]), sysd, seed=3)
    assert n == 256 and int(st.occupation.sum()) == 256
    with pytest.raises(ValueError, match="mismatch"):
        cm.enforce_composition(st, [0.2, 0.3, 0.5], sysd)
    b = cm.ReplicaBatch(sysd, "canonical", [(8, 8, 8)])
    with pytest.raises(RuntimeError, match="finite"):
        b.enforce_composition([np.nan, 1.0], 0)
