"""Pin the oracle (and the table builder) to the reference's own fixtures:
the generated FCC Clexulator (compiled against a shim; vectors committed in
tests/golden by make_fcc_clexulator_golden.py) and its ECI file."""

import json
import os

import numpy as np

from casmcode_clexmonte_gb300.system import ClusterExpansion, fcc_prim

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _fcc_ternary():
    facts = json.load(open(os.path.join(GOLD, "fcc_ternary_eci_facts.json")))
    ce = ClusterExpansion(fcc_prim(4.0, tuple(facts["occupants"])), {2: facts["max_length"]["2"]})
    return ce, facts


def test_builder_orbits_match_reference_eci_file():
    ce, facts = _fcc_ternary()
    ref = facts["orbits"]
    assert ref[0]["n_sites"] == 0  # empty cluster
    assert len(ce.orbits) == len(ref) - 1
    for o, r in zip(ce.orbits, ref[1:]):
        assert o.size == r["n_sites"]
        assert o.mult == r["mult"]
        assert abs(o.max_length - r["max_length"]) < 1e-6
        assert o.n_funcs == len(r["functions"])
        assert o.func_begin == r["functions"][0]["index"]
    assert ce.n_funcs == sum(len(r["functions"]) for r in ref)
    # mixed pair functions carry sqrt(1/2), as "\sqrt{1/2}(...)" in the ECI file
    assert ce.func_coeff[4] == 0.707107 and ce.func_coeff[7] == 0.707107
    # sparse ECI file indexes the same functions
    for idx, val in facts["sparse_eci"]:
        assert 0 <= idx < ce.n_funcs


def test_oracle_multiplicities_match_reference(oracle_mod):
    ce, facts = _fcc_ternary()
    o = oracle_mod.OracleSystem(ce, (6, 6, 6))
    m = o.multiplicities()
    for r in facts["orbits"][1:]:
        for f in r["functions"]:
            assert m[f["index"]] == r["mult"]


def test_oracle_matches_reference_clexulator(oracle_mod):
    g = json.load(open(os.path.join(GOLD, "fcc_ternary_clexulator.json")))
    ce, _ = _fcc_ternary()
    L = g["L"]
    o = oracle_mod.OracleSystem(ce, (L, L, L))
    m = o.multiplicities()
    n_checked = 0
    for case in g["cases"]:
        occ = np.array(case["occ"], dtype=np.int8)
        np.testing.assert_allclose(o.corr(occ), case["corr"], rtol=0, atol=1e-13)
        for d in case["deltas"]:
            _, dc = o.delta(occ, [d["site"]], [d["occ_f"]])
            dcorr = ce.func_coeff * dc / m
            dcorr[0] = 0.0
            np.testing.assert_allclose(dcorr, d["dcorr"], rtol=0, atol=1e-13)
            n_checked += 1
    assert n_checked >= 100


def test_reference_neighbour_list_order_is_symmetric_halves():
    """The probe orders the Clexulator's neighbourhood by r^T W r then
    lexicographically; its global functions must then use one of each +-d
    pair (indices 7-12 and 16-18), which pins the order used above."""
    g = json.load(open(os.path.join(GOLD, "fcc_ternary_clexulator.json")))
    nl = [tuple(x) for x in g["nlist"]]
    assert nl[0] == (0, 0, 0)
    half1 = set(nl[7:13])
    assert all(tuple(-x for x in v) in set(nl[1:7]) for v in half1)
    half2 = set(nl[16:19])
    assert all(tuple(-x for x in v) in set(nl[13:16]) for v in half2)


def test_mt19937_64_known_answer(oracle_mod):
    # C++ standard [rand.predef]: the 10000th output of a default-constructed
    # mt19937_64 (seed 5489) is 9981545732273789042
    assert int(oracle_mod.mt19937_64(5489, 10000)[-1]) == 9981545732273789042


def test_philox_known_answers(oracle_mod):
    # Random123 known-answer vectors for Philox4x32-10
    kat = [
        ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
        ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
        ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
         [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
    ]
    for ctr, key, want in kat:
        assert list(oracle_mod.philox4x32_10(ctr, key)) == want


def _lemire(stream, maxv):
    rng = maxv + 1
    x = next(stream)
    m = x * rng
    lo = m & (2**64 - 1)
    if lo < rng:
        t = (2**64 - rng) % rng
        while lo < t:
            x = next(stream)
            m = x * rng
            lo = m & (2**64 - 1)
    return m >> 64


def test_random_transforms_restated_match_libstdcxx(oracle_mod):
    """The GPU replay restates uniform_int_distribution<long> (Lemire's
    method) and generate_canonical<double,53> on the raw mt19937_64 stream;
    check both restatements against this host's libstdc++."""
    seed = 424242
    rng = np.random.default_rng(1)
    maxv = np.concatenate([rng.integers(0, 2000, 3000), rng.integers(0, 2**40, 1000),
                           [0, 1, 2**62, 2**63 - 1]]).astype(np.int64)
    want, draws = oracle_mod.std_uniform_int(seed, maxv)
    raw = iter(int(v) for v in oracle_mod.mt19937_64(seed, draws + 10))
    got = [_lemire(raw, int(m)) for m in maxv]
    assert got == [int(v) for v in want]
    reals = oracle_mod.std_uniform_real(seed, 5000)
    raw = oracle_mod.mt19937_64(seed, 5000)
    mine = np.array([min(float(int(x)) / 2.0**64, np.nextafter(1.0, 0.0)) for x in raw])
    np.testing.assert_array_equal(mine, reals)
