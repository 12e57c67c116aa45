"""Host-side tables of the product (flower / owned clusters, decoration
tables, colourings) against the oracle's independent cluster enumeration."""

import itertools

import numpy as np
import pytest

from casmcode_clexmonte_gb300 import workloads
from casmcode_clexmonte_gb300.system import (
    ClusterExpansion, Supercell, fcc_prim, make_colouring, neighbour_index_table,
    system_arrays, verify_local_pairs,
)


def table_counts(ce, sc, occ):
    """Function counts from the product's owned-cluster tables (numpy)."""
    part = neighbour_index_table(ce, sc, "owned")
    b, *_ = sc.coords(ce.prim)
    counts = np.zeros(ce.n_funcs, dtype=np.int64)
    n_sf = ce.n_sf
    for bb, own in ce.owned.items():
        sel = np.nonzero(b == bb)[0]
        for ci, c in enumerate(own):
            vals = [occ[sel]] + [occ[part[sel, ci, j]] for j in range(len(c.partners))]
            ok = np.all(np.stack(vals) > 0, axis=0)
            code = np.zeros(len(sel), dtype=np.int64)
            for j, v in enumerate(vals):
                code += (v.astype(np.int64) - 1) * n_sf**j
            f = c.lut[code[ok]]
            np.add.at(counts, f, 1)
    counts[0] = sc.n_uc
    return counts


def table_delta(ce, sc, occ, site, occ_f):
    part = neighbour_index_table(ce, sc, "flowers")
    b, *_ = sc.coords(ce.prim)
    dc = np.zeros(ce.n_funcs, dtype=np.int64)
    n_sf = ce.n_sf
    for ci, c in enumerate(ce.flowers[b[site]]):
        vals = [occ[part[site, ci, j]] for j in range(len(c.partners))]
        if any(v == 0 for v in vals):
            continue
        base = sum((int(v) - 1) * n_sf ** (j + 1) for j, v in enumerate(vals))
        if occ[site] > 0:
            dc[c.lut[base + occ[site] - 1]] -= 1
        if occ_f > 0:
            dc[c.lut[base + occ_f - 1]] += 1
    return dc


CASES = [
    ("fcc_binary", lambda: workloads.fcc_binary_ce(3), (6, 6, 6)),
    ("fcc_ternary", lambda: ClusterExpansion(fcc_prim(4.0, ("A", "B", "Va")), {2: 4.1, 3: 4.01}), (5, 6, 7)),
    ("bcc_ternary", lambda: workloads.bcc_ternary_ce(5), (5, 5, 6)),
]


@pytest.mark.parametrize("name,make,L", CASES)
def test_tables_match_oracle(name, make, L, oracle_mod):
    ce = make()
    if ce.eci.sum() == 0:
        ce.eci = np.random.default_rng(0).normal(0, 0.05, ce.n_funcs)
    sc = Supercell(L)
    o = oracle_mod.OracleSystem(ce, L)
    np.testing.assert_allclose(o.multiplicities()[1:], ce.func_mult[1:])
    rng = np.random.default_rng(7)
    for _ in range(3):
        occ = rng.integers(0, ce.prim.n_occ, o.n_sites).astype(np.int8)
        np.testing.assert_array_equal(table_counts(ce, sc, occ), o.counts(occ) * (np.arange(ce.n_funcs) > 0) + np.eye(ce.n_funcs, dtype=np.int64)[0] * sc.n_uc)
        for _ in range(20):
            s = int(rng.integers(o.n_sites))
            f = int((occ[s] + rng.integers(1, ce.prim.n_occ)) % ce.prim.n_occ)
            _, dco = o.delta(occ, [s], [f])
            np.testing.assert_array_equal(table_delta(ce, sc, occ, s, f), dco)


def test_function_counts_of_benchmark_systems():
    ce = workloads.fcc_binary_ce(0)
    assert ce.n_funcs == 7
    assert [o.mult for o in ce.orbits] == [1, 6, 3, 12, 8, 12]
    assert [len([c for c in ce.flowers[0] if c.orbit == g]) for g in range(6)] == [1, 12, 6, 24, 24, 36]
    be = workloads.bcc_ternary_ce(0)
    assert be.n_funcs == 27
    assert [o.size for o in be.orbits] == [1, 2, 2, 2, 2, 3, 4]
    assert [o.n_funcs for o in be.orbits] == [2, 3, 3, 3, 3, 6, 6]
    for b in (0, 1):
        assert len(be.flowers[b]) == 111


def test_signatures_identify_functions():
    """The oracle identifies functions by edge invariants; they must be
    distinct for distinct functions of the benchmark systems."""
    for ce in (workloads.fcc_binary_ce(0), workloads.bcc_ternary_ce(0)):
        sig = ce.function_signatures()[1:]
        assert len(set(sig)) == len(sig)


@pytest.mark.parametrize("make,L", [
    (lambda: workloads.fcc_binary_ce(0), (10, 10, 10)),
    (lambda: workloads.fcc_binary_ce(0), (8, 8, 8)),
    (lambda: workloads.bcc_ternary_ce(0), (7, 7, 7)),
    (lambda: workloads.bcc_ternary_ce(0), (6, 6, 6)),
])
def test_colouring_and_local_pairs_are_non_interacting(make, L):
    ce = make()
    sc = Supercell(L)
    col = make_colouring(ce, sc)
    assert col.p == 2
    assert verify_local_pairs(ce, sc, col)


def test_system_arrays_shapes():
    ce = workloads.bcc_ternary_ce(0)
    a = system_arrays(ce)
    assert a["n_flower"] == 222 and a["flower_lut"].size == 222 * 16
    assert a["flower_partner_du"].size == 222 * 9
    assert np.all(a["n_neighbour"] == 8)


def test_generated_fcc_header_is_current():
    from casmcode_clexmonte_gb300 import codegen

    with open(codegen.OUT) as f:
        assert f.read() == codegen.fcc_binary_header()
