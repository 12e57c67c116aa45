"""General crystals (CPU): factor groups, the reference's Clex_ZrO_Occ basis
set rebuilt orbit by orbit, and its correlations pinned to the reference's
generated ZrO Clexulator (golden vectors from tests/golden/make_zro_golden.py)."""

import json

import numpy as np
import pytest

from casmcode_clexmonte_gb300 import casm_io, workloads
from casmcode_clexmonte_gb300.crystal import Crystal, CrystalClusterExpansion, canonical
from casmcode_clexmonte_gb300.system import Supercell

from tests.zro_fixture import documents, facts, golden, zro_ce


@pytest.fixture(scope="module")
def ce():
    return zro_ce()


def _owned_counts(ce, L, occ):
    """Integer function counts from the owned-cluster tables (each periodic
    cluster once), occupation basis phi = [occ == 1]."""
    sc = Supercell(tuple(L))
    b, i, j, k = sc.coords(ce.prim)
    occ = np.asarray(occ, dtype=np.int64)
    cnt = np.zeros(ce.n_funcs, dtype=np.int64)
    cnt[0] = sc.n_uc
    for kb in range(ce.prim.n_basis):
        sel = np.nonzero(b == kb)[0]
        for c in ce.owned[kb]:
            v = occ[sel].copy()
            for pb, du in c.partners:
                v = v * occ[sc.index(pb, i[sel] + du[0], j[sel] + du[1], k[sel] + du[2])]
            cnt[c.lut[0]] += int(v.sum())
    return cnt


def test_factor_group_sizes():
    prim, _, _ = documents()
    cr = casm_io.read_crystal(prim)
    assert len(cr.ops) == 24  # hcp-based P6_3/mmc
    assert cr.dof == [2, 3] and cr.fixed_counts() == {"Zr": 2}
    fcc = Crystal("FCC", [[0, 2, 2], [2, 0, 2], [2, 2, 0]], [[0, 0, 0]], [("A", "B")])
    assert len(fcc.ops) == 48
    bcc2 = Crystal("BCC", np.eye(3) * 3.2, [[0, 0, 0], [0.5, 0.5, 0.5]], [("A", "B")] * 2)
    assert len(bcc2.ops) == 96  # 48 rotations x the body-centring translation


def test_zro_orbits_match_reference_basis_set(ce):
    f = facts()
    assert len(ce.orbits) == len(f["orbits"]) - 1 == 73
    assert ce.n_funcs == 74
    for o, ref in zip(ce.orbits, f["orbits"][1:]):
        assert o.size == len(ref["sites"])
        assert o.mult == ref["mult"]
        assert o.max_length == pytest.approx(ref["max_length"], abs=1e-6)
        assert o.min_length == pytest.approx(ref["min_length"], abs=1e-6)
        key = canonical(ce.ops, [(s[0], tuple(s[1:])) for s in ref["sites"]])
        assert canonical(ce.ops, o.proto_sites) == key
    assert [len(ce.flowers[b]) for b in range(2)] == [1591, 1591]
    # every periodic cluster owned once: owned clusters per cell = sum of mult
    assert sum(len(ce.owned[b]) for b in range(2)) == sum(o.mult for o in ce.orbits)
    want = np.zeros(ce.n_funcs)
    for o in f["orbits"]:
        for fn in o["functions"]:
            want[fn["index"]] = fn["eci"]
    np.testing.assert_array_equal(ce.eci, want)


def test_zro_built_order_is_a_permutation_of_the_reference(ce):
    free = CrystalClusterExpansion(ce.crystal, ce.max_length)
    a = sorted((o.size, o.mult, round(o.max_length, 6)) for o in free.orbits)
    b = sorted((o.size, o.mult, round(o.max_length, 6)) for o in ce.orbits)
    assert a == b
    with pytest.raises(ValueError, match="not among"):
        CrystalClusterExpansion(ce.crystal, {2: 5.0}, orbit_order=[[], [(2, (0, 0, 0)), (2, (0, 0, 2))]])


def test_zro_correlations_match_reference_clexulator(ce):
    g = golden()
    assert g["sublat"] == [2, 3]
    L = g["L"]
    n_uc = int(np.prod(L))
    sc = Supercell(tuple(L))
    b, i, j, k = sc.coords(ce.prim)
    mult = ce.func_mult
    for case in g["cases"]:
        occ = np.array(case["occ"], dtype=np.int64)
        cnt = _owned_counts(ce, L, occ)
        corr = ce.func_coeff * cnt / (mult * n_uc)
        corr[0] = 1.0
        np.testing.assert_allclose(corr, case["corr"], rtol=0, atol=1e-14)
        for dl in case["deltas"]:
            l, of = dl["site"], dl["occ_f"]
            dc = np.zeros(ce.n_funcs)
            for c in ce.flowers[int(b[l])]:
                v = 1
                for pb, du in c.partners:
                    v *= occ[sc.index(pb, i[l] + du[0], j[l] + du[1], k[l] + du[2])]
                dc[c.lut[0]] += v * (of - occ[l])
            dcorr = ce.func_coeff * dc / mult
            dcorr[0] = 0.0
            np.testing.assert_allclose(dcorr, dl["dcorr"], rtol=0, atol=1e-14)


def test_oracle_zro_matches_reference_clexulator(ce, oracle_mod):
    g = golden()
    o = oracle_mod.OracleSystem(ce, g["L"])
    m = o.multiplicities()
    for f in range(1, ce.n_funcs):
        assert m[f] == ce.orbits[ce.func_orbit[f]].mult
    for case in g["cases"]:
        occ = np.array(case["occ"], dtype=np.int8)
        np.testing.assert_allclose(o.corr(occ), case["corr"], rtol=0, atol=1e-14)
        for dl in case["deltas"]:
            _, dc = o.delta(occ, [dl["site"]], [dl["occ_f"]])
            dcorr = ce.func_coeff * dc / m
            dcorr[0] = 0.0
            np.testing.assert_allclose(dcorr, dl["dcorr"], rtol=0, atol=1e-14)
        # the formation energy is the correlations . ECI per unit cell
        assert o.energy(occ) == pytest.approx(float(np.dot(case["corr"], ce.eci)) * o.n_uc,
                                              rel=1e-12, abs=1e-9)


def test_zro_composition_axes(ce):
    # a = 0.5 - 0.25 Va + 0.25 O per unit cell over (Zr, Va, O): the rows of
    # R^T over the dof species (Va, O)
    np.testing.assert_allclose(ce.param_RT, [[-0.25, 0.25]])
    x = ce.param_RT @ (np.array([0.5, 1.5]) - np.array([2.0, 0.0]))
    np.testing.assert_allclose(x, [0.75])
    _, _, axes = documents()
    bad = json.loads(json.dumps(axes))
    bad["origin"] = [[1.0], [3.0], [0.0]]
    with pytest.raises(ValueError, match="origin"):
        casm_io.composition_axes_RT(bad, ce.prim.occupants, ce.crystal.fixed_counts())


def test_general_builder_reproduces_cubic_fcc():
    """The crystal builder on the FCC prim gives the cubic builder's orbits,
    functions and energies."""
    cube = workloads.fcc_binary_ce(2)
    p = cube.prim
    lat = p.lattice * p.grid
    cr = Crystal("FCC", lat, [[0, 0, 0]], [p.occupants])
    gen = CrystalClusterExpansion(cr, cube.max_length)
    assert [(o.size, o.mult, round(o.max_length, 6)) for o in gen.orbits] == \
        [(o.size, o.mult, round(o.max_length, 6)) for o in cube.orbits]
    gen.eci = cube.eci.copy()
    L = (6, 6, 6)
    rng = np.random.default_rng(5)
    occ = rng.integers(0, 2, 216)
    np.testing.assert_array_equal(_owned_counts(gen, L, occ)[1:], _owned_counts(cube, L, occ)[1:])


def test_eci_json_round_trip_zro(ce, tmp_path):
    path = str(tmp_path / "eci.json")
    casm_io.write_eci_json(ce, path)
    doc = json.load(open(path))
    back = casm_io.read_cluster_expansion(doc["prim"], path)
    assert back.n_funcs == ce.n_funcs
    np.testing.assert_array_equal(back.eci, ce.eci)
    assert [(o.size, o.mult) for o in back.orbits] == [(o.size, o.mult) for o in ce.orbits]


def test_summary_writer_follows_zro_composition_axes(tmp_path):
    """mol_composition in summary.json over Zr, Va, O from the system's
    composition axes (Zr(2)Va(2-2a)O(2a))."""
    _, _, axes = documents()
    path = str(tmp_path / "summary.json")
    w = casm_io.SummaryWriter(path, "semigrand_canonical", ["Va", "O"], n_sites_per_uc=2,
                              composition_axes=axes)
    stats = {"mean_potential": -1.0, "mean_formation": -1.1, "var_potential": 1e-4,
             "mean_comp": [0.25], "cov_comp": [[1e-4]], "cov_e_comp": [1e-5],
             "n_samples": 100.0, "n_accepted": 40, "n_proposed": 100}
    w.append(temperature=1200.0, n_unitcells=512, stats=stats, param_chem_pot=[-0.5])
    w.write()
    data = json.load(open(path))
    mc = data["statistics"]["mol_composition"]
    assert mc["component_names"] == ["Zr", "Va", "O"]
    assert [mc[c]["mean"][0] for c in ("Zr", "Va", "O")] == pytest.approx([2.0, 1.5, 0.5])


def test_local_swaps_connect_every_site(ce):
    """Canonical local-swap displacements are the partners of the shortest
    pair orbits, taken until the swaps connect every site with a degree of
    freedom (graph over the sublattices connected, cycle translations
    generating Z^3). FCC: the nearest neighbours. ZrO: the O-O pairs along c
    only link the octahedral sites of one column (a conserved O count per
    column colour would make the canonical chain non-ergodic), so the
    in-plane O-O pairs are added."""
    from casmcode_clexmonte_gb300.system import _lattice_index, _swaps_connect

    assert _lattice_index([(1, 0, 0), (0, 1, 0), (0, 0, 1)]) == 1
    assert _lattice_index([(1, 1, 0), (0, 1, 1), (1, 0, 1)]) == 2
    assert _lattice_index([(1, 1, 0), (0, 1, 1), (1, 0, 1), (1, 0, 0)]) == 1
    assert _lattice_index([(0, 0, 1), (0, 0, 2)]) == 0
    fcc = workloads.fcc_binary_ce(0)
    shortest = min((o for o in fcc.orbits if o.size == 2), key=lambda o: o.max_length).index
    assert fcc.local_swap_orbits() == {shortest}
    assert len(fcc.neighbour_partners(0)) == 12
    pairs = sorted((o for o in ce.orbits if o.size == 2), key=lambda o: o.max_length)
    subl = sorted(ce.flowers)
    only_c = [(b, c.partners[0][0], tuple(c.partners[0][1])) for b in subl for c in ce.flowers[b]
              if c.orbit == pairs[0].index]
    assert all(du[0] == 0 and du[1] == 0 for _, _, du in only_c)
    assert not _swaps_connect(subl, only_c)
    sel = ce.local_swap_orbits()
    assert pairs[0].index in sel and len(sel) == 2
    edges = [(b, pb, tuple(du)) for b in subl for pb, du in ce.neighbour_partners(b)]
    assert _swaps_connect(subl, edges)
    assert all(len(ce.neighbour_partners(b)) <= 16 for b in subl)
