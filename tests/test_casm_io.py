"""Reference-format files: prim.json and basis-set/ECI JSON in, ECI JSON and
summary.json out (CPU only)."""

import json
import os

import numpy as np
import pytest

from casmcode_clexmonte_gb300 import casm_io, workloads
from casmcode_clexmonte_gb300.casm_io import (
    SummaryWriter,
    equilibration_index,
    read_cluster_expansion,
    read_prim,
    write_eci_json,
)

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _fcc_ternary_docs():
    """prim.json and formation_energy_eci.json documents with the content of
    the reference's FCC_binary_vacancy fixture (orbit structure and ECI from
    the committed facts)."""
    facts = json.load(open(os.path.join(GOLD, "fcc_ternary_eci_facts.json")))
    prim = {
        "title": "FCC_binary_vacancy",
        "coordinate_mode": "Fractional",
        "lattice_vectors": [[0.0, 2.0, 2.0], [2.0, 0.0, 2.0], [2.0, 2.0, 0.0]],
        "basis": [{"coordinate": [0.0, 0.0, 0.0], "occupants": facts["occupants"]}],
    }
    orbits = []
    for k, o in enumerate(facts["orbits"]):
        funcs = []
        for f in o["functions"]:
            d = {"linear_function_index": f["index"]}
            if f["eci"] != 0.0:
                d["eci"] = f["eci"]
            funcs.append(d)
        orbits.append({
            "linear_orbit_index": k, "mult": o["mult"], "cluster_functions": funcs,
            "prototype": {"sites": [[0, 0, 0, 0]] * o["n_sites"], "max_length": o["max_length"]},
        })
    eci = {
        "bspecs": {
            "basis_function_specs": {"dof_specs": {"occ": {"site_basis_functions": "OCCUPATION"}}},
            "cluster_specs": {"method": "periodic_max_length", "params": {
                "orbit_branch_specs": {k: {"max_length": v} for k, v in facts["max_length"].items()}}},
        },
        "orbits": orbits,
    }
    return prim, eci, facts


def test_read_prim_fcc_matches_builder():
    prim, _, _ = _fcc_ternary_docs()
    p = read_prim(prim)
    assert p.grid == pytest.approx(2.0)
    assert p.lattice.tolist() == [[0, 1, 1], [1, 0, 1], [1, 1, 0]]
    assert p.occupants == ("A", "B", "Va")


def test_read_cluster_expansion_reference_fixture():
    prim, eci, facts = _fcc_ternary_docs()
    ce = read_cluster_expansion(prim, eci)
    want = np.zeros(ce.n_funcs)
    for o in facts["orbits"]:
        for f in o["functions"]:
            want[f["index"]] = f["eci"]
    np.testing.assert_array_equal(ce.eci, want)
    ce2 = read_cluster_expansion(prim, eci, sparse_eci=facts["sparse_eci"])
    want2 = np.zeros(ce.n_funcs)
    for i, v in facts["sparse_eci"]:
        want2[i] = v
    np.testing.assert_array_equal(ce2.eci, want2)


def test_read_energy_matches_reference_clexulator(oracle_mod):
    """Energy of the file-built expansion = reference correlations . ECI."""
    prim, eci, _ = _fcc_ternary_docs()
    ce = read_cluster_expansion(prim, eci)
    gold = json.load(open(os.path.join(GOLD, "fcc_ternary_clexulator.json")))
    L = gold["L"]
    o = oracle_mod.OracleSystem(ce, (L, L, L))
    for case in gold["cases"]:
        occ = np.asarray(case["occ"], dtype=np.int8)
        corr = np.asarray(case["corr"], dtype=np.float64)
        assert o.energy(occ) / L ** 3 == pytest.approx(float(corr @ ce.eci), abs=1e-12)


def test_mismatched_orbits_are_rejected():
    prim, eci, _ = _fcc_ternary_docs()
    bad = json.loads(json.dumps(eci))
    bad["orbits"][2]["mult"] = 7
    with pytest.raises(ValueError, match="orbit 2"):
        read_cluster_expansion(prim, bad)
    bad = json.loads(json.dumps(eci))
    bad["bspecs"]["basis_function_specs"]["dof_specs"]["occ"]["site_basis_functions"] = "CHEBYCHEV"
    with pytest.raises(ValueError, match="not supported"):
        read_cluster_expansion(prim, bad)
    mixed = json.loads(json.dumps(prim))
    mixed["basis"].append({"coordinate": [0.5, 0.5, 0.5], "occupants": ["A", "B"]})
    with pytest.raises(ValueError, match="same occupants"):
        read_prim(mixed)


@pytest.mark.parametrize("make", [lambda: workloads.fcc_binary_ce(3),
                                  lambda: workloads.bcc_ternary_ce(3)])
def test_eci_json_round_trip(make, tmp_path):
    ce = make()
    path = str(tmp_path / "eci.json")
    write_eci_json(ce, path)
    doc = json.load(open(path))
    back = read_cluster_expansion(doc["prim"], path)
    assert back.n_funcs == ce.n_funcs
    np.testing.assert_array_equal(back.eci, ce.eci)
    assert [(o.size, o.mult, o.n_funcs) for o in back.orbits] == \
        [(o.size, o.mult, o.n_funcs) for o in ce.orbits]
    np.testing.assert_array_equal(back.func_coeff, ce.func_coeff)


def test_equilibration_index():
    rng = np.random.default_rng(0)
    flat = rng.normal(0.0, 0.01, 4000)
    assert equilibration_index(flat, 0.005) == 0
    transient = flat.copy()
    transient[:800] += np.linspace(1.0, 0.0, 800)
    k = equilibration_index(transient, 0.005)
    assert k is not None and 200 <= k <= 800
    walk = np.cumsum(rng.normal(0.0, 1.0, 4000))
    assert equilibration_index(walk, 1e-3) is None


# restatement of the reference tests' summary.json checks
# (python/tests/conftest.py:141-259)
def _validate(data, size, canonical, convergence):
    def block(sub, keys):
        for x in keys:
            assert x in sub
            if "component_names" in sub[x]:
                for y in sub[x]["component_names"]:
                    assert len(sub[x][y]) == size
            elif "value" in sub[x]:
                assert sub[x]["shape"] == []
                assert len(sub[x]["value"]) == size
            else:
                assert len(sub[x]) == size

    if canonical:
        cond = ["temperature", "param_composition", "mol_composition"]
        ana = ["heat_capacity"]
    else:
        cond = ["temperature", "param_chem_pot"]
        ana = ["heat_capacity", "mol_susc", "param_susc", "mol_thermochem_susc",
               "param_thermochem_susc"]
    block(data["analysis"], ana)
    cc = ["N_samples", "N_samples_for_statistics", "acceptance_rate", "count", "elapsed_clocktime"]
    if convergence:
        cc += ["N_samples_for_all_to_equilibrate", "all_converged", "all_equilibrated"]
    block(data["completion_check_results"], cc)
    block(data["conditions"], cond)
    st = data["statistics"]
    for x in ["clex.formation_energy", "mol_composition", "param_composition", "potential_energy"]:
        assert x in st
        if "component_names" in st[x]:
            for y in st[x]["component_names"]:
                for z in ["mean", "calculated_precision"]:
                    assert len(st[x][y][z]) == size
        else:
            assert st[x]["shape"] == []
            for z in ["mean", "calculated_precision"]:
                assert len(st[x]["value"][z]) == size
    if convergence:
        assert "is_converged" in st["potential_energy"]["value"]
        if not canonical:
            assert "is_converged" in st["param_composition"]["a"]


def _fake_stats(rng, nc):
    cov = np.eye(nc) * 1e-4
    return dict(n_samples=500.0, mean_potential=-0.1, var_potential=2e-6, mean_formation=-0.09,
                mean_comp=np.full(nc, 0.3), cov_comp=cov, cov_e_comp=np.full(nc, 1e-5),
                n_proposed=10000, n_accepted=2500)


@pytest.mark.parametrize("method,components", [("canonical", ["A", "B"]),
                                               ("semigrand_canonical", ["A", "B", "C"])])
@pytest.mark.parametrize("convergence", [False, True])
def test_summary_layout(method, components, convergence, tmp_path):
    rng = np.random.default_rng(1)
    nc = len(components) - 1
    req = {"potential_energy": 1e-3, "param_composition": 1e-3} if convergence else None
    path = str(tmp_path / "out" / "summary.json")
    w = SummaryWriter(path, method, components, n_sites_per_uc=2, requested_precision=req)
    temps = [300.0, 400.0, 500.0]
    for T in temps:
        pot = -0.1 + rng.normal(0, 1e-3, 500)
        comp = 0.3 + rng.normal(0, 1e-3, (500, nc))
        w.append(temperature=T, n_unitcells=1000, stats=_fake_stats(rng, nc),
                 samples=(pot, comp), param_chem_pot=np.zeros(nc), elapsed_s=1.0, count=500)
    w.write()
    data = json.load(open(path))
    _validate(data, len(temps), method == "canonical", convergence)
    kb = casm_io.KB
    assert data["analysis"]["heat_capacity"]["value"][0] == pytest.approx(
        2e-6 * 1000 / (kb * 300.0 ** 2))
    # mol composition per unit cell of a 2-site cell: origin 2 A, axes 2 (e_k - e_A)
    mol = data["statistics"]["mol_composition"]
    assert mol["A"]["mean"][0] == pytest.approx(2 * (1 - 0.3 * nc))
    assert mol["B"]["mean"][0] == pytest.approx(0.6)
    if method == "semigrand_canonical":
        ps = data["analysis"]["param_susc"]
        assert ps["component_names"] == ["a,a", "b,a", "a,b", "b,b"]
        assert ps["a,a"][0] == pytest.approx(1e-4 * 1000 / (kb * 300.0))
        ms = data["analysis"]["mol_susc"]
        assert ms["B,B"][0] == pytest.approx(4 * ps["a,a"][0])
        assert ms["A,A"][0] == pytest.approx(4 * 2 * ps["a,a"][0])


def _write_project(tmp_path, sparse: bool, axes=None):
    """A CASM project directory in the reference's layout (system.json,
    basis_sets/bset.default/{bspecs,basis}.json, coefficients)."""
    prim, eci, facts = _fcc_ternary_docs()
    bdir = tmp_path / "basis_sets" / "bset.default"
    bdir.mkdir(parents=True)
    json.dump(eci["bspecs"], open(bdir / "bspecs.json", "w"))
    basis = json.loads(json.dumps(eci))
    for o in basis["orbits"]:
        for f in o["cluster_functions"]:
            f.pop("eci", None)
    json.dump(basis, open(bdir / "basis.json", "w"))
    if sparse:
        json.dump(facts["sparse_eci"], open(tmp_path / "eci.json", "w"))
    else:
        json.dump(eci, open(tmp_path / "eci.json", "w"))
    system = {
        "prim": prim,
        "composition_axes": axes or {"components": ["A", "B", "Va"], "origin": [1.0, 0.0, 0.0],
                                     "a": [0.0, 1.0, 0.0], "b": [0.0, 0.0, 1.0],
                                     "independent_compositions": 2},
        "basis_sets": {"default": {"source": "basis_sets/bset.default/FCC_Clexulator_default.cc"}},
        "clex": {"formation_energy": {"basis_set": "default", "coefficients": "eci.json"}},
    }
    json.dump(system, open(tmp_path / "system.json", "w"))
    return str(tmp_path / "system.json"), facts


@pytest.mark.parametrize("sparse", [False, True])
def test_read_system_json(sparse, tmp_path):
    path, facts = _write_project(tmp_path, sparse)
    ce = casm_io.read_system(path)
    want = np.zeros(ce.n_funcs)
    for i, v in facts["sparse_eci"]:
        want[i] = v
    np.testing.assert_array_equal(ce.eci, want)
    from casmcode_clexmonte_gb300.system import composition_RT, system_arrays

    np.testing.assert_allclose(ce.param_RT, composition_RT(1, 3))
    np.testing.assert_allclose(system_arrays(ce)["param_RT"], composition_RT(1, 3).reshape(-1))


def test_read_system_composition_axes(tmp_path):
    # axes listed in another component order and with the end members swapped
    axes = {"components": ["Va", "A", "B"], "origin": [0.0, 1.0, 0.0],
            "a": [1.0, 0.0, 0.0], "b": [0.0, 0.0, 1.0]}
    path, _ = _write_project(tmp_path, False, axes)
    ce = casm_io.read_system(path)
    # a = Va content, b = B content: rows of R^T select those species
    RT = ce.param_RT
    x = RT @ (np.array([0.5, 0.2, 0.3]) - np.array([1.0, 0.0, 0.0]))  # A, B, Va per unit cell
    np.testing.assert_allclose(x, [0.3, 0.2])
    bad = {"components": ["A", "B", "Va"], "origin": [0.0, 1.0, 0.0],
           "a": [1.0, 0.0, 0.0], "b": [0.0, 0.0, 1.0]}
    path2, _ = _write_project(tmp_path / "p2", False, bad)
    with pytest.raises(ValueError, match="origin"):
        casm_io.read_system(path2)
