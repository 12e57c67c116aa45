"""The reference's Clex_ZrO_Occ system (hcp Zr, octahedral O/Va sites) from
the committed facts: prim.json, formation_energy_eci.json and system.json
documents in the reference's schema, and the cluster expansion read from
them by ``casm_io``."""

import json
import os

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def facts() -> dict:
    return json.load(open(os.path.join(GOLD, "zro_facts.json")))


def documents():
    """(prim, formation_energy_eci, composition_axes) documents."""
    f = facts()
    orbits = []
    for k, o in enumerate(f["orbits"]):
        funcs = []
        for fn in o["functions"]:
            d = {"linear_function_index": fn["index"]}
            if fn["eci"] != 0.0:
                d["eci"] = fn["eci"]
            funcs.append(d)
        orbits.append({
            "linear_orbit_index": k, "mult": o["mult"], "cluster_functions": funcs,
            "prototype": {"sites": o["sites"], "max_length": o["max_length"],
                          "min_length": o["min_length"]},
        })
    eci = {
        "bspecs": {
            "basis_function_specs": {"dof_specs": {"occ": {"site_basis_functions": "OCCUPATION"}}},
            "cluster_specs": {"method": "periodic_max_length", "params": {
                "orbit_branch_specs": {k: {"max_length": v} for k, v in f["max_length"].items()}}},
        },
        "orbits": orbits,
    }
    return f["prim"], eci, f["composition_axes"]


def zro_ce():
    from casmcode_clexmonte_gb300 import casm_io

    prim, eci, axes = documents()
    ce = casm_io.read_cluster_expansion(prim, eci)
    ce.param_RT = casm_io.composition_axes_RT(axes, ce.prim.occupants, ce.crystal.fixed_counts())
    return ce


def golden() -> dict:
    return json.load(open(os.path.join(GOLD, "zro_clexulator.json")))
