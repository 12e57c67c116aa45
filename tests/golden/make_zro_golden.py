"""Generate the golden vectors that pin the general-crystal path (hcp Zr with
octahedral O/Va sites, the reference's Clex_ZrO_Occ fixture).

Run in a container where the reference sources are mounted (default
/root/reference, or $REFERENCE_ROOT). It

1. compiles the reference's generated ZrO Clexulator against the shim
   (``oracle/build_ref.sh zro``) and runs the probe, which writes global
   correlations and delta point correlations for seeded random O/Va
   configurations of an 8 x 8 x 6 supercell -> tests/golden/zro_clexulator.json;
2. extracts the prim, composition axes, cluster specs and orbits (prototype
   sites, multiplicities, lengths, function indices, ECI) of the reference's
   Clex_ZrO_Occ/{prim,system,formation_energy_eci}.json
   -> tests/golden/zro_facts.json.
"""

import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
# the reference tree: $REFERENCE_ROOT, else its read-only mount in the
# container that generates the fixtures
REF = os.environ.get("REFERENCE_ROOT", "/root/reference")
if not os.path.isdir(REF):
    sys.exit(f"reference sources not found at {REF}: set REFERENCE_ROOT to the reference tree")


def main():
    probe = subprocess.run(
        [os.path.join(ROOT, "oracle", "build_ref.sh"), "zro"], check=True, capture_output=True,
        text=True,
    ).stdout.strip().splitlines()[-1]
    out = subprocess.run([probe, "8", "8", "6", "2", "24", "20261204"], check=True,
                         capture_output=True, text=True).stdout
    data = json.loads(out)
    data["source"] = (
        "tests/unit/clexmonte/data/Clex_ZrO_Occ/basis_sets/bset.formation_energy/"
        "ZrO_Clexulator_formation_energy.cc via oracle/ref_probe_xtal.cc"
    )
    with open(os.path.join(HERE, "zro_clexulator.json"), "w") as f:
        json.dump(data, f, separators=(",", ":"))

    d = os.path.join(REF, "tests/unit/clexmonte/data/Clex_ZrO_Occ")
    prim = json.load(open(os.path.join(d, "prim.json")))
    system = json.load(open(os.path.join(d, "system.json")))
    eci = json.load(open(os.path.join(d, "formation_energy_eci.json")))
    orbits = []
    for o in eci["orbits"]:
        orbits.append({
            "mult": o["mult"],
            "sites": o["prototype"]["sites"],
            "max_length": o["prototype"]["max_length"],
            "min_length": o["prototype"]["min_length"],
            "functions": [{"index": cf["linear_function_index"], "eci": cf.get("eci", 0.0)}
                          for cf in o["cluster_functions"]],
        })
    facts = {
        "source": "tests/unit/clexmonte/data/Clex_ZrO_Occ/{prim,system,formation_energy_eci}.json",
        "prim": prim,
        "composition_axes": system["composition_axes"],
        "max_length": {k: v["max_length"] for k, v in
                       eci["bspecs"]["cluster_specs"]["params"]["orbit_branch_specs"].items()},
        "orbits": orbits,
    }
    with open(os.path.join(HERE, "zro_facts.json"), "w") as f:
        json.dump(facts, f, indent=0)
    print("wrote golden fixtures")


if __name__ == "__main__":
    sys.exit(main())
