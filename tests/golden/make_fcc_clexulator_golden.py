"""Generate the golden vectors that pin the oracle to the reference.

Run in a container where the reference sources are mounted (default
/root/reference, or $REFERENCE_ROOT). It

1. compiles the reference's generated FCC Clexulator against the shim
   (oracle/build_ref.sh) and runs the probe, which writes global correlations
   and delta point correlations for seeded random A/B/Va configurations
   -> tests/golden/fcc_ternary_clexulator.json;
2. extracts the orbit multiplicities, function counts and ECI values of the
   reference's FCC_binary_vacancy/formation_energy_eci.json and
   formation_energy_sparse_eci.json
   -> tests/golden/fcc_ternary_eci_facts.json.
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
        [os.path.join(ROOT, "oracle", "build_ref.sh")], check=True, capture_output=True, text=True
    ).stdout.strip().splitlines()[-1]
    out = subprocess.run([probe, "6", "3", "40", "20251203"], check=True, capture_output=True, text=True).stdout
    data = json.loads(out)
    data["source"] = (
        "tests/unit/clexmonte/data/FCC_binary_vacancy/basis_sets/bset.default/"
        "FCC_binary_vacancy_Clexulator_default.cc via oracle/ref_probe_fcc.cc"
    )
    with open(os.path.join(HERE, "fcc_ternary_clexulator.json"), "w") as f:
        json.dump(data, f)

    d = os.path.join(REF, "tests/unit/clexmonte/data/FCC_binary_vacancy")
    eci = json.load(open(os.path.join(d, "formation_energy_eci.json")))
    sparse = json.load(open(os.path.join(d, "formation_energy_sparse_eci.json")))
    orbits = []
    for o in eci["orbits"]:
        funcs = [
            {"index": cf["linear_function_index"], "eci": cf.get("eci", 0.0)}
            for cf in o["cluster_functions"]
        ]
        orbits.append(
            {
                "mult": o["mult"],
                "n_sites": len(o["prototype"]["sites"]),
                "max_length": o["prototype"]["max_length"],
                "functions": funcs,
            }
        )
    facts = {
        "source": "tests/unit/clexmonte/data/FCC_binary_vacancy/formation_energy_eci.json",
        "occupants": eci["prim"]["basis"][0]["occupants"],
        "max_length": {k: v["max_length"] for k, v in eci["bspecs"]["cluster_specs"]["params"]["orbit_branch_specs"].items()},
        "orbits": orbits,
        "sparse_eci": sparse,
    }
    with open(os.path.join(HERE, "fcc_ternary_eci_facts.json"), "w") as f:
        json.dump(facts, f, indent=1)
    print("wrote golden fixtures")


if __name__ == "__main__":
    sys.exit(main())
