#!/bin/bash
# Compile the reference's generated FCC Clexulator, where it lies in the
# reference tree, against the shim in oracle/ref_shim, into oracle/_ref/.
# Needs the reference sources (present only where they are mounted).
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${REFERENCE_ROOT:-/root/reference}"
SRC="$REF/tests/unit/clexmonte/data/FCC_binary_vacancy/basis_sets/bset.default/FCC_binary_vacancy_Clexulator_default.cc"
[ -f "$SRC" ] || { echo "reference sources not found: $SRC" >&2; exit 2; }
mkdir -p "$HERE/_ref"
g++ -O1 -std=c++17 -I "$HERE/ref_shim" "$SRC" "$HERE/ref_probe_fcc.cc" -o "$HERE/_ref/fcc_clexulator_probe"
echo "$HERE/_ref/fcc_clexulator_probe"
