#!/bin/bash
# Compile a generated Clexulator of the reference, where it lies in the
# reference tree, against the shim in oracle/ref_shim, into oracle/_ref/.
# Needs the reference sources (present only where they are mounted).
#   build_ref.sh        FCC_binary_vacancy bset.default (one sublattice)
#   build_ref.sh zro    Clex_ZrO_Occ bset.formation_energy (hcp Zr + O/Va)
#   build_ref.sh fcc-time  timing probe of the FCC Clexulator's delta evaluation
# Prints the path of the built probe on its last line.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
# The reference tree: $REFERENCE_ROOT, else the read-only mount of the
# reference sources in the build container. Exit status 2 when absent.
REF="${REFERENCE_ROOT:-/root/reference}"
if [ ! -d "$REF" ]; then
  echo "reference sources not found at $REF (set REFERENCE_ROOT)" >&2
  exit 2
fi
DATA="$REF/tests/unit/clexmonte/data"
mkdir -p "$HERE/_ref"
case "${1:-fcc}" in
  fcc)
    SRC="$DATA/FCC_binary_vacancy/basis_sets/bset.default/FCC_binary_vacancy_Clexulator_default.cc"
    [ -f "$SRC" ] || { echo "reference sources not found: $SRC" >&2; exit 2; }
    g++ -O1 -std=c++17 -I "$HERE/ref_shim" "$SRC" "$HERE/ref_probe_fcc.cc" -o "$HERE/_ref/fcc_clexulator_probe"
    echo "$HERE/_ref/fcc_clexulator_probe"
    ;;
  fcc-time)
    SRC="$DATA/FCC_binary_vacancy/basis_sets/bset.default/FCC_binary_vacancy_Clexulator_default.cc"
    [ -f "$SRC" ] || { echo "reference sources not found: $SRC" >&2; exit 2; }
    g++ -O3 -std=c++17 -I "$HERE/ref_shim" "$SRC" "$HERE/ref_time_fcc.cc" -o "$HERE/_ref/fcc_clexulator_time"
    echo "$HERE/_ref/fcc_clexulator_time"
    ;;
  zro)
    SRC="$DATA/Clex_ZrO_Occ/basis_sets/bset.formation_energy/ZrO_Clexulator_formation_energy.cc"
    [ -f "$SRC" ] || { echo "reference sources not found: $SRC" >&2; exit 2; }
    g++ -O1 -std=c++17 -I "$HERE/ref_shim" -DPROBE_FACTORY=make_ZrO_Clexulator_formation_energy \
      "$SRC" "$HERE/ref_probe_xtal.cc" -o "$HERE/_ref/zro_clexulator_probe"
    echo "$HERE/_ref/zro_clexulator_probe"
    ;;
  *)
    echo "unknown probe: $1" >&2
    exit 2
    ;;
esac
