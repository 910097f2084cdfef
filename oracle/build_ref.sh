#!/usr/bin/env bash
# ORACLE — test infrastructure only.
#
# Builds the reference's own code from its sources where they lie (read-only)
# into oracle/_ref/, for pinning the oracle and generating golden fixtures:
#   _ref/MD          the reference driver MD.cpp, flags as its Makefile:2-3
#                    plus -ffp-contract=off (no FMA contraction on any host)
#   _ref/ref_dump    oracle/ref_dump.cpp linked against the reference headers
#   _ref/liposome    generate/liposome.cpp
#   _ref/bilayer     generate/bilayer.cpp
# Usage: oracle/build_ref.sh reference_root   (or $SMD_REFERENCE_ROOT)
set -euo pipefail
REF="${1:-${SMD_REFERENCE_ROOT:-}}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ -z "$REF" ] || [ ! -f "$REF/MD.cpp" ]; then
  echo "reference sources not found (give their root as the argument or in SMD_REFERENCE_ROOT); nothing to build" >&2
  exit 0
fi
mkdir -p "$OUT"
CXX="${CXX:-g++}"
FLAGS="-O3 -std=c++11 -ffp-contract=off"
$CXX $FLAGS -fopenmp "$REF/MD.cpp" -o "$OUT/MD" &
$CXX $FLAGS -fopenmp -I"$REF" "$HERE/ref_dump.cpp" -o "$OUT/ref_dump" &
$CXX $FLAGS -I"$REF/generate" "$REF/generate/liposome.cpp" -o "$OUT/liposome" &
$CXX $FLAGS -I"$REF/generate" "$REF/generate/bilayer.cpp" -o "$OUT/bilayer" &
wait
echo "built reference tools into $OUT"
