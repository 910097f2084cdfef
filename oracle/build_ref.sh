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
#   _ref/MDcuda      the reference's own FP32 CUDA driver MDcuda.cu, unmodified,
#                    for sm_103a (C++17: CUDA 13's thrust requires it), when nvcc
#                    is present.  It is built as a check that the reference GPU
#                    port compiles for GB300; the binary is for this host's
#                    architecture and cannot run where no reference sources are.
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
NVCC="$(command -v nvcc || echo /usr/local/cuda/bin/nvcc)"
if [ -x "$NVCC" ] && [ -f "$REF/MDcuda.cu" ]; then
  (cd "$OUT" && "$NVCC" -gencode arch=compute_103a,code=sm_103a -O3 -std=c++17 "$REF/MDcuda.cu" -o "$OUT/MDcuda") &
fi
wait
echo "built reference tools into $OUT"
