#!/usr/bin/env bash
# Builds the reference's own CPU k-means (comparisons/CPU_Kmeans) from the
# sources where they lie in the reference tree into oracle/_ref/, for use as a
# checker of the oracle restatement (tests) and as the reference CPU baseline.
#
#   oracle/build_ref.sh [REFERENCE_ROOT]
#   oracle/build_ref.sh --print-root          (prints the resolved root)
#
# The root is the argument, else $KM_REFERENCE_ROOT, else /root/reference;
# nothing else in the repository names the reference tree's location.
#
# Only the reference's kmeans.cpp and its headers are compiled, together with
# oracle/ref_shim.cpp (a C entry point); the reference's header-only dataset
# reader/writer (src/include/input_parser.hpp) is compiled with
# oracle/ref_io_shim.cpp.  The reference's main.cpp is not used:
# it calls a stale 11-argument parse_input_args (main.cpp:22) that no longer
# matches utils.hpp:92-99.  -ffp-contract=off keeps every float operation
# separately rounded, which is what the reference's makefile build does on
# x86-64 (no FMA without -march), and makes an aarch64 build agree with it.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
if [ "${1:-}" = "--print-root" ]; then
  echo "${KM_REFERENCE_ROOT:-/root/reference}"
  exit 0
fi
REF="${1:-${KM_REFERENCE_ROOT:-/root/reference}}"
SRC="$REF/comparisons/CPU_Kmeans/src/kmeans.cpp"
if [ ! -f "$SRC" ]; then
  echo "build_ref.sh: reference sources not found under $REF; skipping" >&2
  exit 0
fi
mkdir -p "$HERE/_ref"
g++ -O2 -std=c++17 -ffp-contract=off -fPIC -shared -w \
    -I"$REF/src/include" -I"$REF/comparisons/CPU_Kmeans/include" \
    "$HERE/ref_shim.cpp" "$SRC" -o "$HERE/_ref/libref_kmeans.so"
echo "built $HERE/_ref/libref_kmeans.so"
# the reference's dataset reader/writer (header-only), behind C entry points
g++ -O2 -std=c++17 -fPIC -shared -w -I"$REF/src/include" \
    "$HERE/ref_io_shim.cpp" -o "$HERE/_ref/libref_io.so"
echo "built $HERE/_ref/libref_io.so"
