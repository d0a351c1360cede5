#!/usr/bin/env bash
# Builds the UNMODIFIED reference (UAlex322/GraphAlgo) into a test-only shared
# library, oracle/_ref/libref.so, straight from its own sources:
#   include/*.h, src/main.cpp (its main() renamed), src/mmio.cpp
# plus the harness oracle/ref/ref_harness.cpp and an empty stand-in for the
# missing bin_reader.h. Nothing is copied out of the reference tree.
# The reference's own CMake build is not used.
#
#   REF=/path/to/GraphAlgo oracle/build_ref.sh
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
REF="${REF:-/root/reference}"
if [ ! -f "$REF/include/matrix_la.h" ]; then
    echo "reference sources not found under $REF; skipping" >&2
    exit 0
fi
out="$here/_ref"
mkdir -p "$out"
# The reference prints with the CPU's native char signedness; -fsigned-char
# keeps the MSA state bytes identical on Arm and x86.
g++ -O3 -std=c++17 -fopenmp -fPIC -shared -fsigned-char -ffp-contract=off -w \
    -I"$here/ref/stub" -I"$REF/include" -I"$REF/src" \
    "$here/ref/ref_harness.cpp" "$REF/src/mmio.cpp" \
    -o "$out/libref.so"
# where the sources were, for the tests that read the reference's graph files
printf '%s\n' "$REF" > "$out/source_dir"
echo "built $out/libref.so"
