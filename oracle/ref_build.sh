#!/usr/bin/env bash
# Compiles the parts of the reference that build standalone (its vendored dSFMT and the
# header-only Random.hpp) from the reference tree into oracle/_ref/ for cross-checking
# the oracle's restated RNG. Outputs go to oracle/_ref/ only (git-ignored). The rest of
# the reference does not build (missing Cell.hpp/MD.hpp/CIL.hpp/Units.hpp, Boost, HDF5).
set -euo pipefail
REF=${CIL_REFERENCE_DIR:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -f "$REF/mt/dSFMT.c" ] || [ ! -f "$REF/Random.hpp" ]; then
  echo "reference tree not found at $REF; nothing to build" >&2
  exit 0
fi
mkdir -p "$OUT"
gcc -O2 -fPIC -DDSFMT_MEXP=19937 -I"$REF/mt" -c "$REF/mt/dSFMT.c" -o "$OUT/dSFMT.o"
g++ -O2 -fPIC -std=c++11 -DDSFMT_MEXP=19937 -I"$REF" -c "$REF/Random.cpp" -o "$OUT/Random.o"
g++ -O2 -fPIC -std=c++11 -DDSFMT_MEXP=19937 -I"$REF" -c "$HERE/ref_random_shim.cpp" -o "$OUT/shim.o"
g++ -shared -o "$OUT/libref_random.so" "$OUT/shim.o" "$OUT/Random.o" "$OUT/dSFMT.o"
echo "built $OUT/libref_random.so"
