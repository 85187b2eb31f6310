#!/usr/bin/env bash
# Compiles the parts of the reference that build standalone from the reference tree into
# oracle/_ref/ (git-ignored):
#   libref_random.so - its vendored dSFMT and Random.cpp, to cross-check the oracle's
#                      restated RNG;
#   libref_gsd.so    - its vendored GSD 1.0 library gsd.c, to read the files the frame writer
#                      writes and to write the golden files it must reproduce byte for byte.
# The rest of the reference does not build (missing Cell.hpp/MD.hpp/CIL.hpp/Units.hpp,
# Boost, HDF5).
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
if [ -f "$REF/gsd.c" ]; then
  gcc -O2 -fPIC -shared -I"$REF" "$REF/gsd.c" -o "$OUT/libref_gsd.so"
  echo "built $OUT/libref_gsd.so"
fi
