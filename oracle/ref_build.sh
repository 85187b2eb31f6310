#!/usr/bin/env bash
# Compiles the parts of the reference that build standalone from the reference tree into
# oracle/_ref/ (git-ignored):
#   libref_random.so - its vendored dSFMT and Random.cpp, to cross-check the oracle's
#                      restated RNG;
#   libref_gsd.so    - its vendored GSD 1.0 library gsd.c, to read the files the frame writer
#                      writes and to write the golden files it must reproduce byte for byte;
#   libref_utils.so  - its Utils.hpp (Nint, BoundingBox, LinkListOrtho2D/3D), with
#                      oracle/boost_shim standing in for the two Boost headers it includes, to
#                      pin the oracle's box and link-list geometry;
#   libref_force.so  - its MD.cuh Lennard-Jones law (LJParams::elemForce) compiled as host C++
#                      with the stand-ins of oracle/ref_stubs for the headers its tree lacks, to
#                      pin the oracle's LJ force.
# The rest of the reference does not build (its .cu files, the missing CIL.hpp, HDF5).
set -euo pipefail
REF=${CIL_REFERENCE_DIR:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -f "$REF/mt/dSFMT.c" ] || [ ! -f "$REF/Random.hpp" ]; then
  echo "reference tree not found at $REF; nothing to build" >&2
  exit 0
fi
mkdir -p "$OUT"
# where the tree was found, for the tests that read the reference's own files (oracle/refdir.py)
(cd "$REF" && pwd) > "$OUT/reference_dir"
gcc -O2 -fPIC -DDSFMT_MEXP=19937 -I"$REF/mt" -c "$REF/mt/dSFMT.c" -o "$OUT/dSFMT.o"
g++ -O2 -fPIC -std=c++11 -DDSFMT_MEXP=19937 -I"$REF" -c "$REF/Random.cpp" -o "$OUT/Random.o"
g++ -O2 -fPIC -std=c++11 -DDSFMT_MEXP=19937 -I"$REF" -c "$HERE/ref_random_shim.cpp" -o "$OUT/shim.o"
g++ -shared -o "$OUT/libref_random.so" "$OUT/shim.o" "$OUT/Random.o" "$OUT/dSFMT.o"
echo "built $OUT/libref_random.so"
if [ -f "$REF/Utils.hpp" ]; then
  # -DNDEBUG: the reference's asserts (positions inside the box) are not part of what is pinned
  g++ -O2 -fPIC -shared -std=c++11 -DNDEBUG -ffp-contract=off -I"$HERE/boost_shim" -I"$REF" \
      "$HERE/ref_utils_shim.cpp" -o "$OUT/libref_utils.so"
  echo "built $OUT/libref_utils.so"
fi
if [ -f "$REF/MD.cuh" ]; then
  g++ -O2 -fPIC -shared -std=c++14 -DNDEBUG -ffp-contract=off -D__host__= -D__device__= -D__global__= \
      -DSIMIO_HPP -I"$HERE/ref_stubs" -I"$HERE/boost_shim" -I"$REF" -w \
      "$HERE/ref_force_shim.cpp" -o "$OUT/libref_force.so"
  echo "built $OUT/libref_force.so"
fi
if [ -f "$REF/gsd.c" ]; then
  gcc -O2 -fPIC -shared -I"$REF" "$REF/gsd.c" -o "$OUT/libref_gsd.so"
  echo "built $OUT/libref_gsd.so"
fi
