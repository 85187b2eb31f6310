#!/usr/bin/env bash
# Builds the oracle (test infrastructure) into oracle/_build/liboracle.so.
# Strict IEEE arithmetic: no FMA contraction, no fast-math (the reference's own
# -Ofast -ffast-math flags, include.mk:6-9, are deliberately not used).
set -euo pipefail
HERE=$(cd "$(dirname "$0")" && pwd)
mkdir -p "$HERE/_build"
g++ -std=c++17 -O2 -ffp-contract=off -fno-fast-math -fopenmp -fPIC -shared \
    -o "$HERE/_build/liboracle.so" "$HERE/cil_oracle.cpp" "$HERE/cil_cycle_oracle.cpp"
echo "built $HERE/_build/liboracle.so"
