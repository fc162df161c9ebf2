#!/bin/sh
# Builds the CPU oracle (test infrastructure only) into oracle/_build/.
# -ffp-contract=off keeps a*b+c unfused, as the reference's FP64 radius test is
# evaluated on x86-64 without FMA.
set -e
here="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$here/_build"
out="$here/_build/liboracle.so"
if [ ! -f "$out" ] || [ "$here/aboria_oracle.cpp" -nt "$out" ]; then
  g++ -O2 -std=c++17 -fopenmp -fPIC -shared -ffp-contract=off \
      -o "$out" "$here/aboria_oracle.cpp"
fi
echo "$out"
