#!/usr/bin/env bash
# Builds the CPU oracle (test infrastructure) from oracle.cpp in two forms:
#   oracle/_build/liboracle.so        strict IEEE arithmetic (-fno-fast-math
#                                     -ffp-contract=off): the parity checker
#   oracle/_build/liboracle_tuned.so  the reference's release intent
#                                     (-O3 -ffast-math -funroll-loops, as its
#                                     CMakeLists.txt release flags): the timed
#                                     CPU leg
# Portable flags only: the same recipe runs on x86_64 and aarch64 hosts. No
# CPU-family tuning: a build with -mcpu=neoverse-v2 stopped with an illegal
# instruction on the GPU host.
set -euo pipefail
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
mkdir -p "$here/_build"
g++ -O3 -fno-fast-math -ffp-contract=off -fopenmp -fPIC -shared -std=c++17 \
    -o "$here/_build/liboracle.so.tmp" "$here/oracle.cpp" &
strict=$!
g++ -O3 -ffast-math -funroll-loops -fopenmp -fPIC -shared -std=c++17 \
    -o "$here/_build/liboracle_tuned.so.tmp" "$here/oracle.cpp" &
tuned=$!
wait $strict
wait $tuned
mv "$here/_build/liboracle.so.tmp" "$here/_build/liboracle.so"
mv "$here/_build/liboracle_tuned.so.tmp" "$here/_build/liboracle_tuned.so"
