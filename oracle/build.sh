#!/usr/bin/env bash
# Builds the CPU oracle (test infrastructure) from oracle.cpp in two forms:
#   oracle/_build/liboracle.so        strict IEEE arithmetic (-fno-fast-math
#                                     -ffp-contract=off): the parity checker
#   oracle/_build/liboracle_tuned.so  the reference's release intent
#                                     (-O3 -ffast-math -funroll-loops, as its
#                                     CMakeLists.txt release flags): the timed
#                                     CPU leg
# The same recipe runs on x86_64 and aarch64 hosts. On a Neoverse V2 host
# (Grace) the timed build is tuned for that core, named explicitly; where the
# kernel exposes no SVE (the Features line of /proc/cpuinfo), SVE code
# generation is switched off, since SVE instructions would stop with an
# illegal instruction there. If the compiler refuses the tuning flags, the
# build falls back to the untuned release flags.
set -euo pipefail
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
mkdir -p "$here/_build"
tune=""
if [ "$(uname -m)" = "aarch64" ] && grep -qi "0xd4f" /proc/cpuinfo 2>/dev/null; then
  if grep -i "^Features" /proc/cpuinfo | head -1 | grep -qw sve; then
    tune="-mcpu=neoverse-v2"
  else
    tune="-mcpu=neoverse-v2+nosve+nosve2"
  fi
fi
g++ -O3 -fno-fast-math -ffp-contract=off -fopenmp -fPIC -shared -std=c++17 \
    -o "$here/_build/liboracle.so.tmp" "$here/oracle.cpp" &
strict=$!
( g++ -O3 -ffast-math -funroll-loops $tune -fopenmp -fPIC -shared -std=c++17 \
      -o "$here/_build/liboracle_tuned.so.tmp" "$here/oracle.cpp" 2>/dev/null ||
  g++ -O3 -ffast-math -funroll-loops -fopenmp -fPIC -shared -std=c++17 \
      -o "$here/_build/liboracle_tuned.so.tmp" "$here/oracle.cpp" ) &
tuned=$!
wait $strict
wait $tuned
mv "$here/_build/liboracle.so.tmp" "$here/_build/liboracle.so"
mv "$here/_build/liboracle_tuned.so.tmp" "$here/_build/liboracle_tuned.so"
echo "$tune" > "$here/_build/tuned_flags.txt"
