#!/usr/bin/env bash
# Builds the CPU oracle (test infrastructure) into oracle/_build/liboracle.so.
# Portable flags only: the same recipe runs on x86_64 and aarch64 hosts.
set -euo pipefail
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
mkdir -p "$here/_build"
g++ -O3 -fno-fast-math -ffp-contract=off -fopenmp -fPIC -shared -std=c++17 \
    -o "$here/_build/liboracle.so.tmp" "$here/oracle.cpp"
mv "$here/_build/liboracle.so.tmp" "$here/_build/liboracle.so"
