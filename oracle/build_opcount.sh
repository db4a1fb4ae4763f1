#!/usr/bin/env bash
# Builds the operation-counting oracle (test infrastructure) into
# oracle/_build/liboracle_opcount.so: oracle.cpp with every double (except on
# lines marked keep-double) replaced by the counting type of opcount.h and the
# std:: math calls by its overloads; no OpenMP (the counters are plain
# integers).
set -euo pipefail
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
mkdir -p "$here/_build"
sed -e '/keep-double/!s/\bdouble\b/Real/g' \
    -e 's/std::numeric_limits<Real>/std::numeric_limits<double>/g' \
    -e 's/std::\(abs\|fabs\|sqrt\|exp\|cos\|sin\|atan\|pow\|copysign\|max\|min\)(/oc::\1(/g' \
    "$here/oracle.cpp" > "$here/_build/oracle_opcount.cpp"
g++ -O1 -std=c++17 -fPIC -shared -DORC_OPCOUNT -include "$here/opcount.h" -I"$here" \
    -o "$here/_build/liboracle_opcount.so.tmp" "$here/_build/oracle_opcount.cpp"
mv "$here/_build/liboracle_opcount.so.tmp" "$here/_build/liboracle_opcount.so"
