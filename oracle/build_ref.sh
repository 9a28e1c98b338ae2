#!/bin/sh
# Builds oracle/_ref/libtiraref.so: tiralib's own CPU tensor-voting functions,
# compiled unmodified from the reference headers with the glm / Boost
# stand-ins in oracle/shim.  Test infrastructure only (see oracle/ref/tira_ref.cpp).
# Usage: oracle/build_ref.sh <path to the tiralib checkout>
set -e
REF="${1:?path to the tiralib checkout}"
HERE="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$HERE/_ref"
g++ -std=c++20 -O2 -ffp-contract=off -fPIC -shared -w \
    -I"$REF" -I"$HERE/shim" \
    "$HERE/ref/tira_ref.cpp" -o "$HERE/_ref/libtiraref.so"
