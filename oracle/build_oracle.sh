#!/bin/sh
# Builds oracle/_build/libtvoracle.so from the C restatement (test infrastructure).
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$HERE/_build"
gcc -std=c11 -O2 -ffp-contract=off -fPIC -shared -fopenmp -Wall -Wno-unused-function \
    "$HERE/tvoracle_eig.c" "$HERE/tvoracle_filter.c" "$HERE/tvoracle_vote.c" "$HERE/tvoracle_mlp.c" \
    -lm -o "$HERE/_build/libtvoracle.so"
