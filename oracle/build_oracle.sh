#!/bin/sh
# Builds the CPU oracle (test infrastructure) into oracle/_build/liboracle.so.
# -ffp-contract=off keeps gcc from fusing multiply-adds (it does so by
# default on aarch64), so the oracle rounds exactly like the reference.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
mkdir -p "$HERE/_build"
gcc -O3 -fPIC -shared -fopenmp -ffp-contract=off -fno-fast-math -std=gnu99 \
    -Wall -Wno-unused-function \
    -o "$HERE/_build/liboracle.so" "$HERE/tsph_oracle.c" -lm
echo "built $HERE/_build/liboracle.so"
