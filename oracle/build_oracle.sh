#!/bin/sh
# Build the CPU oracle (test infrastructure; never linked into the product).
# IEEE semantics are required: no fast-math, no FMA contraction (gcc on aarch64
# contracts by default, so -ffp-contract=off is explicit).
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$HERE/_build"
gcc -O2 -std=c11 -fPIC -shared -fopenmp -ffp-contract=off -fno-fast-math \
    -o "$HERE/_build/libfteik_oracle.so" "$HERE/fteik_oracle.c" -lm
