#!/bin/sh
# Build the CPU oracle (test infrastructure; never linked into the product).
#
# libfteik_oracle.so is the checker: IEEE semantics are required, so no
# fast-math and no FMA contraction (gcc on aarch64 contracts by default, so
# -ffp-contract=off is explicit).
#
# libfteik_oracle_fast.so is the same source built only to be timed as the CPU
# baseline, with the floating-point licences the reference's numba build takes
# (fteikpy/_common.py:12: contract, arcp, nsz, afn; not nnan or reassoc):
# -O3, contraction, reciprocal multiplication, no signed zeros, no errno from
# sqrt. It is not bitwise and is never used to check results. No -march/-mcpu
# flag: the same build has to run on x86_64 and aarch64 hosts.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$HERE/_build"
gcc -O2 -std=c11 -fPIC -shared -fopenmp -ffp-contract=off -fno-fast-math \
    -o "$HERE/_build/libfteik_oracle.so" "$HERE/fteik_oracle.c" -lm
gcc -O3 -std=c11 -fPIC -shared -fopenmp -ffp-contract=fast -freciprocal-math \
    -fno-signed-zeros -fno-math-errno -fno-trapping-math \
    -o "$HERE/_build/libfteik_oracle_fast.so" "$HERE/fteik_oracle.c" -lm
