#!/usr/bin/env bash
# Builds the CPU oracle (TEST INFRASTRUCTURE ONLY) into oracle/_build/.
# -ffp-contract=off keeps every float expression unfused, as the oracle's
# bit-level comparisons assume; -fopenmp parallelises the per-particle
# density/force/advance loops for the timed CPU baseline. adjoint64.c is the
# FP64 frozen-structure model and adjoint the adjoint tests check against.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
mkdir -p "$HERE/_build"
gcc -std=gnu11 -O2 -ffp-contract=off -fno-fast-math -fopenmp -fPIC -shared \
    "$HERE/fluids_oracle.c" "$HERE/adjoint64.c" -lm -o "$HERE/_build/libfluids_oracle.so"
echo "build_oracle: built $HERE/_build/libfluids_oracle.so"
