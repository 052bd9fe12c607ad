#!/usr/bin/env bash
# Builds oracle tier 1 (TEST INFRASTRUCTURE ONLY): the reference's own kernel
# source fluids4.0/fluid_kernels.cu compiled as host C++ through ref_shim.h,
# into oracle/_ref/libfluids_ref.so. Reads the reference tree in place
# (default /root/reference, or $FLUIDS_REF_ROOT); writes only oracle/_ref/.
# Exits 0 without building when the reference tree is absent.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${FLUIDS_REF_ROOT:-/root/reference}/fluids4.0"
if [ ! -f "$REF/fluid_kernels.cu" ]; then
    echo "build_ref: reference tree not found at $REF; skipping" >&2
    exit 0
fi
CUDA_INC="${CUDA_HOME:-/usr/local/cuda}/include"
mkdir -p "$HERE/_ref"
# -ffp-contract=off: no FMA contraction, so float expressions round exactly
# as written (the reference's CPU semantics; also what aarch64 gcc needs).
g++ -std=c++14 -O2 -ffp-contract=off -fno-fast-math -fopenmp -fPIC -shared \
    -w -I"$REF" -I"$CUDA_INC" -include "$HERE/ref_shim.h" \
    "$HERE/ref_wrap.cpp" -o "$HERE/_ref/libfluids_ref.so"
echo "build_ref: built $HERE/_ref/libfluids_ref.so"
