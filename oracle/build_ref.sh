#!/usr/bin/env bash
# Builds oracle tier 1 (TEST INFRASTRUCTURE ONLY): the reference's own kernel
# source fluids4.0/fluid_kernels.cu compiled as host C++ through ref_shim.h,
# into oracle/_ref/libfluids_ref.so, and as a GPU module for sm_103a into
# oracle/_ref/fluid_kernels_sm103a.fatbin. Reads the reference tree in place
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

# The same kernel source as a GPU module for sm_103a, with the code-generation
# flags of the reference's own build (fluids4.0/CMakeLists.txt:91: -O3
# --use_fast_math --maxrregcount=32; its PTX target becomes sm_103a code).
# oracle/ref_gpu.py loads it through the driver API, as FluidSystem loads its
# module, to check the product against the reference's GPU results and to
# time the reference on the same GPU.
NVCC="${CUDA_HOME:-/usr/local/cuda}/bin/nvcc"
if [ -x "$NVCC" ]; then
    "$NVCC" -fatbin -std=c++14 -gencode arch=compute_103a,code=sm_103a -O3 --use_fast_math \
        --maxrregcount=32 -w -I"$REF" -o "$HERE/_ref/fluid_kernels_sm103a.fatbin" "$REF/fluid_kernels.cu"
    echo "build_ref: built $HERE/_ref/fluid_kernels_sm103a.fatbin"
fi
