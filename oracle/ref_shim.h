/*
 * ref_shim.h -- TEST INFRASTRUCTURE ONLY (oracle tier 1).
 *
 * Force-included (g++ -include) ahead of the reference's own kernel source
 * fluids4.0/fluid_kernels.cu so that g++ compiles it as plain host C++.
 * Each CUDA thread index becomes a host global that ref_wrap.cpp sets before
 * calling a kernel body for one particle; atomicAdd becomes a serial add, so
 * running particles in index order gives the canonical within-cell order
 * (gndx = number of earlier particles in the same cell).
 *
 * Nothing here is part of the product; only tests/, bench.py's CPU arm and
 * the smoke check load the library built from it.
 */
#pragma once

/* Execution-space qualifiers vanish on the host. Defined before
 * crt/host_defines.h is reached so it keeps these definitions. */
#define __global__
#define __device__
#define __host__
#define __shared__
#define __constant__
#define __forceinline__ inline

/* curand: only the off-path emit/randomInit kernels use it; they are never
 * called. Pre-claim the headers' include guards and supply the one type. */
#define CURAND_KERNEL_H_
#define CURAND_H_
typedef struct { unsigned int d; } curandState_t;
static inline void curand_init(unsigned long long, unsigned long long,
                               unsigned long long, curandState_t *s) { s->d = 0; }
static inline unsigned int curand(curandState_t *s) { return s->d++; }

#include <cuda_runtime.h>   /* float3/int3/uint3 and make_* (host-usable) */

/* Thread coordinates of the one "thread" being run. */
extern thread_local uint3 blockIdx;
extern thread_local uint3 blockDim;
extern thread_local uint3 threadIdx;

static inline unsigned int __mul24(unsigned int a, unsigned int b) { return a * b; }
static inline void __syncthreads(void) {}
static inline unsigned int atomicAdd(unsigned int *p, int v) {
    unsigned int old = *p;
    *p = old + (unsigned int)v;
    return old;
}
