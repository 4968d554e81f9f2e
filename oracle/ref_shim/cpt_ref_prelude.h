/* Test infrastructure for the oracle (never part of the shipped library).
 *
 * Force-included (g++ -include) in front of every translation unit of the reference
 * that the recipe in oracle/Makefile compiles as host C++.  It supplies the few
 * CUDA-device names the reference's path uses so that its own kernels can run as
 * ordinary host functions:
 *   - __clzll: count leading zeros of a 64-bit word, 64 for zero (PTX clz.b64 semantics),
 *     used by findSplit/delta (BVH.cuh:94,111,127);
 *   - threadIdx/blockIdx/blockDim: thread-local launch coordinates read by
 *     render (Render.cu:20-21) and generateMortonCodes (Device.cuh:136). */
#pragma once
#include <cuda_runtime.h>

static inline int __clzll(long long x)
{
    return x == 0 ? 64 : __builtin_clzll((unsigned long long)x);
}

extern thread_local uint3 threadIdx;
extern thread_local uint3 blockIdx;
extern thread_local dim3 blockDim;
