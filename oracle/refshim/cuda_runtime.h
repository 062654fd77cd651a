/* Minimal stand-in for <cuda_runtime.h> used ONLY to compile the reference's
 * src/core3d/cuda/CUDA_kernels.cu as host C++ so its tet local solver
 * (localSolverTet1) can be called on the CPU to pin the oracle.  The kernels in
 * that file compile into plain functions that are never called. */
#pragma once
#include <algorithm>
#include <cmath>
#define __device__
#define __global__
#define __shared__
#define __host__
struct float3 { float x, y, z; };
struct float4 { float x, y, z, w; };
struct uint3 { unsigned x, y, z; };
static inline float3 make_float3(float x, float y, float z) { float3 r{x, y, z}; return r; }
static uint3 threadIdx, blockIdx, blockDim, gridDim;
static inline void __syncthreads() {}
/* device min/max on floats are fminf/fmaxf */
static inline float min(float a, float b) { return fminf(a, b); }
static inline float max(float a, float b) { return fmaxf(a, b); }
using std::sqrt;
