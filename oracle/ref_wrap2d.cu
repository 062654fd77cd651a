// Wraps the reference's 2D kernels (src/core2d/cuda/CUDA_kernels.cu) as extern "C"
// kernels in a cubin for the GPU parity tests.  Test infrastructure only.
#include <cuda_runtime.h>
#pragma push_macro("__global__")
#undef __global__
#define __global__ __device__
#include "cuda/CUDA_kernels.cu"
#pragma pop_macro("__global__")

extern "C" __global__ void ref2d_fim(float* tm, float* tmo, int* vm, int* vmo, float* e0, float* e1, float* e2,
                                     float* sp, int* bs, int* con, int* al, int nact, int maxF, int maxV, float sd) {
  FIMCuda(tm, tmo, vm, vmo, e0, e1, e2, sp, bs, con, al, nact, maxF, maxV, sd);
}
extern "C" __global__ void ref2d_check(float* tm, float* tmo, int* vm, int* vmo, float* e0, float* e1, float* e2,
                                       float* sp, int* bs, int* con, int* al, int nold, int maxF, int maxV, int ntot,
                                       int sd) {
  run_check_neighbor(tm, tmo, vm, vmo, e0, e1, e2, sp, bs, con, al, nold, maxF, maxV, ntot, sd);
}
extern "C" __global__ void ref2d_reduce(int* con, int* bc, int* al, int n, int* bs) {
  run_reduction(con, bc, al, n, bs);
}
