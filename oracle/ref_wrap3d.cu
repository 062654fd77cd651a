// Wraps the reference's 3D kernels (src/core3d/cuda/CUDA_kernels.cu, compiled from
// the reference tree by build_oracle.py) as extern "C" kernels in a cubin, so the
// GPU parity tests can run the reference's own device arithmetic on the same
// inputs as the product.  Test infrastructure only.
#include <cuda_runtime.h>
#pragma push_macro("__global__")
#undef __global__
#define __global__ __device__
#include "cuda/CUDA_kernels.cu"
#pragma pop_macro("__global__")

extern "C" __global__ void ref3d_fim(float3* m0, float3* m1, float4* tT, float* vT, float* sp, int* vm, int* vmo,
                                     int* bs, bool* con, int* al, int maxIn, int mapIn, int mapOut, int nIter) {
  FIMCuda(m0, m1, tT, vT, sp, vm, vmo, bs, con, al, maxIn, mapIn, mapOut, nIter);
}
extern "C" __global__ void ref3d_check(float3* m0, float3* m1, float4* tT, float* sp, int* vm, int* vmo, int* bs,
                                       bool* con, int* al, int maxIn, int mapIn, int mapOut) {
  run_check_neghbor(m0, m1, tT, sp, vm, vmo, bs, con, al, maxIn, mapIn, mapOut);
}
extern "C" __global__ void ref3d_copyout(float4* tT, float* vT, int* vm, int* vmo, int* bs, int* al, int maxIn,
                                         int maxTets, int mapIn, int mapOut) {
  CopyOutBack(tT, vT, vm, vmo, bs, al, maxIn, maxTets, mapIn, mapOut);
}
extern "C" __global__ void ref3d_reduce(bool* con, bool* bc, int* al, int n, int* bs) {
  run_reduction(con, bc, al, n, bs);
}
// element-wise local solver on packed inputs (9 floats per call)
extern "C" __global__ void ref3d_local_solver(const float* in, float* out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const float* a = in + 9 * (size_t)i;
    out[i] = localSolverTet1(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8]);
  }
}
