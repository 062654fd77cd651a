// Host build of the reference's tet local solver, for pinning the oracle only.
// Compiled from the reference source where it lies (see build_oracle.py) with the
// stand-in header in refshim/; nothing here is part of the product.
#include "cuda/CUDA_kernels.cu"

// the kernels' dynamic shared-memory arrays, never used on the host
char s_array[1];
float s_run_check_neghbor_array[1];

extern "C" float ref_tet_local_solver(float TA, float TB, float TC, float ACAC, float ACBC, float ACCD,
                                      float BCBC, float BCCD, float CDCD) {
  return localSolverTet1(TA, TB, TC, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD);
}
