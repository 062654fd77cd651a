// Host half of the reference's 3D set-up, for pinning the product's 3D host set-up
// only (test infrastructure; nothing here is part of the product).  Built by
// build_oracle.py with nvcc, as the reference's own build compiles these files,
// together with the reference's src/core3d/cuda/meshFIM3dEikonal.cu,
// tetmesh.cu and CUDA_kernels.cu where they lie (stand-ins for cusp and metis.h in
// refshim_nvcc/), into _ref/libref_host3d.so.  No CUDA call is made.
//
// ref_tet_gram runs TetMesh::init (tetmesh.cu:9-80: 0/1 index base, speed vector
// to per-tet metric) and then meshFIM3dEikonal::gettetmem (meshFIM3dEikonal.cu:
// 650-678: the six metric edge products vMv, Vec.h:479-483) for every tet, and
// returns the metric and the products the reference's GetTetMem stores per slot.
#include <vector>

#include "meshFIM3dEikonal.h"

// meshFIM3dEikonal.cu calls METIS only from GraphPartition_METIS2, which the pin
// never runs; the symbol must exist for the library to load.
extern "C" void METIS_PartGraphKway(int*, int*, int*, int*, int*, int*, int*, int* nparts, int*, int* edgecut,
                                    int*) {
  if (edgecut) *edgecut = -1;
  (void)nparts;
}

extern "C" int ref_tet_gram(int nv, const float* xyz, int nt, const int* tets, const float* speeds, int nspeeds,
                            float* metric_out, float* gram_out) {
  std::vector<float> pts(xyz, xyz + 3 * (size_t)nv);
  std::vector<int> tl(tets, tets + 4 * (size_t)nt);
  std::vector<float> sm;
  if (speeds && nspeeds > 0) sm.assign(speeds, speeds + nspeeds);
  TetMesh mesh;
  mesh.init(pts.data(), nv, nullptr, 0, tl.data(), nt, nullptr, sm, false);
  meshFIM3dEikonal fim;
  fim.SetMesh(&mesh);
  std::vector<float> tm;
  for (int t = 0; t < nt; ++t) {
    fim.gettetmem(tm, mesh.tets[t]);
    for (int k = 0; k < 6; ++k) {
      gram_out[6 * (size_t)t + k] = tm[k];
      metric_out[6 * (size_t)t + k] = mesh.tets[t].M[k];
    }
  }
  return 0;
}
