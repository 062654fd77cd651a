// fim_oracle.cpp — TEST INFRASTRUCTURE ONLY.
//
// A CPU restatement of the reference block-partitioned Fast Iterative Method
// (SCI-Solver_Eikonal) used as the checker for the GB300 CUDA path: the parity
// tests, smoke() and bench.py's cpu_baseline leg call it.  Nothing in the product
// library links or calls this file.
//
// It follows the reference's own data layout (padded per-block element slots that
// each carry their own copy of the vertex travel times, plus per-vertex lists of
// slot addresses) and its host schedule line by line, so that it is an independent
// second implementation of the same scheme rather than a copy of the product's
// compact layout.  Citations are paths inside the reference project.
//
//   3D:  src/core3d/cuda/meshFIM3dEikonal.cu  (PartitionTets :568-648,
//        GenerateData :285-566, GetTetMem :680-827, GetVertMem :829-923)
//        src/core3d/cuda/CUDA_kernels.cu     (FIMCuda :383-489,
//        run_check_neghbor :493-602, CopyOutBack :604-668, run_reduction :7-33,
//        localSolverTet1 :69-225)
//   2D:  src/core2d/cuda/meshFIM2d_eikonal.cu (PartitionFaces :254-347,
//        GenerateData :349-864)
//        src/core2d/cuda/CUDA_kernels.cu     (FIMCuda :36-409,
//        run_check_neighbor :415-799, run_reduction :8-30; triangle update :143-204)
//
// Every routine is instantiated for float (the reference arithmetic: FP32 with the
// two FP64 divisions the reference source writes) and for double (the "FP64 run of
// the same scheme" used to state the error of every FP32 result).
//
// Build: g++ -O2 -ffp-contract=off -fopenmp -shared -fPIC (oracle/build_oracle.py).
// -ffp-contract=off keeps every product rounded on its own, like the reference's
// host compile on x86-64; the GPU contracts a*b+c into FMA, so GPU-vs-oracle
// comparisons carry a tolerance while GPU-vs-reference-kernel comparisons are
// bitwise.

#include "oracle_scheme.hpp"
#include "tet_fusion_model.hpp"

using namespace oracle;

static double g_last_loop_seconds = 0;

extern "C" {

// Local updates, exposed for unit tests (precision 32 or 64).
float oracle_tet_update_f32(float TA, float TB, float TC, float ACAC, float ACBC, float ACCD,
                            float BCBC, float BCCD, float CDCD) {
  return tet_update<float>(TA, TB, TC, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD);
}
double oracle_tet_update_f64(double TA, double TB, double TC, double ACAC, double ACBC,
                             double ACCD, double BCBC, double BCCD, double CDCD) {
  return tet_update<double>(TA, TB, TC, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD);
}
float oracle_tri_update_f32(float TA, float TB, float TC, float LAB, float LBC, float LAC, float F) {
  return tri_update<float>(TA, TB, TC, LAB, LBC, LAC, F);
}

// Whole 3D solve.  tets are 0-based; M holds 6 metric entries per tet.  Returns the
// number of outer iterations (the length of the reference's iteration history), or
// -1 on bad input.  `out_final` receives the last snapshot of d_vertT mapped to
// vertices (0 for blocks that never ran, like the reference's cudaMemset buffer).
int oracle3d_solve(int nv, const float* xyz, int nt, const int* tets, const float* M,
                   const int* part, int nb, const int* seeds, int nseeds, int max_iters,
                   int nsweeps, int precision, int nthreads, float* out_final, float* history,
                   int hist_cap, long long* updates, int* max_tets) {
  if (nv <= 0 || nt <= 0 || nb <= 0) return -1;
  for (int v = 0; v < nv; ++v) if (part[v] < 0 || part[v] >= nb) return -1;
  auto run = [&](auto& o) {
    o.nv = nv; o.nt = nt; o.nb = nb; o.xyz = xyz; o.tets = tets; o.M = M; o.part = part;
    const int it = o.solve(seeds, nseeds, max_iters, nsweeps, nthreads, out_final, history, hist_cap, updates);
    if (max_tets) *max_tets = o.maxTets;
    g_last_loop_seconds = o.loopSeconds;
    return it;
  };
  if (precision == 64) { Oracle3D<double> o; return run(o); }
  Oracle3D<float> o;
  return run(o);
}

// Whole 2D solve on an oriented mesh with its virtual faces (see the product's
// triangle-mesh preparation).  speed_inv is per face; init_vals are the vertex
// values the reference keeps in TriMesh::vertT (used by its all-vertices
// convergence test).  Same return convention as oracle3d_solve.
int oracle2d_solve(int nv, const float* xyz, int nf, const int* faces, const float* speed_inv,
                   const uint8_t* obtuse, const int* vf_off, const int* vf_verts,
                   const float* vf_speed_inv, const int* part, int nb, const int* seeds,
                   int nseeds, const float* init_vals, int max_iters, int nsweeps, int precision,
                   int nthreads, float* out_final, float* history, int hist_cap,
                   long long* updates, int* max_faces) {
  if (nv <= 0 || nf <= 0 || nb <= 0) return -1;
  for (int v = 0; v < nv; ++v) if (part[v] < 0 || part[v] >= nb) return -1;
  auto run = [&](auto& o) {
    o.nv = nv; o.nf = nf; o.nb = nb; o.xyz = xyz; o.faces = faces; o.speedInv = speed_inv;
    o.obtuse = obtuse; o.vfOff = vf_off; o.vfVerts = vf_verts; o.vfSpeedInv = vf_speed_inv;
    o.part = part;
    const int it = o.solve(seeds, nseeds, init_vals, max_iters, nsweeps, nthreads, out_final,
                           history, hist_cap, updates);
    if (max_faces) *max_faces = o.maxFaces;
    return it;
  };
  if (precision == 64) { Oracle2D<double> o; return run(o); }
  Oracle2D<float> o;
  return run(o);
}

// Recursive coordinate bisection, restated so the CPU baseline and the reference
// arm of the benchmark run on the product's default partition without loading the
// product.  The reference partitions with METIS (meshFIM3dEikonal.cu:153-237); the
// product's default is this bisection: split the longest bounding-box axis of the
// point set so the lower part gets floor(n * floor(k/2) / k) points, points ordered
// by (coordinate, vertex id), parts [first, first + floor(k/2)) below and the rest
// above.  Same labels as the product's partitioner (a test holds them equal); this
// version sorts each level instead of selecting, and runs on one thread.
static void rcb_split(std::vector<int>& ids, size_t lo, size_t hi, int nparts, int first, const float* xyz,
                      int* labels) {
  const size_t n = hi - lo;
  if (nparts <= 1 || n <= 1) {
    for (size_t i = lo; i < hi; ++i) labels[ids[i]] = first;
    return;
  }
  float mn[3], mx[3];
  for (int d = 0; d < 3; ++d) mn[d] = mx[d] = xyz[3 * (size_t)ids[lo] + d];
  for (size_t i = lo + 1; i < hi; ++i)
    for (int d = 0; d < 3; ++d) {
      const float c = xyz[3 * (size_t)ids[i] + d];
      mn[d] = std::min(mn[d], c);
      mx[d] = std::max(mx[d], c);
    }
  int ax = 0;
  for (int d = 1; d < 3; ++d)
    if (mx[d] - mn[d] > mx[ax] - mn[ax]) ax = d;
  std::sort(ids.begin() + lo, ids.begin() + hi, [&](int a, int b) {
    const float ca = xyz[3 * (size_t)a + ax], cb = xyz[3 * (size_t)b + ax];
    return ca < cb || (ca == cb && a < b);
  });
  const int pl = nparts / 2;
  const size_t nl = (size_t)(((long long)n * pl) / nparts);
  rcb_split(ids, lo, lo + nl, pl, first, xyz, labels);
  rcb_split(ids, lo + nl, hi, nparts - pl, first + pl, xyz, labels);
}

// Block count of the product's partition rule: the reference's METIS block counts
// (2D nv / k, meshFIM2d_eikonal.cu; 3D ceil(nv / k), meshFIM3dEikonal.cu), at least
// 2 and at most nv.  Labels go to `labels` (nv ints); returns the block count.
int oracle_partition_rcb(int nv, const float* xyz, int verts_per_block, int dim, int* labels) {
  if (nv <= 0 || !xyz || !labels) return -1;
  const long long k = verts_per_block > 0 ? verts_per_block : 1;
  long long nb = (dim == 2) ? (long long)nv / k : ((long long)nv + k - 1) / k;
  nb = std::max(2ll, std::min(nb, (long long)nv));
  std::vector<int> ids(nv);
  for (int v = 0; v < nv; ++v) ids[v] = v;
  rcb_split(ids, 0, (size_t)nv, (int)nb, 0, xyz, labels);
  return (int)nb;
}

// The CPU model of the reference kernel's fused roundings (tet_fusion_model.hpp):
// n cases of 10 inputs -> 4 outputs each under masks[4].
void oracle_tet_group_fused(const float* in, int n, const unsigned long long* masks, float* out) {
  const uint64_t m[4] = {masks[0], masks[1], masks[2], masks[3]};
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) fusion::tet_group(m, in + 10 * (size_t)i, out + 4 * (size_t)i);
}

// Mismatches of apex k of the model under mask m against want (4 per case).
int oracle_tet_fusion_mismatch(const float* in, const float* want, int n, int k, unsigned long long m) {
  int bad = 0;
#pragma omp parallel for reduction(+ : bad) schedule(static)
  for (int i = 0; i < n; ++i) {
    uint64_t masks[4] = {0, 0, 0, 0};
    masks[k] = m;
    float o[4];
    fusion::tet_group(masks, in + 10 * (size_t)i, o);
    const float w = want[4 * (size_t)i + k];
    bad += std::memcmp(&o[k], &w, sizeof(float)) != 0;
  }
  return bad;
}

// FP64 fixed-point residual of travel times T: per vertex the smallest FP64 tet
// update over its incident tets (the four apex updates of the sweep above, from the
// FP64 edge products), LARGENUM where no update is finite.  Used to state how far a
// result is from a fixed point of the scheme, for the GPU result and for the FP64
// run of the scheme itself.
int oracle3d_fp64_candidates(int nv, const float* xyz, int nt, const int* tets, const float* M, const float* T,
                             double* cand) {
  if (nv <= 0 || nt <= 0) return -1;
  Oracle3D<double> o;
  o.nv = nv; o.nt = nt; o.xyz = xyz; o.tets = tets; o.M = M;
  for (int v = 0; v < nv; ++v) cand[v] = (double)kLarge3D;
  for (int t = 0; t < nt; ++t) {
    double g[6];
    o.tet_gram(t, g);
    const double ACBC = g[0], BCCD = g[1], ACCD = g[2], ADBD = g[3], ACAD = g[4], BCBD = g[5];
    const double ADBC = ACBC + BCCD, ACBD = ACBC + ACCD, CDBD = ADBD - ACBD, ADCD = ADBD - ADBC;
    const double CDCD = ADCD - ACCD, ADAD = ADCD + ACAD, ACAC = ACAD - ACCD, BDBD = BCBD + CDBD;
    const double BCBC = BCBD - BCCD;
    const int* v = tets + 4 * (size_t)t;
    const double TA = T[v[0]], TB = T[v[1]], TC = T[v[2]], TD = T[v[3]];
    const double u[4] = {tet_update<double>(TB, TD, TC, BCBC, -BCCD, -ACBC, CDCD, ACCD, ACAC),
                         tet_update<double>(TA, TD, TC, ACAC, -ACCD, -ACBC, CDCD, BCCD, BCBC),
                         tet_update<double>(TA, TB, TD, ADAD, ADBD, -ADCD, BDBD, -CDBD, CDCD),
                         tet_update<double>(TA, TB, TC, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD)};
    for (int k = 0; k < 4; ++k)
      if (u[k] >= 0.0 && u[k] < cand[v[k]]) cand[v[k]] = u[k];
  }
  return 0;
}

int oracle_num_threads(void) { return n_threads(0); }

// Wall time of the outer iterations of the last oracle3d_solve (its layout set-up
// excluded), for rates comparable with the device's solve time.
double oracle_last_loop_seconds(void) { return g_last_loop_seconds; }

}  // extern "C"
