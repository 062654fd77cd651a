// oracle_scheme.hpp — TEST INFRASTRUCTURE ONLY.
// The reference scheme restated for the CPU (templates shared by fim_oracle.cpp,
// the CPU oracle, and ref_gpu_driver.cpp, which feeds the same padded layouts to
// the reference's own kernels).  See fim_oracle.cpp for the full description.
#pragma once

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <set>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace oracle {

// ---------------------------------------------------------------------------
// Constants of the scheme.
//   3D: LARGENUM 1000000000 (src/core3d/include/tetmesh.h:34-36),
//       SMALLNUM 0.00000001 (tetmesh.h:37-39), EPS 1e-5 as a double
//       (src/core3d/include/CUDADefines.h:20).
//   2D: LARGENUM 10000000.0 (src/core2d/include/TriMesh.h:11-13),
//       EPS 1e-5f (src/core2d/include/CUDADefines.h:21), 6 slots per vertex
//       (VERTMEMLENGTH / VERTMEMLENGTHOUTSIDE, :15-16), convergence flags strided
//       by REDUCTIONSHARESIZE 64 with a 32-thread reduction (:17,
//       meshFIM2d_eikonal.cu:720-722).
// ---------------------------------------------------------------------------
constexpr double kLarge3D = 1000000000.0;
constexpr double kSmall3D = 0.00000001;
constexpr double kEps3D = 1e-5;
constexpr double kLarge2D = 10000000.0;
constexpr float kEps2D = 1e-5f;
constexpr int kSlots2D = 6;
constexpr int kReduce2D = 32;

inline float rmin(float a, float b) { return fminf(a, b); }
inline double rmin(double a, double b) { return fmin(a, b); }
inline float rsqrt_(float a) { return sqrtf(a); }
inline double rsqrt_(double a) { return sqrt(a); }

// (-q ± sqrt(delta)) / (2.0*p): the literal 2.0 makes the reference divide in
// double and narrow the quotient to float (CUDA_kernels.cu:93,102,127,139,...).
inline float root_quot(float num, float p) { return (float)((double)num / (2.0 * (double)p)); }
inline double root_quot(double num, double p) { return num / (2.0 * p); }
// (s*lambda1 + t) / (h + SMALLNUM): SMALLNUM is a double literal (:200,:210).
inline float small_quot(float num, float h) { return (float)((double)num / ((double)h + kSmall3D)); }
inline double small_quot(double num, double h) { return num / (h + kSmall3D); }

// Tet local update of apex D from A, B, C under metric Gram terms
// (restates localSolverTet1, src/core3d/cuda/CUDA_kernels.cu:69-225; statement
// order and association are kept because they decide the rounding).
template <typename R>
R tet_update(R TA, R TB, R TC, R ACAC, R ACBC, R ACCD, R BCBC, R BCCD, R CDCD) {
  const R LARGE = (R)kLarge3D;
  if (TA >= LARGE && TB >= LARGE && TC >= LARGE) return LARGE;
  R p, q, r, l1, l2, l3, delta, TE;
  R fBC = LARGE, fAB = LARGE, fAC = LARGE, TD = LARGE;
  const R TAC = TC - TA;
  const R TBC = TC - TB;
  const R TAB = TB - TA;

  // face BC (lambda1 = 0)
  p = BCBC * TBC * TBC - BCBC * BCBC;
  q = (BCCD + BCCD) * TBC * TBC - 2 * BCBC * BCCD;
  r = TBC * TBC * CDCD - BCCD * BCCD;
  delta = q * q - 4 * p * r;
  if (delta >= 0.0) {
    l1 = 0.0;
    l2 = root_quot(-q + rsqrt_(delta), p);
    l3 = 1 - l1 - l2;
    if (l2 >= 0 && l2 <= 1) {
      TE = TB * l2 + TC * l3;
      fBC = rmin(fBC, TE + rsqrt_((l2 * BCBC + BCCD) * l2 + (l2 * BCCD + CDCD)));
    }
    l1 = 0.0;
    l2 = root_quot(-q - rsqrt_(delta), p);
    l3 = 1 - l1 - l2;
    if (l2 >= 0 && l2 <= 1) {
      TE = TB * l2 + TC * l3;
      fBC = rmin(fBC, TE + rsqrt_((l2 * BCBC + BCCD) * l2 + (l2 * BCCD + CDCD)));
    }
  }
  fBC = rmin(fBC, rmin(TB + rsqrt_((BCBC + BCCD) + (BCCD + CDCD)), TC + rsqrt_(CDCD)));

  // face AB (lambda3 = 0)
  const R gx = ACAC - ACBC, gy = ACBC - BCBC, gz = ACCD - BCCD;
  p = (TAB * TAB * ACAC - gx * gx) + (BCBC * TAB * TAB - gy * gy) -
      ((ACBC + ACBC) * TAB * TAB - 2 * gx * gy);
  q = -(BCBC * TAB * TAB - gy * gy) * 2 + ((ACBC + ACBC) * TAB * TAB - 2 * gx * gy) +
      ((ACCD + ACCD) * TAB * TAB - 2 * gx * gz) - ((BCCD + BCCD) * TAB * TAB - 2 * gy * gz);
  r = (TAB * TAB * BCBC - gy * gy) + ((BCCD + BCCD) * TAB * TAB - 2 * gy * gz) +
      (TAB * TAB * CDCD - gz * gz);
  delta = q * q - 4 * p * r;
  if (delta >= 0.0) {
    l1 = root_quot(-q + rsqrt_(delta), p);
    l2 = 1 - l1;
    if (l1 >= 0 && l1 <= 1) {
      TE = TA * l1 + TB * l2;
      fAB = rmin(fAB, TE + rsqrt_((l1 * ACAC + l2 * ACBC + ACCD) * l1 +
                                  (l1 * ACBC + l2 * BCBC + BCCD) * l2 +
                                  (l1 * ACCD + l2 * BCCD + CDCD)));
    }
    l1 = root_quot(-q - rsqrt_(delta), p);
    l2 = 1 - l1;
    if (l1 >= 0 && l1 <= 1) {
      TE = TA * l1 + TB * l2;
      fAB = rmin(fAB, TE + rsqrt_((l1 * ACAC + l2 * ACBC + ACCD) * l1 +
                                  (l1 * ACBC + l2 * BCBC + BCCD) * l2 +
                                  (l1 * ACCD + l2 * BCCD + CDCD)));
    }
  }
  fAB = rmin(fAB, rmin(TB + rsqrt_((BCBC + BCCD) + (BCCD + CDCD)),
                       TA + rsqrt_((ACAC + ACCD) + (ACCD + CDCD))));

  // face AC (lambda2 = 0)
  p = ACAC * TAC * TAC - ACAC * ACAC;
  q = (ACCD + ACCD) * TAC * TAC - 2 * ACAC * ACCD;
  r = TAC * TAC * CDCD - ACCD * ACCD;
  delta = q * q - 4 * p * r;
  if (delta >= 0.0) {
    l1 = root_quot(-q + rsqrt_(delta), p);
    l2 = 0.0;
    l3 = 1 - l1 - l2;
    if (l1 >= 0 && l1 <= 1) {
      TE = TA * l1 + TC * l3;
      fAC = rmin(fAC, TE + rsqrt_((l1 * ACAC + ACCD) * l1 + (l1 * ACCD + CDCD)));
    }
    l1 = root_quot(-q - rsqrt_(delta), p);
    l2 = 0.0;
    l3 = 1 - l1 - l2;
    if (l1 >= 0 && l1 <= 1) {
      // the reference keeps the zero-weight TB term in this second candidate
      TE = TA * l1 + TB * l2 + TC * l3;
      fAC = rmin(fAC, TE + rsqrt_((l1 * ACAC + ACCD) * l1 + (l1 * ACCD + CDCD)));
    }
  }
  fAC = rmin(fAC, rmin(TA + rsqrt_((ACAC + ACCD) + (ACCD + CDCD)), TC + rsqrt_(CDCD)));

  // interior of face ABC: lambda2 = (s*lambda1 + t)/(h + SMALLNUM)
  const R s = TAC * ACBC - TBC * ACAC;
  const R t = TAC * BCCD - TBC * ACCD;
  const R h = -(TAC * BCBC - TBC * ACBC);
  p = (TAC * TAC * ACAC - ACAC * ACAC) * h * h + (BCBC * TAC * TAC - ACBC * ACBC) * s * s +
      ((ACBC + ACBC) * TAC * TAC - 2 * ACAC * ACBC) * s * h;
  q = (BCBC * TAC * TAC - ACBC * ACBC) * 2 * s * t +
      ((ACBC + ACBC) * TAC * TAC - 2 * ACAC * ACBC) * t * h +
      ((ACCD + ACCD) * TAC * TAC - 2 * ACAC * ACCD) * h * h +
      ((BCCD + BCCD) * TAC * TAC - 2 * ACBC * ACCD) * s * h;
  r = (TAC * TAC * BCBC - ACBC * ACBC) * t * t +
      ((BCCD + BCCD) * TAC * TAC - 2 * ACBC * ACCD) * t * h +
      (TAC * TAC * CDCD - ACCD * ACCD) * h * h;
  delta = q * q - 4 * p * r;
  if (delta >= 0.0) {
    for (int sgn = 0; sgn < 2; ++sgn) {
      l1 = root_quot(sgn == 0 ? -q + rsqrt_(delta) : -q - rsqrt_(delta), p);
      l2 = small_quot(s * l1 + t, h);
      l3 = 1 - l1 - l2;
      if (l1 >= 0 && l1 <= 1 && l2 >= 0 && l2 <= 1 && l3 >= 0 && l3 <= 1) {
        TE = TA * l1 + TB * l2 + TC * l3;
        TD = rmin(TD, TE + rsqrt_((l1 * ACAC + l2 * ACBC + ACCD) * l1 +
                                  (l1 * ACBC + l2 * BCBC + BCCD) * l2 +
                                  (l1 * ACCD + l2 * BCCD + CDCD)));
      }
    }
  }
  TD = rmin(TD, rmin(fBC, rmin(fAB, fAC)));
  return TD;
}

// Triangle update of corner C from A and B (restates the inline update of
// src/core2d/cuda/CUDA_kernels.cu:143-204).  F is the face's inverse speed.
template <typename R>
R tri_update(R TA, R TB, R TC, R LAB, R LBC, R LAC, R F) {
  const R LARGE = (R)kLarge2D;
  auto MIN = [](R a, R b) { return (a < b) ? a : b; };  // the MIN macro, not fminf
  R TC1 = LARGE, TC2 = LARGE;
  const R TAB = TB - TA;
  const R a = (F * F * LAB * LAB - TAB * TAB) * LAB * LAB;
  const R EdgeTA = TA + LAC * F;
  const R EdgeTB = TB + LBC * F;
  if (a > 0) {
    const R cosA = (LAC * LAC + LAB * LAB - LBC * LBC) / (2 * LAC * LAB);
    const R b = 2 * LAB * LAC * cosA * (TAB * TAB - F * F * LAB * LAB);
    const R delta = 4 * LAC * LAC * a * TAB * TAB * (1 - cosA * cosA);
    const R l1 = (-b + rsqrt_(delta)) / (2 * a);
    const R l2 = (-b - rsqrt_(delta)) / (2 * a);
    if (l1 >= 0 && l1 <= 1) {
      const R LAD = l1 * LAB;
      const R LCD = rsqrt_(LAC * LAC + LAD * LAD - 2 * LAC * LAD * cosA);
      TC1 = l1 * TAB + TA + LCD * F;
    }
    if (l2 >= 0 && l2 <= 1) {
      const R LAD = l2 * LAB;
      const R LCD = rsqrt_(LAC * LAC + LAD * LAD - 2 * LAC * LAD * cosA);
      TC2 = l2 * TAB + TA + LCD * F;
    }
    return MIN(TC, MIN(TC2, MIN(TC1, MIN(EdgeTA, EdgeTB))));
  }
  return MIN(TC, MIN(EdgeTA, EdgeTB));
}

int n_threads(int req) {
#ifdef _OPENMP
  return req > 0 ? req : omp_get_max_threads();
#else
  (void)req;
  return 1;
#endif
}

// ===========================================================================
// 3D
// ===========================================================================
template <typename R>
struct Oracle3D {
  int nv = 0, nt = 0, nb = 0;
  const float* xyz = nullptr;
  const int* tets = nullptr;
  const float* M = nullptr;  // 6 per tet: M00 M01 M02 M11 M12 M22
  const int* part = nullptr;

  std::vector<std::vector<int>> inVerts;   // m_PartitionInVerts (ascending ids)
  std::vector<int> blockSize;
  int maxInVert = 0;
  std::vector<std::vector<int>> blkIn, blkNb;  // m_PartitionTets / m_PartitionNbTets
  int maxTets = 0;
  std::vector<std::vector<int>> blkNbrs;   // m_BlockNeighbor (sorted)
  std::vector<R> gram;                     // 6 per slot: tetMem0 xyz, tetMem1 xyz
  std::vector<R> slotT;                    // d_tetT (4 per slot)
  std::vector<std::vector<int>> vmap;      // m_blockVertMapping
  std::vector<int> vmIn, vmOut;            // d_vertMem / d_vertMemOutside (absolute, -1 pad)
  int maxMapIn = 0, maxMapOut = 0;
  std::vector<R> vertT;                    // d_vertT
  std::vector<uint8_t> con;                // d_con
  std::vector<uint8_t> blockCon;

  // PartitionTets (meshFIM3dEikonal.cu:568-648).  No virtual tets exist: the
  // reference's TetMesh::IsNonObtuse always returns 1 (tetmesh.cu:188-217).
  void partition() {
    inVerts.assign(nb, {});
    blockSize.assign(nb, 0);
    for (int v = 0; v < nv; ++v) { inVerts[part[v]].push_back(v); blockSize[part[v]]++; }
    maxInVert = 0;
    for (int b = 0; b < nb; ++b) maxInVert = std::max(maxInVert, blockSize[b]);
    blkIn.assign(nb, {});
    blkNb.assign(nb, {});
    for (int i = 0; i < nt; ++i) {
      std::set<int> labels;
      for (int m = 0; m < 4; ++m) labels.insert(part[tets[4 * i + m]]);
      if (labels.size() == 1) blkIn[*labels.begin()].push_back(i);
      else for (int l : labels) blkNb[l].push_back(i);
    }
    maxTets = 0;
    for (int b = 0; b < nb; ++b)
      maxTets = std::max<int>(maxTets, (int)(blkIn[b].size() + blkNb[b].size()));
    // block neighbours from vertex adjacency: two vertices are neighbours when
    // they share a tet (TetMesh::need_neighbors, tetmesh.cu:82-111)
    std::vector<std::set<int>> nbs(nb);
    for (int i = 0; i < nt; ++i)
      for (int a = 0; a < 4; ++a)
        for (int c = 0; c < 4; ++c) {
          int la = part[tets[4 * i + a]], lc = part[tets[4 * i + c]];
          if (la != lc) nbs[la].insert(lc);
        }
    blkNbrs.assign(nb, {});
    for (int b = 0; b < nb; ++b) blkNbrs[b].assign(nbs[b].begin(), nbs[b].end());
  }

  // gettetmem (meshFIM3dEikonal.cu:650-678) with vMv (core3d/include/Vec.h:479-483)
  void tet_gram(int t, R* g) const {
    const int* v = tets + 4 * t;
    R P[4][3];
    for (int k = 0; k < 4; ++k)
      for (int d = 0; d < 3; ++d) P[k][d] = (R)xyz[3 * v[k] + d];
    auto sub = [](const R* a, const R* b, R* o) { o[0] = a[0] - b[0]; o[1] = a[1] - b[1]; o[2] = a[2] - b[2]; };
    R AC[3], AD[3], BC[3], CD[3], BD[3];
    sub(P[2], P[0], AC); sub(P[3], P[0], AD); sub(P[2], P[1], BC); sub(P[3], P[2], CD); sub(P[3], P[1], BD);
    R m[6];
    for (int k = 0; k < 6; ++k) m[k] = (R)M[6 * t + k];
    auto vMv = [&](const R* a, const R* b) -> R {
      return (a[0] * m[0] + a[1] * m[1] + a[2] * m[2]) * b[0] +
             (a[0] * m[1] + a[1] * m[3] + a[2] * m[4]) * b[1] +
             (a[0] * m[2] + a[1] * m[4] + a[2] * m[5]) * b[2];
    };
    g[0] = vMv(AC, BC); g[1] = vMv(BC, CD); g[2] = vMv(AC, CD);
    g[3] = vMv(AD, BD); g[4] = vMv(AC, AD); g[5] = vMv(BC, BD);
  }

  // GetTetMem + GetVertMem (meshFIM3dEikonal.cu:680-923)
  void layout() {
    const size_t nslot = (size_t)nb * maxTets;
    gram.assign(nslot * 6, (R)0);
    slotT.assign(nslot * 4, (R)kLarge3D);
    vmap.assign(nv, {});
    auto put = [&](int b, int j, int t) {
      tet_gram(t, &gram[((size_t)b * maxTets + j) * 6]);
      const int base = (b * maxTets + j) * 4;
      for (int k = 0; k < 4; ++k) vmap[tets[4 * t + k]].push_back(base + k);
    };
    for (int b = 0; b < nb; ++b)
      for (size_t j = 0; j < blkIn[b].size(); ++j) put(b, (int)j, blkIn[b][j]);
    for (int b = 0; b < nb; ++b)
      for (size_t k = 0; k < blkNb[b].size(); ++k) put(b, (int)(blkIn[b].size() + k), blkNb[b][k]);

    std::vector<std::vector<int>> in(nv), out(nv);
    for (int b = 0; b < nb; ++b) {
      const int lo = b * maxTets * 4, hi = lo + maxTets * 4;
      for (int v : inVerts[b])
        for (int a : vmap[v]) (a >= lo && a < hi ? in[v] : out[v]).push_back(a);
    }
    maxMapIn = maxMapOut = 0;
    for (int v = 0; v < nv; ++v) {
      maxMapIn = std::max<int>(maxMapIn, (int)in[v].size());
      maxMapOut = std::max<int>(maxMapOut, (int)out[v].size());
    }
    vmIn.assign((size_t)nb * maxInVert * std::max(maxMapIn, 1), -1);
    vmOut.assign((size_t)nb * maxInVert * std::max(maxMapOut, 1), -1);
    for (int b = 0; b < nb; ++b)
      for (size_t m = 0; m < inVerts[b].size(); ++m) {
        const int v = inVerts[b][m];
        for (size_t n = 0; n < in[v].size(); ++n)
          vmIn[((size_t)b * maxInVert + m) * maxMapIn + n] = in[v][n];
        for (size_t n = 0; n < out[v].size(); ++n)
          vmOut[((size_t)b * maxInVert + m) * maxMapOut + n] = out[v][n];
      }
  }

  // FIMCuda (nsweeps = 2, CUDA_kernels.cu:383-489) and run_check_neghbor
  // (1 sweep, flags only, :493-602).  Each CUDA thread owns one slot in the update
  // phase and one vertex in the reconcile phase, so a serial walk is exact.
  void visit(int b, int nsweeps, bool check, std::vector<R>& sT) {
    const size_t base = (size_t)b * maxTets * 4;
    const int nslots = (int)(blkIn[b].size() + blkNb[b].size());  // padding stays LARGENUM
    sT.assign(slotT.begin() + base, slotT.begin() + base + (size_t)maxTets * 4);
    const int size = blockSize[b];
    std::vector<R> oldT(size), newT(size);
    for (int it = 0; it < nsweeps; ++it) {
      for (int k = 0; k < size; ++k) {
        const int a0 = vmIn[((size_t)b * maxInVert + k) * maxMapIn + 0];
        oldT[k] = a0 >= 0 ? sT[a0 - base] : (R)kLarge3D;
      }
      for (int j = 0; j < nslots; ++j) {
        const R* g = &gram[((size_t)b * maxTets + j) * 6];
        const R ACBC = g[0], BCCD = g[1], ACCD = g[2], ADBD = g[3], ACAD = g[4], BCBD = g[5];
        const R ADBC = ACBC + BCCD, ACBD = ACBC + ACCD, CDBD = ADBD - ACBD, ADCD = ADBD - ADBC;
        const R CDCD = ADCD - ACCD, ADAD = ADCD + ACAD, ACAC = ACAD - ACCD, BDBD = BCBD + CDBD;
        const R BCBC = BCBD - BCCD;
        R* T = &sT[(size_t)j * 4];
        const R TA = T[0], TB = T[1], TC = T[2], TD = T[3];
        T[3] = rmin(TD, tet_update<R>(TA, TB, TC, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD));
        T[0] = rmin(TA, tet_update<R>(TB, TD, TC, BCBC, -BCCD, -ACBC, CDCD, ACCD, ACAC));
        T[1] = rmin(TB, tet_update<R>(TA, TD, TC, ACAC, -ACCD, -ACBC, CDCD, BCCD, BCBC));
        T[2] = rmin(TC, tet_update<R>(TA, TB, TD, ADAD, ADBD, -ADCD, BDBD, -CDBD, CDCD));
      }
      for (int k = 0; k < size; ++k) {
        const int* lst = &vmIn[((size_t)b * maxInVert + k) * maxMapIn];
        R m = (R)kLarge3D;
        for (int j = 0; j < maxMapIn && lst[j] > -1; ++j) m = rmin(m, sT[lst[j] - base]);
        for (int j = 0; j < maxMapIn && lst[j] > -1; ++j) sT[lst[j] - base] = m;
        newT[k] = m;
      }
    }
    for (int k = 0; k < size; ++k) {
      const size_t vi = (size_t)b * maxInVert + k;
      if (check) {
        const R res = oldT[k] - newT[k];
        con[vi] = ((double)res < kEps3D) ? 1 : 0;
      } else {
        R res = oldT[k] - newT[k];
        if (res < 0.) res = -res;
        con[vi] = ((double)res < kEps3D) ? 1 : 0;
        vertT[vi] = newT[k];
      }
    }
  }

  // CopyOutBack (CUDA_kernels.cu:604-668): push owned T into every slot copy.
  void copy_out(int b) {
    for (int k = 0; k < blockSize[b]; ++k) {
      const size_t vi = (size_t)b * maxInVert + k;
      const R T = vertT[vi];
      const int* li = &vmIn[vi * maxMapIn];
      for (int j = 0; j < maxMapIn && li[j] > -1; ++j) slotT[li[j]] = T;
      const int* lo = &vmOut[vi * maxMapOut];
      for (int j = 0; j < maxMapOut && lo[j] > -1; ++j) slotT[lo[j]] = T;
    }
  }

  bool reduce(int b) const {
    for (int k = 0; k < blockSize[b]; ++k)
      if (!con[(size_t)b * maxInVert + k]) return false;
    return true;
  }

  // Outer loop of GenerateData (meshFIM3dEikonal.cu:332-542).
  int solve(const int* seeds, int nseeds, int maxIters, int nsweeps, int nthreads,
            float* out_final, float* history, int hist_cap, long long* updates) {
    partition();
    layout();
    vertT.assign((size_t)nb * maxInVert, (R)0);  // cudaMemset(d_vertT, 0)
    con.assign((size_t)nb * maxInVert, 0);
    blockCon.assign(nb, 1);
    enum { FARP = 0, ACTIVE = 1 };
    std::vector<int> label(nb, FARP);
    std::set<int> activeSet;
    for (int i = 0; i < nseeds; ++i) {
      const int s = seeds[i];
      activeSet.insert(part[s]);
      blockCon[part[s]] = 0;
      label[part[s]] = ACTIVE;
      for (int a : vmap[s]) slotT[a] = 0;
    }
    std::vector<int> act(activeSet.begin(), activeSet.end()), fresh;
    long long nupd = 0;
    int iters = 0;
    const int nth = n_threads(nthreads);
    std::vector<float> snap(nv);
    auto snapshot = [&](float* dst) {
      for (int b = 0; b < nb; ++b)
        for (size_t j = 0; j < inVerts[b].size(); ++j)
          dst[inVerts[b][j]] = (float)vertT[(size_t)b * maxInVert + j];
    };
    size_t total = 0;
    const auto loop0 = std::chrono::steady_clock::now();
    while (!act.empty()) {
      if (++total > (size_t)maxIters) break;
      const int na = (int)act.size();
#pragma omp parallel num_threads(nth)
      {
        std::vector<R> sT;
#pragma omp for schedule(dynamic, 1)
        for (int i = 0; i < na; ++i) visit(act[i], nsweeps, false, sT);
      }
#pragma omp parallel for num_threads(nth) schedule(dynamic, 4)
      for (int i = 0; i < na; ++i) copy_out(act[i]);
      for (int b : act) { blockCon[b] = reduce(b) ? 1 : 0; nupd += (long long)blockSize[b] * nsweeps; }
      for (int b : act) label[b] = blockCon[b] ? FARP : ACTIVE;
      fresh.clear();
      for (int b : act)
        if (blockCon[b])
          for (int nbk : blkNbrs[b])
            if (label[nbk] == FARP) { label[nbk] = ACTIVE; fresh.push_back(nbk); }
      std::vector<int> next;
      for (int b : act) if (!blockCon[b]) next.push_back(b);
      if (!fresh.empty()) {
        const int nf = (int)fresh.size();
#pragma omp parallel num_threads(nth)
        {
          std::vector<R> sT;
#pragma omp for schedule(dynamic, 1)
          for (int i = 0; i < nf; ++i) visit(fresh[i], 1, true, sT);
        }
        for (int b : fresh) {
          blockCon[b] = reduce(b) ? 1 : 0;
          nupd += blockSize[b];
          if (!blockCon[b]) next.push_back(b); else label[b] = FARP;
        }
      }
      act.swap(next);
      ++iters;
      if (history && iters <= hist_cap) snapshot(history + (size_t)(iters - 1) * nv);
    }
    loopSeconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - loop0).count();
    snapshot(snap.data());
    if (out_final) std::memcpy(out_final, snap.data(), sizeof(float) * nv);
    if (updates) *updates = nupd;
    return iters;
  }
  double loopSeconds = 0;  // wall time of the outer iterations (after the layout set-up)
};

// ===========================================================================
// 2D
// ===========================================================================
template <typename R>
struct Oracle2D {
  int nv = 0, nf = 0, nb = 0;
  const float* xyz = nullptr;
  const int* faces = nullptr;      // oriented faces, 3 per face
  const float* speedInv = nullptr; // per face
  const uint8_t* obtuse = nullptr; // bit k set: corner k fails IsNonObtuse
  const int* vfOff = nullptr;      // virtual faces per face (CSR, nf+1)
  const int* vfVerts = nullptr;    // 3 per virtual face
  const float* vfSpeedInv = nullptr;
  const int* part = nullptr;

  struct Slot { int v[3]; R e[3]; R F; };
  std::vector<std::vector<int>> verts;              // m_PartitionVerts
  std::vector<int> blockSize;
  int maxVert = 0, maxFaces = 0;
  std::vector<std::vector<Slot>> blkSlots;          // inside, boundary, virtual
  std::vector<std::vector<int>> blkNbrs;
  std::vector<int> insideCount;                     // inside faces lead each block's slots
  std::vector<R> triMem, triMemOut;                 // 3 per slot
  std::vector<R> edge;                              // 3 per slot
  std::vector<R> spd;                               // 1 per slot
  std::vector<std::vector<int>> vmap;               // blockVertMapping
  std::vector<int> vmIn, vmOut;                     // 6 per vertex (absolute, padded)
  std::vector<uint8_t> con, blockCon;

  Slot make_slot(const int* v, float F) const {
    Slot s;
    for (int k = 0; k < 3; ++k) s.v[k] = v[k];
    // edge lengths 01, 12, 20 (TriMesh::need_faceedges, TriMesh_connectivity.cu:54-75)
    for (int k = 0; k < 3; ++k) {
      const float* a = xyz + 3 * v[k];
      const float* b = xyz + 3 * v[(k + 1) % 3];
      const R dx = (R)b[0] - (R)a[0], dy = (R)b[1] - (R)a[1], dz = (R)b[2] - (R)a[2];
      s.e[k] = rsqrt_(dx * dx + dy * dy + dz * dz);
    }
    s.F = (R)F;
    return s;
  }

  // GraphPartition bookkeeping + PartitionFaces (meshFIM2d_eikonal.cu:254-347)
  void partition() {
    verts.assign(nb, {});
    blockSize.assign(nb, 0);
    for (int v = 0; v < nv; ++v) { verts[part[v]].push_back(v); blockSize[part[v]]++; }
    maxVert = 0;
    for (int b = 0; b < nb; ++b) maxVert = std::max(maxVert, blockSize[b]);
    std::vector<std::vector<int>> inF(nb), nbF(nb);
    std::vector<std::vector<Slot>> virt(nb);
    std::vector<std::set<int>> nbs(nb);
    for (int i = 0; i < nf; ++i) {
      const int* f = faces + 3 * i;
      for (int k = 0; k < 3; ++k)
        if (obtuse[i] & (1 << k))
          for (int j = vfOff[i]; j < vfOff[i + 1]; ++j)
            virt[part[f[k]]].push_back(make_slot(vfVerts + 3 * j, vfSpeedInv[j]));
      const int l0 = part[f[0]], l1 = part[f[1]], l2 = part[f[2]];
      if (l0 == l1 && l1 == l2) {
        inF[l0].push_back(i);
      } else {
        std::set<int> ls{l0, l1, l2};
        std::vector<int> lv(ls.begin(), ls.end());
        // the reference pushes the face once per distinct label in the order
        // l0 (then l2 or l1); only membership and order within a block matter
        for (int l : lv) nbF[l].push_back(i);
        for (int a : lv) for (int c : lv) if (a != c) nbs[a].insert(c);
      }
    }
    blkSlots.assign(nb, {});
    insideCount.assign(nb, 0);
    maxFaces = 0;
    for (int b = 0; b < nb; ++b) {
      insideCount[b] = (int)inF[b].size();
      for (int i : inF[b]) blkSlots[b].push_back(make_slot(faces + 3 * i, speedInv[i]));
      for (int i : nbF[b]) blkSlots[b].push_back(make_slot(faces + 3 * i, speedInv[i]));
      for (auto& s : virt[b]) blkSlots[b].push_back(s);
      maxFaces = std::max<int>(maxFaces, (int)blkSlots[b].size());
    }
    blkNbrs.assign(nb, {});
    for (int b = 0; b < nb; ++b) blkNbrs[b].assign(nbs[b].begin(), nbs[b].end());
  }

  // Slot arrays + vertex mapping (meshFIM2d_eikonal.cu:404-614)
  void layout(const int* seeds, int nseeds) {
    const size_t nslot = (size_t)nb * maxFaces;
    triMem.assign(nslot * 3, (R)kLarge2D);
    edge.assign(nslot * 3, (R)0);
    spd.assign(nslot, (R)0);
    vmap.assign(nv, {});
    for (int b = 0; b < nb; ++b) {
      for (size_t j = 0; j < blkSlots[b].size(); ++j) {
        const Slot& s = blkSlots[b][j];
        const size_t si = (size_t)b * maxFaces + j;
        for (int k = 0; k < 3; ++k) edge[si * 3 + k] = s.e[k];
        spd[si] = s.F;
      }
    }
    // order of blockVertMapping: pass 1 = inside faces of all blocks, pass 2 =
    // boundary + virtual faces of all blocks
    const std::vector<int>& nIn = insideCount;
    for (int b = 0; b < nb; ++b)
      for (int j = 0; j < nIn[b]; ++j)
        for (int k = 0; k < 3; ++k)
          vmap[blkSlots[b][j].v[k]].push_back((b * maxFaces + j) * 3 + k);
    for (int b = 0; b < nb; ++b)
      for (int j = nIn[b]; j < (int)blkSlots[b].size(); ++j)
        for (int k = 0; k < 3; ++k)
          vmap[blkSlots[b][j].v[k]].push_back((b * maxFaces + j) * 3 + k);
    // own-block slot to the front (:487-507)
    for (int v = 0; v < nv; ++v) {
      if (vmap[v].empty()) continue;
      const int lo = part[v] * maxFaces * 3, hi = lo + maxFaces * 3;
      const int tmp = vmap[v][0];
      if (tmp < lo || tmp >= hi)
        for (size_t j = 0; j < vmap[v].size(); ++j)
          if (vmap[v][j] >= lo && vmap[v][j] < hi) { vmap[v][0] = vmap[v][j]; vmap[v][j] = tmp; break; }
    }
    vmIn.assign((size_t)nb * maxVert * kSlots2D, -1);
    vmOut.assign((size_t)nb * maxVert * kSlots2D, -1);
    for (int b = 0; b < nb; ++b) {
      const int lo = b * maxFaces * 3, hi = lo + maxFaces * 3;
      for (size_t m = 0; m < verts[b].size(); ++m) {
        const int v = verts[b][m];
        int ni = 0, no = 0;
        for (int a : vmap[v]) {
          if (a >= lo && a < hi) { if (ni < kSlots2D) vmIn[((size_t)b * maxVert + m) * kSlots2D + ni] = a; ++ni; }
          else { if (no < kSlots2D) vmOut[((size_t)b * maxVert + m) * kSlots2D + no] = a; ++no; }
        }
      }
    }
    for (int i = 0; i < nseeds; ++i)
      for (int a : vmap[seeds[i]]) triMem[a] = 0;
  }


  // FIMCuda (7 sweeps) / run_check_neighbor (1 sweep): read `src`, write `dst`.
  void visit(int b, int nsweeps, bool check, const std::vector<R>& src, std::vector<R>& dst,
             std::vector<R>& sT) {
    const size_t base = (size_t)b * maxFaces * 3;
    const int nslots = (int)blkSlots[b].size();
    sT.assign(src.begin() + base, src.begin() + base + (size_t)maxFaces * 3);
    const int size = blockSize[b];
    std::vector<R> oldT(size, (R)kLarge2D), newT(size, (R)kLarge2D);
    for (int it = 0; it < nsweeps; ++it) {
      for (int k = 0; k < size; ++k) {
        const int a0 = vmIn[((size_t)b * maxVert + k) * kSlots2D];
        oldT[k] = a0 >= 0 ? sT[a0 - base] : (R)kLarge2D;
      }
      for (int j = 0; j < nslots; ++j) {
        R* T = &sT[(size_t)j * 3];
        const R o0 = T[0], o1 = T[1], o2 = T[2];
        if (o0 >= (R)kLarge2D && o1 >= (R)kLarge2D && o2 >= (R)kLarge2D) continue;
        const R* e = &edge[((size_t)b * maxFaces + j) * 3];
        const R F = spd[(size_t)b * maxFaces + j];
        T[0] = tri_update<R>(o1, o2, o0, e[1], e[2], e[0], F);
        T[1] = tri_update<R>(o2, o0, o1, e[2], e[0], e[1], F);
        T[2] = tri_update<R>(o0, o1, o2, e[0], e[1], e[2], F);
      }
      for (int k = 0; k < size; ++k) {
        const int* lst = &vmIn[((size_t)b * maxVert + k) * kSlots2D];
        R m = (R)kLarge2D;
        for (int j = 0; j < kSlots2D && lst[j] > -1; ++j) m = (m < sT[lst[j] - base]) ? m : sT[lst[j] - base];
        newT[k] = m;
        for (int j = 0; j < kSlots2D && lst[j] > -1; ++j) sT[lst[j] - base] = m;
      }
    }
    for (int k = 0; k < size; ++k) {
      const size_t vi = (size_t)b * maxVert + k;
      if (check) {
        const R res = oldT[k] - newT[k];
        con[vi] = (res < (R)kEps2D) ? 1 : 0;
      } else {
        R res = oldT[k] - newT[k];
        if (res < 0.) res = -res;
        con[vi] = (res <= (R)kEps2D) ? 1 : 0;
      }
      const int* li = &vmIn[vi * kSlots2D];
      for (int j = 0; j < kSlots2D && li[j] > -1; ++j) dst[li[j]] = newT[k];
      const int* lo = &vmOut[vi * kSlots2D];
      for (int j = 0; j < kSlots2D && lo[j] > -1; ++j) dst[lo[j]] = newT[k];
    }
  }

  // 32-thread reduction: only the first 32 owned vertices decide (CUDA_kernels.cu:8-30)
  bool reduce(int b) const {
    const int n = std::min(blockSize[b], kReduce2D);
    for (int k = 0; k < n; ++k)
      if (!con[(size_t)b * maxVert + k]) return false;
    return true;
  }

  int solve(const int* seeds, int nseeds, const float* initVals, int maxIters, int nsweeps,
            int nthreads, float* out_final, float* history, int hist_cap, long long* updates) {
    partition();
    layout(seeds, nseeds);
    triMemOut = triMem;
    con.assign((size_t)nb * maxVert, 0);
    blockCon.assign(nb, 1);
    enum { FARP = 0, ACTIVE = 1 };
    std::vector<int> label(nb, FARP);
    std::set<int> activeSet;
    for (int i = 0; i < nseeds; ++i) { activeSet.insert(part[seeds[i]]); label[part[seeds[i]]] = ACTIVE; blockCon[part[seeds[i]]] = 0; }
    std::vector<int> act(activeSet.begin(), activeSet.end());
    std::vector<R> prev(nv);
    for (int v = 0; v < nv; ++v) prev[v] = (R)initVals[v];
    auto first_slot = [&](int v) -> R { return vmap[v].empty() ? (R)kLarge2D : triMem[vmap[v][0]]; };
    long long nupd = 0;
    int iters = 0, total = 0;
    const int nth = n_threads(nthreads);
    while (!act.empty()) {
      if (++total > maxIters) break;
      const int na = (int)act.size();
#pragma omp parallel num_threads(nth)
      {
        std::vector<R> sT;
#pragma omp for schedule(dynamic, 1)
        for (int i = 0; i < na; ++i) visit(act[i], nsweeps, false, triMem, triMemOut, sT);
      }
      for (int b : act) { blockCon[b] = reduce(b) ? 1 : 0; nupd += (long long)blockSize[b] * nsweeps; }
      std::vector<int> list = act;
      for (int b : act)
        if (blockCon[b])
          for (int nbk : blkNbrs[b])
            if (label[nbk] == FARP) { label[nbk] = ACTIVE; list.push_back(nbk); }
      const int nl = (int)list.size();
#pragma omp parallel num_threads(nth)
      {
        std::vector<R> sT;
#pragma omp for schedule(dynamic, 1)
        for (int i = 0; i < nl; ++i) visit(list[i], 1, true, triMemOut, triMem, sT);
      }
      for (int b : list) { blockCon[b] = reduce(b) ? 1 : 0; nupd += blockSize[b]; }
      std::vector<int> next;
      for (int b = 0; b < nb; ++b) {
        if (!blockCon[b]) { label[b] = ACTIVE; next.push_back(b); } else label[b] = FARP;
      }
      bool allConv = true;
      for (int v = 0; v < nv; ++v) {
        const R cur = first_slot(v);
        R diff = prev[v] - cur;
        if (diff < 0) diff = -diff;
        const bool c = (diff <= (R)kEps2D) && ((double)cur < kLarge2D);
        allConv = allConv && c;
        prev[v] = cur;
      }
      ++iters;
      if (history && iters <= hist_cap)
        for (int v = 0; v < nv; ++v) history[(size_t)(iters - 1) * nv + v] = (float)prev[v];
      act.swap(next);
      if (allConv) break;
    }
    if (out_final)
      for (int v = 0; v < nv; ++v) out_final[v] = (float)first_slot(v);
    if (updates) *updates = nupd;
    return iters;
  }
};

}  // namespace oracle
