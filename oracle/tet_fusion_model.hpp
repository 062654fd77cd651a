// tet_fusion_model.hpp — TEST INFRASTRUCTURE ONLY.
//
// A CPU model of how the reference's tet update (localSolverTet1,
// src/core3d/cuda/CUDA_kernels.cu:69-225) rounds when nvcc compiles it into
// FIMCuda (CUDA_kernels.cu:454-457): nvcc fuses every product that feeds a sum
// into one multiply-add, and in a sum or difference of two products it fuses one
// of the two.  Bit S of a mask says which one at site S (set: the second product,
// x*y - z*w -> fma(-z, w, x*y); clear: the first, fma(x, y, -(z*w))).  Everything
// else is the reference's expression trees with IEEE operations; the two FP64
// quotients are evaluated in FP64 as the reference source writes them.
//
// fit_tet_fusion.py fits one mask per apex update of a slot to the reference
// kernel's own outputs on single-tet blocks (oracle/ref_gpu_driver.cpp
// refgpu_tet_blocks); the product's explicitly rounded update takes the fitted
// masks.  Compile with -ffp-contract=off (fim_oracle.cpp is).
#pragma once
#include <cmath>
#include <cstdint>

namespace oracle {
namespace fusion {

constexpr float kL = 1000000000.0f;  // LARGENUM (src/core3d/include/tetmesh.h)

inline bool bit(uint64_t m, int s) { return (m >> s) & 1ull; }
inline float ms(uint64_t m, int s, float x, float y, float z, float w) {  // x*y - z*w
  return bit(m, s) ? std::fma(-z, w, x * y) : std::fma(x, y, -(z * w));
}
inline float ma(uint64_t m, int s, float x, float y, float z, float w) {  // x*y + z*w
  return bit(m, s) ? std::fma(z, w, x * y) : std::fma(x, y, z * w);
}
inline float root(float num, float p) { return (float)((double)num / (2.0 * (double)p)); }
inline float small(float num, float h) { return (float)((double)num / ((double)h + 0.00000001)); }
inline float dist3(uint64_t m, int s, float l1, float l2, float ACAC, float ACBC, float ACCD, float BCBC, float BCCD,
                   float CDCD) {
  const float X = ma(m, s, l1, ACAC, l2, ACBC) + ACCD;
  const float Y = ma(m, s + 1, l1, ACBC, l2, BCBC) + BCCD;
  const float Z = ma(m, s + 2, l1, ACCD, l2, BCCD) + CDCD;
  return ma(m, s + 3, X, l1, Y, l2) + Z;
}
inline float dist2(float l, float XX, float XY, float YY) {
  return std::fma(std::fma(l, XX, XY), l, std::fma(l, XY, YY));
}

// Update of apex D from A, B, C with the roundings of mask m (sites 0..50).
inline float tet_update(uint64_t m, float TA, float TB, float TC, float ACAC, float ACBC, float ACCD, float BCBC,
                        float BCCD, float CDCD) {
  if (TA >= kL && TB >= kL && TC >= kL) return kL;
  float p, q, r, l1, l2, l3, delta;
  float fBC = kL, fAB = kL, fAC = kL, TD = kL;
  const float TAC = TC - TA, TBC = TC - TB, TAB = TB - TA;
  p = ms(m, 0, BCBC * TBC, TBC, BCBC, BCBC);
  q = ms(m, 1, (BCCD + BCCD) * TBC, TBC, 2 * BCBC, BCCD);
  r = ms(m, 2, TBC * TBC, CDCD, BCCD, BCCD);
  delta = ms(m, 3, q, q, 4 * p, r);
  if (delta >= 0.0f) {
    for (int sg = 0; sg < 2; ++sg) {
      l2 = root(sg ? -q - std::sqrt(delta) : -q + std::sqrt(delta), p);
      l3 = 1.0f - l2;
      if (l2 >= 0 && l2 <= 1)
        fBC = std::fmin(fBC, ma(m, 4 + sg, TB, l2, TC, l3) + std::sqrt(dist2(l2, BCBC, BCCD, CDCD)));
    }
  }
  const float eB = TB + std::sqrt((BCBC + BCCD) + (BCCD + CDCD)), eC = TC + std::sqrt(CDCD);
  const float eA = TA + std::sqrt((ACAC + ACCD) + (ACCD + CDCD));
  fBC = std::fmin(fBC, std::fmin(eB, eC));
  const float gx = ACAC - ACBC, gy = ACBC - BCBC, gz = ACCD - BCCD;
  const float P2 = ms(m, 7, BCBC * TAB, TAB, gy, gy);
  const float P3 = ms(m, 8, (ACBC + ACBC) * TAB, TAB, 2 * gx, gy);
  p = (ms(m, 6, TAB * TAB, ACAC, gx, gx) + P2) - P3;
  const float P5 = ms(m, 10, (BCCD + BCCD) * TAB, TAB, 2 * gy, gz);
  q = ((-P2 * 2 + P3) + ms(m, 9, (ACCD + ACCD) * TAB, TAB, 2 * gx, gz)) - P5;
  r = (ms(m, 11, TAB * TAB, BCBC, gy, gy) + P5) + ms(m, 12, TAB * TAB, CDCD, gz, gz);
  delta = ms(m, 13, q, q, 4 * p, r);
  if (delta >= 0.0f) {
    for (int sg = 0; sg < 2; ++sg) {
      l1 = root(sg ? -q - std::sqrt(delta) : -q + std::sqrt(delta), p);
      l2 = 1 - l1;
      if (l1 >= 0 && l1 <= 1)
        fAB = std::fmin(fAB, ma(m, sg ? 19 : 14, TA, l1, TB, l2) +
                                 std::sqrt(dist3(m, sg ? 20 : 15, l1, l2, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD)));
    }
  }
  fAB = std::fmin(fAB, std::fmin(eB, eA));
  p = ms(m, 24, ACAC * TAC, TAC, ACAC, ACAC);
  const float qAC = ms(m, 25, (ACCD + ACCD) * TAC, TAC, 2 * ACAC, ACCD);
  const float rAC = ms(m, 26, TAC * TAC, CDCD, ACCD, ACCD);
  delta = ms(m, 27, qAC, qAC, 4 * p, rAC);
  if (delta >= 0.0f) {
    for (int sg = 0; sg < 2; ++sg) {
      l1 = root(sg ? -qAC - std::sqrt(delta) : -qAC + std::sqrt(delta), p);
      l3 = 1 - l1;
      if (l1 >= 0 && l1 <= 1) {
        const float TE = sg ? std::fma(TC, l3, ma(m, 29, TA, l1, TB, 0.0f)) : ma(m, 28, TA, l1, TC, l3);
        fAC = std::fmin(fAC, TE + std::sqrt(dist2(l1, ACAC, ACCD, CDCD)));
      }
    }
  }
  fAC = std::fmin(fAC, std::fmin(eA, eC));
  const float s = ms(m, 30, TAC, ACBC, TBC, ACAC);
  const float t = ms(m, 31, TAC, BCCD, TBC, ACCD);
  const float h = -ms(m, 32, TAC, BCBC, TBC, ACBC);
  const float A1 = ms(m, 33, TAC * TAC, ACAC, ACAC, ACAC);
  const float A2 = ms(m, 34, BCBC * TAC, TAC, ACBC, ACBC);
  const float A3 = ms(m, 35, (ACBC + ACBC) * TAC, TAC, 2 * ACAC, ACBC);
  const float A4 = ms(m, 37, (BCCD + BCCD) * TAC, TAC, 2 * ACBC, ACCD);
  p = std::fma(A3 * s, h, ma(m, 36, A1 * h, h, A2 * s, s));
  q = std::fma(A4 * s, h, std::fma(qAC * h, h, ma(m, 38, (A2 * 2) * s, t, A3 * t, h)));
  r = std::fma(rAC * h, h, ma(m, 40, ms(m, 39, TAC * TAC, BCBC, ACBC, ACBC) * t, t, A4 * t, h));
  delta = ms(m, 41, q, q, 4 * p, r);
  if (delta >= 0.0f) {
    for (int sg = 0; sg < 2; ++sg) {
      l1 = root(sg ? -q - std::sqrt(delta) : -q + std::sqrt(delta), p);
      l2 = small(std::fma(s, l1, t), h);
      l3 = 1 - l1 - l2;
      if (l1 >= 0 && l1 <= 1 && l2 >= 0 && l2 <= 1 && l3 >= 0 && l3 <= 1)
        TD = std::fmin(TD, std::fma(TC, l3, ma(m, sg ? 47 : 42, TA, l1, TB, l2)) +
                               std::sqrt(dist3(m, sg ? 48 : 43, l1, l2, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD)));
    }
  }
  return std::fmin(TD, std::fmin(fBC, std::fmin(fAB, fAC)));
}

// The four apex updates of a slot as FIMCuda runs them (CUDA_kernels.cu:429-457):
// in = TA TB TC TD and the stored products ACBC BCCD ACCD ADBD ACAD BCBD;
// out[k] = min(T_k, update of apex k) under masks[k] (k = 0..3: A, B, C, D).
inline void tet_group(const uint64_t masks[4], const float in[10], float out[4]) {
  const float TA = in[0], TB = in[1], TC = in[2], TD = in[3];
  const float ACBC = in[4], BCCD = in[5], ACCD = in[6], ADBD = in[7], ACAD = in[8], BCBD = in[9];
  const float ADBC = ACBC + BCCD, ACBD = ACBC + ACCD, CDBD = ADBD - ACBD, ADCD = ADBD - ADBC;
  const float CDCD = ADCD - ACCD, ADAD = ADCD + ACAD, ACAC = ACAD - ACCD, BDBD = BCBD + CDBD, BCBC = BCBD - BCCD;
  out[3] = std::fmin(TD, tet_update(masks[3], TA, TB, TC, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD));
  out[0] = std::fmin(TA, tet_update(masks[0], TB, TD, TC, BCBC, -BCCD, -ACBC, CDCD, ACCD, ACAC));
  out[1] = std::fmin(TB, tet_update(masks[1], TA, TD, TC, ACAC, -ACCD, -ACBC, CDCD, BCCD, BCBC));
  out[2] = std::fmin(TC, tet_update(masks[2], TA, TB, TD, ADAD, ADBD, -ADCD, BDBD, -CDBD, CDCD));
}

}  // namespace fusion
}  // namespace oracle
