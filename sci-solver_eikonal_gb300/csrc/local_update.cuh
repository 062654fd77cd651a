// local_update.cuh — tet and triangle local updates for the GB300 FIM kernels.
//
// The arithmetic reproduces the reference updates bit for bit:
//   tet:      localSolverTet1, src/core3d/cuda/CUDA_kernels.cu:69-225
//   triangle: inline update in FIMCuda, src/core2d/cuda/CUDA_kernels.cu:143-204
// Every expression keeps the reference's association and operand order, because
// nvcc's multiply-add contraction (on by default, as in the reference build) pairs
// products with sums by position; the same expression trees give the same fused
// roundings.
//
// The reference divides in FP64 in two places: `(-q ± sqrt(delta)) / (2.0*p)` and
// `(s*lambda1 + t) / (h + 1e-8)` (the 2.0 and the 1e-8 literal are doubles).  GB300
// runs FP64 at 1/64 of the FP32 rate, so this file computes both quotients in FP32
// with the same final bits:
//   * root_quot: an IEEE float division by 2p.  For float operands a double
//     quotient rounded to float equals the correctly rounded float quotient
//     (53 >= 2*24 + 2, the innocuous double rounding bound), so the only cases left
//     are |p| so large that 2p overflows in float; those take the FP64 path.
//   * small_quot: the denominator h + 1e-8 is carried as an unevaluated float pair,
//     the quotient is corrected with an exact FMA residual, and the result is
//     accepted only when it lies clearly away from a rounding boundary; otherwise
//     (about once in a million calls) the FP64 division runs.
#pragma once

#include <cuda_runtime.h>

namespace eikgb {

constexpr float kLarge3DDev = 1000000000.0f;
constexpr float kLarge2DDev = 10000000.0f;

// Rare paths (FP64 divisions) and the whole of small_quot stay out of line: the
// four inlined tet updates of a slot are large, and moving code that runs once in
// a million calls out of them cuts instruction-cache misses (the sweep kernels ran
// 10% faster on a 65^3 cube, same bits).  Calls do not change the arithmetic.
__device__ __noinline__ float root_quot_slow(float num, float p) {
  return (float)((double)num / (2.0 * (double)p));
}

__device__ __forceinline__ float root_quot(float num, float p) {
  if (fabsf(p) < 0x1p126f) return num / (2.0f * p);
  return root_quot_slow(num, p);
}

__device__ __noinline__ float small_quot_slow(float num, float h) {
  return (float)((double)num / ((double)h + 0.00000001));
}

__device__ __noinline__ float small_quot(float num, float h) {
  const float c1 = 0x1.5798eep-27f;  // RN_f(1e-8)
  const float c2 = 0x1.18461cp-54f;  // RN_f(1e-8 - c1)
  // two-sum h + c1 = s + e exactly
  const float s = __fadd_rn(h, c1);
  const float bb = __fsub_rn(s, h);
  const float e = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(c1, bb));
  const float lo0 = __fadd_rn(e, c2);
  const float hi = __fadd_rn(s, lo0);
  const float lo = __fsub_rn(lo0, __fsub_rn(hi, s));
  // reject non-finite inputs, cancellation of h against 1e-8 (the pair then
  // misses the last bits of the double denominator), and tiny/huge values
  const float ah = fabsf(hi);
  if (!(ah > 1e-10f && ah < 1e30f) || !(fabsf(num) < 1e30f)) return small_quot_slow(num, h);
  const float q = __fdiv_rn(num, hi);
  const float aq = fabsf(q);
  if (q == 0.0f) {
    if (num == 0.0f) return q;  // signed zero of num / D
    return small_quot_slow(num, h);
  }
  if (!(aq > 1e-30f && aq < 1e30f)) return small_quot_slow(num, h);
  // N/D = q + (N - q*hi - q*lo)/(hi + lo); fma gives N - q*hi exactly
  const float r = __fmaf_rn(-q, hi, num);
  const float t = __fmaf_rn(-q, lo, r);
  const float corr = __fdiv_rn(t, hi);
  const float R = __fadd_rn(q, corr);
  // distance of the estimate from R, in units of R's half ulp
  const unsigned rb = __float_as_uint(R);
  if ((rb & 0x007fffffu) == 0u) return small_quot_slow(num, h);  // binade edge
  const float d = __fadd_rn(__fsub_rn(q, R), corr);              // ~ N/D - R
  const float half_ulp = __uint_as_float(((rb >> 23) & 0xffu) - 24u << 23);
  const float margin = __fmul_rn(fabsf(R), 0x1p-36f);
  if (fabsf(d) > half_ulp - margin) return small_quot_slow(num, h);
  return R;
}

// Tet update of apex D from A, B, C (metric Gram terms of the apex ordering).
__device__ __forceinline__ float tet_update(float TA, float TB, float TC, float ACAC, float ACBC,
                                            float ACCD, float BCBC, float BCCD, float CDCD) {
  if (TA >= kLarge3DDev && TB >= kLarge3DDev && TC >= kLarge3DDev) return kLarge3DDev;
  float p, q, r, l1, l2, l3, delta, TE;
  float fBC = kLarge3DDev, fAB = kLarge3DDev, fAC = kLarge3DDev, TD = kLarge3DDev;
  const float TAC = TC - TA;
  const float TBC = TC - TB;
  const float TAB = TB - TA;

  // ---- candidate on face BC (lambda1 = 0) ----
  p = BCBC * TBC * TBC - BCBC * BCBC;
  q = (BCCD + BCCD) * TBC * TBC - 2 * BCBC * BCCD;
  r = TBC * TBC * CDCD - BCCD * BCCD;
  delta = q * q - 4 * p * r;
  if (delta >= 0.0f) {
    l2 = root_quot(-q + sqrtf(delta), p);
    l3 = 1.0f - l2;
    if (l2 >= 0 && l2 <= 1) {
      TE = TB * l2 + TC * l3;
      fBC = fminf(fBC, TE + sqrtf((l2 * BCBC + BCCD) * l2 + (l2 * BCCD + CDCD)));
    }
    l2 = root_quot(-q - sqrtf(delta), p);
    l3 = 1.0f - l2;
    if (l2 >= 0 && l2 <= 1) {
      TE = TB * l2 + TC * l3;
      fBC = fminf(fBC, TE + sqrtf((l2 * BCBC + BCCD) * l2 + (l2 * BCCD + CDCD)));
    }
  }
  fBC = fminf(fBC, fminf(TB + sqrtf((BCBC + BCCD) + (BCCD + CDCD)), TC + sqrtf(CDCD)));

  // ---- candidate on face AB (lambda3 = 0) ----
  const float gx = ACAC - ACBC, gy = ACBC - BCBC, gz = ACCD - BCCD;
  p = (TAB * TAB * ACAC - gx * gx) + (BCBC * TAB * TAB - gy * gy) -
      ((ACBC + ACBC) * TAB * TAB - 2 * gx * gy);
  q = -(BCBC * TAB * TAB - gy * gy) * 2 + ((ACBC + ACBC) * TAB * TAB - 2 * gx * gy) +
      ((ACCD + ACCD) * TAB * TAB - 2 * gx * gz) - ((BCCD + BCCD) * TAB * TAB - 2 * gy * gz);
  r = (TAB * TAB * BCBC - gy * gy) + ((BCCD + BCCD) * TAB * TAB - 2 * gy * gz) +
      (TAB * TAB * CDCD - gz * gz);
  delta = q * q - 4 * p * r;
  if (delta >= 0.0f) {
    l1 = root_quot(-q + sqrtf(delta), p);
    l2 = 1 - l1;
    if (l1 >= 0 && l1 <= 1) {
      TE = TA * l1 + TB * l2;
      fAB = fminf(fAB, TE + sqrtf((l1 * ACAC + l2 * ACBC + ACCD) * l1 +
                                  (l1 * ACBC + l2 * BCBC + BCCD) * l2 +
                                  (l1 * ACCD + l2 * BCCD + CDCD)));
    }
    l1 = root_quot(-q - sqrtf(delta), p);
    l2 = 1 - l1;
    if (l1 >= 0 && l1 <= 1) {
      TE = TA * l1 + TB * l2;
      fAB = fminf(fAB, TE + sqrtf((l1 * ACAC + l2 * ACBC + ACCD) * l1 +
                                  (l1 * ACBC + l2 * BCBC + BCCD) * l2 +
                                  (l1 * ACCD + l2 * BCCD + CDCD)));
    }
  }
  fAB = fminf(fAB, fminf(TB + sqrtf((BCBC + BCCD) + (BCCD + CDCD)),
                         TA + sqrtf((ACAC + ACCD) + (ACCD + CDCD))));

  // ---- candidate on face AC (lambda2 = 0) ----
  p = ACAC * TAC * TAC - ACAC * ACAC;
  q = (ACCD + ACCD) * TAC * TAC - 2 * ACAC * ACCD;
  r = TAC * TAC * CDCD - ACCD * ACCD;
  delta = q * q - 4 * p * r;
  if (delta >= 0.0f) {
    l1 = root_quot(-q + sqrtf(delta), p);
    l3 = 1 - l1;
    if (l1 >= 0 && l1 <= 1) {
      TE = TA * l1 + TC * l3;
      fAC = fminf(fAC, TE + sqrtf((l1 * ACAC + ACCD) * l1 + (l1 * ACCD + CDCD)));
    }
    l1 = root_quot(-q - sqrtf(delta), p);
    l3 = 1 - l1;
    if (l1 >= 0 && l1 <= 1) {
      // the second candidate keeps a zero-weight TB term, as the reference does
      TE = TA * l1 + TB * 0.0f + TC * l3;
      fAC = fminf(fAC, TE + sqrtf((l1 * ACAC + ACCD) * l1 + (l1 * ACCD + CDCD)));
    }
  }
  fAC = fminf(fAC, fminf(TA + sqrtf((ACAC + ACCD) + (ACCD + CDCD)), TC + sqrtf(CDCD)));

  // ---- candidate inside face ABC: lambda2 = (s*lambda1 + t)/(h + 1e-8) ----
  const float s = TAC * ACBC - TBC * ACAC;
  const float t = TAC * BCCD - TBC * ACCD;
  const float h = -(TAC * BCBC - TBC * ACBC);
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
  if (delta >= 0.0f) {
    l1 = root_quot(-q + sqrtf(delta), p);
    l2 = small_quot(s * l1 + t, h);
    l3 = 1 - l1 - l2;
    if (l1 >= 0 && l1 <= 1 && l2 >= 0 && l2 <= 1 && l3 >= 0 && l3 <= 1) {
      TE = TA * l1 + TB * l2 + TC * l3;
      TD = fminf(TD, TE + sqrtf((l1 * ACAC + l2 * ACBC + ACCD) * l1 +
                                (l1 * ACBC + l2 * BCBC + BCCD) * l2 +
                                (l1 * ACCD + l2 * BCCD + CDCD)));
    }
    l1 = root_quot(-q - sqrtf(delta), p);
    l2 = small_quot(s * l1 + t, h);
    l3 = 1 - l1 - l2;
    if (l1 >= 0 && l1 <= 1 && l2 >= 0 && l2 <= 1 && l3 >= 0 && l3 <= 1) {
      TE = TA * l1 + TB * l2 + TC * l3;
      TD = fminf(TD, TE + sqrtf((l1 * ACAC + l2 * ACBC + ACCD) * l1 +
                                (l1 * ACBC + l2 * BCBC + BCCD) * l2 +
                                (l1 * ACCD + l2 * BCCD + CDCD)));
    }
  }
  TD = fminf(TD, fminf(fBC, fminf(fAB, fAC)));
  return TD;
}

// Square root of a non-negative candidate distance for the FP64 update: the
// argument is formed in FP64 (where the cancellation is), the root taken in FP32
// (relative error below 1e-7, far inside the scheme's 1e-5 tolerance), which
// spares the slow FP64 unit.
__device__ __forceinline__ double sqrt_pos(double x) { return (double)sqrtf((float)x); }

// The same tet update carried out in FP64 (precision mode: slots of sliver or
// ill-conditioned tets).  Same candidates and order as tet_update; the metric
// edge products come from FP64 setup values, quotients are FP64 (one reciprocal
// per candidate face); only the candidate roots use sqrt_pos.
__device__ __forceinline__ double tet_update_f64(double TA, double TB, double TC, double ACAC, double ACBC,
                                                 double ACCD, double BCBC, double BCCD, double CDCD) {
  const double L = (double)kLarge3DDev;
  if (TA >= L && TB >= L && TC >= L) return L;
  double p, q, r, l1, l2, l3, delta, TE;
  double fBC = L, fAB = L, fAC = L, TD = L;
  const double TAC = TC - TA, TBC = TC - TB, TAB = TB - TA;
  // face BC
  p = BCBC * TBC * TBC - BCBC * BCBC;
  q = (BCCD + BCCD) * TBC * TBC - 2 * BCBC * BCCD;
  r = TBC * TBC * CDCD - BCCD * BCCD;
  delta = q * q - 4 * p * r;
  if (delta >= 0.0) {
    const double sd = sqrt(delta), i2p = 1.0 / (2.0 * p);
    for (int sg = 0; sg < 2; ++sg) {
      l2 = (-q + (sg ? -sd : sd)) * i2p;
      l3 = 1.0 - l2;
      if (l2 >= 0 && l2 <= 1) {
        TE = TB * l2 + TC * l3;
        fBC = fmin(fBC, TE + sqrt_pos((l2 * BCBC + BCCD) * l2 + (l2 * BCCD + CDCD)));
      }
    }
  }
  fBC = fmin(fBC, fmin(TB + sqrt_pos((BCBC + BCCD) + (BCCD + CDCD)), TC + sqrt_pos(CDCD)));
  // face AB
  const double gx = ACAC - ACBC, gy = ACBC - BCBC, gz = ACCD - BCCD;
  p = (TAB * TAB * ACAC - gx * gx) + (BCBC * TAB * TAB - gy * gy) - ((ACBC + ACBC) * TAB * TAB - 2 * gx * gy);
  q = -(BCBC * TAB * TAB - gy * gy) * 2 + ((ACBC + ACBC) * TAB * TAB - 2 * gx * gy) +
      ((ACCD + ACCD) * TAB * TAB - 2 * gx * gz) - ((BCCD + BCCD) * TAB * TAB - 2 * gy * gz);
  r = (TAB * TAB * BCBC - gy * gy) + ((BCCD + BCCD) * TAB * TAB - 2 * gy * gz) + (TAB * TAB * CDCD - gz * gz);
  delta = q * q - 4 * p * r;
  if (delta >= 0.0) {
    const double sd = sqrt(delta), i2p = 1.0 / (2.0 * p);
    for (int sg = 0; sg < 2; ++sg) {
      l1 = (-q + (sg ? -sd : sd)) * i2p;
      l2 = 1 - l1;
      if (l1 >= 0 && l1 <= 1) {
        TE = TA * l1 + TB * l2;
        fAB = fmin(fAB, TE + sqrt_pos((l1 * ACAC + l2 * ACBC + ACCD) * l1 + (l1 * ACBC + l2 * BCBC + BCCD) * l2 +
                                  (l1 * ACCD + l2 * BCCD + CDCD)));
      }
    }
  }
  fAB = fmin(fAB, fmin(TB + sqrt_pos((BCBC + BCCD) + (BCCD + CDCD)), TA + sqrt_pos((ACAC + ACCD) + (ACCD + CDCD))));
  // face AC
  p = ACAC * TAC * TAC - ACAC * ACAC;
  q = (ACCD + ACCD) * TAC * TAC - 2 * ACAC * ACCD;
  r = TAC * TAC * CDCD - ACCD * ACCD;
  delta = q * q - 4 * p * r;
  if (delta >= 0.0) {
    const double sd = sqrt(delta), i2p = 1.0 / (2.0 * p);
    for (int sg = 0; sg < 2; ++sg) {
      l1 = (-q + (sg ? -sd : sd)) * i2p;
      l3 = 1 - l1;
      if (l1 >= 0 && l1 <= 1) {
        TE = TA * l1 + TC * l3;
        fAC = fmin(fAC, TE + sqrt_pos((l1 * ACAC + ACCD) * l1 + (l1 * ACCD + CDCD)));
      }
    }
  }
  fAC = fmin(fAC, fmin(TA + sqrt_pos((ACAC + ACCD) + (ACCD + CDCD)), TC + sqrt_pos(CDCD)));
  // inside face ABC
  const double s = TAC * ACBC - TBC * ACAC;
  const double t = TAC * BCCD - TBC * ACCD;
  const double h = -(TAC * BCBC - TBC * ACBC);
  p = (TAC * TAC * ACAC - ACAC * ACAC) * h * h + (BCBC * TAC * TAC - ACBC * ACBC) * s * s +
      ((ACBC + ACBC) * TAC * TAC - 2 * ACAC * ACBC) * s * h;
  q = (BCBC * TAC * TAC - ACBC * ACBC) * 2 * s * t + ((ACBC + ACBC) * TAC * TAC - 2 * ACAC * ACBC) * t * h +
      ((ACCD + ACCD) * TAC * TAC - 2 * ACAC * ACCD) * h * h +
      ((BCCD + BCCD) * TAC * TAC - 2 * ACBC * ACCD) * s * h;
  r = (TAC * TAC * BCBC - ACBC * ACBC) * t * t + ((BCCD + BCCD) * TAC * TAC - 2 * ACBC * ACCD) * t * h +
      (TAC * TAC * CDCD - ACCD * ACCD) * h * h;
  delta = q * q - 4 * p * r;
  if (delta >= 0.0) {
    const double sd = sqrt(delta), i2p = 1.0 / (2.0 * p), ih = 1.0 / (h + 0.00000001);
    for (int sg = 0; sg < 2; ++sg) {
      l1 = (-q + (sg ? -sd : sd)) * i2p;
      l2 = (s * l1 + t) * ih;
      l3 = 1 - l1 - l2;
      if (l1 >= 0 && l1 <= 1 && l2 >= 0 && l2 <= 1 && l3 >= 0 && l3 <= 1) {
        TE = TA * l1 + TB * l2 + TC * l3;
        TD = fmin(TD, TE + sqrt_pos((l1 * ACAC + l2 * ACBC + ACCD) * l1 + (l1 * ACBC + l2 * BCBC + BCCD) * l2 +
                                (l1 * ACCD + l2 * BCCD + CDCD)));
      }
    }
  }
  return fmin(TD, fmin(fBC, fmin(fAB, fAC)));
}

// Triangle update of corner C from A and B; F is the inverse speed.  Uses the
// reference's MIN macro semantics ((a)<(b)?(a):(b)), not fminf.
__device__ __forceinline__ float mn2(float a, float b) { return (a < b) ? a : b; }

//
// kHoisted: inside the reference's multi-sweep FIMCuda the products LenAC*F and
// LenBC*F do not change between sweeps and are rounded once before the sweeps,
// so the edge candidates there are TA + RN(LenAC*F); the single-sweep check
// kernel fuses them into one multiply-add.  EA, EB carry the pre-rounded products
// in the first form and are ignored in the second.
template <bool kHoisted>
__device__ __forceinline__ float tri_update(float TA, float TB, float TC, float LenAB, float LenBC,
                                            float LenAC, float F, float EA, float EB) {
  float TC1 = kLarge2DDev, TC2 = kLarge2DDev;
  const float TAB = TB - TA;
  const float a = (F * F * LenAB * LenAB - TAB * TAB) * LenAB * LenAB;
  const float EdgeTA = kHoisted ? TA + EA : TA + LenAC * F;
  const float EdgeTB = kHoisted ? TB + EB : TB + LenBC * F;
  if (a > 0.0f) {
    const float cosA = (LenAC * LenAC + LenAB * LenAB - LenBC * LenBC) / (2.0f * LenAC * LenAB);
    const float b = 2.0f * LenAB * LenAC * cosA * (TAB * TAB - F * F * LenAB * LenAB);
    const float delta = 4.0f * LenAC * LenAC * a * TAB * TAB * (1.0f - cosA * cosA);
    const float l1 = (-b + sqrtf(delta)) / (2.0f * a);
    const float l2 = (-b - sqrtf(delta)) / (2.0f * a);
    if (l1 >= 0.0f && l1 <= 1.0f) {
      const float LenAD = l1 * LenAB;
      const float LenCD = sqrtf(LenAC * LenAC + LenAD * LenAD - 2 * LenAC * LenAD * cosA);
      TC1 = l1 * TAB + TA + LenCD * F;
    }
    if (l2 >= 0.0f && l2 <= 1.0f) {
      const float LenAD = l2 * LenAB;
      const float LenCD = sqrtf(LenAC * LenAC + LenAD * LenAD - 2 * LenAC * LenAD * cosA);
      TC2 = l2 * TAB + TA + LenCD * F;
    }
    return mn2(TC, mn2(TC2, mn2(TC1, mn2(EdgeTA, EdgeTB))));
  }
  return mn2(TC, mn2(EdgeTA, EdgeTB));
}

}  // namespace eikgb
