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

// ---------------------------------------------------------------------------
// Explicitly rounded tet update.
//
// nvcc fuses a product into an adjacent sum (one FMA rounding instead of two), and
// in a sum or difference of two products it picks one of them; which one depends
// on the code around the expression, so the reference's four inlined updates in
// FIMCuda (CUDA_kernels.cu:454-457) do not all round alike, and the same source in
// a different kernel shape can round differently.  Here every product, sum,
// quotient and square root is one IEEE operation (__fmul_rn, __fadd_rn, __fmaf_rn,
// __fdiv_rn, __fsqrt_rn) that the compiler cannot fuse or split, so the result no
// longer depends on the surrounding code, and a template mask states, for each sum
// or difference of two products, which product the reference's kernel fuses: bit S
// set = the second product is fused (x*y - z*w -> fma(-z, w, x*y)), clear = the
// first (fma(x, y, -(z*w))).
//
// The four masks below reproduce the reference kernel's own roundings for the four
// apex updates of a slot: they were fitted to, and reproduce bit for bit, the
// reference's FIMCuda run on 500,000 single-tet blocks (one sweep, so each vertex
// ends at that apex's update) covering jittered-cube tets with scalar metrics,
// slivers and random shapes with anisotropic metrics, and uniform random times;
// every site of the mask is exercised by those inputs (the one exception, site 29,
// is TB*0 beside TA*l1, where both choices give the same value).  A GPU test holds
// the group to the reference kernel on fresh inputs.
// ---------------------------------------------------------------------------
constexpr unsigned long long kFuseApexA = 0x6301902630000ull;  // update of A from B, D, C
constexpr unsigned long long kFuseApexB = 0x6301902630000ull;  // B from A, D, C
constexpr unsigned long long kFuseApexC = 0x4203182420002ull;  // C from A, B, D
constexpr unsigned long long kFuseApexD = 0x0000001100000000ull;  // D from A, B, C

// Sites in R take their choice from the runtime mask m instead of M (one body
// serving several masks): the same two operations, operands picked by selects.
template <unsigned long long M, unsigned long long R, int S>
__device__ __forceinline__ float x_ms(unsigned long long m, float x, float y, float z, float w) {  // x*y - z*w
  if constexpr (((R >> S) & 1ull) != 0) {
    const bool b = ((m >> S) & 1ull) != 0;
    const float pr = __fmul_rn(b ? x : z, b ? y : w);
    return __fmaf_rn(b ? -z : x, b ? w : y, b ? pr : -pr);
  } else if constexpr (((M >> S) & 1ull) != 0) {
    return __fmaf_rn(-z, w, __fmul_rn(x, y));
  } else {
    return __fmaf_rn(x, y, -__fmul_rn(z, w));
  }
}
template <unsigned long long M, unsigned long long R, int S>
__device__ __forceinline__ float x_ma(unsigned long long m, float x, float y, float z, float w) {  // x*y + z*w
  if constexpr (((R >> S) & 1ull) != 0) {
    const bool b = ((m >> S) & 1ull) != 0;
    const float pr = __fmul_rn(b ? x : z, b ? y : w);
    return __fmaf_rn(b ? z : x, b ? w : y, pr);
  } else if constexpr (((M >> S) & 1ull) != 0) {
    return __fmaf_rn(z, w, __fmul_rn(x, y));
  } else {
    return __fmaf_rn(x, y, __fmul_rn(z, w));
  }
}
// (l1*XX + l2*XY + XZ)*l1 + (l1*XY + l2*YY + YZ)*l2 + (l1*XZ + l2*YZ + ZZ): the metric
// length of the path from the apex to the point l1 A + l2 B + l3 C (sites S..S+3)
template <unsigned long long M, unsigned long long R, int S>
__device__ __forceinline__ float x_dist3(unsigned long long m, float l1, float l2, float ACAC, float ACBC,
                                         float ACCD, float BCBC, float BCCD, float CDCD) {
  const float X = __fadd_rn(x_ma<M, R, S>(m, l1, ACAC, l2, ACBC), ACCD);
  const float Y = __fadd_rn(x_ma<M, R, S + 1>(m, l1, ACBC, l2, BCBC), BCCD);
  const float Z = __fadd_rn(x_ma<M, R, S + 2>(m, l1, ACCD, l2, BCCD), CDCD);
  return __fadd_rn(x_ma<M, R, S + 3>(m, X, l1, Y, l2), Z);
}
// (l*XX + XY)*l + (l*XY + YY): the same on an edge
__device__ __forceinline__ float x_dist2(float l, float XX, float XY, float YY) {
  return __fmaf_rn(__fmaf_rn(l, XX, XY), l, __fmaf_rn(l, XY, YY));
}
__device__ __forceinline__ float x_root(float num, float p) {
  if (fabsf(p) < 0x1p126f) return __fdiv_rn(num, __fmul_rn(2.0f, p));
  return root_quot_slow(num, p);
}

// localSolverTet1 (CUDA_kernels.cu:69-225) with the roundings of mask M: the update
// of apex D from A, B, C; the candidate order and every expression tree are the
// reference's.
template <unsigned long long M, unsigned long long R = 0>
__device__ __forceinline__ float tet_update_x(float TA, float TB, float TC, float ACAC, float ACBC, float ACCD,
                                              float BCBC, float BCCD, float CDCD, unsigned long long m = 0) {
  if (TA >= kLarge3DDev && TB >= kLarge3DDev && TC >= kLarge3DDev) return kLarge3DDev;
  float p, q, r, l1, l2, l3, delta;
  float fBC = kLarge3DDev, fAB = kLarge3DDev, fAC = kLarge3DDev, TD = kLarge3DDev;
  const float TAC = __fsub_rn(TC, TA), TBC = __fsub_rn(TC, TB), TAB = __fsub_rn(TB, TA);
  // ---- face BC (lambda1 = 0) ----
  p = x_ms<M, R, 0>(m, __fmul_rn(BCBC, TBC), TBC, BCBC, BCBC);
  q = x_ms<M, R, 1>(m, __fmul_rn(__fadd_rn(BCCD, BCCD), TBC), TBC, __fmul_rn(2.0f, BCBC), BCCD);
  r = x_ms<M, R, 2>(m, __fmul_rn(TBC, TBC), CDCD, BCCD, BCCD);
  delta = x_ms<M, R, 3>(m, q, q, __fmul_rn(4.0f, p), r);
  if (delta >= 0.0f) {
    const float sd = __fsqrt_rn(delta);
    l2 = x_root(__fadd_rn(-q, sd), p);
    l3 = __fsub_rn(1.0f, l2);
    if (l2 >= 0 && l2 <= 1)
      fBC = fminf(fBC, __fadd_rn(x_ma<M, R, 4>(m, TB, l2, TC, l3), __fsqrt_rn(x_dist2(l2, BCBC, BCCD, CDCD))));
    l2 = x_root(__fsub_rn(-q, sd), p);
    l3 = __fsub_rn(1.0f, l2);
    if (l2 >= 0 && l2 <= 1)
      fBC = fminf(fBC, __fadd_rn(x_ma<M, R, 5>(m, TB, l2, TC, l3), __fsqrt_rn(x_dist2(l2, BCBC, BCCD, CDCD))));
  }
  const float eB = __fadd_rn(TB, __fsqrt_rn(__fadd_rn(__fadd_rn(BCBC, BCCD), __fadd_rn(BCCD, CDCD))));
  const float eC = __fadd_rn(TC, __fsqrt_rn(CDCD));
  fBC = fminf(fBC, fminf(eB, eC));
  // ---- face AB (lambda3 = 0) ----
  const float gx = __fsub_rn(ACAC, ACBC), gy = __fsub_rn(ACBC, BCBC), gz = __fsub_rn(ACCD, BCCD);
  const float TAB2 = __fmul_rn(TAB, TAB);
  const float P1 = x_ms<M, R, 6>(m, TAB2, ACAC, gx, gx);
  const float P2 = x_ms<M, R, 7>(m, __fmul_rn(BCBC, TAB), TAB, gy, gy);
  const float P3 = x_ms<M, R, 8>(m, __fmul_rn(__fadd_rn(ACBC, ACBC), TAB), TAB, __fmul_rn(2.0f, gx), gy);
  p = __fsub_rn(__fadd_rn(P1, P2), P3);
  const float P4 = x_ms<M, R, 9>(m, __fmul_rn(__fadd_rn(ACCD, ACCD), TAB), TAB, __fmul_rn(2.0f, gx), gz);
  const float P5 = x_ms<M, R, 10>(m, __fmul_rn(__fadd_rn(BCCD, BCCD), TAB), TAB, __fmul_rn(2.0f, gy), gz);
  q = __fsub_rn(__fadd_rn(__fadd_rn(__fmul_rn(-P2, 2.0f), P3), P4), P5);
  r = __fadd_rn(__fadd_rn(x_ms<M, R, 11>(m, TAB2, BCBC, gy, gy), P5), x_ms<M, R, 12>(m, TAB2, CDCD, gz, gz));
  delta = x_ms<M, R, 13>(m, q, q, __fmul_rn(4.0f, p), r);
  if (delta >= 0.0f) {
    const float sd = __fsqrt_rn(delta);
    l1 = x_root(__fadd_rn(-q, sd), p);
    l2 = __fsub_rn(1.0f, l1);
    if (l1 >= 0 && l1 <= 1)
      fAB = fminf(fAB, __fadd_rn(x_ma<M, R, 14>(m, TA, l1, TB, l2),
                                 __fsqrt_rn(x_dist3<M, R, 15>(m, l1, l2, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD))));
    l1 = x_root(__fsub_rn(-q, sd), p);
    l2 = __fsub_rn(1.0f, l1);
    if (l1 >= 0 && l1 <= 1)
      fAB = fminf(fAB, __fadd_rn(x_ma<M, R, 19>(m, TA, l1, TB, l2),
                                 __fsqrt_rn(x_dist3<M, R, 20>(m, l1, l2, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD))));
  }
  const float eA = __fadd_rn(TA, __fsqrt_rn(__fadd_rn(__fadd_rn(ACAC, ACCD), __fadd_rn(ACCD, CDCD))));
  fAB = fminf(fAB, fminf(eB, eA));
  // ---- face AC (lambda2 = 0) ----
  const float TAC2 = __fmul_rn(TAC, TAC);
  p = x_ms<M, R, 24>(m, __fmul_rn(ACAC, TAC), TAC, ACAC, ACAC);
  const float qAC = x_ms<M, R, 25>(m, __fmul_rn(__fadd_rn(ACCD, ACCD), TAC), TAC, __fmul_rn(2.0f, ACAC), ACCD);
  const float rAC = x_ms<M, R, 26>(m, TAC2, CDCD, ACCD, ACCD);
  delta = x_ms<M, R, 27>(m, qAC, qAC, __fmul_rn(4.0f, p), rAC);
  if (delta >= 0.0f) {
    const float sd = __fsqrt_rn(delta);
    l1 = x_root(__fadd_rn(-qAC, sd), p);
    l3 = __fsub_rn(1.0f, l1);
    if (l1 >= 0 && l1 <= 1)
      fAC = fminf(fAC, __fadd_rn(x_ma<M, R, 28>(m, TA, l1, TC, l3), __fsqrt_rn(x_dist2(l1, ACAC, ACCD, CDCD))));
    l1 = x_root(__fsub_rn(-qAC, sd), p);
    l3 = __fsub_rn(1.0f, l1);
    // the second candidate keeps a zero-weight TB term, as the reference does
    if (l1 >= 0 && l1 <= 1)
      fAC = fminf(fAC, __fadd_rn(__fmaf_rn(TC, l3, x_ma<M, R, 29>(m, TA, l1, TB, 0.0f)),
                                 __fsqrt_rn(x_dist2(l1, ACAC, ACCD, CDCD))));
  }
  fAC = fminf(fAC, fminf(eA, eC));
  // ---- inside face ABC: lambda2 = (s*lambda1 + t)/(h + 1e-8) ----
  const float s = x_ms<M, R, 30>(m, TAC, ACBC, TBC, ACAC);
  const float t = x_ms<M, R, 31>(m, TAC, BCCD, TBC, ACCD);
  const float h = -x_ms<M, R, 32>(m, TAC, BCBC, TBC, ACBC);
  const float A1 = x_ms<M, R, 33>(m, TAC2, ACAC, ACAC, ACAC);
  const float A2 = x_ms<M, R, 34>(m, __fmul_rn(BCBC, TAC), TAC, ACBC, ACBC);
  const float A3 = x_ms<M, R, 35>(m, __fmul_rn(__fadd_rn(ACBC, ACBC), TAC), TAC, __fmul_rn(2.0f, ACAC), ACBC);
  const float A4 = x_ms<M, R, 37>(m, __fmul_rn(__fadd_rn(BCCD, BCCD), TAC), TAC, __fmul_rn(2.0f, ACBC), ACCD);
  p = __fmaf_rn(__fmul_rn(A3, s), h, x_ma<M, R, 36>(m, __fmul_rn(A1, h), h, __fmul_rn(A2, s), s));
  q = __fmaf_rn(__fmul_rn(A4, s), h,
                __fmaf_rn(__fmul_rn(qAC, h), h, x_ma<M, R, 38>(m, __fmul_rn(__fmul_rn(A2, 2.0f), s), t, __fmul_rn(A3, t), h)));
  r = __fmaf_rn(__fmul_rn(rAC, h), h, x_ma<M, R, 40>(m, __fmul_rn(x_ms<M, R, 39>(m, TAC2, BCBC, ACBC, ACBC), t), t,
                                                   __fmul_rn(A4, t), h));
  delta = x_ms<M, R, 41>(m, q, q, __fmul_rn(4.0f, p), r);
  if (delta >= 0.0f) {
    const float sd = __fsqrt_rn(delta);
    l1 = x_root(__fadd_rn(-q, sd), p);
    l2 = small_quot(__fmaf_rn(s, l1, t), h);
    l3 = __fsub_rn(__fsub_rn(1.0f, l1), l2);
    if (l1 >= 0 && l1 <= 1 && l2 >= 0 && l2 <= 1 && l3 >= 0 && l3 <= 1)
      TD = fminf(TD, __fadd_rn(__fmaf_rn(TC, l3, x_ma<M, R, 42>(m, TA, l1, TB, l2)),
                               __fsqrt_rn(x_dist3<M, R, 43>(m, l1, l2, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD))));
    l1 = x_root(__fsub_rn(-q, sd), p);
    l2 = small_quot(__fmaf_rn(s, l1, t), h);
    l3 = __fsub_rn(__fsub_rn(1.0f, l1), l2);
    if (l1 >= 0 && l1 <= 1 && l2 >= 0 && l2 <= 1 && l3 >= 0 && l3 <= 1)
      TD = fminf(TD, __fadd_rn(__fmaf_rn(TC, l3, x_ma<M, R, 47>(m, TA, l1, TB, l2)),
                               __fsqrt_rn(x_dist3<M, R, 48>(m, l1, l2, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD))));
  }
  return fminf(TD, fminf(fBC, fminf(fAB, fAC)));
}

// The same update with the edge-face candidates (faces BC, AB, AC) evaluated
// without branches: both roots of each face are computed whatever the
// discriminant's sign, and a candidate enters the minimum only where the branching
// form would have taken it (a negative discriminant gives NaN roots, which fail
// the [0, 1] tests).  Every value is the explicitly rounded one of tet_update_x and
// the minimum does not depend on the order of its operands, so the result is the
// same bits; the interior face keeps its branch (its second quotient has a slow
// path that a NaN input would take).
template <unsigned long long M, unsigned long long R = 0>
__device__ __forceinline__ float tet_update_xb(float TA, float TB, float TC, float ACAC, float ACBC, float ACCD,
                                               float BCBC, float BCCD, float CDCD, unsigned long long m = 0) {
  if (TA >= kLarge3DDev && TB >= kLarge3DDev && TC >= kLarge3DDev) return kLarge3DDev;
  const float L = kLarge3DDev;
  const float TAC = __fsub_rn(TC, TA), TBC = __fsub_rn(TC, TB), TAB = __fsub_rn(TB, TA);
  // ---- face BC (lambda1 = 0) ----
  float fBC;
  {
    const float p = x_ms<M, R, 0>(m, __fmul_rn(BCBC, TBC), TBC, BCBC, BCBC);
    const float q = x_ms<M, R, 1>(m, __fmul_rn(__fadd_rn(BCCD, BCCD), TBC), TBC, __fmul_rn(2.0f, BCBC), BCCD);
    const float r = x_ms<M, R, 2>(m, __fmul_rn(TBC, TBC), CDCD, BCCD, BCCD);
    const float delta = x_ms<M, R, 3>(m, q, q, __fmul_rn(4.0f, p), r);
    const bool ok = delta >= 0.0f;
    const float sd = __fsqrt_rn(delta);
    const float a2 = x_root(__fadd_rn(-q, sd), p), a3 = __fsub_rn(1.0f, a2);
    const float b2 = x_root(__fsub_rn(-q, sd), p), b3 = __fsub_rn(1.0f, b2);
    const float ca = __fadd_rn(x_ma<M, R, 4>(m, TB, a2, TC, a3), __fsqrt_rn(x_dist2(a2, BCBC, BCCD, CDCD)));
    const float cb = __fadd_rn(x_ma<M, R, 5>(m, TB, b2, TC, b3), __fsqrt_rn(x_dist2(b2, BCBC, BCCD, CDCD)));
    // seeded with LARGENUM as the branching form (a NaN candidate is ignored)
    fBC = fminf(fminf(L, (ok && a2 >= 0 && a2 <= 1) ? ca : L), (ok && b2 >= 0 && b2 <= 1) ? cb : L);
  }
  const float eB = __fadd_rn(TB, __fsqrt_rn(__fadd_rn(__fadd_rn(BCBC, BCCD), __fadd_rn(BCCD, CDCD))));
  const float eC = __fadd_rn(TC, __fsqrt_rn(CDCD));
  const float eA = __fadd_rn(TA, __fsqrt_rn(__fadd_rn(__fadd_rn(ACAC, ACCD), __fadd_rn(ACCD, CDCD))));
  // ---- face AB (lambda3 = 0) ----
  float fAB;
  {
    const float gx = __fsub_rn(ACAC, ACBC), gy = __fsub_rn(ACBC, BCBC), gz = __fsub_rn(ACCD, BCCD);
    const float TAB2 = __fmul_rn(TAB, TAB);
    const float P1 = x_ms<M, R, 6>(m, TAB2, ACAC, gx, gx);
    const float P2 = x_ms<M, R, 7>(m, __fmul_rn(BCBC, TAB), TAB, gy, gy);
    const float P3 = x_ms<M, R, 8>(m, __fmul_rn(__fadd_rn(ACBC, ACBC), TAB), TAB, __fmul_rn(2.0f, gx), gy);
    const float p = __fsub_rn(__fadd_rn(P1, P2), P3);
    const float P4 = x_ms<M, R, 9>(m, __fmul_rn(__fadd_rn(ACCD, ACCD), TAB), TAB, __fmul_rn(2.0f, gx), gz);
    const float P5 = x_ms<M, R, 10>(m, __fmul_rn(__fadd_rn(BCCD, BCCD), TAB), TAB, __fmul_rn(2.0f, gy), gz);
    const float q = __fsub_rn(__fadd_rn(__fadd_rn(__fmul_rn(-P2, 2.0f), P3), P4), P5);
    const float r = __fadd_rn(__fadd_rn(x_ms<M, R, 11>(m, TAB2, BCBC, gy, gy), P5), x_ms<M, R, 12>(m, TAB2, CDCD, gz, gz));
    const float delta = x_ms<M, R, 13>(m, q, q, __fmul_rn(4.0f, p), r);
    const bool ok = delta >= 0.0f;
    const float sd = __fsqrt_rn(delta);
    const float a1 = x_root(__fadd_rn(-q, sd), p), a2 = __fsub_rn(1.0f, a1);
    const float b1 = x_root(__fsub_rn(-q, sd), p), b2 = __fsub_rn(1.0f, b1);
    const float ca = __fadd_rn(x_ma<M, R, 14>(m, TA, a1, TB, a2),
                               __fsqrt_rn(x_dist3<M, R, 15>(m, a1, a2, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD)));
    const float cb = __fadd_rn(x_ma<M, R, 19>(m, TA, b1, TB, b2),
                               __fsqrt_rn(x_dist3<M, R, 20>(m, b1, b2, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD)));
    // seeded with LARGENUM as the branching form (a NaN candidate is ignored)
    fAB = fminf(fminf(L, (ok && a1 >= 0 && a1 <= 1) ? ca : L), (ok && b1 >= 0 && b1 <= 1) ? cb : L);
  }
  // ---- face AC (lambda2 = 0) ----
  const float TAC2 = __fmul_rn(TAC, TAC);
  const float qAC = x_ms<M, R, 25>(m, __fmul_rn(__fadd_rn(ACCD, ACCD), TAC), TAC, __fmul_rn(2.0f, ACAC), ACCD);
  const float rAC = x_ms<M, R, 26>(m, TAC2, CDCD, ACCD, ACCD);
  float fAC;
  {
    const float p = x_ms<M, R, 24>(m, __fmul_rn(ACAC, TAC), TAC, ACAC, ACAC);
    const float delta = x_ms<M, R, 27>(m, qAC, qAC, __fmul_rn(4.0f, p), rAC);
    const bool ok = delta >= 0.0f;
    const float sd = __fsqrt_rn(delta);
    const float a1 = x_root(__fadd_rn(-qAC, sd), p), a3 = __fsub_rn(1.0f, a1);
    const float b1 = x_root(__fsub_rn(-qAC, sd), p), b3 = __fsub_rn(1.0f, b1);
    const float ca = __fadd_rn(x_ma<M, R, 28>(m, TA, a1, TC, a3), __fsqrt_rn(x_dist2(a1, ACAC, ACCD, CDCD)));
    // the second candidate keeps a zero-weight TB term, as the reference does
    const float cb = __fadd_rn(__fmaf_rn(TC, b3, x_ma<M, R, 29>(m, TA, b1, TB, 0.0f)),
                               __fsqrt_rn(x_dist2(b1, ACAC, ACCD, CDCD)));
    // seeded with LARGENUM as the branching form (a NaN candidate is ignored)
    fAC = fminf(fminf(L, (ok && a1 >= 0 && a1 <= 1) ? ca : L), (ok && b1 >= 0 && b1 <= 1) ? cb : L);
  }
  const float edges = fminf(fminf(fBC, fminf(eB, eC)), fminf(fminf(fAB, fminf(eB, eA)), fminf(fAC, fminf(eA, eC))));
  // ---- inside face ABC: lambda2 = (s*lambda1 + t)/(h + 1e-8) ----
  const float s = x_ms<M, R, 30>(m, TAC, ACBC, TBC, ACAC);
  const float t = x_ms<M, R, 31>(m, TAC, BCCD, TBC, ACCD);
  const float h = -x_ms<M, R, 32>(m, TAC, BCBC, TBC, ACBC);
  const float A1 = x_ms<M, R, 33>(m, TAC2, ACAC, ACAC, ACAC);
  const float A2 = x_ms<M, R, 34>(m, __fmul_rn(BCBC, TAC), TAC, ACBC, ACBC);
  const float A3 = x_ms<M, R, 35>(m, __fmul_rn(__fadd_rn(ACBC, ACBC), TAC), TAC, __fmul_rn(2.0f, ACAC), ACBC);
  const float A4 = x_ms<M, R, 37>(m, __fmul_rn(__fadd_rn(BCCD, BCCD), TAC), TAC, __fmul_rn(2.0f, ACBC), ACCD);
  const float p = __fmaf_rn(__fmul_rn(A3, s), h, x_ma<M, R, 36>(m, __fmul_rn(A1, h), h, __fmul_rn(A2, s), s));
  const float q = __fmaf_rn(__fmul_rn(A4, s), h,
                            __fmaf_rn(__fmul_rn(qAC, h), h,
                                      x_ma<M, R, 38>(m, __fmul_rn(__fmul_rn(A2, 2.0f), s), t, __fmul_rn(A3, t), h)));
  const float r = __fmaf_rn(__fmul_rn(rAC, h), h, x_ma<M, R, 40>(m, __fmul_rn(x_ms<M, R, 39>(m, TAC2, BCBC, ACBC, ACBC), t), t,
                                                               __fmul_rn(A4, t), h));
  const float delta = x_ms<M, R, 41>(m, q, q, __fmul_rn(4.0f, p), r);
  float TD = L;
  if (delta >= 0.0f) {
    const float sd = __fsqrt_rn(delta);
    float l1 = x_root(__fadd_rn(-q, sd), p);
    float l2 = small_quot(__fmaf_rn(s, l1, t), h);
    float l3 = __fsub_rn(__fsub_rn(1.0f, l1), l2);
    if (l1 >= 0 && l1 <= 1 && l2 >= 0 && l2 <= 1 && l3 >= 0 && l3 <= 1)
      TD = fminf(TD, __fadd_rn(__fmaf_rn(TC, l3, x_ma<M, R, 42>(m, TA, l1, TB, l2)),
                               __fsqrt_rn(x_dist3<M, R, 43>(m, l1, l2, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD))));
    l1 = x_root(__fsub_rn(-q, sd), p);
    l2 = small_quot(__fmaf_rn(s, l1, t), h);
    l3 = __fsub_rn(__fsub_rn(1.0f, l1), l2);
    if (l1 >= 0 && l1 <= 1 && l2 >= 0 && l2 <= 1 && l3 >= 0 && l3 <= 1)
      TD = fminf(TD, __fadd_rn(__fmaf_rn(TC, l3, x_ma<M, R, 47>(m, TA, l1, TB, l2)),
                               __fsqrt_rn(x_dist3<M, R, 48>(m, l1, l2, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD))));
  }
  return fminf(TD, edges);
}

// tet_update_x with the four faces' quadratic coefficients and discriminants
// formed before any root is taken: the four chains are independent and can
// interleave; the roots keep their branches.  Same operations, same bits.
template <unsigned long long M, unsigned long long R = 0>
__device__ __forceinline__ float tet_update_xd(float TA, float TB, float TC, float ACAC, float ACBC, float ACCD,
                                               float BCBC, float BCCD, float CDCD, unsigned long long m = 0) {
  if (TA >= kLarge3DDev && TB >= kLarge3DDev && TC >= kLarge3DDev) return kLarge3DDev;
  const float L = kLarge3DDev;
  const float TAC = __fsub_rn(TC, TA), TBC = __fsub_rn(TC, TB), TAB = __fsub_rn(TB, TA);
  // face BC
  const float pBC = x_ms<M, R, 0>(m, __fmul_rn(BCBC, TBC), TBC, BCBC, BCBC);
  const float qBC = x_ms<M, R, 1>(m, __fmul_rn(__fadd_rn(BCCD, BCCD), TBC), TBC, __fmul_rn(2.0f, BCBC), BCCD);
  const float rBC = x_ms<M, R, 2>(m, __fmul_rn(TBC, TBC), CDCD, BCCD, BCCD);
  const float dBC = x_ms<M, R, 3>(m, qBC, qBC, __fmul_rn(4.0f, pBC), rBC);
  // face AB
  const float gx = __fsub_rn(ACAC, ACBC), gy = __fsub_rn(ACBC, BCBC), gz = __fsub_rn(ACCD, BCCD);
  const float TAB2 = __fmul_rn(TAB, TAB);
  const float P2 = x_ms<M, R, 7>(m, __fmul_rn(BCBC, TAB), TAB, gy, gy);
  const float P3 = x_ms<M, R, 8>(m, __fmul_rn(__fadd_rn(ACBC, ACBC), TAB), TAB, __fmul_rn(2.0f, gx), gy);
  const float pAB = __fsub_rn(__fadd_rn(x_ms<M, R, 6>(m, TAB2, ACAC, gx, gx), P2), P3);
  const float P5 = x_ms<M, R, 10>(m, __fmul_rn(__fadd_rn(BCCD, BCCD), TAB), TAB, __fmul_rn(2.0f, gy), gz);
  const float qAB = __fsub_rn(__fadd_rn(__fadd_rn(__fmul_rn(-P2, 2.0f), P3),
                                        x_ms<M, R, 9>(m, __fmul_rn(__fadd_rn(ACCD, ACCD), TAB), TAB, __fmul_rn(2.0f, gx), gz)),
                              P5);
  const float rAB = __fadd_rn(__fadd_rn(x_ms<M, R, 11>(m, TAB2, BCBC, gy, gy), P5), x_ms<M, R, 12>(m, TAB2, CDCD, gz, gz));
  const float dAB = x_ms<M, R, 13>(m, qAB, qAB, __fmul_rn(4.0f, pAB), rAB);
  // face AC
  const float TAC2 = __fmul_rn(TAC, TAC);
  const float pAC = x_ms<M, R, 24>(m, __fmul_rn(ACAC, TAC), TAC, ACAC, ACAC);
  const float qAC = x_ms<M, R, 25>(m, __fmul_rn(__fadd_rn(ACCD, ACCD), TAC), TAC, __fmul_rn(2.0f, ACAC), ACCD);
  const float rAC = x_ms<M, R, 26>(m, TAC2, CDCD, ACCD, ACCD);
  const float dAC = x_ms<M, R, 27>(m, qAC, qAC, __fmul_rn(4.0f, pAC), rAC);
  // face ABC
  const float s = x_ms<M, R, 30>(m, TAC, ACBC, TBC, ACAC);
  const float t = x_ms<M, R, 31>(m, TAC, BCCD, TBC, ACCD);
  const float h = -x_ms<M, R, 32>(m, TAC, BCBC, TBC, ACBC);
  const float A1 = x_ms<M, R, 33>(m, TAC2, ACAC, ACAC, ACAC);
  const float A2 = x_ms<M, R, 34>(m, __fmul_rn(BCBC, TAC), TAC, ACBC, ACBC);
  const float A3 = x_ms<M, R, 35>(m, __fmul_rn(__fadd_rn(ACBC, ACBC), TAC), TAC, __fmul_rn(2.0f, ACAC), ACBC);
  const float A4 = x_ms<M, R, 37>(m, __fmul_rn(__fadd_rn(BCCD, BCCD), TAC), TAC, __fmul_rn(2.0f, ACBC), ACCD);
  const float p = __fmaf_rn(__fmul_rn(A3, s), h, x_ma<M, R, 36>(m, __fmul_rn(A1, h), h, __fmul_rn(A2, s), s));
  const float q = __fmaf_rn(__fmul_rn(A4, s), h,
                            __fmaf_rn(__fmul_rn(qAC, h), h,
                                      x_ma<M, R, 38>(m, __fmul_rn(__fmul_rn(A2, 2.0f), s), t, __fmul_rn(A3, t), h)));
  const float r = __fmaf_rn(__fmul_rn(rAC, h), h, x_ma<M, R, 40>(m, __fmul_rn(x_ms<M, R, 39>(m, TAC2, BCBC, ACBC, ACBC), t), t,
                                                               __fmul_rn(A4, t), h));
  const float delta = x_ms<M, R, 41>(m, q, q, __fmul_rn(4.0f, p), r);
  const float eB = __fadd_rn(TB, __fsqrt_rn(__fadd_rn(__fadd_rn(BCBC, BCCD), __fadd_rn(BCCD, CDCD))));
  const float eC = __fadd_rn(TC, __fsqrt_rn(CDCD));
  const float eA = __fadd_rn(TA, __fsqrt_rn(__fadd_rn(__fadd_rn(ACAC, ACCD), __fadd_rn(ACCD, CDCD))));
  float fBC = L, fAB = L, fAC = L, TD = L, l1, l2, l3;
  if (dBC >= 0.0f) {
    const float sd = __fsqrt_rn(dBC);
    l2 = x_root(__fadd_rn(-qBC, sd), pBC);
    l3 = __fsub_rn(1.0f, l2);
    if (l2 >= 0 && l2 <= 1)
      fBC = fminf(fBC, __fadd_rn(x_ma<M, R, 4>(m, TB, l2, TC, l3), __fsqrt_rn(x_dist2(l2, BCBC, BCCD, CDCD))));
    l2 = x_root(__fsub_rn(-qBC, sd), pBC);
    l3 = __fsub_rn(1.0f, l2);
    if (l2 >= 0 && l2 <= 1)
      fBC = fminf(fBC, __fadd_rn(x_ma<M, R, 5>(m, TB, l2, TC, l3), __fsqrt_rn(x_dist2(l2, BCBC, BCCD, CDCD))));
  }
  fBC = fminf(fBC, fminf(eB, eC));
  if (dAB >= 0.0f) {
    const float sd = __fsqrt_rn(dAB);
    l1 = x_root(__fadd_rn(-qAB, sd), pAB);
    l2 = __fsub_rn(1.0f, l1);
    if (l1 >= 0 && l1 <= 1)
      fAB = fminf(fAB, __fadd_rn(x_ma<M, R, 14>(m, TA, l1, TB, l2),
                                 __fsqrt_rn(x_dist3<M, R, 15>(m, l1, l2, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD))));
    l1 = x_root(__fsub_rn(-qAB, sd), pAB);
    l2 = __fsub_rn(1.0f, l1);
    if (l1 >= 0 && l1 <= 1)
      fAB = fminf(fAB, __fadd_rn(x_ma<M, R, 19>(m, TA, l1, TB, l2),
                                 __fsqrt_rn(x_dist3<M, R, 20>(m, l1, l2, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD))));
  }
  fAB = fminf(fAB, fminf(eB, eA));
  if (dAC >= 0.0f) {
    const float sd = __fsqrt_rn(dAC);
    l1 = x_root(__fadd_rn(-qAC, sd), pAC);
    l3 = __fsub_rn(1.0f, l1);
    if (l1 >= 0 && l1 <= 1)
      fAC = fminf(fAC, __fadd_rn(x_ma<M, R, 28>(m, TA, l1, TC, l3), __fsqrt_rn(x_dist2(l1, ACAC, ACCD, CDCD))));
    l1 = x_root(__fsub_rn(-qAC, sd), pAC);
    l3 = __fsub_rn(1.0f, l1);
    if (l1 >= 0 && l1 <= 1)
      fAC = fminf(fAC, __fadd_rn(__fmaf_rn(TC, l3, x_ma<M, R, 29>(m, TA, l1, TB, 0.0f)),
                                 __fsqrt_rn(x_dist2(l1, ACAC, ACCD, CDCD))));
  }
  fAC = fminf(fAC, fminf(eA, eC));
  if (delta >= 0.0f) {
    const float sd = __fsqrt_rn(delta);
    l1 = x_root(__fadd_rn(-q, sd), p);
    l2 = small_quot(__fmaf_rn(s, l1, t), h);
    l3 = __fsub_rn(__fsub_rn(1.0f, l1), l2);
    if (l1 >= 0 && l1 <= 1 && l2 >= 0 && l2 <= 1 && l3 >= 0 && l3 <= 1)
      TD = fminf(TD, __fadd_rn(__fmaf_rn(TC, l3, x_ma<M, R, 42>(m, TA, l1, TB, l2)),
                               __fsqrt_rn(x_dist3<M, R, 43>(m, l1, l2, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD))));
    l1 = x_root(__fsub_rn(-q, sd), p);
    l2 = small_quot(__fmaf_rn(s, l1, t), h);
    l3 = __fsub_rn(__fsub_rn(1.0f, l1), l2);
    if (l1 >= 0 && l1 <= 1 && l2 >= 0 && l2 <= 1 && l3 >= 0 && l3 <= 1)
      TD = fminf(TD, __fadd_rn(__fmaf_rn(TC, l3, x_ma<M, R, 47>(m, TA, l1, TB, l2)),
                               __fsqrt_rn(x_dist3<M, R, 48>(m, l1, l2, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD))));
  }
  return fminf(TD, fminf(fBC, fminf(fAB, fAC)));
}

#ifndef EIK_TET_BRANCHFREE
#define EIK_TET_BRANCHFREE 0
#endif
#if EIK_TET_BRANCHFREE == 1
#define EIK_TET_UPDATE tet_update_xb
#elif EIK_TET_BRANCHFREE == 2
#define EIK_TET_UPDATE tet_update_xd
#else
#define EIK_TET_UPDATE tet_update_x
#endif

// The remaining metric edge products of a slot from its six stored ones
// (CUDA_kernels.cu:429-437), in the order the tet updates take them.
struct TetGram {
  float ACAC, ACBC, ACCD, BCBC, BCCD, CDCD, ADAD, ADBD, ADCD, BDBD, CDBD;
};
__device__ __forceinline__ TetGram tet_gram9(float ACBC, float BCCD, float ACCD, float ADBD, float ACAD, float BCBD) {
  TetGram g;
  const float ADBC = __fadd_rn(ACBC, BCCD);
  const float ACBD = __fadd_rn(ACBC, ACCD);
  g.CDBD = __fsub_rn(ADBD, ACBD);
  g.ADCD = __fsub_rn(ADBD, ADBC);
  g.CDCD = __fsub_rn(g.ADCD, ACCD);
  g.ADAD = __fadd_rn(g.ADCD, ACAD);
  g.ACAC = __fsub_rn(ACAD, ACCD);
  g.BDBD = __fadd_rn(BCBD, g.CDBD);
  g.BCBC = __fsub_rn(BCBD, BCCD);
  g.ACBC = ACBC;
  g.BCCD = BCCD;
  g.ACCD = ACCD;
  g.ADBD = ADBD;
  return g;
}

#ifndef EIK_TET_NOINLINE
#define EIK_TET_NOINLINE 1
#endif
#ifndef EIK_TET_ONEBODY
#define EIK_TET_ONEBODY 2
#endif
#if EIK_TET_ONEBODY == 2
// two out-of-line bodies: apexes A, B and C share one (their masks differ at 8
// sites, taken at run time through selects), apex D has its own: little code for
// the instruction cache, few selects (65^3 sweep kernel 2% faster than one body for
// all four kinds, 4-6% faster than one body per mask; same bits)
constexpr unsigned long long kFuseAll = kFuseApexA & kFuseApexB & kFuseApexC;
constexpr unsigned long long kFuseRt = (kFuseApexA ^ kFuseApexB) | (kFuseApexA ^ kFuseApexC);
__device__ __noinline__ float tet_update_rt(float TA, float TB, float TC, float ACAC, float ACBC, float ACCD,
                                            float BCBC, float BCCD, float CDCD, unsigned long long m) {
  return EIK_TET_UPDATE<kFuseAll, kFuseRt>(TA, TB, TC, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD, m);
}
__device__ __noinline__ float tet_update_d(float TA, float TB, float TC, float ACAC, float ACBC, float ACCD,
                                           float BCBC, float BCCD, float CDCD) {
  return EIK_TET_UPDATE<kFuseApexD>(TA, TB, TC, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD);
}
template <unsigned long long M>
__device__ __forceinline__ float tet_update_call(float TA, float TB, float TC, float ACAC, float ACBC, float ACCD,
                                                 float BCBC, float BCCD, float CDCD) {
  if constexpr (M == kFuseApexD) return tet_update_d(TA, TB, TC, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD);
  else return tet_update_rt(TA, TB, TC, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD, M);
}
#elif EIK_TET_ONEBODY
// one out-of-line body for all four apex kinds: the sites where their masks agree
// are fixed at compile time, the 13 others (kFuseRt) follow the kind's mask at run
// time through selects; a third of the code for the instruction cache (65^3 sweep
// kernel 2-4% faster than one body per mask, same bits)
constexpr unsigned long long kFuseAll = kFuseApexA & kFuseApexB & kFuseApexC & kFuseApexD;
constexpr unsigned long long kFuseRt =
    (kFuseApexA ^ kFuseApexB) | (kFuseApexA ^ kFuseApexC) | (kFuseApexA ^ kFuseApexD);
__device__ __noinline__ float tet_update_rt(float TA, float TB, float TC, float ACAC, float ACBC, float ACCD,
                                            float BCBC, float BCCD, float CDCD, unsigned long long m) {
  return EIK_TET_UPDATE<kFuseAll, kFuseRt>(TA, TB, TC, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD, m);
}
template <unsigned long long M>
__device__ __forceinline__ float tet_update_call(float TA, float TB, float TC, float ACAC, float ACBC, float ACCD,
                                                 float BCBC, float BCCD, float CDCD) {
  return tet_update_rt(TA, TB, TC, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD, M);
}
#elif EIK_TET_NOINLINE
// one out-of-line body per mask (apexes A and B share theirs): less code for the
// instruction cache than four inlined copies (the item sweep kernel ran 6% faster on
// the 65^3 workload, same bits)
template <unsigned long long M>
__device__ __noinline__ float tet_update_call(float TA, float TB, float TC, float ACAC, float ACBC, float ACCD,
                                              float BCBC, float BCCD, float CDCD) {
  return EIK_TET_UPDATE<M>(TA, TB, TC, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD);
}
#else
template <unsigned long long M>
__device__ __forceinline__ float tet_update_call(float TA, float TB, float TC, float ACAC, float ACBC, float ACCD,
                                                 float BCBC, float BCCD, float CDCD) {
  return EIK_TET_UPDATE<M>(TA, TB, TC, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD);
}
#endif

// The update of apex k (0..3 = A, B, C, D) of a slot with corner times T, as the
// reference's FIMCuda computes it for that apex (its arguments and its roundings).
template <int K>
__device__ __forceinline__ float apex_update(const float T[4], const TetGram& g) {
  if constexpr (K == 3)
    return tet_update_call<kFuseApexD>(T[0], T[1], T[2], g.ACAC, g.ACBC, g.ACCD, g.BCBC, g.BCCD, g.CDCD);
  if constexpr (K == 0)
    return tet_update_call<kFuseApexA>(T[1], T[3], T[2], g.BCBC, -g.BCCD, -g.ACBC, g.CDCD, g.ACCD, g.ACAC);
  if constexpr (K == 1)
    return tet_update_call<kFuseApexB>(T[0], T[3], T[2], g.ACAC, -g.ACCD, -g.ACBC, g.CDCD, g.BCCD, g.BCBC);
  if constexpr (K == 2)
    return tet_update_call<kFuseApexC>(T[0], T[1], T[3], g.ADAD, g.ADBD, -g.ADCD, g.BDBD, -g.CDBD, g.CDCD);
  return kLarge3DDev;
}

// The operations of the wide (precision mode) update, named so the update reads
// like the FP32 one.
__device__ __forceinline__ double w_make(double a, double) { return a; }
__device__ __forceinline__ double w_min(double a, double b) { return fmin(a, b); }
__device__ __forceinline__ double w_sqrt(double a) { return sqrt(a); }
__device__ __forceinline__ double w_recip(double a) { return 1.0 / a; }
__device__ __forceinline__ bool w_ge0(double a) { return a >= 0.0; }
__device__ __forceinline__ bool w_in01(double a) { return a >= 0 && a <= 1; }
__device__ __forceinline__ bool w_large(double a) { return a >= (double)kLarge3DDev; }
__device__ __forceinline__ float w_float(double a) { return (float)a; }

// Square root of a non-negative candidate distance for the FP64 update: the
// argument is formed in FP64 (where the cancellation is), the root taken in FP32 (relative error below 1e-7, far inside the scheme's 1e-5 tolerance), which
// spares the slow FP64 unit.
__device__ __forceinline__ double sqrt_pos(double x) { return (double)sqrtf((float)x); }

// The same tet update carried out in FP64 (precision mode: slots of sliver or
// ill-conditioned tets), written over a type R for the helpers above.  Same
// candidates and order as tet_update; the metric edge products come from FP64 setup
// values, quotients are FP64 (one reciprocal per candidate face); only the candidate
// roots use sqrt_pos.  (A double-float R, two FP32 numbers per value, ran slower on
// GB300 than the FP64 unit and was dropped.)
template <typename R>
__device__ __forceinline__ R tet_update_wide(R TA, R TB, R TC, R ACAC, R ACBC, R ACCD, R BCBC, R BCCD, R CDCD) {
  const R L = w_make((double)kLarge3DDev, R{});
  if (w_large(TA) && w_large(TB) && w_large(TC)) return L;
  const R one = w_make(1.0, R{}), eps8 = w_make(0.00000001, R{});
  R p, q, r, l1, l2, l3, delta, TE;
  R fBC = L, fAB = L, fAC = L, TD = L;
  const R TAC = TC - TA, TBC = TC - TB, TAB = TB - TA;
  // face BC
  p = BCBC * TBC * TBC - BCBC * BCBC;
  q = (BCCD + BCCD) * TBC * TBC - 2.0f * BCBC * BCCD;
  r = TBC * TBC * CDCD - BCCD * BCCD;
  delta = q * q - 4.0f * p * r;
  if (w_ge0(delta)) {
    const R sd = w_sqrt(delta), i2p = w_recip(2.0f * p);
    for (int sg = 0; sg < 2; ++sg) {
      l2 = (-q + (sg ? -sd : sd)) * i2p;
      l3 = one - l2;
      if (w_in01(l2)) {
        TE = TB * l2 + TC * l3;
        fBC = w_min(fBC, TE + sqrt_pos((l2 * BCBC + BCCD) * l2 + (l2 * BCCD + CDCD)));
      }
    }
  }
  fBC = w_min(fBC, w_min(TB + sqrt_pos((BCBC + BCCD) + (BCCD + CDCD)), TC + sqrt_pos(CDCD)));
  // face AB
  const R gx = ACAC - ACBC, gy = ACBC - BCBC, gz = ACCD - BCCD;
  p = (TAB * TAB * ACAC - gx * gx) + (BCBC * TAB * TAB - gy * gy) - ((ACBC + ACBC) * TAB * TAB - 2.0f * gx * gy);
  q = -(BCBC * TAB * TAB - gy * gy) * w_make(2.0, R{}) + ((ACBC + ACBC) * TAB * TAB - 2.0f * gx * gy) +
      ((ACCD + ACCD) * TAB * TAB - 2.0f * gx * gz) - ((BCCD + BCCD) * TAB * TAB - 2.0f * gy * gz);
  r = (TAB * TAB * BCBC - gy * gy) + ((BCCD + BCCD) * TAB * TAB - 2.0f * gy * gz) + (TAB * TAB * CDCD - gz * gz);
  delta = q * q - 4.0f * p * r;
  if (w_ge0(delta)) {
    const R sd = w_sqrt(delta), i2p = w_recip(2.0f * p);
    for (int sg = 0; sg < 2; ++sg) {
      l1 = (-q + (sg ? -sd : sd)) * i2p;
      l2 = one - l1;
      if (w_in01(l1)) {
        TE = TA * l1 + TB * l2;
        fAB = w_min(fAB, TE + sqrt_pos((l1 * ACAC + l2 * ACBC + ACCD) * l1 + (l1 * ACBC + l2 * BCBC + BCCD) * l2 +
                                       (l1 * ACCD + l2 * BCCD + CDCD)));
      }
    }
  }
  fAB = w_min(fAB, w_min(TB + sqrt_pos((BCBC + BCCD) + (BCCD + CDCD)), TA + sqrt_pos((ACAC + ACCD) + (ACCD + CDCD))));
  // face AC
  p = ACAC * TAC * TAC - ACAC * ACAC;
  q = (ACCD + ACCD) * TAC * TAC - 2.0f * ACAC * ACCD;
  r = TAC * TAC * CDCD - ACCD * ACCD;
  delta = q * q - 4.0f * p * r;
  if (w_ge0(delta)) {
    const R sd = w_sqrt(delta), i2p = w_recip(2.0f * p);
    for (int sg = 0; sg < 2; ++sg) {
      l1 = (-q + (sg ? -sd : sd)) * i2p;
      l3 = one - l1;
      if (w_in01(l1)) {
        TE = TA * l1 + TC * l3;
        fAC = w_min(fAC, TE + sqrt_pos((l1 * ACAC + ACCD) * l1 + (l1 * ACCD + CDCD)));
      }
    }
  }
  fAC = w_min(fAC, w_min(TA + sqrt_pos((ACAC + ACCD) + (ACCD + CDCD)), TC + sqrt_pos(CDCD)));
  // inside face ABC
  const R s = TAC * ACBC - TBC * ACAC;
  const R t = TAC * BCCD - TBC * ACCD;
  const R h = -(TAC * BCBC - TBC * ACBC);
  p = (TAC * TAC * ACAC - ACAC * ACAC) * h * h + (BCBC * TAC * TAC - ACBC * ACBC) * s * s +
      ((ACBC + ACBC) * TAC * TAC - 2.0f * ACAC * ACBC) * s * h;
  q = (BCBC * TAC * TAC - ACBC * ACBC) * w_make(2.0, R{}) * s * t +
      ((ACBC + ACBC) * TAC * TAC - 2.0f * ACAC * ACBC) * t * h +
      ((ACCD + ACCD) * TAC * TAC - 2.0f * ACAC * ACCD) * h * h +
      ((BCCD + BCCD) * TAC * TAC - 2.0f * ACBC * ACCD) * s * h;
  r = (TAC * TAC * BCBC - ACBC * ACBC) * t * t + ((BCCD + BCCD) * TAC * TAC - 2.0f * ACBC * ACCD) * t * h +
      (TAC * TAC * CDCD - ACCD * ACCD) * h * h;
  delta = q * q - 4.0f * p * r;
  if (w_ge0(delta)) {
    const R sd = w_sqrt(delta), i2p = w_recip(2.0f * p), ih = w_recip(h + eps8);
    for (int sg = 0; sg < 2; ++sg) {
      l1 = (-q + (sg ? -sd : sd)) * i2p;
      l2 = (s * l1 + t) * ih;
      l3 = one - l1 - l2;
      if (w_in01(l1) && w_in01(l2) && w_in01(l3)) {
        TE = TA * l1 + TB * l2 + TC * l3;
        TD = w_min(TD, TE + sqrt_pos((l1 * ACAC + l2 * ACBC + ACCD) * l1 + (l1 * ACBC + l2 * BCBC + BCCD) * l2 +
                                     (l1 * ACCD + l2 * BCCD + CDCD)));
      }
    }
  }
  return w_min(TD, w_min(fBC, w_min(fAB, fAC)));
}
__device__ __forceinline__ double tet_update_f64(double TA, double TB, double TC, double ACAC, double ACBC,
                                                 double ACCD, double BCBC, double BCCD, double CDCD) {
  return tet_update_wide<double>(TA, TB, TC, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD);
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
