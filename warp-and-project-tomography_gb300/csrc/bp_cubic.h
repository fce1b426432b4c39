// The reference's cubics in double, evaluated without the FP64 pipe where the
// result is certain: the backprojection's bicubic weights (WaP_Tomo.cpp:
// 208-222, cubic_cert below) and the flow pyramid's cubic growth (CImg.h:
// 28432-28610, grow_cert at the end).
//
// cubicInterpolate(float p[4], float x) computes, in C's promotion order,
//   p1 + (0.5 x) * ((p2 - p0)_f + x * ((((2 p0 - 5 p1) + 4 p2) - p3)
//                                      + x * ((3 (p1 - p2)_f + p3) - p0)))
// where (.)_f are float subtractions and everything else is double, and the
// caller stores the double result in a float.  This GPU computes FP64 at a
// small fraction of its FP32 rate, so cubic_cert evaluates the same
// expression in float-float arithmetic (an unevaluated sum hi + lo of two
// floats, built from error-free transformations) together with a rigorous
// bound B on its distance from the double evaluation, and returns the float
// nearest to hi + lo only when every value within B of hi + lo rounds to the
// same float.  Then that float is also the rounding of the double result.
// Otherwise (a result near a rounding boundary, heavy cancellation, zero,
// subnormal, huge or non-finite values) it reports failure and the caller
// takes the double path.
//
// The bound.  Each float-float operation below returns its exact result plus
// an error of at most 2^-46 (|a| + |b|) for a sum and 2^-46 |a b| for a
// product of its (already perturbed) operands, barring underflow, whose
// absolute errors (below 2^-149 each) the added term 2^-126 covers.  For an expression tree whose
// operations all err that way, the result differs from the exact value by at
// most ((1 + e)^k - 1) T, where T is the same tree evaluated on the absolute
// values of its inputs and k the number of operations (products count the
// operations of both operands): k <= 16 here, so the float-float value is
// within 2^-41.9 T of the exact value, and the double evaluation (unit
// roundoff 2^-53, same tree) within 2^-48.9 T.  B = 2^-40 T + 2^-126 covers
// both.  T is accumulated with upward rounding.
//
// The functions are __host__ __device__ so that a host harness can compare
// them with the double expression on many inputs; on the device every
// operation is an explicit round-to-nearest intrinsic (no contraction).
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define BPC_HD __host__ __device__ __forceinline__
#else
#define BPC_HD inline
#endif

namespace wap {
namespace bpc {

#if defined(__CUDA_ARCH__)
BPC_HD float add(float a, float b) { return __fadd_rn(a, b); }
BPC_HD float sub(float a, float b) { return __fsub_rn(a, b); }
BPC_HD float mul(float a, float b) { return __fmul_rn(a, b); }
BPC_HD float fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
BPC_HD float add_up(float a, float b) { return __fadd_ru(a, b); }
BPC_HD float mul_up(float a, float b) { return __fmul_ru(a, b); }
BPC_HD float fma_up(float a, float b, float c) { return __fmaf_ru(a, b, c); }
BPC_HD uint32_t bits(float a) { return __float_as_uint(a); }
BPC_HD float from_bits(uint32_t u) { return __uint_as_float(u); }
#else
// Host build (the test harness, -ffp-contract=off): upward-rounded operations
// are replaced by the round-to-nearest result pushed one float up, which is
// never below the upward rounding for the non-negative operands used here.
BPC_HD float add(float a, float b) { return a + b; }
BPC_HD float sub(float a, float b) { return a - b; }
BPC_HD float mul(float a, float b) { return a * b; }
BPC_HD float fma(float a, float b, float c) { return fmaf(a, b, c); }
BPC_HD float add_up(float a, float b) { return nextafterf(a + b, INFINITY); }
BPC_HD float mul_up(float a, float b) { return nextafterf(a * b, INFINITY); }
BPC_HD float fma_up(float a, float b, float c) { return nextafterf(fmaf(a, b, c), INFINITY); }
BPC_HD uint32_t bits(float a) {
  uint32_t u;
  memcpy(&u, &a, 4);
  return u;
}
BPC_HD float from_bits(uint32_t u) {
  float a;
  memcpy(&a, &u, 4);
  return a;
}
#endif

struct FF {
  float h, l;  // value h + l, |l| <= half an ulp of h
};

// s + e = a + b exactly (Knuth's two-sum).
BPC_HD FF two_sum(float a, float b) {
  const float s = add(a, b);
  const float bb = sub(s, a);
  return FF{s, add(sub(a, sub(s, bb)), sub(b, bb))};
}
// s + e = a + b exactly when |a| >= |b| or a == 0 (Dekker's fast two-sum).
BPC_HD FF fast_two_sum(float a, float b) {
  const float s = add(a, b);
  return FF{s, sub(b, sub(s, a))};
}
// p + e = a b exactly (barring underflow).
BPC_HD FF two_prod(float a, float b) {
  const float p = mul(a, b);
  return FF{p, fma(a, b, -p)};
}
// Sums renormalise with two_sum: after cancellation the correction term can
// exceed the leading one, where the fast form would not be exact.
BPC_HD FF ff_add_f(FF a, float b) {
  const FF s = two_sum(a.h, b);
  return two_sum(s.h, add(s.l, a.l));
}
BPC_HD FF ff_add(FF a, FF b) {
  const FF s = two_sum(a.h, b.h);
  return two_sum(s.h, add(s.l, add(a.l, b.l)));
}
// |fma(a.l, b, p.l)| <= 2^-23 |p.h|, so the fast renormalisation is exact.
BPC_HD FF ff_mul_f(FF a, float b) {
  const FF p = two_prod(a.h, b);
  return fast_two_sum(p.h, fma(a.l, b, p.l));
}

// The float that every value within b of v = (h, l) rounds to, if there is
// one: true and *out = h.  Requires h normal, not too small for its half-gap
// to be representable, and |l| + b strictly inside the half-gap on l's side
// (a power of two has the half-size gap below it).
constexpr float kRelBound = 9.094947017729282e-13f;  // 2^-40
constexpr float kAbsBound = 1.1754943508222875e-38f;  // 2^-126

BPC_HD float bound(float t) { return add_up(mul_up(t, kRelBound), kAbsBound); }

BPC_HD bool certain_rounding(FF v, float b, float *out) {
  const uint32_t u = bits(v.h) & 0x7fffffffu;
  const uint32_t e = u & 0x7f800000u;
  if (e < (26u << 23) || e >= 0x7f800000u) return false;  // tiny, zero, subnormal, inf, NaN
  const float half_ulp = from_bits(e - (24u << 23));      // 2^(exponent - 24)
  const float gap = ((u & 0x007fffffu) == 0u) ? mul(half_ulp, 0.5f) : half_ulp;
  const float need = add_up(fabsf(v.l), b);
  if (!(need < gap)) return false;
  *out = v.h;
  return true;
}

// cubicInterpolate of WaP_Tomo.cpp:208-211 by the certified float-float route.
BPC_HD bool cubic_cert(float p0, float p1, float p2, float p3, float x, float *out) {
  const float f1 = sub(p1, p2), f2 = sub(p2, p0);  // the reference's float subtractions
  // inner = (3 f1 + p3) - p0
  FF inner = ff_add_f(ff_add_f(two_prod(3.0f, f1), p3), -p0);
  // mid = (((2 p0 - 5 p1) + 4 p2) - p3) + x inner
  FF mid = ff_add_f(ff_add_f(ff_add_f(two_prod(-5.0f, p1), mul(2.0f, p0)), mul(4.0f, p2)), -p3);
  mid = ff_add(mid, ff_mul_f(inner, x));
  // outer = f2 + x mid; result = p1 + (0.5 x) outer
  const FF outer = ff_add_f(ff_mul_f(mid, x), f2);
  const FF res = ff_add_f(ff_mul_f(outer, mul(0.5f, x)), p1);
  // T: the same tree on absolute values, rounded upward
  const float ax = fabsf(x);
  const float ta = add_up(fma_up(3.0f, fabsf(f1), fabsf(p3)), fabsf(p0));
  float tm = add_up(fma_up(5.0f, fabsf(p1), mul(2.0f, fabsf(p0))), mul(4.0f, fabsf(p2)));
  tm = add_up(add_up(tm, fabsf(p3)), mul_up(ax, ta));
  const float to = fma_up(ax, tm, fabsf(f2));
  const float t = fma_up(mul(0.5f, ax), to, fabsf(p1));
  return certain_rounding(res, bound(t), out);
}

// (float)((double)v + alpha * (double)g), the reference's update of a voxel
// (WaP_Tomo.cpp:1618, alpha a double), certified the same way; alpha is given
// as ah + al with ah = (float)alpha, al = (float)(alpha - ah), so that
// |alpha - (ah + al)| <= 2^-48 |alpha|.
BPC_HD bool update_cert(float v, float g, float ah, float al, float *out) {
  FF p = two_prod(ah, g);
  p = fast_two_sum(p.h, fma(al, g, p.l));
  const FF r = ff_add_f(p, v);
  const float t = fma_up(fabsf(ah), fabsf(g), fabsf(v));
  return certain_rounding(r, bound(t), out);
}

// a * (bh + bl) for a float-float a and a double weight given as the float
// pair bh + bl: the leading product exactly (two_prod), the cross terms with
// one rounding each, a.l * bl (below 2^-48 of the product) dropped.
BPC_HD FF ff_mul_pair(FF a, float bh, float bl) {
  const FF p = two_prod(a.h, bh);
  return fast_two_sum(p.h, fma(a.h, bl, fma(a.l, bh, p.l)));
}

// CImg's cubic growth of an image axis (CImg.h:28432-28610, interpolation
// type 5), which the flow pyramid evaluates in double:
//   val1 + 0.5 (t (-val0 + val2) + t2 (((2 val0 - 5 val1) + 4 val2) - val3)
//               + t3 (((-val0 + 3 val1) - 3 val2) + val3))
// with float samples val0..val3 and the double weights t, t2 = t t and
// t3 = t2 t, each passed as a float pair tp[2q] + tp[2q+1] within 2^-48 of
// it; the caller stores the double result in a float.  Certified as
// cubic_cert is: at most 21 float-float operations (counting the weights'
// representation) put the float-float value within 2^-41.6 T of the exact
// value and the double evaluation's 13 roundings within 2^-49.3 T, so the
// same B = 2^-40 T + 2^-126 covers both.
BPC_HD bool grow_cert(float v0, float v1, float v2, float v3, const float *tp, float *out) {
  const FF A = two_sum(-v0, v2);
  FF B = ff_add_f(ff_add_f(ff_add_f(two_prod(-5.0f, v1), mul(2.0f, v0)), mul(4.0f, v2)), -v3);
  FF C = ff_add(ff_add_f(two_prod(3.0f, v1), -v0), two_prod(-3.0f, v2));
  C = ff_add_f(C, v3);
  FF S = ff_add(ff_mul_pair(A, tp[0], tp[1]), ff_mul_pair(B, tp[2], tp[3]));
  S = ff_add(S, ff_mul_pair(C, tp[4], tp[5]));
  const FF val = ff_add_f(FF{mul(0.5f, S.h), mul(0.5f, S.l)}, v1);
  // T: the same tree on absolute values, rounded upward
  const float a0 = fabsf(v0), a1 = fabsf(v1), a2 = fabsf(v2), a3 = fabsf(v3);
  const float w1 = add_up(fabsf(tp[0]), fabsf(tp[1])), w2 = add_up(fabsf(tp[2]), fabsf(tp[3])),
              w3 = add_up(fabsf(tp[4]), fabsf(tp[5]));
  const float sa = add_up(a0, a2);
  const float sb = add_up(add_up(fma_up(5.0f, a1, mul(2.0f, a0)), mul(4.0f, a2)), a3);
  const float sc = add_up(fma_up(3.0f, a2, fma_up(3.0f, a1, a0)), a3);
  const float ts = fma_up(w3, sc, fma_up(w2, sb, mul_up(w1, sa)));
  const float t = fma_up(0.5f, ts, a1);
  return certain_rounding(val, bound(t), out);
}

}  // namespace bpc
}  // namespace wap
