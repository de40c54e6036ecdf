// Float-float arithmetic: a value as the unevaluated sum hi + lo of two
// floats (about 48 significant bits), with the error-free transformations of
// Knuth (TwoSum), Dekker (Fast2Sum) and the fused multiply-add (TwoProd).
//
// The kernels whose result must be the reference's float64 expression rounded
// to float32 (integration's signed distance, fusion's running mean) evaluate
// the expression in float-float instead of float64: GB300's float64 rate is
// about 1/64 of its float32 rate, and those kernels were bound by it.  The
// float-float value differs from the reference's double by far less than the
// bound `tol` each caller states (a few float64 roundings plus the
// float-float error), so rounding it to float gives the reference's float
// unless the value lies within `tol` of a rounding boundary (the midpoint of
// two neighbouring floats).  round_checked reports that case, and the caller
// then evaluates the reference's float64 expression itself.
//
// Every operation is spelled with its rounding (__fadd_rn, __fmul_rn,
// __fmaf_rn) so that no compiler contraction changes the transformations.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

struct FF {
  float hi, lo;
};

// s + e == a + b exactly, s = fl(a + b)
__device__ __forceinline__ FF ff_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

// the same when |a| >= |b| (or a == 0)
__device__ __forceinline__ FF ff_fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

// p + e == a * b exactly (barring underflow)
__device__ __forceinline__ FF ff_two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return {p, __fmaf_rn(a, b, -p)};
}

// a double as a float pair: hi = (float)d, lo = (float)(d - hi); hi + lo
// equals d to within 2^-48 of |d|
__device__ __forceinline__ FF ff_from_double(double d) {
  const float hi = __double2float_rn(d);
  return {hi, __double2float_rn(d - (double)hi)};
}

__host__ __forceinline__ void ff_split_host(double d, float &hi, float &lo) {
  hi = (float)d;
  lo = (float)(d - (double)hi);
}

// a + b with an error of a few 2^-48 of |a| + |b| (the accurate sum of two
// float-float values)
__device__ __forceinline__ FF ff_add(FF a, FF b) {
  const FF s = ff_two_sum(a.hi, b.hi);
  const FF t = ff_two_sum(a.lo, b.lo);
  const FF v = ff_fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
  return ff_fast_two_sum(v.hi, __fadd_rn(t.lo, v.lo));
}

// a + b with an error of a few 2^-48 of |a| + |b| too, in fewer operations:
// the low parts are summed in one rounding (the bound is relative to the
// operands' magnitudes, not to the sum's, which is what the callers' bounds
// need)
__device__ __forceinline__ FF ff_add_short(FF a, FF b) {
  const FF s = ff_two_sum(a.hi, b.hi);
  return ff_fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ FF ff_neg(FF a) { return {-a.hi, -a.lo}; }

// Float nearest to hi + lo (round to nearest even).  ambiguous is set when a
// value within tol of hi + lo could round to another float -- a rounding
// boundary lies within tol -- or when the result is zero or not finite.
__device__ __forceinline__ float ff_round_checked(FF v, float tol, bool &ambiguous) {
  const FF r = ff_fast_two_sum(v.hi, v.lo);  // r.hi = fl(hi + lo), hi + lo = r.hi + r.lo
  const float f = r.hi;
  const float a = fabsf(f);
  if (!(a > 0.f) || !isfinite(a)) {
    ambiguous = true;
    return f;
  }
  // spacings to the neighbouring floats below and above |f| (they differ at
  // powers of two); the boundaries are half of them away
  const float down = __fsub_rn(a, __int_as_float(__float_as_int(a) - 1));
  const float up = __fsub_rn(__int_as_float(__float_as_int(a) + 1), a);
  const float e = fabsf(r.lo);
  ambiguous = fabsf(__fsub_rn(e, __fmul_rn(0.5f, down))) <= tol || fabsf(__fsub_rn(e, __fmul_rn(0.5f, up))) <= tol ||
              tol >= __fmul_rn(0.25f, down);  // spacings too fine for the bound
  return f;
}

// FUSE_BY_MERGE's running mean (w1 * d1 + w2 * d2) / (w1 + w2) (SDF.cpp:
// 212-236) rounded to float, as the reference's float64 expression rounds
// it: the products are exact in float64 and in float-float, the sum and the
// quotient round once each in float64 (2^-53) and to about 2^-47 here, so
// `tol` is 2^-38 of the terms' magnitude.  False (out unset) when the
// float-float result cannot decide -- weights of 2^24 or more, values not
// finite, a rounding boundary within tol -- and the caller evaluates the
// float64 expression.
__device__ __forceinline__ bool ff_merge_mean(int32_t w1, float d1, int32_t w2, float d2, float &out) {
  if (w1 <= 0 || w2 <= 0 || w1 >= (1 << 23) || w2 >= (1 << 23) || !isfinite(d1) || !isfinite(d2)) return false;
  const float a = (float)w1, b = (float)w2, den = (float)(w1 + w2);  // exact below 2^24
  const FF p1 = ff_two_prod(a, d1), p2 = ff_two_prod(b, d2);
  const FF p = ff_add(p1, p2);
  const float q1 = __fdiv_rn(p.hi, den);
  // p.hi - q1 * den is exact for a correctly rounded q1
  const float rem = __fadd_rn(__fmaf_rn(-q1, den, p.hi), p.lo);
  const FF q = ff_fast_two_sum(q1, __fdiv_rn(rem, den));
  const float tol = __fmul_rn(__fdiv_rn(__fadd_rn(fabsf(p1.hi), fabsf(p2.hi)), den), 0x1p-38f);
  bool ambiguous;
  const float r = ff_round_checked(q, tol, ambiguous);
  if (ambiguous) return false;
  out = r;
  return true;
}
