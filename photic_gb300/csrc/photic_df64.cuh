// photic_df64.cuh -- double-float arithmetic on the FP32 pipes and the
// photic cost written with it.
//
// GB300 executes FP64 at 1/64 of its FP32 rate, so the fast path keeps the
// cost in an unevaluated sum of two floats (hi + lo, about 48 significant
// bits) built from error-free transformations: Knuth's TwoSum, Dekker's
// FastTwoSum and the FMA-based TwoProd (Dekker 1971; Shewchuk 1997).  Every
// product-sum below is written with explicit __fmaf_rn / __fadd_rn /
// __fmul_rn, so the result does not depend on compiler contraction.
//
// Transcendentals (own implementations, from the mathematics):
//   exp: x = k ln2 + j/64 + r with |r| <= 1/128 (three-part ln2 for an exact
//        reduction), exp(j/64) from a double-float table, exp(r) by its
//        Taylor series to r^5 (tail below 1e-16 relative).
//   log: one Newton step y + x exp(-y) - 1 from the float logarithm.
//   sqrt: one Newton step on the float reciprocal square root.
#pragma once
#include <stdint.h>

#include "photic_params.h"

namespace photic {

struct df64 {
  float hi, lo;
};

__device__ __forceinline__ df64 df_make(float hi, float lo) { return df64{hi, lo}; }
__device__ __forceinline__ df64 df_from_float(float a) { return df64{a, 0.0f}; }
// Conversion from double uses the FP64 pipe: set-up only, never per evaluation.
__device__ __forceinline__ df64 df_from_double(double a) {
  float hi = __double2float_rn(a);
  float lo = __double2float_rn(a - (double)hi);
  return df64{hi, lo};
}
__device__ __forceinline__ double df_to_double(df64 a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ df64 fast_two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float e = __fsub_rn(b, __fsub_rn(s, a));
  return df64{s, e};
}
__device__ __forceinline__ df64 two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return df64{s, e};
}
__device__ __forceinline__ df64 two_prod(float a, float b) {
  float p = __fmul_rn(a, b);
  float e = __fmaf_rn(a, b, -p);
  return df64{p, e};
}

__device__ __forceinline__ df64 df_add(df64 a, df64 b) {
  df64 s = two_sum(a.hi, b.hi);
  df64 t = two_sum(a.lo, b.lo);
  s.lo = __fadd_rn(s.lo, t.hi);
  s = fast_two_sum(s.hi, s.lo);
  s.lo = __fadd_rn(s.lo, t.lo);
  return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df64 df_neg(df64 a) { return df64{-a.hi, -a.lo}; }
__device__ __forceinline__ df64 df_sub(df64 a, df64 b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ df64 df_add_f(df64 a, float b) {
  df64 s = two_sum(a.hi, b);
  s.lo = __fadd_rn(s.lo, a.lo);
  return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df64 df_mul(df64 a, df64 b) {
  float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}
__device__ __forceinline__ df64 df_mul_f(df64 a, float b) {
  float p = __fmul_rn(a.hi, b);
  float e = __fmaf_rn(a.hi, b, -p);
  e = __fmaf_rn(a.lo, b, e);
  return fast_two_sum(p, e);
}
// a / b with two correction steps (relative error ~2^-47).
__device__ __forceinline__ df64 df_div(df64 a, df64 b) {
  float r = __frcp_rn(b.hi);
  float q1 = __fmul_rn(a.hi, r);
  df64 p = df_mul_f(b, q1);
  df64 s = df_sub(a, p);
  float q2 = __fmul_rn(s.hi, r);
  p = df_mul_f(b, q2);
  s = df_sub(s, p);
  float q3 = __fmul_rn(s.hi, r);
  df64 q = fast_two_sum(q1, q2);
  return df_add_f(q, q3);
}
__device__ __forceinline__ df64 df_div_f(df64 a, float b) {
  float r = __frcp_rn(b);
  float q1 = __fmul_rn(a.hi, r);
  df64 p = two_prod(q1, b);
  df64 s = df_sub(a, p);
  float q2 = __fmul_rn(s.hi, r);
  p = two_prod(q2, b);
  s = df_sub(s, p);
  float q3 = __fmul_rn(s.hi, r);
  df64 q = fast_two_sum(q1, q2);
  return df_add_f(q, q3);
}
__device__ __forceinline__ df64 df_sqrt(df64 a) {
  if (a.hi <= 0.0f) return df64{0.0f, 0.0f};
  float x = rsqrtf(a.hi);
  float y = __fmul_rn(a.hi, x);
  df64 yy = two_prod(y, y);
  df64 d = df_sub(a, yy);
  float c = __fmul_rn(__fmul_rn(d.hi, x), 0.5f);
  return fast_two_sum(y, c);
}
__device__ __forceinline__ df64 df_abs(df64 a) { return a.hi < 0.0f ? df_neg(a) : a; }

__device__ __forceinline__ bool df_lt(df64 a, df64 b) {
  return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
}
__device__ __forceinline__ bool df_le(df64 a, df64 b) {
  return a.hi < b.hi || (a.hi == b.hi && a.lo <= b.lo);
}

// exp of a double-float.  Arguments below -87 flush to 0 (the cost only
// exponentiates non-positive numbers; exp(-87) is far below any weight).
__device__ __forceinline__ df64 df_exp(df64 a, const float *Thi, const float *Tlo) {
  if (a.hi < -87.0f) return df64{0.0f, 0.0f};
  if (a.hi > 87.0f) return df64{__int_as_float(0x7f800000), 0.0f};
  // ln2 = L0 + L1 + L2; L0 has 15 significant bits, so k * L0 is exact
  // for |k| < 512.
  const float L0 = 0.693145751953125f, L1 = 1.42860677e-06f, L2 = 5.49560397e-14f;
  float k = rintf(__fmul_rn(a.hi, 1.44269504f));
  df64 r = two_sum(a.hi, -__fmul_rn(k, L0));
  r.lo = __fadd_rn(r.lo, a.lo);
  r = fast_two_sum(r.hi, r.lo);
  r = df_sub(r, two_prod(k, L1));
  r = df_add_f(r, -__fmul_rn(k, L2));
  float j = rintf(__fmul_rn(r.hi, 64.0f));
  r = df_add_f(r, -__fmul_rn(j, 0.015625f));  // j/64 exact
  // exp(r) = 1 + r + r^2/2 + r^3/6 + r^4/24 + r^5/120, |r| <= 1/128
  df64 r2 = df_mul(r, r);
  df64 r3 = df_mul(r2, r);
  float rf = r.hi;
  float tail = __fmul_rn(__fmul_rn(r2.hi, r2.hi),
                         __fmaf_rn(rf, 0.00833333377f, 0.0416666679f));
  const df64 sixth = df64{0.166666672f, -4.96705303e-09f};
  df64 p = df_add_f(r, 1.0f);
  p = df_add(p, df64{__fmul_rn(r2.hi, 0.5f), __fmul_rn(r2.lo, 0.5f)});
  p = df_add(p, df_mul(r3, sixth));
  p = df_add_f(p, tail);
  int ji = (int)j + 32;
  p = df_mul(p, df64{Thi[ji], Tlo[ji]});
  int ki = (int)k;
  float s = __int_as_float((ki + 127) << 23);  // 2^k, |k| <= 126 here
  return df64{__fmul_rn(p.hi, s), __fmul_rn(p.lo, s)};
}

__device__ __forceinline__ df64 df_log(df64 a, const float *Thi, const float *Tlo) {
  float y0 = logf(a.hi);
  df64 e = df_exp(df64{-y0, 0.0f}, Thi, Tlo);
  df64 t = df_mul(a, e);
  t = df_add_f(t, -1.0f);
  return df_add_f(t, y0);
}

// (long)(10 * y) with the x86-64 result for NaN / out of range, for y >= 0
// or y < 0 alike (truncation towards zero of hi + lo).
__device__ __forceinline__ long long df_trunc10(df64 y) {
  df64 v = df_mul_f(y, 10.0f);
  if (!(fabsf(v.hi) < 9.2233720e18f)) return (long long)(-9223372036854775807LL - 1);
  float t = truncf(v.hi);
  long long r = (long long)t;
  if (t == v.hi) {
    if (v.hi > 0.0f && v.lo < 0.0f) r -= 1;
    else if (v.hi < 0.0f && v.lo > 0.0f) r += 1;
  }
  return r;
}

}  // namespace photic
