// df64.h -- double-float arithmetic: a value is hi + lo with two FP32 words
// (|lo| <= ulp(hi)/2), about 48 significant bits.  Error-free transforms
// (Knuth TwoSum, FMA-based TwoProd; Dekker 1971, Hida/Li/Bailey "QD" 2001)
// on the FP32 pipes, which on GB300 issue 64x the FP64 rate.
//
// Device code uses the _rn intrinsics so the compiler can neither contract
// nor reorder the compensated sequences; the host build (the CPU check of
// the same element math) must be compiled with -ffp-contract=off.
#pragma once

#include <cmath>

#ifdef __CUDACC__
#define DF_HD __host__ __device__ __forceinline__
#else
#define DF_HD inline
#endif

namespace nalu_gb300 {

struct df64 {
  float hi, lo;
};

#ifdef __CUDA_ARCH__
DF_HD float f_add(float a, float b) { return __fadd_rn(a, b); }
DF_HD float f_sub(float a, float b) { return __fsub_rn(a, b); }
DF_HD float f_mul(float a, float b) { return __fmul_rn(a, b); }
DF_HD float f_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
#else
DF_HD float f_add(float a, float b) { return a + b; }
DF_HD float f_sub(float a, float b) { return a - b; }
DF_HD float f_mul(float a, float b) { return a * b; }
DF_HD float f_fma(float a, float b, float c) { return std::fma(a, b, c); }
#endif

// s + e = a + b exactly
DF_HD df64 two_sum(float a, float b) {
  const float s = f_add(a, b);
  const float bb = f_sub(s, a);
  const float e = f_add(f_sub(a, f_sub(s, bb)), f_sub(b, bb));
  return {s, e};
}
// requires |a| >= |b| (or a == 0)
DF_HD df64 quick_two_sum(float a, float b) {
  const float s = f_add(a, b);
  return {s, f_sub(b, f_sub(s, a))};
}

DF_HD df64 df_from_double(double x) {
  const float hi = (float)x;
  const float lo = (float)(x - (double)hi);
  return {hi, lo};
}
DF_HD double df_to_double(df64 a) { return (double)a.hi + (double)a.lo; }
DF_HD df64 df_zero() { return {0.0f, 0.0f}; }

DF_HD df64 df_neg(df64 a) { return {-a.hi, -a.lo}; }

DF_HD df64 df_add(df64 a, df64 b) {
  df64 s = two_sum(a.hi, b.hi);
  s.lo = f_add(s.lo, f_add(a.lo, b.lo));
  return quick_two_sum(s.hi, s.lo);
}
DF_HD df64 df_sub(df64 a, df64 b) { return df_add(a, df_neg(b)); }

DF_HD df64 df_mul(df64 a, df64 b) {
  const float p = f_mul(a.hi, b.hi);
  float e = f_fma(a.hi, b.hi, -p);
  e = f_fma(a.hi, b.lo, e);
  e = f_fma(a.lo, b.hi, e);
  return quick_two_sum(p, e);
}
// a * c with c a float constant
DF_HD df64 df_mul_f(df64 a, float c) {
  const float p = f_mul(a.hi, c);
  float e = f_fma(a.hi, c, -p);
  e = f_fma(a.lo, c, e);
  return quick_two_sum(p, e);
}
// a * c with c a power of two (exact)
DF_HD df64 df_scale2(df64 a, float c) { return {f_mul(a.hi, c), f_mul(a.lo, c)}; }

// a * b + c
DF_HD df64 df_fma(df64 a, df64 b, df64 c) {
  const float p = f_mul(a.hi, b.hi);
  float e = f_fma(a.hi, b.hi, -p);
  e = f_fma(a.hi, b.lo, e);
  e = f_fma(a.lo, b.hi, e);
  df64 s = two_sum(p, c.hi);
  s.lo = f_add(s.lo, f_add(e, c.lo));
  return quick_two_sum(s.hi, s.lo);
}

// a * b - c * d
DF_HD df64 df_cross(df64 a, df64 b, df64 c, df64 d) { return df_sub(df_mul(a, b), df_mul(c, d)); }

// 1 / a: FP32 reciprocal refined by one Newton step in df64
DF_HD df64 df_rcp(df64 a) {
  const float x0 = 1.0f / a.hi;
  // r = 1 - a * x0  (in df64), then x = x0 + x0 * r
  const df64 ax = df_mul_f(a, x0);
  const df64 r = df_sub(df64{1.0f, 0.0f}, ax);
  const df64 corr = df_mul_f(r, x0);
  return df_add(df64{x0, 0.0f}, corr);
}

DF_HD bool df_gt(df64 a, double b) { return df_to_double(a) > b; }

}  // namespace nalu_gb300
