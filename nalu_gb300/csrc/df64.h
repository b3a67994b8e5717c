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
#include <cstdint>
#include <cstring>

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

// ---- conversions by integer bit manipulation (no FP64 instructions) ----
#ifdef __CUDA_ARCH__
DF_HD uint64_t d2u(double d) { return (uint64_t)__double_as_longlong(d); }
DF_HD double u2d(uint64_t u) { return __longlong_as_double((long long)u); }
DF_HD uint32_t f2u(float f) { return __float_as_uint(f); }
DF_HD float u2f(uint32_t u) { return __uint_as_float(u); }
DF_HD int clz32(uint32_t v) { return __clz(v); }
#else
DF_HD uint64_t d2u(double d) { uint64_t u; std::memcpy(&u, &d, 8); return u; }
DF_HD double u2d(uint64_t u) { double d; std::memcpy(&d, &u, 8); return d; }
DF_HD uint32_t f2u(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
DF_HD float u2f(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
DF_HD int clz32(uint32_t v) { return v ? __builtin_clz(v) : 32; }
#endif

#ifdef __CUDA_ARCH__
DF_HD double hilo2d(uint32_t hi, uint32_t lo) { return __hiloint2double((int)hi, (int)lo); }
#else
DF_HD double hilo2d(uint32_t hi, uint32_t lo) { return u2d(((uint64_t)hi << 32) | lo); }
#endif

// Exact widening of f * 2^k to a double, built in the two 32-bit halves of
// the result: sign, exponent rebased by 1023 - 127 + k, the 23 significand
// bits shifted into place.  Normal floats; zero and float subnormals
// (|f| < 2^-126) map to zero.  |k| <= 800 keeps every normal float's
// exponent inside the FP64 range (the element math uses |k| <= 124).
DF_HD double f2d_bits(float f, int k = 0) {
  const uint32_t u = f2u(f);
  const uint32_t e = (u >> 23) & 0xffu;
  const uint32_t hi = (u & 0x80000000u) | ((e + (uint32_t)(896 + k)) << 20) | ((u >> 3) & 0xfffffu);
  return e == 0 ? 0.0 : hilo2d(hi, u << 29);
}

// (hi + lo) * 2^k as a double: both widen exactly and their sum (<= 48
// significant bits) is exact in FP64, so one FP64 add is the only FP64
// instruction.  The power-of-two factor undoes an exact scaling of the
// inputs (per-element coordinate normalisation) at no cost.
DF_HD double df_to_double_bits(df64 a, int k = 0) { return f2d_bits(a.hi, k) + f2d_bits(a.lo, k); }

// 2^k as a float, k in [-126, 127]
DF_HD float pow2f(int k) { return u2f((uint32_t)(k + 127) << 23); }
// unbiased binary exponent of a double (-1023 for zero and subnormals)
DF_HD int dexp(double d) { return (int)((d2u(d) >> 52) & 0x7ff) - 1023; }

// Split d * 2^-k into hi (nearest float) + lo (the remaining significand
// bits, truncated to 24) with integer instructions only (the scaling is an
// exponent shift, exact).  |d| 2^-k must lie in [2^-100, 2^127); smaller
// magnitudes return 0 (below anything the element math sees relative to its
// inputs), which keeps lo a normal float.
DF_HD df64 df_split_bits(double d, int k = 0) {
  const uint64_t b = d2u(d);
  const int e = (int)((b >> 52) & 0x7ff);
  const int E = e - 1023 - k;
  if (e == 0 || E < -100) return {0.0f, 0.0f};
  const uint32_t sgn = (uint32_t)(b >> 32) & 0x80000000u;
  const uint64_t sig = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);  // 53 bits
  uint32_t hs = (uint32_t)(sig >> 29);                              // top 24 bits
  int32_t rem = (int32_t)(sig & ((1ull << 29) - 1));                // low 29 bits
  if (rem >= (1 << 28)) {                                           // round hi to nearest
    hs += 1;
    rem -= (1 << 29);
  }
  int Eh = E;
  if (hs == (1u << 24)) {
    hs >>= 1;
    Eh += 1;
  }
  const float hi = u2f(sgn | ((uint32_t)(Eh + 127) << 23) | (hs & 0x7fffffu));
  float lo = 0.0f;
  if (rem != 0) {
    const uint32_t lsgn = rem < 0 ? (sgn ^ 0x80000000u) : sgn;
    const uint32_t ar = (uint32_t)(rem < 0 ? -rem : rem);
    const int msb = 31 - clz32(ar);
    const uint32_t mant = msb > 23 ? (ar >> (msb - 23)) : (ar << (23 - msb));
    const int el = msb + E - 52 + 127;
    if (el > 0) lo = u2f(lsgn | ((uint32_t)el << 23) | (mant & 0x7fffffu));
  }
  return {hi, lo};
}
DF_HD df64 df_zero() { return {0.0f, 0.0f}; }

DF_HD df64 df_neg(df64 a) { return {-a.hi, -a.lo}; }

DF_HD df64 df_add(df64 a, df64 b) {
  df64 s = two_sum(a.hi, b.hi);
  s.lo = f_add(s.lo, f_add(a.lo, b.lo));
  return quick_two_sum(s.hi, s.lo);
}
DF_HD df64 df_sub(df64 a, df64 b) { return df_add(a, df_neg(b)); }

// a + b as an unnormalised pair (TwoSum of the leading parts, the low parts
// added in FP32, no renormalisation: 8 operations instead of 11), for inputs
// of products that take unnormalised pairs (df_cross, df_mul)
DF_HD df64 df_add_lazy(df64 a, df64 b) {
  const df64 s = two_sum(a.hi, b.hi);
  return {s.hi, f_add(s.lo, f_add(a.lo, b.lo))};
}

// a + b + c as an unnormalised pair: two TwoSums of the leading parts, the
// low parts and the TwoSum errors added in FP32 (16 operations instead of
// two df_add, 22).  The pair's hi + lo is the sum to about 2^-47 (|a| + |b|
// + |c|); widening hi and lo to FP64 separately and adding them (as
// df_to_double_bits does) renormalises it.
DF_HD df64 df_sum3_lazy(df64 a, df64 b, df64 c) {
  const df64 s = two_sum(a.hi, b.hi);
  const df64 t = two_sum(s.hi, c.hi);
  return {t.hi, f_add(f_add(s.lo, t.lo), f_add(f_add(a.lo, b.lo), c.lo))};
}

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

// df_split_bits for an input field value.  Magnitudes of 2^127 and above,
// infinities and NaN (df_split_in_range false) take the float conversion
// instead (the nearest float, inf past FLT_MAX, or NaN) rather than a wrapped
// exponent; the per-node passes that call it flag such inputs, since the
// widening back to FP64 (f2d_bits) does not carry inf or NaN.  Magnitudes
// below 2^-100 become zero, as in df_split_bits.
DF_HD bool df_split_in_range(double d) { return (int)((d2u(d) >> 52) & 0x7ff) < 1023 + 127; }
DF_HD df64 df_split_input(double d) {
  if (!df_split_in_range(d)) return {(float)d, 0.0f};
  return df_split_bits(d);
}

// The nodal input of the df64 continuity kernels, rho u + tau gp, as a
// normalised pair with no FP64 instruction: the inputs split by integer
// operations (df_split_input, ~2^-48 relative), then two double-float
// products and a sum (at most ~2^-45.9 of |rho u| + |tau gp| against FP64 on
// random inputs).  An FP64 product, sum and conversion take 6 FP64-pipe
// instructions per component, which made the per-node pass FP64-bound on
// GB300.
DF_HD df64 df_nodal_w(df64 rho, double u, df64 tau, double gp) {
  return df_add(df_mul(rho, df_split_input(u)), df_mul(tau, df_split_input(gp)));
}

// a + b + c + d: three TwoSums of the leading parts, the low parts and the
// TwoSum errors added in FP32, one renormalisation (27 operations instead of
// three df_add, 33)
DF_HD df64 df_sum4(df64 a, df64 b, df64 c, df64 d) {
  const df64 s = two_sum(a.hi, b.hi);
  const df64 t = two_sum(s.hi, c.hi);
  const df64 u = two_sum(t.hi, d.hi);
  const float lo = f_add(f_add(f_add(s.lo, t.lo), u.lo), f_add(f_add(a.lo, b.lo), f_add(c.lo, d.lo)));
  return quick_two_sum(u.hi, lo);
}

// a0 b0 + a1 b1 + a2 b2: three FMA-based TwoProds, their leading parts
// summed by two TwoSums, every error term added in FP32, one renormalisation
// (31 FP32 operations instead of df_mul + 2 df_fma, 37)
DF_HD df64 df_dot3(df64 a0, df64 b0, df64 a1, df64 b1, df64 a2, df64 b2) {
  const float p0 = f_mul(a0.hi, b0.hi), p1 = f_mul(a1.hi, b1.hi), p2 = f_mul(a2.hi, b2.hi);
  float e0 = f_fma(a0.hi, b0.hi, -p0);
  e0 = f_fma(a0.hi, b0.lo, e0);
  e0 = f_fma(a0.lo, b0.hi, e0);
  float e1 = f_fma(a1.hi, b1.hi, -p1);
  e1 = f_fma(a1.hi, b1.lo, e1);
  e1 = f_fma(a1.lo, b1.hi, e1);
  float e2 = f_fma(a2.hi, b2.hi, -p2);
  e2 = f_fma(a2.hi, b2.lo, e2);
  e2 = f_fma(a2.lo, b2.hi, e2);
  const df64 s = two_sum(p0, p1);
  const df64 t = two_sum(s.hi, p2);
  return quick_two_sum(t.hi, f_add(f_add(s.lo, t.lo), f_add(f_add(e0, e1), e2)));
}

// a * b - c * d: both products with FMA error terms, one TwoSum of the
// leading parts, one renormalisation (19 FP32 operations instead of 25)
DF_HD df64 df_cross(df64 a, df64 b, df64 c, df64 d) {
  const float p = f_mul(a.hi, b.hi);
  float e = f_fma(a.hi, b.hi, -p);
  e = f_fma(a.hi, b.lo, e);
  e = f_fma(a.lo, b.hi, e);
  const float q = f_mul(c.hi, d.hi);
  float g = f_fma(c.hi, d.hi, -q);
  g = f_fma(c.hi, d.lo, g);
  g = f_fma(c.lo, d.hi, g);
  df64 s = two_sum(p, -q);
  s.lo = f_add(s.lo, f_sub(e, g));
  return quick_two_sum(s.hi, s.lo);
}

// a * b - c * d as an unnormalised pair (df_cross without its final
// renormalisation: 16 operations), for products that take unnormalised pairs
DF_HD df64 df_cross_lazy(df64 a, df64 b, df64 c, df64 d) {
  const float p = f_mul(a.hi, b.hi);
  float e = f_fma(a.hi, b.hi, -p);
  e = f_fma(a.hi, b.lo, e);
  e = f_fma(a.lo, b.hi, e);
  const float q = f_mul(c.hi, d.hi);
  float g = f_fma(c.hi, d.hi, -q);
  g = f_fma(c.hi, d.lo, g);
  g = f_fma(c.lo, d.hi, g);
  const df64 s = two_sum(p, -q);
  return {s.hi, f_add(s.lo, f_sub(e, g))};
}
// a * b + c as an unnormalised pair (df_fma without its final
// renormalisation: 12 operations), for accumulations whose result is only
// added to or widened to FP64
DF_HD df64 df_fma_lazy(df64 a, df64 b, df64 c) {
  const float p = f_mul(a.hi, b.hi);
  float e = f_fma(a.hi, b.hi, -p);
  e = f_fma(a.hi, b.lo, e);
  e = f_fma(a.lo, b.hi, e);
  const df64 s = two_sum(p, c.hi);
  return {s.hi, f_add(s.lo, f_add(e, c.lo))};
}
// a * b as an unnormalised pair (df_mul without its final renormalisation)
DF_HD df64 df_mul_lazy(df64 a, df64 b) {
  const float p = f_mul(a.hi, b.hi);
  float e = f_fma(a.hi, b.hi, -p);
  e = f_fma(a.hi, b.lo, e);
  e = f_fma(a.lo, b.hi, e);
  return {p, e};
}

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
