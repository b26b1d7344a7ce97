// dfloat.cuh -- double-float arithmetic (an unevaluated sum hi + lo of two
// FP32 numbers, ~48 significant bits) for kernels whose FP64 work would
// otherwise be bound by GB300's FP64 rate, a small fraction of its FP32 rate.
//
// Building blocks (Dekker 1971, Knuth TAOCP vol. 2 4.2.2): two_sum and
// fast_two_sum give a + b exactly as a double-float, two_prod gives a * b
// exactly with one fused multiply-add.  All operations use the _rn
// intrinsics, so the compiler neither contracts nor reorders them.
//
// df_exp_neg: e^y for y <= 0 by Tang's table-driven method (P. T. P. Tang,
// "Table-driven implementation of the exponential function in IEEE
// floating-point arithmetic", ACM TOMS 15(2), 1989): y = (64 m + j) ln2/64 + r,
// |r| <= ln2/128, e^y = 2^m 2^(j/64) e^r, with 2^(j/64) from a 64-entry
// double-float table and e^r from its Taylor series.  ln2/64 is split
// Cody-Waite style into C1 (11 significant bits, so k * C1 is exact for
// |k| < 2^13) + C2 + C3.  Relative error below 5e-14 + |y| 4e-15 (the
// double-float y itself carries ~48 bits) for y >= -70; below
// that the low word turns subnormal (FP32-level accuracy down to -87), and 0
// is returned below -87 (the FP32 range ends there): the caller handles sums
// made of such terms.
#pragma once

#include <cstdint>

namespace centre {

struct dfl {
  float hi, lo;
};

__device__ __forceinline__ dfl df_make(float hi, float lo) {
  dfl r;
  r.hi = hi;
  r.lo = lo;
  return r;
}

// exact a + b (any magnitudes)
__device__ __forceinline__ dfl two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return df_make(s, e);
}

// exact a + b for |a| >= |b|
__device__ __forceinline__ dfl fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return df_make(s, __fsub_rn(b, __fsub_rn(s, a)));
}

// exact a * b
__device__ __forceinline__ dfl two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return df_make(p, __fmaf_rn(a, b, -p));
}

__device__ __forceinline__ dfl df_add(dfl x, dfl y) {
  const dfl s = two_sum(x.hi, y.hi);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo)));
}

__device__ __forceinline__ dfl df_mul(dfl x, dfl y) {
  const dfl p = two_prod(x.hi, y.hi);
  return fast_two_sum(p.hi, __fmaf_rn(x.hi, y.lo, __fmaf_rn(x.lo, y.hi, p.lo)));
}

__device__ __forceinline__ dfl df_mul_f(dfl x, float f) {
  const dfl p = two_prod(x.hi, f);
  return fast_two_sum(p.hi, __fmaf_rn(x.lo, f, p.lo));
}

__host__ __device__ __forceinline__ double df_value(float hi, float lo) {
  return (double)hi + (double)lo;
}

__device__ __forceinline__ dfl df_from_double(double x) {
  const float hi = __double2float_rn(x);
  return df_make(hi, __double2float_rn(x - (double)hi));
}

// 2^(j/64), j = 0..63, as double-floats: tab[2j] = hi, tab[2j+1] = lo
// (filled on the host from exp2 in double precision).
constexpr int kDfExpTable = 64;

__device__ __forceinline__ dfl df_exp_neg(dfl y, const float *__restrict__ tab) {
  if (!(y.hi >= -87.0f)) return df_make(0.0f, 0.0f);
  // k = round(y * 64 / ln2)
  const float kf = rintf(__fmul_rn(y.hi, 92.332481384277344f));
  const int k = (int)kf;
  const int j = k & 63;
  const int m = k >> 6;                      // floor(k / 64): k = 64 m + j
  // r = y - k ln2/64, ln2/64 = C1 + C2 + C3
  const float C1 = 0x1.62cp-7f, C2 = 0x1.217f7ep-18f, C3 = -0x1.c611p-43f;
  const float r1 = __fmaf_rn(-kf, C1, y.hi);         // exact
  dfl r = two_sum(r1, y.lo);
  r = df_add(r, two_prod(-kf, C2));
  r = fast_two_sum(r.hi, __fmaf_rn(-kf, C3, r.lo));
  // e^r = 1 + r + r^2/2 + r^3 (1/6 + r/24 + r^2/120), |r| <= ln2/128
  const dfl r2 = df_mul(r, r);
  const float t = __fmul_rn(__fmul_rn(r.hi, r2.hi),
                            __fmaf_rn(r.hi, __fmaf_rn(r.hi, 1.0f / 120.0f, 1.0f / 24.0f),
                                      1.0f / 6.0f));
  dfl s = df_add(r, df_make(__fmul_rn(r2.hi, 0.5f), __fmul_rn(r2.lo, 0.5f)));
  s = fast_two_sum(s.hi, __fadd_rn(s.lo, t));
  const dfl e = df_add(df_make(1.0f, 0.0f), s);
  dfl res = df_mul(df_make(tab[2 * j], tab[2 * j + 1]), e);
  // times 2^m (m >= -126 here: 2^m is a normal float)
  const float scale = __int_as_float((127 + m) << 23);
  res.hi = __fmul_rn(res.hi, scale);
  res.lo = __fmul_rn(res.lo, scale);
  return res;
}

}  // namespace centre
