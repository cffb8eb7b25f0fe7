// Pairs of floats (hi + lo, about 48 significant bits) for the few alpha
// solves whose entropy difference FP32 cannot resolve to the tolerance.
// Error-free transformations: Knuth's TwoSum, and TwoProd through one fused
// multiply-add (Dekker's product without the splitting).  Every operation is
// spelled with the _rn intrinsics so that the compiler neither contracts nor
// reorders them.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace elbm {

struct df {
  float hi, lo;
};

__device__ __forceinline__ df df_make(float a) { return df{a, 0.f}; }

__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return df{s, e};
}

__device__ __forceinline__ df fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return df{s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ df df_add(df x, df y) {
  const df s = two_sum(x.hi, y.hi);
  const df t = two_sum(x.lo, y.lo);
  df r = fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
  return fast_two_sum(r.hi, __fadd_rn(r.lo, t.lo));
}

__device__ __forceinline__ df df_neg(df x) { return df{-x.hi, -x.lo}; }

__device__ __forceinline__ df df_mul(df x, df y) {
  const float p = __fmul_rn(x.hi, y.hi);
  float e = __fmaf_rn(x.hi, y.hi, -p);
  e = __fmaf_rn(x.hi, y.lo, __fmaf_rn(x.lo, y.hi, e));
  return fast_two_sum(p, e);
}

__device__ __forceinline__ df df_mul_f(df x, float b) {
  const float p = __fmul_rn(x.hi, b);
  const float e = __fmaf_rn(x.lo, b, __fmaf_rn(x.hi, b, -p));
  return fast_two_sum(p, e);
}

// x / y: a float quotient, then two corrections from the exact residual.
__device__ __forceinline__ df df_div(df x, df y) {
  const float q1 = __fdiv_rn(x.hi, y.hi);
  df r = df_add(x, df_neg(df_mul_f(y, q1)));
  const float q2 = __fdiv_rn(r.hi, y.hi);
  r = df_add(r, df_neg(df_mul_f(y, q2)));
  const float q3 = __fdiv_rn(r.hi, y.hi);
  const df q = fast_two_sum(q1, q2);
  return df_add(q, df_make(q3));
}

// ln(1 + x) for 1 + x > 0.  With 1 + x = m 2^e, m in [sqrt(1/2), sqrt(2)),
// s = (m - 1)/(m + 1) (|s| <= 0.1716) and ln m = 2 s A(s^2),
// A(z) = 1 + z/3 + z^2/5 + z^3/7 + z^4 T(z) (the series of atanh(s)/s);
// the first four coefficients are pairs, the tail T (z^4 <= 7.6e-7) is a
// plain FP32 Horner sum.
__device__ __forceinline__ df df_log1p(df x) {
  const df v = df_add(df_make(1.0f), x);
  int e = (int)((__float_as_uint(v.hi) >> 23) & 0xffu) - 127;
  float scale = __uint_as_float((uint32_t)(127 - e) << 23);
  df m = df{__fmul_rn(v.hi, scale), __fmul_rn(v.lo, scale)};
  if (m.hi > 1.41421356f) {
    e += 1;
    m.hi = __fmul_rn(m.hi, 0.5f);
    m.lo = __fmul_rn(m.lo, 0.5f);
  }
  const df num = fast_two_sum(__fsub_rn(m.hi, 1.0f), m.lo);  // m.hi - 1 is exact (Sterbenz)
  const df den = df_add(df_make(1.0f), m);
  const df s = df_div(num, den);
  const df z = df_mul(s, s);
  // tail T(z) = 1/9 + z/11 + z^2/13 + ... to FP32 rounding (z <= 0.0295)
  float t = 1.0f / 23.0f;
#pragma unroll
  for (int k = 10; k >= 4; --k) t = __fmaf_rn(t, z.hi, 1.0f / (2 * k + 1));
  constexpr double c3 = 1.0 / 3.0, c5 = 1.0 / 5.0, c7 = 1.0 / 7.0;
  const df C3{(float)c3, (float)(c3 - (double)(float)c3)};
  const df C5{(float)c5, (float)(c5 - (double)(float)c5)};
  const df C7{(float)c7, (float)(c7 - (double)(float)c7)};
  df A = df_add(C7, df_mul_f(z, t));
  A = df_add(C5, df_mul(z, A));
  A = df_add(C3, df_mul(z, A));
  A = df_add(df_make(1.0f), df_mul(z, A));
  const df lnm = df_mul(df_mul_f(s, 2.0f), A);
  constexpr double ln2 = 0.693147180559945309417232121458;
  const df LN2{(float)ln2, (float)(ln2 - (double)(float)ln2)};
  return df_add(df_mul_f(LN2, (float)e), lnm);
}

}  // namespace elbm
