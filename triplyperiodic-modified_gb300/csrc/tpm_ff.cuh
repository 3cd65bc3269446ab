// Float-float ("double-float") arithmetic for the mixed path's Poisson
// refinement.  A value is the unevaluated sum hi + lo of two floats (x, y of a
// float2).  GB300 issues FP64 at 1/58 of its FP32 rate, so the refinement's
// residual is summed here, on the FP32 pipe, at about 2^-46 relative
// precision instead of FP64's 2^-53.
//
// Methods: Knuth's TwoSum (TAOCP vol. 2, 4.2.2, theorem B), Dekker's
// FastTwoSum and the FMA form of his exact product (T. J. Dekker, "A
// floating-point technique for extending the available precision", Numer.
// Math. 18, 1971).  These error-free transformations need every add rounded
// to nearest and kept in program order: the kernels that use them are built
// without fast-math and with --fmad=false (no contraction besides the
// explicit fmaf below).
#pragma once

#include <cuda_runtime.h>

namespace tpm {

// s + e == a + b exactly (TwoSum, 6 adds)
__device__ __forceinline__ float2 ff_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  const float e = (a - (s - bb)) + (b - bb);
  return make_float2(s, e);
}

// s + e == a + b exactly when |a| >= |b| or a == 0 (FastTwoSum, 3 adds)
__device__ __forceinline__ float2 ff_fast_two_sum(float a, float b) {
  const float s = a + b;
  return make_float2(s, b - (s - a));
}

// a + b for a pair a and a pair b that need not be normalised; the error is
// within 2^-46 (|a| + |b|), which is what a residual summed from terms of
// both signs needs (the "sloppy" add: one TwoSum on the high parts)
__device__ __forceinline__ float2 ff_add(float2 a, float2 b) {
  const float2 s = ff_two_sum(a.x, b.x);
  return ff_fast_two_sum(s.x, s.y + (a.y + b.y));
}

// a - b to within 2^-46 |a - b| (both pairs' parts through TwoSum: the
// difference of two close sums keeps its relative precision)
__device__ __forceinline__ float2 ff_sub(float2 a, float2 b) {
  float2 s = ff_two_sum(a.x, -b.x);
  const float2 t = ff_two_sum(a.y, -b.y);
  s = ff_fast_two_sum(s.x, s.y + t.x);
  return ff_fast_two_sum(s.x, s.y + t.y);
}

// a - b within 2^-46 (|a| + |b|) (one TwoSum on the high parts: for pairs
// whose difference need not keep its own relative precision)
__device__ __forceinline__ float2 ff_sub_sloppy(float2 a, float2 b) {
  const float2 s = ff_two_sum(a.x, -b.x);
  return make_float2(s.x, s.y + (a.y - b.y));
}

// a + b for a pair a and a float b, within 2^-46 (|a| + |b|)
__device__ __forceinline__ float2 ff_add_f(float2 a, float b) {
  const float2 s = ff_two_sum(a.x, b);
  return ff_fast_two_sum(s.x, s.y + a.y);
}

// a * b, unnormalised: a.x b.x exactly (FMA) plus the other three partial
// products, within 2^-45 |a b| for pairs from ff_from_double (|lo| < 2^-23
// |hi|: the roundings of the cross terms).  a.y b.y is kept: for truncated
// splits the low parts carry the sign of their values, so dropping it would
// bias every product by up to 2^-46.
__device__ __forceinline__ float2 ff_mul(float2 a, float2 b) {
  const float p = a.x * b.x;
  float e = fmaf(a.y, b.y, fmaf(a.x, b.x, -p));
  e = fmaf(a.x, b.y, e);
  e = fmaf(a.y, b.x, e);
  return make_float2(p, e);
}

// A double as a pair with |x - (hi + lo)| <= 2^-48 |x| for 2^-74 <= |x| <
// 2^128, by integer operations on its bits only (conversion instructions
// issue on the FP64 pipe, and a branch around them is if-converted into
// evaluating them for every value): hi is x truncated to 24 significant
// bits, lo the remaining 29 bits rounded to 24.  Below 2^-74 lo is dropped
// (an error under 2^-97), below 2^-126 x flushes to a signed zero; from 2^128
// on hi is an infinity of x's sign (nan for nan) and lo zero.
__device__ __forceinline__ float2 ff_from_double(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned int hw = (unsigned int)(b >> 32), lw = (unsigned int)b;
  const int e = (int)((hw >> 20) & 0x7ffu);  // biased binary exponent
  const unsigned int sgn = hw & 0x80000000u;
  // float exponent e - 1023 + 127, the 20 high and 3 next significand bits
  const unsigned int mant = ((hw & 0xfffffu) << 3) | (lw >> 29);
  unsigned int hb = sgn | ((unsigned int)(e - 896) << 23) | mant;
  hb = e < 897 ? sgn : hb;
  hb = e > 1150 ? (sgn | 0x7f800000u | ((e == 2047 && ((hw & 0xfffffu) | lw)) ? 0x400000u : 0u))
                : hb;
  // the low 29 significand bits are worth t * 2^(e - 1075), and 2^(e - 1075)
  // is the float with biased exponent e - 948 (>= 1 in range)
  const float t = __uint2float_rn(lw & 0x1fffffffu);
  const bool lo_ok = e >= 949 && e <= 1150;
  const float scale = __uint_as_float(lo_ok ? ((unsigned int)(e - 948) << 23) : 0u);
  const float lo = t * scale;
  return make_float2(__uint_as_float(hb), __uint_as_float(__float_as_uint(lo) | sgn));
}

// x truncated to a float (within 2^-23 |x|; below 2^-126 a signed zero, from
// 2^128 on an infinity of x's sign, nan for nan) by integer operations only:
// the FP32 copy of an FP64 value without an FP64-pipe conversion
__device__ __forceinline__ float ff_hi(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned int hw = (unsigned int)(b >> 32), lw = (unsigned int)b;
  const int e = (int)((hw >> 20) & 0x7ffu);
  const unsigned int sgn = hw & 0x80000000u;
  unsigned int hb = sgn | ((unsigned int)(e - 896) << 23) | ((hw & 0xfffffu) << 3) | (lw >> 29);
  hb = e < 897 ? sgn : hb;
  hb = e > 1150 ? (sgn | 0x7f800000u | ((e == 2047 && ((hw & 0xfffffu) | lw)) ? 0x400000u : 0u))
                : hb;
  return __uint_as_float(hb);
}

// A float as a double, exactly, by integer operations only; subnormal floats
// (below 2^-126) flush to a signed zero.
__device__ __forceinline__ double ff_f2d(float f) {
  const unsigned int u = __float_as_uint(f);
  const unsigned int ef = (u >> 23) & 0xffu;
  const unsigned long long sgn = (unsigned long long)(u & 0x80000000u) << 32;
  const unsigned long long ed = ef == 0xffu ? 0x7ffull : (unsigned long long)(ef + 896u);
  const unsigned long long bits = sgn | (ed << 52) | ((unsigned long long)(u & 0x7fffffu) << 29);
  return __longlong_as_double((long long)(ef == 0u ? sgn : bits));
}

// u = ip + fr with ip = trunc(u) (toward zero) and fr = u - ip truncated to a
// float, and up = (|fr| >= 1/2) decided on the exact bits; by integer
// operations only (the FP64 route is a truncating conversion, a conversion
// back and a subtraction, all on the FP64 pipe).  For |u| < 2^31; beyond,
// ip saturates and fr is 0.
__device__ __forceinline__ void ff_int_frac(double u, int &ip, float &fr, bool &up) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(u);
  const bool neg = (b >> 63) != 0;
  const int e = (int)((b >> 52) & 0x7ffu) - 1023;  // |u| in [2^e, 2^(e+1))
  const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  // e >= 0: integer part m >> (52 - e), fraction bits fb worth fb * 2^-(52 - e)
  const int sh = 52 - (e < 0 ? 0 : (e > 30 ? 30 : e));
  const unsigned long long fb = m & ((1ull << sh) - 1ull);
  const int lz = __clzll((long long)(fb | 1ull));
  const unsigned long long nb = (fb << lz) << 1;  // fraction bits after the leading one
  const unsigned int fbits =
      fb ? (((unsigned int)(63 - lz - sh + 127) << 23) | (unsigned int)(nb >> 41)) : 0u;
  int ia = (int)(m >> sh);
  float fa = __uint_as_float(fbits);
  bool half = ((fb >> (sh - 1)) & 1ull) != 0;
  if (e < 0) {  // |u| < 1: no integer part, the fraction is |u|
    ia = 0;
    fa = __uint_as_float(__float_as_uint(ff_hi(u)) & 0x7fffffffu);
    half = e == -1;
  }
  if (e > 30) {
    ia = 0x7fffffff;
    fa = 0.f;
    half = false;
  }
  ip = neg ? -ia : ia;
  fr = neg ? -fa : fa;
  up = half;
}

// u = ip + fr with ip = trunc(u) and the fraction fr = u - ip as a
// normalised pair, by integer operations only.  The fraction's bits split at
// bit 29 into two integers that convert to floats: the high part exactly, the
// low part rounded to 24 bits, so |fr - (u - ip)| <= 2^(e - 48) for
// 2^e <= |u| < 2^(e + 1) (2^-41 for |u| < 256), and exactly ff_from_double(u)
// for |u| < 1.  For |u| < 2^31; beyond, ip saturates and fr is 0.
__device__ __forceinline__ void ff_int_frac2(double u, int &ip, float2 &fr) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(u);
  const bool neg = (b >> 63) != 0;
  const int e = (int)((b >> 52) & 0x7ffu) - 1023;
  const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  const int sh = 52 - (e < 0 ? 0 : (e > 30 ? 30 : e));  // fraction = fb 2^-sh
  const unsigned long long fb = m & ((1ull << sh) - 1ull);
  // fb = fh 2^29 + fl: fh < 2^23 converts exactly, and fh 2^(29 - sh) > fl 2^-sh
  // whenever fh > 0, so FastTwoSum normalises the pair
  const float hi = __uint2float_rn((unsigned int)(fb >> 29)) *
                   __uint_as_float((unsigned int)(127 + 29 - sh) << 23);
  const float lo = __uint2float_rn((unsigned int)(fb & 0x1fffffffull)) *
                   __uint_as_float((unsigned int)(127 - sh) << 23);
  float2 f = ff_fast_two_sum(hi, lo);
  int ia = (int)(m >> sh);
  if (e < 0) {  // |u| < 1: no integer part, the fraction is |u|
    ia = 0;
    f = ff_from_double(__longlong_as_double((long long)(b & 0x7fffffffffffffffull)));
  }
  if (e > 30) {
    ia = 0x7fffffff;
    f = make_float2(0.f, 0.f);
  }
  ip = neg ? -ia : ia;
  fr = neg ? make_float2(-f.x, -f.y) : f;
}

// hi + lo as a double (two exact conversions and one FP64 addition)
__device__ __forceinline__ double ff_to_double(float2 a) { return ff_f2d(a.x) + ff_f2d(a.y); }

// double -> T and back for code templated on its compute type: for float by
// integer operations (truncation down, exact up), for double the identity
template <typename T>
__device__ __forceinline__ T ff_cast(double x) { return (T)x; }
template <>
__device__ __forceinline__ float ff_cast<float>(double x) { return ff_hi(x); }
__device__ __forceinline__ double ff_widen(double x) { return x; }
__device__ __forceinline__ double ff_widen(float x) { return ff_f2d(x); }

// a normalised so that |lo| <= ulp(hi) / 2 (for pairs whose lo is already
// small against hi, as ff_mul leaves them)
__device__ __forceinline__ float2 ff_norm(float2 a) { return ff_fast_two_sum(a.x, a.y); }

// 1/h for a pair h with |lo| <= 2^-23 |hi| and hi a normal float, within
// 2^-45 |1/h|, on the FP32 pipe.  y = 1/hi rounded; 1 - hi y is exact as one
// FMA for a correctly rounded reciprocal, and e = 1 - h y follows with the
// low part; then 1/h = y / (1 - e) = y (1 + e + e^2) up to e^3 (|e| < 2^-22).
__device__ __forceinline__ float2 ff_rcp(float2 h) {
  const float y = __frcp_rn(h.x);
  const float r = fmaf(-h.x, y, 1.0f);
  const float e = fmaf(-h.y, y, r);
  return ff_fast_two_sum(y, y * fmaf(e, e, e));
}

}  // namespace tpm
