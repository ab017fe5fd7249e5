// Float-float ("double-single") arithmetic on the FP32 pipes.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi),
// about 48 significant bits. GB300 runs FP32 FMA 73x faster than FP64 FMA
// (36.6 vs 0.50 T instructions/s measured), so stencils that need FP64-class
// accuracy are evaluated in this arithmetic instead of native FP64.
// Algorithms: Knuth's TwoSum, Dekker's Fast2Sum, and the FMA-based exact
// product (error-free transformations), combined as in the classic
// double-word arithmetic of Dekker (1971); the sum is the cheap variant whose
// error is relative to the larger operand, which is what these stencils
// need (their terms are summed, never divided by a small difference).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ns {

struct ff {
  float hi, lo;
};

__device__ __forceinline__ ff ff_make(float h, float l) { ff r; r.hi = h; r.lo = l; return r; }

__device__ __forceinline__ ff fast2sum(float a, float b) {  // requires |a| >= |b|
  const float s = a + b;
  return ff_make(s, b - (s - a));
}

__device__ __forceinline__ ff two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return ff_make(s, (a - (s - bb)) + (b - bb));
}

__device__ __forceinline__ ff operator+(ff x, ff y) {
  ff s = two_sum(x.hi, y.hi);
  return fast2sum(s.hi, s.lo + (x.lo + y.lo));
}
__device__ __forceinline__ ff operator-(ff x) { return ff_make(-x.hi, -x.lo); }
__device__ __forceinline__ ff operator-(ff x, ff y) { return x + (-y); }

__device__ __forceinline__ ff operator*(ff x, ff y) {
  const float p = x.hi * y.hi;
  float e = fmaf(x.hi, y.hi, -p);
  e = fmaf(x.hi, y.lo, e);
  e = fmaf(x.lo, y.hi, e);
  return fast2sum(p, e);
}

// product with a float (exact float inputs such as 0.125, 2, 3 stay exact in hi)
__device__ __forceinline__ ff operator*(float c, ff x) {
  const float p = x.hi * c;
  float e = fmaf(x.hi, c, -p);
  e = fmaf(x.lo, c, e);
  return fast2sum(p, e);
}

// multiplication by a power of two: exact
__device__ __forceinline__ ff ff_scale2(ff x, float pow2) { return ff_make(x.hi * pow2, x.lo * pow2); }

__device__ __forceinline__ ff ff_add_f(ff x, float y) {
  ff s = two_sum(x.hi, y);
  return fast2sum(s.hi, s.lo + x.lo);
}

__device__ __forceinline__ ff ff_abs(ff x) { return x.hi < 0.f ? -x : x; }

// Split an FP64 value into hi + lo with integer operations only (no FP64
// instruction): hi keeps the leading 24 bits of the significand (truncated),
// lo the next 24 (rounded). Values outside the normal float range fall back to
// a plain conversion.
__device__ __forceinline__ ff ff_from_double(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  if ((b << 1) == 0ull) return ff_make(0.f, 0.f);
  const int e = (int)((b >> 52) & 0x7ff);
  const int fe = e - 1023 + 127;
  if (fe <= 24 || fe >= 255) return ff_make((float)x, 0.f);
  const unsigned sign = (unsigned)(b >> 63) << 31;
  const unsigned long long m = (b & 0xfffffffffffffull) | (1ull << 52);
  const unsigned hm = (unsigned)(m >> 29);
  const float hi = __uint_as_float(sign | ((unsigned)fe << 23) | (hm & 0x7fffffu));
  const unsigned lm = (unsigned)(m & 0x1fffffffu);  // 29 bits
  // lo = lm * 2^(e - 1075): lm as a float, exponent shifted by (e - 1075)
  float lo = __uint2float_rn(lm);
  const int sh = e - 1075;  // in [-1074, 971]; normal range checked above keeps lo >= 2^-126 or 0
  lo = ldexpf(lo, sh);
  return ff_make(hi, sign ? -lo : lo);
}

__device__ __forceinline__ double ff_to_double(ff x) { return (double)x.hi + (double)x.lo; }

}  // namespace ns
