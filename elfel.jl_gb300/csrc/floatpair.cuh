// Float-pair ("double-float") arithmetic for FP64-bound kernels.
//
// GB300 executes FP64 at 1/64 of its FP32 rate (measured 1.26 vs 78.5
// TFLOP/s), so element kernels whose results must carry ~1e-14 relative
// accuracy can run their arithmetic on the FP32 pipe as unevaluated sums
// hi + lo of two floats (48 significant bits).  The algorithms are the
// published error-free transformations:
//   two_sum        Knuth, TAOCP vol. 2, 4.2.2 (Møller 1965)
//   quick_two_sum  Dekker 1971 (|a| >= |b|)
//   two_prod       the FMA form of Dekker's exact product
//   add / mul / div  the double-double algorithms of Hida, Li and Bailey's
//                  QD library (2001), on float pairs as in Thall (2006),
//                  "Extended-precision floating-point numbers for GPU
//                  computation"
// Every operation is an explicit round-to-nearest intrinsic, so the compiler
// can neither contract nor reassociate them.
//
// Conversions from and to double use integer operations on the IEEE bit
// patterns (no FP64 instruction): split_scaled() keeps 47 of the 53 bits of a
// double, join_scaled() rebuilds the double with one FP64 add.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace elfel {

struct f2 {
  float hi, lo;
};

__device__ __forceinline__ f2 quick_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ f2 two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}

__device__ __forceinline__ f2 two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return {p, __fmaf_rn(a, b, -p)};
}

// a + b keeping only the error of the leading terms (QD's "sloppy" addition):
// accurate when a and b have the same sign, as for sums of squares.
__device__ __forceinline__ f2 f2_add_same_sign(f2 a, f2 b) {
  const f2 s = two_sum(a.hi, b.hi);
  return quick_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

// a + b with both error terms kept (the accurate QD addition).
__device__ __forceinline__ f2 f2_add(f2 a, f2 b) {
  f2 s = two_sum(a.hi, b.hi);
  const f2 t = two_sum(a.lo, b.lo);
  s = quick_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
  return quick_two_sum(s.hi, __fadd_rn(s.lo, t.lo));
}

__device__ __forceinline__ f2 f2_neg(f2 a) { return {-a.hi, -a.lo}; }

__device__ __forceinline__ f2 f2_sub(f2 a, f2 b) { return f2_add(a, f2_neg(b)); }

__device__ __forceinline__ f2 f2_mul(f2 a, f2 b) {
  f2 p = two_prod(a.hi, b.hi);
  p.lo = __fmaf_rn(a.hi, b.lo, p.lo);
  p.lo = __fmaf_rn(a.lo, b.hi, p.lo);
  return quick_two_sum(p.hi, p.lo);
}

__device__ __forceinline__ f2 f2_mul_f(f2 a, float b) {
  f2 p = two_prod(a.hi, b);
  p.lo = __fmaf_rn(a.lo, b, p.lo);
  return quick_two_sum(p.hi, p.lo);
}

// a / b: three quotient terms, each from the remainder of the previous ones
// (QD's accurate division).  The terms need not be correctly rounded -- each
// remainder is formed exactly enough to correct the previous term -- so they
// use one approximate reciprocal of b.hi (b.hi nonzero and finite).
__device__ __forceinline__ f2 f2_div(f2 a, f2 b) {
  const float rb = __fdividef(1.0f, b.hi);
  const float q1 = __fmul_rn(a.hi, rb);
  f2 r = f2_sub(a, f2_mul_f(b, q1));
  const float q2 = __fmul_rn(r.hi, rb);
  r = f2_sub(r, f2_mul_f(b, q2));
  const float q3 = __fmul_rn(r.hi, rb);
  return quick_two_sum(q1, __fadd_rn(q2, q3));  // |q2 + q3| is far below ulp(q1)
}

// Biased exponent field of a double.
__device__ __forceinline__ int dexp(double x) { return (int)((__double_as_longlong(x) >> 52) & 0x7ff); }

// x * 2^-k as a float pair with the leading 47 bits of x's significand: hi
// takes the top 24, lo the next 23 (both truncated; relative error < 2^-46).
// lo is formed without an int-to-float conversion: 2^23 + i has the bit
// pattern 0x4b000000 | i, and subtracting 2^23 from it is exact.  Returns
// false (and zero) when x * 2^-k is outside [2^-68, 2^127] in magnitude and
// not zero.
// The zero test masks the sign with an explicit integer and.b64: written in
// C++ it is recognised as the comparison x == 0.0 and issued on the FP64 pipe.
__device__ __forceinline__ long long and_b64(long long a, long long m) {
  long long r;
  asm("and.b64 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(m));
  return r;
}

__device__ __forceinline__ bool split_scaled(double x, int k, f2* out) {
  const long long b = __double_as_longlong(x);
  *out = {0.0f, 0.0f};
  if (and_b64(b, 0x7fffffffffffffffLL) == 0) return true;
  const int ex = (int)((b >> 52) & 0x7ff) - k;  // biased exponent of x * 2^-k
  if (ex < 955 || ex > 1150) return false;
  const unsigned sign = (unsigned)((unsigned long long)b >> 63) << 31;
  const float hi = __uint_as_float(sign | ((unsigned)(ex - 896) << 23) | (unsigned)((b >> 29) & 0x7fffff));
  const unsigned i = (unsigned)(b >> 6) & 0x7fffff;                 // significand bits 28..6
  const float m = __fsub_rn(__uint_as_float(0x4b000000u | i), 8388608.0f);  // = i, exactly
  // lo = i * 2^(ex - 1023 - 46), the power of two as a normal float
  const float lo = __uint_as_float(__float_as_uint(__fmul_rn(m, __uint_as_float((unsigned)(ex - 942) << 23))) | sign);
  *out = quick_two_sum(hi, lo);
  return true;
}

// A float (normal or zero) times 2^e as a double, built from its bits.
__device__ __forceinline__ double f2d_bits(float f, int e) {
  const unsigned b = __float_as_uint(f);
  const unsigned ef = (b >> 23) & 0xff;
  if (ef == 0) return 0.0;
  const unsigned long long d = ((unsigned long long)(b >> 31) << 63) |
                               ((unsigned long long)(ef + 896 + e) << 52) |
                               ((unsigned long long)(b & 0x7fffff) << 29);
  return __longlong_as_double((long long)d);
}

// (v.hi + v.lo) * 2^e rounded once to double.  The caller keeps e and the
// magnitudes such that every exponent stays in the normal double range.
__device__ __forceinline__ double join_scaled(f2 v, int e) {
  return __dadd_rn(f2d_bits(v.hi, e), f2d_bits(v.lo, e));
}


}  // namespace elfel
