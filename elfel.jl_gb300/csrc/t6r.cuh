// The exact-rational T6 heat record (straight-sided elements, quadrature
// rules exact for the gradient products): the 21 stored K entries of an
// element are b0..b6 (its 7 K bases), -4 or -8 times b1, b3, b4, or zero.
// Shared by the integration kernels, which write records or bases, and the
// tile reduction, which expands bases; both use t6r_scale, so the values
// agree bit for bit.
#pragma once
#include <stdint.h>

namespace elfel {

// The exact-rational T6 record is determined by 8 base values: the stored K
// entries k0..k5, k9 (= k14 = k20) and the load at the midside nodes; every
// other entry is one of them times -4 or -8, or zero (t6r_expand).
// t6r_scale: code 0: b; 1: -4 b; 2: -8 b; 3: +0, by integer operations only:
// normal values are scaled exactly by an exponent add; a result above the
// double range is the infinity of its sign, infinities and NaNs keep their
// exponent, and subnormal values (below 2^-1022, negligible next to any entry
// of an element record) become zero of their sign.
// The sign flip is an explicit integer XOR: written as an XOR in C++ it is
// recognised as a floating-point negation and issued on the FP64 pipe.
__device__ __forceinline__ long long t6r_xor(long long a, long long m) {
  long long r;
  asm("xor.b64 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(m));
  return r;
}

__device__ __forceinline__ double t6r_scale(double b, int code) {
  const long long bits = t6r_xor(__double_as_longlong(b), (long long)(1ull << 63));  // -b
  const long long sign = bits & (long long)(1ull << 63);
  const int ex = (int)((bits >> 52) & 0x7ff);
  const int m = code == 1 ? 2 : 3;
  long long r = bits + ((long long)m << 52);
  r = ex == 0 ? sign : r;                                                        // zero or subnormal
  r = ex == 0x7ff ? bits : r;                                                    // inf, NaN
  r = (ex != 0 && ex != 0x7ff && ex + m > 2046) ? (sign | 0x7ff0000000000000LL) : r;  // overflow
  const double scaled = __longlong_as_double(r);
  return code == 0 ? b : (code == 3 ? 0.0 : scaled);
}

// t6r_scale(b, 1) and t6r_scale(b, 2) from one decode of b (the same bits).
__device__ __forceinline__ void t6r_scale48(double b, double* m4, double* m8) {
  const long long bits = t6r_xor(__double_as_longlong(b), (long long)(1ull << 63));  // -b
  const long long sign = bits & (long long)(1ull << 63);
  const int ex = (int)((bits >> 52) & 0x7ff);
  const bool zero = ex == 0, special = ex == 0x7ff;
  const long long inf = sign | 0x7ff0000000000000LL;
  long long r4 = bits + (2LL << 52), r8 = bits + (3LL << 52);
  r4 = zero ? sign : (special ? bits : (ex + 2 > 2046 ? inf : r4));
  r8 = zero ? sign : (special ? bits : (ex + 3 > 2046 ? inf : r8));
  *m4 = __longlong_as_double(r4);
  *m8 = __longlong_as_double(r8);
}

// Value table of one element for the tile reduction, entry j at v[j * ld]:
// b0..b6, +0, -4 b1, -4 b3, -4 b4, -8 b1, -8 b3, -8 b4.
constexpr int kT6RTable = 14;
// Stored K entry k (0..20, column-packed upper triangle) -> its table index.
constexpr uint8_t kT6REntry[21] = {0, 1, 2, 3, 4, 5, 8, 8, 7, 6, 7, 10, 10, 12, 6, 9, 7, 9, 13, 11, 6};

// kT6REntry[s] in device code: 4-bit fields of two packed words.
__device__ __forceinline__ int t6r_entry(int s) {
  return s < 16 ? (int)((0x96caa76788543210ull >> (4 * s)) & 15u) : (int)((0x6bd97u >> (4 * (s - 16))) & 15u);
}

__device__ __forceinline__ void t6r_table(const double* b, double* v, int ld = 1) {
#pragma unroll
  for (int k = 0; k < 7; ++k) v[k * ld] = b[k];
  v[7 * ld] = 0.0;
  t6r_scale48(b[1], v + 8 * ld, v + 11 * ld);
  t6r_scale48(b[3], v + 9 * ld, v + 12 * ld);
  t6r_scale48(b[4], v + 10 * ld, v + 13 * ld);
}

}  // namespace elfel
