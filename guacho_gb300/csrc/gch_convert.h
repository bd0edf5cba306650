// gch_convert.h -- FP64 <-> FP32 conversions on the integer pipes.
//
// On GB300 a conversion between FP64 and FP32 issues to the FP64 pipe, which
// runs at 1/57 of the FP32 rate, and the FP32 paths that keep u in FP64
// convert every value they load or store.  These functions produce the same
// bits with a handful of integer operations on the two 32-bit halves:
//
//   d2f_rn(x)  round to nearest, ties to even.  |x| in [2^-126, 2^128)
//              (every value a physical state holds) takes the fast path;
//              a rounding carry out of the largest binade gives infinity,
//              as IEEE 754 does.  Outside that range: |x| >= 2^128 or
//              infinity -> signed infinity; NaN -> NaN; |x| < 2^-126 ->
//              signed zero (the FP32 units of these paths flush subnormals).
//   f2d(x)     exact.  Normal numbers and zero take the fast path;
//              infinity and NaN map to themselves; subnormal inputs, which
//              flush-to-zero FP32 arithmetic never produces, become zero.
//   ge_pos(x, lo)  x >= lo for a positive finite floor lo (below).
//
// The fast path of d2f_rn rounds with a single 64-bit add: the 29 mantissa
// bits that FP32 drops are added to 2^28 - 1 plus the lowest kept bit, so the
// sum carries into the kept bits exactly when the dropped part is above one
// half ulp, or equal to it with an odd kept part (Knuth, TAOCP vol. 2,
// 4.2.1; the same bit-level round-to-nearest-even that softfloat libraries
// use).  A carry out of the mantissa increments the exponent field.
//
// Plain C++ as well, so that host tests check them against the C casts.
#pragma once

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define GCH_HD __host__ __device__ __forceinline__
#else
#define GCH_HD inline
#endif

namespace gch {

GCH_HD uint64_t bits_of(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t b;
  memcpy(&b, &x, sizeof(b));
  return b;
#endif
}
GCH_HD uint32_t bits_of(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  uint32_t b;
  memcpy(&b, &x, sizeof(b));
  return b;
#endif
}
GCH_HD float float_of(uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(b);
#else
  float f;
  memcpy(&f, &b, sizeof(f));
  return f;
#endif
}
GCH_HD double double_of(uint32_t hi, uint32_t lo) {
#if defined(__CUDA_ARCH__)
  return __hiloint2double((int)hi, (int)lo);
#else
  const uint64_t b = ((uint64_t)hi << 32) | lo;
  double d;
  memcpy(&d, &b, sizeof(d));
  return d;
#endif
}

// FP64 exponent fields of 2^-126 and 2^128, in the high word
constexpr uint32_t kD2fLoHi = 897u << 20;
constexpr uint32_t kD2fHiHi = 1151u << 20;

// double -> float, round to nearest even
GCH_HD float d2f_rn(double x) {
  const uint64_t b = bits_of(x);
  const uint32_t hi = (uint32_t)(b >> 32);
  const uint32_t ahi = hi & 0x7FFFFFFFu;
  const uint32_t sign = hi ^ ahi;
  if (ahi - kD2fLoHi < kD2fHiHi - kD2fLoHi) {
    const uint64_t a = b & 0x7FFFFFFFFFFFFFFFull;
    const uint64_t r = a + (0x0FFFFFFFull + ((a >> 29) & 1u));
    // exponent field rebased from 1023 to 127: (e - 896) << 23
    return float_of(sign | ((uint32_t)(r >> 29) - (896u << 23)));
  }
  if (ahi < kD2fLoHi) return float_of(sign);
  // |x| >= 2^128: infinity, or NaN when the fraction is not zero.  Tested
  // on the two 32-bit halves: the same test on the 64-bit pattern was
  // compiled as an FP64 unordered comparison, an FP64-pipe instruction on
  // every zero input (which takes this path too).
  const bool nan = ahi > 0x7FF00000u || (ahi == 0x7FF00000u && (uint32_t)b != 0u);
  return float_of(sign | (nan ? 0x7FC00000u : 0x7F800000u));
}

// float -> double, exact
GCH_HD double f2d(float x) {
  const uint32_t b = bits_of(x);
  const uint32_t a = b & 0x7FFFFFFFu;
  const uint32_t sign = b ^ a;
  if (a - 0x00800000u < 0x7F800000u - 0x00800000u)
    // exponent field rebased from 127 to 1023: + 896 << 20
    return double_of(sign | ((a >> 3) + (896u << 20)), b << 29);
  if (a < 0x00800000u) return double_of(sign, 0u);
  return double_of(sign | 0x7FF00000u | ((a & 0x7FFFFFu) >> 3), b << 29);
}

// x >= lo for a positive finite lo, false for NaN, on the integer pipes.
// Non-negative doubles order as their bit patterns (IEEE 754 totalOrder);
// as unsigned patterns, NaNs with the sign bit clear lie above +infinity and
// every value with the sign bit set (negatives, -0, negative NaNs) above
// those.  So x >= lo exactly when bits(x) - bits(lo) wraps to no more than
// bits(+inf) - bits(lo).  `ge_pos(x, lo) ? x : lo` is then tmax_(x, lo)
// (x > lo ? x : lo) bit for bit: equal operands have equal bits.
GCH_HD bool ge_pos(double x, double lo) {
  const uint64_t l = bits_of(lo);
  return bits_of(x) - l <= 0x7FF0000000000000ull - l;
}

}  // namespace gch
