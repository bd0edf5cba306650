// gch_ddiv.h -- correctly rounded FP64 division on the integer and FP32 pipes.
//
// An IEEE FP64 divide costs about ten FP64-pipe operations, and the FP64
// pipe of GB300 runs at 1/57 of the FP32 rate, while the integer and FP32
// pipes of the FP64 stage kernels stay mostly idle.  ddiv_rn(a, b) returns
// the same bits as a / b (round to nearest, ties to even) with 64-bit
// integer arithmetic and three FP32 digit estimates:
//
//   a = X 2^(ea-1075), b = Y 2^(eb-1075) with X, Y in [2^52, 2^53).
//   Q = floor(X 2^55 / Y) in [2^54, 2^56) is built as three digits of 19, 18
//   and 18 bits, schoolbook division with estimated digits (Knuth, TAOCP
//   vol. 2, 4.3.1): each digit is the partial remainder R times a correctly
//   rounded FP32 reciprocal of Y, rounded to an integer, and R <- R 2^s - q Y.
//   R is exact in 64-bit two's complement: its true value stays below Y in
//   magnitude, so the arithmetic modulo 2^64 loses nothing.
//
//   Digit error: the reciprocal of the top 29 bits of Y is within 2^-22.9
//   relative, the top 40 bits of R are within 2^-24, and one FP32 product
//   adds 2^-24, so |q - R 2^s / Y| <= 1/2 + |R/Y| 2^(s-22) + 2^-9.  Starting
//   from |R/Y| < 2 the remainder bound is 0.752 Y after the 19-bit digit and
//   0.549 Y, 0.537 Y after the 18-bit ones, so one step (R < 0: Q - 1,
//   R + Y) makes Q the floor quotient and R its remainder.
//
//   Rounding: Q has 56 bits (X >= Y) or 55 bits; the 53 kept bits are
//   followed by 3 or 2 dropped bits, and R != 0 is the sticky bit.
//
// The fast path takes normal a and b whose quotient exponent is normal
// before rounding (a carry out of the largest binade gives infinity, as
// IEEE 754 does).  A zero over a normal number gives the signed zero
// directly.  Other zeros, subnormals, infinities, NaNs and quotients near
// the ends of the exponent range go to the hardware division.  The same code
// runs on the host (FP32 reciprocal by IEEE division, which rounds like
// __frcp_rn), so host tests check the digits the device computes.
#pragma once

#include <stdint.h>

#include "gch_convert.h"

namespace gch {

GCH_HD float rcp_rn(float x) {
#if defined(__CUDA_ARCH__)
  return __frcp_rn(x);
#else
  return 1.0f / x;
#endif
}
GCH_HD int32_t f2i_rn(float x) {
#if defined(__CUDA_ARCH__)
  return __float2int_rn(x);
#else
  // round half to even, as the device conversion (|x| < 2^22 here)
  const float f = (float)(int32_t)x;  // truncated
  const float d = x - f;              // exact, |d| < 1
  int32_t i = (int32_t)f;
  if (d > 0.5f || (d == 0.5f && (i & 1))) ++i;
  if (d < -0.5f || (d == -0.5f && (i & 1))) --i;
  return i;
#endif
}

// one schoolbook digit of s bits: q ~ R 2^s / Y, R <- R 2^s - q Y, Q <- Q 2^s + q
GCH_HD void ddiv_digit(int64_t& R, int64_t& Q, int64_t Y, float rs, int s) {
  const float rf = (float)(int32_t)(R >> 24);   // |R| < 2^54: fits in 30 bits
  const int32_t q = f2i_rn(rf * rs);
  // q Y reaches 2^74: the product is taken modulo 2^64 in unsigned arithmetic
  R = (int64_t)(((uint64_t)R << s) - (uint64_t)(int64_t)q * (uint64_t)Y);
  Q = (int64_t)(((uint64_t)Q << s) + (uint64_t)(int64_t)q);
}

GCH_HD double ddiv_rn(double a, double b) {
  const uint64_t ba = bits_of(a), bb = bits_of(b);
  const int ea = (int)((ba >> 52) & 0x7FF), eb = (int)((bb >> 52) & 0x7FF);
  const int e0 = ea - eb + 1022;  // biased exponent of the quotient for X < Y
  if ((unsigned)(ea - 1) < 2046u && (unsigned)(eb - 1) < 2046u && (unsigned)(e0 - 1) < 2045u) {
    const int64_t X = (int64_t)((ba & 0xFFFFFFFFFFFFFull) | (1ull << 52));
    const int64_t Y = (int64_t)((bb & 0xFFFFFFFFFFFFFull) | (1ull << 52));
    const float r = rcp_rn((float)(int32_t)(Y >> 24));  // ~ 2^24 / Y
    int64_t R = X, Q = 0;
    ddiv_digit(R, Q, Y, r * 524288.0f, 19);
    ddiv_digit(R, Q, Y, r * 262144.0f, 18);
    ddiv_digit(R, Q, Y, r * 262144.0f, 18);
    if (R < 0) { Q -= 1; R += Y; }
    const int wide = (int)(Q >> 55);           // 1 when X >= Y (56-bit Q)
    const int sh = 2 + wide;
    const uint64_t M = (uint64_t)Q >> sh;      // 53 kept bits
    const uint32_t low = (uint32_t)Q & ((1u << sh) - 1u);
    const uint32_t half = 1u << (sh - 1);
    const uint64_t up = (low > half || (low == half && (R != 0 || (M & 1u)))) ? 1u : 0u;
    const uint64_t e = (uint64_t)(e0 + wide);
    const uint64_t bits = ((ba ^ bb) & 0x8000000000000000ull)
                          | ((e << 52) + (M - (1ull << 52)) + up);
    return double_of((uint32_t)(bits >> 32), (uint32_t)bits);
  }
  // a zero over a normal number: the zero with the quotient's sign (IEEE is
  // exact here).  Exactly zero fields make these common in the Riemann
  // solvers (Bz and vz of a 2.5-D problem, static gas where S_M - u = 0).
  if ((ba << 1) == 0 && (unsigned)(eb - 1) < 2046u)
    return double_of((uint32_t)((ba ^ bb) >> 32) & 0x80000000u, 0u);
  return a / b;
}

}  // namespace gch
