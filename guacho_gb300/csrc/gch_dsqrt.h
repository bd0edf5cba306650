// gch_dsqrt.h -- correctly rounded FP64 square root on the integer and FP32
// pipes.
//
// The FP64 wave speeds (cfast, csound) and the HLLD Alfven speeds take about
// twenty square roots per cell and stage.  An IEEE FP64 square root is a
// sequence of FP64-pipe operations, and that pipe bounds the plain FP64 step
// on GB300.  dsqrt_rn(x) returns the same bits as sqrt(x) (round to nearest)
// with 64-bit integer arithmetic and FP32 estimates, by the classical
// digit-by-digit square root with an exact remainder (the schoolbook method,
// e.g. Brent and Zimmermann, Modern Computer Arithmetic, 1.5.1), here with
// two digits and two Newton-style corrections of the root:
//
//   x = X 2^E, X in [2^52, 2^53).  With E odd, X' = 2X and E' = E - 1, else
//   X' = X, E' = E; then N = X' 2^52 is in [2^104, 2^106), Q = floor(sqrt(N))
//   in [2^52, 2^53), and sqrt(x) = sqrt(N) 2^(E'/2 - 26).
//
//   1. Q1 ~ sqrt(X') in [2^26, 2^27) from an FP32 reciprocal square root of
//      the top 30 bits of X' (within 23 of the root), R1 = X' - Q1^2 exact,
//      and one correction Q1 += round(R1 / 2Q1): |Q1 - sqrt(X')| <= 0.51,
//      so |R1| < 2^28.
//   2. the second digit q2 ~ R1 2^25 / Q1 from the FP32 reciprocal of Q1
//      (within 17 of the digit): Q = Q1 2^26 + q2, and the remainder
//      R = N - Q^2 = R1 2^52 - Q1 q2 2^27 - q2^2, exact in 64-bit two's
//      complement because its true value is below 2^59 in magnitude.
//   3. Q += round(R / 2Q), R updated exactly: |Q - sqrt(N)| <= 0.5 + 2^-17,
//      so one step (R < 0: Q - 1, R + 2Q - 1) makes Q the floor root and R
//      its remainder, 0 <= R <= 2Q.
//
//   Rounding: sqrt(N) >= Q + 1/2 exactly when R > Q (N is an integer, so
//   sqrt(N) is never a half-integer and there are no ties).  The result
//   Q + (R > Q) <= 2^53 is always a normal number; a root that rounds up to
//   2^53 carries into the exponent field.
//
// The fast path takes positive normal x.  Zero, subnormals, infinity, NaN
// and negative numbers go to the hardware square root.  The same code runs
// on the host (FP32 estimates by IEEE operations), so host tests check the
// digits the device computes.
#pragma once

#include <math.h>
#include <stdint.h>

#include "gch_ddiv.h"

namespace gch {

GCH_HD float rsqrt_rn(float x) {
#if defined(__CUDA_ARCH__)
  return __frsqrt_rn(x);
#else
  return 1.0f / sqrtf(x);
#endif
}

GCH_HD double dsqrt_rn(double x) {
  const uint64_t b = bits_of(x);
  const int e = (int)(b >> 52);  // with the sign bit: negative x gives e >= 2048
  if ((unsigned)(e - 1) < 2046u) {
    const int odd = (e - 1075) & 1;
    const int half = (e - 1075 - odd) / 2;  // exact: an even number halved
    const int64_t Xp = (int64_t)(((b & 0xFFFFFFFFFFFFFull) | (1ull << 52)) << odd);
    // 1. Q1 ~ sqrt(X'): xs = X' 2^-24 (top 30 bits), y ~ 2^12 / sqrt(X')
    const float xs = (float)(int32_t)(Xp >> 24);
    const float y = rsqrt_rn(xs);
    int32_t Q1 = f2i_rn(xs * y * 4096.0f);
    int64_t R1 = Xp - (int64_t)Q1 * Q1;
    // R1 / (2 Q1) with 1 / Q1 ~ y 2^-12; |R1| < 2^33, so R1 >> 8 fits 32 bits
    const int32_t d = f2i_rn((float)(int32_t)(R1 >> 8) * y * 0.03125f);
    R1 -= (int64_t)d * (2 * (int64_t)Q1 + d);
    Q1 += d;
    // 2. q2 ~ R1 2^25 / Q1
    const float rq = rcp_rn((float)Q1);
    const int32_t q2 = f2i_rn((float)(int32_t)R1 * rq * 33554432.0f);
    int64_t Q = ((int64_t)Q1 << 26) + q2;
    int64_t R = (int64_t)(((uint64_t)R1 << 52) - ((uint64_t)((int64_t)Q1 * q2) << 27) -
                          (uint64_t)((int64_t)q2 * q2));
    // 3. R / (2Q) with 1 / Q ~ rq 2^-26; |R| < 2^59, so R >> 30 fits 32 bits
    const int32_t dl = f2i_rn((float)(int32_t)(R >> 30) * rq * 8.0f);
    R = (int64_t)((uint64_t)R - (uint64_t)((int64_t)dl * (2 * Q + dl)));
    Q += dl;
    if (R < 0) {
      R += 2 * Q - 1;
      Q -= 1;
    }
    const uint64_t up = R > Q ? 1u : 0u;
    const uint64_t bits = ((uint64_t)(half + 1049) << 52) + ((uint64_t)Q + up - (1ull << 52));
    return double_of((uint32_t)(bits >> 32), (uint32_t)bits);
  }
  return sqrt(x);
}

}  // namespace gch
