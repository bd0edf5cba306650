// convert_cases.h -- the inputs of the conversion and division checks:
// random bit patterns, values around the FP32 range, exact rounding ties of
// the 29 bits FP64 -> FP32 drops and their neighbours, operands of nearby
// magnitudes, dividends one ulp either side of b times a 53-bit quotient
// (quotients next to a rounding boundary), radicands within two ulps of the
// square of a 53-bit root and of the square of a midpoint between two roots
// (roots next to a rounding boundary), and the special values.  The
// host check (convert_check.cpp) and the device check (convert_check_gpu.cu)
// feed the same cases to their callbacks, seeded alike.
#pragma once

#include <stdint.h>
#include <string.h>

#include <cfloat>
#include <cmath>
#include <random>

template <class D2F, class F2D, class DIV, class SQ>
void convert_cases(long n, D2F&& d2f, F2D&& f2d, DIV&& div, SQ&& sq) {
  std::mt19937_64 g(20260001);
  for (long i = 0; i < n; ++i) {
    // any bit pattern
    const uint64_t b = g();
    double x;
    memcpy(&x, &b, 8);
    d2f(x);
    // values around the FP32 range
    const double y = std::ldexp((double)(g() >> 11) * 0x1p-53 + 0.5, (int)(g() % 300) - 150);
    d2f(y);
    d2f(-y);
    // exact ties of the 29 dropped bits, and their neighbours
    uint64_t t;
    memcpy(&t, &y, 8);
    t = (t & ~0x1FFFFFFFull) | 0x10000000ull;
    for (int k = -1; k <= 1; ++k) {
      const uint64_t tk = t + (uint64_t)(int64_t)k;
      memcpy(&x, &tk, 8);
      d2f(x);
    }
    uint32_t fb = (uint32_t)g();
    float f;
    memcpy(&f, &fb, 4);
    f2d(f);
    // division: any bit patterns, operands of nearby magnitudes, and
    // dividends one ulp either side of b times a 53-bit quotient, whose
    // quotients sit next to a rounding boundary
    const uint64_t ub = g(), vb = g();
    double da, db;
    memcpy(&da, &ub, 8);
    memcpy(&db, &vb, 8);
    div(da, db);
    const double c = std::ldexp((double)(g() >> 11) * 0x1p-53 + 0.5, (int)(g() % 80) - 40);
    div(y, c);
    div(-c, y);
    div(c, c);
    div(3.0 * c, 3.0);
    const uint64_t mb = (0x3FFull << 52) | (g() >> 12);
    double q;
    memcpy(&q, &mb, 8);
    const double p = q * c;
    div(p, c);
    div(std::nextafter(p, 0.0), c);
    div(std::nextafter(p, INFINITY), c);
    // square roots: any positive or negative bit pattern, and radicands next
    // to r^2 and to (r + half an ulp)^2 for a 53-bit r of any magnitude
    sq(da);
    sq(std::fabs(da));
    const double r = std::ldexp(q, (int)(g() % 1000) - 500);
    const double mid = r + std::ldexp(0.5, std::ilogb(r) - 52);
    for (double s0 : {r * r, mid * mid}) {
      double lo = s0, hi = s0;
      sq(s0);
      for (int k = 0; k < 2; ++k) {
        lo = std::nextafter(lo, 0.0);
        hi = std::nextafter(hi, INFINITY);
        sq(lo);
        sq(hi);
      }
    }
  }
  const double special[] = {0.0, -0.0, INFINITY, -INFINITY, NAN, -NAN, DBL_MAX, -DBL_MAX,
                            FLT_MAX, -FLT_MAX, (double)FLT_MAX * (1 + 0x1p-25),
                            (double)FLT_MAX * (1 + 0x1p-24), 0x1.ffffffeffffffp127,
                            0x1.fffffff0000000p127, 0x1p128, 0x1p-126, -0x1p-126, 0x1p-127,
                            0x1.fffffffffffffp-127, 1.0, 1e-15, 1e-16, 1e-300, 5e-324};
  for (double s : special) d2f(s);
  const float fspecial[] = {0.0f, -0.0f, INFINITY, -INFINITY, NAN, FLT_MAX, FLT_MIN, -FLT_MIN,
                            0x1p-127f, 1.0f, -1.0f, 1e-15f};
  for (float s : fspecial) f2d(s);
  for (double s : special)
    for (double t : special) div(s, t);
  for (double s : special) sq(s);
  const double sspecial[] = {0x1p-1022, 0x1.0000000000001p-1022, 0x1.fffffffffffffp1023,
                             0x1p-1074, 4.0, 2.0, 0x1.fffffffffffffp-1, 0x1.0000000000001p0};
  for (double s : sspecial) sq(s);
}
