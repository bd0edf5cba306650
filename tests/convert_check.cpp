// Host check of gch_convert.h and gch_ddiv.h: the integer-pipe FP64 <-> FP32
// conversions against the C casts, with the flush rule the header states
// (results and FP32 inputs below 2^-126 in magnitude become signed zero),
// and the integer-pipe FP64 division against the IEEE division.
// Usage: convert_check <n_random>; prints "checked N bad B", exits 1 on a mismatch.
#include "gch_convert.h"
#include "gch_ddiv.h"

#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

using gch::bits_of;

static float want_d2f(double x) {
  if (std::isnan(x)) return NAN;
  if (std::fabs(x) < 0x1p-126) return std::signbit(x) ? -0.0f : 0.0f;
  return (float)x;
}
static double want_f2d(float f) {
  if (((bits_of(f) >> 23) & 0xFFu) == 0) return std::signbit(f) ? -0.0 : 0.0;
  return (double)f;
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? atol(argv[1]) : 1000000;
  long checked = 0, bad = 0;
  auto d2f = [&](double x) {
    ++checked;
    const float got = gch::d2f_rn(x), want = want_d2f(x);
    const bool ok = std::isnan(want) ? std::isnan(got) : bits_of(got) == bits_of(want);
    if (!ok && bad++ < 8) printf("d2f_rn(%a) = %a, want %a\n", x, got, want);
  };
  auto f2d = [&](float f) {
    ++checked;
    const double got = gch::f2d(f), want = want_f2d(f);
    const bool ok = std::isnan(want) ? std::isnan(got) : bits_of(got) == bits_of(want);
    if (!ok && bad++ < 8) printf("f2d(%a) = %a, want %a\n", f, got, want);
  };
  auto div = [&](double a, double b) {
    ++checked;
    const double got = gch::ddiv_rn(a, b), want = a / b;
    const bool ok = std::isnan(want) ? std::isnan(got) : bits_of(got) == bits_of(want);
    if (!ok && bad++ < 8) printf("ddiv_rn(%a, %a) = %a, want %a\n", a, b, got, want);
  };
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
  }
  const double special[] = {0.0, -0.0, INFINITY, -INFINITY, NAN, -NAN, DBL_MAX, -DBL_MAX,
                            FLT_MAX, -FLT_MAX, (double)FLT_MAX * (1 + 0x1p-25),
                            (double)FLT_MAX * (1 + 0x1p-24), 0x1.ffffffefffffffp127,
                            0x1.fffffff0000000p127, 0x1p128, 0x1p-126, -0x1p-126, 0x1p-127,
                            0x1.fffffffffffffp-127, 1.0, 1e-15, 1e-16, 1e-300, 5e-324};
  for (double s : special) d2f(s);
  const float fspecial[] = {0.0f, -0.0f, INFINITY, -INFINITY, NAN, FLT_MAX, FLT_MIN, -FLT_MIN,
                            0x1p-127f, 1.0f, -1.0f, 1e-15f};
  for (float s : fspecial) f2d(s);
  for (double s : special)
    for (double t : special) div(s, t);
  printf("checked %ld bad %ld\n", checked, bad);
  return bad ? 1 : 0;
}
