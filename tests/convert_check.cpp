// Host check of gch_convert.h, gch_ddiv.h and gch_dsqrt.h: the integer-pipe
// FP64 <-> FP32 conversions against the C casts, with the flush rule the
// header states (results and FP32 inputs below 2^-126 in magnitude become
// signed zero), and the integer-pipe FP64 division and square root against
// the IEEE division and square root, and the integer-pipe floor comparison
// against the C comparison.
// Usage: convert_check <n_random>; prints "checked N bad B", exits 1 on a mismatch.
#include "gch_convert.h"
#include "gch_ddiv.h"
#include "gch_dsqrt.h"
#include "convert_cases.h"

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
  auto sq = [&](double a) {
    ++checked;
    const double got = gch::dsqrt_rn(a), want = std::sqrt(a);
    const bool ok = std::isnan(want) ? std::isnan(got) : bits_of(got) == bits_of(want);
    if (!ok && bad++ < 8) printf("dsqrt_rn(%a) = %a, want %a\n", a, got, want);
  };
  // ge_pos against the C comparison, for the floors the FP32 + FP64 u
  // path uses and the ends of the positive range
  const double floors[] = {1e-15, 1e-16, 1.0, DBL_MIN, 0x1p-1074, DBL_MAX};
  auto ge = [&](double x) {
    for (double lo : floors) {
      ++checked;
      if (gch::ge_pos(x, lo) != (x >= lo) && bad++ < 8)
        printf("ge_pos(%a, %a) = %d, want %d\n", x, lo, (int)gch::ge_pos(x, lo), (int)(x >= lo));
    }
  };
  auto d2f_ge = [&](double x) {
    d2f(x);
    ge(x);
  };
  auto sq_ge = [&](double a) {
    sq(a);
    ge(a);
  };
  for (double lo : floors)
    for (double x : {lo, std::nextafter(lo, 0.0), std::nextafter(lo, INFINITY), -lo, 0.0, -0.0,
                     (double)INFINITY, -(double)INFINITY, (double)NAN, -(double)NAN})
      ge(x);
  convert_cases(n, d2f_ge, f2d, div, sq_ge);
  printf("checked %ld bad %ld\n", checked, bad);
  return bad ? 1 : 0;
}
