// gch_tc.cu -- thermal conduction (src/thermal_cond.f90): the FP64 path
// (compiled without multiply-add contraction, the reference's arithmetic),
// the host-side super-step arithmetic, and the dispatch on the precision
// mode.  The kernels are in gch_tc.cuh.
#include "gch_tc.cuh"

namespace gch {

// :625-636 superstep.  real**integer with a variable exponent is evaluated
// by binary (square-and-multiply) exponentiation in the reference build;
// this restates it.
static double powi_sq(double x, int m) {
  unsigned n = m < 0 ? 0u - (unsigned)m : (unsigned)m;
  double y = (n % 2u) ? x : 1.0;
  while (n >>= 1) {
    x = x * x;
    if (n % 2u) y = y * x;
  }
  return m < 0 ? 1.0 / y : y;
}

double tc_superstep(int N, double snu) {
  const double a = powi_sq(1.0 + snu, 2 * N), b = powi_sq(1.0 - snu, 2 * N);
  return (double)N / (2.0 * snu) * (a - b) / (a + b);
}

// :646-654 substep
double tc_substep(int j, int N, double nu) {
  const double pi = std::acos(-1.0);
  return 1.0 / ((nu - 1.0) * std::cos(pi * (double)(2 * j - 1) / (2.0 * (double)N)) + nu + 1.0);
}

// :664-681 ST_steps: the first N in 1..199 whose super step exceeds fs, or
// 200 (the Fortran DO index after a loop that did not exit)
void tc_st_steps(double fs, int* Ns, double* fstep) {
  const double snu = std::sqrt(kNu);
  int j;
  for (j = 1; j <= kJmax; ++j)
    if (tc_superstep(j, snu) > fs) break;
  *Ns = j;
  *fstep = fs / tc_superstep(j, snu);
}

int tc_run(gch_domain* d, double dt_CFL) {
  if (d->mode == GCH_FP32_KAHAN) return tc_run_kahan(d, dt_CFL);
  if (d->mode == GCH_FP32_MIXED) return tc_run_mixed(d, dt_CFL);
  return tc_run_t<PolFP64>(d, dt_CFL);
}

}  // namespace gch
