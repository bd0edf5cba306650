// gch_tc.cu -- thermal conduction (src/thermal_cond.f90) on the device.
//
// tstep ends with thermal_conduction() when th_cond != 0
// (src/hydro_solver.f90:227): Spitzer conduction, isotropic (heatfluxes,
// :189-267) or split along and across B (MHD_heatfluxes, :277-487), with
// optional saturation, advanced by Chebyshev super time steps
// (:625-681, :690-768).  Per conduction substep:
//   k_tc_flux     the heat flux through the +x, +y and +z faces of every
//                 cell 0..n (the reference's F(5), G(5), H(5))
//   k_tc_update   u(5) of the interior from the flux divergence
//   k_tc_bounds   thermal_bounds (:496-616): the first ghost layer of u(5),
//                 periodic copies then the outflow copies of every wall
//   k_tc_prim     calcprim over the whole array: rho, p and T
// The conduction timescale is a min-reduction on the device (k_tc_dtcond);
// the super-step count and the substep sizes are scalars formed on the host
// with the reference's arithmetic, so conduction needs one host round trip
// per timestep.  All arithmetic is FP64 on every precision path (u is read
// and written in its stored type); this unit is compiled without
// multiply-add contraction, so only pow() (T^2.5) may round differently from
// the host's libm.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#include "gch_domain.h"
#include "gch_policy.cuh"

namespace gch {
namespace {

constexpr double kRg = 8.3145e7;     // gas constant (cgs), src/constants.f90:35
constexpr double kPh = 0.4;          // saturation parameter, thermal_cond.f90:36
constexpr double kNu = 0.01;         // super-step damping factor, :37
constexpr double kRed = 0.25;        // tstep_red_factor, :41
constexpr double kClight = 3.e10;    // :195, :281
constexpr int kJmax = 199;           // ST_steps search limit, :670

// :142-178 Spitzer conductivities
__device__ __forceinline__ double ksp(double T) { return 6.e-7 * pow(T, 2.5); }
__device__ __forceinline__ double ksp_parl(double T) { return 9.2181e-7 * pow(T, 2.5); }
__device__ __forceinline__ double ksp_perp(double T, double dens, double B2) {
  return 0.30089e+33 * dens / (B2 * sqrt(T)) * dens;
}

struct TcArgs {
  double rsc, rhosc, vsc, vsc2, bsc2, Psc, gamma;
  int saturation;
};

// calcprim (src/hydro_core.f90:245-320) of every cell into w: rho, p, T
template <class TU, int NEQ>
__global__ void k_tc_prim(KParams p, const TU* __restrict__ u, double* __restrict__ w) {
  const int ax = blockIdx.x * blockDim.x + threadIdx.x;
  const int ay = blockIdx.y * blockDim.y + threadIdx.y;
  const int az = blockIdx.z;
  if (ax >= p.NX || ay >= p.NY) return;
  const long long c = cell_index(p, ax, ay, az);
  double uu[NEQ], pp[NEQ], T;
#pragma unroll
  for (int q = 0; q < NEQ; ++q) uu[q] = to_d(u[q * p.fs + c]);
  unsigned pfl = 0;
  Ops<PolFP64>::u2prim<NEQ>(p, uu, pp, pfl, &T);
  w[c] = pp[0];
  w[p.fs + c] = pp[4];
  w[2 * p.fs + c] = T;
}

// get_dt_cond (:78-110): min over the interior of rho/Ksp(T), one atomic per
// block on the bits of the positive double
__global__ void k_tc_dtcond(KParams p, const double* __restrict__ w,
                            unsigned long long* __restrict__ out) {
  const int ci = blockIdx.x * blockDim.x + threadIdx.x;
  const int cj = blockIdx.y * blockDim.y + threadIdx.y;
  const int ck = blockIdx.z;
  double v = 1.7976931348623157e308;  // huge(1.)
  if (ci < p.nx && cj < p.ny) {
    const long long c = cell_index(p, ci + NG, cj + NG, ck + NG);
    v = w[c] / ksp(w[2 * p.fs + c]);
  }
  for (int o = 16; o > 0; o >>= 1) v = tmin_(v, __shfl_xor_sync(0xffffffffu, v, o));
  __shared__ double red[8];
  const int t = threadIdx.y * blockDim.x + threadIdx.x;
  if ((t & 31) == 0) red[t >> 5] = v;
  __syncthreads();
  if (t == 0) {
    for (int i = 1; i < (int)(blockDim.x * blockDim.y) / 32; ++i) v = tmin_(v, red[i]);
    atomicMin(out, (unsigned long long)__double_as_longlong(v));
  }
}

__global__ void k_tc_init(unsigned long long* out) { *out = 0x7FEFFFFFFFFFFFFFull; }

// One face of heatfluxes (:196-263): from cell a to its +1 neighbour b along
// an axis of spacing d
__device__ __forceinline__ double heatflux_iso(const KParams& p, const TcArgs& t,
                                               const double* w, long long a, long long b,
                                               double d) {
  const double yhp = 1.0;
  const double Ta = w[2 * p.fs + a], Tb = w[2 * p.fs + b];
  if (Ta == Tb) return 0.0;
  const double meanP = 0.5 * (w[p.fs + a] + w[p.fs + b]);
  const double meanDens = 0.5 * (w[a] + w[b]);
  const double meanT = 0.5 * (Ta + Tb);
  const double dT = (Tb - Ta) / (d * t.rsc);
  double coef;
  if (t.saturation) {
    double cs = sqrt(t.gamma * meanP / meanDens);  // csound, src/hydro_core.f90:544-553
    cs = tmin_(cs * sqrt(t.vsc2), kClight);
    coef = tmin_(ksp(meanT), 5. * kPh * cs * meanP * t.Psc / fabs(dT));
  } else {
    coef = ksp(meanT);
  }
  return -coef * dT * yhp;
}

// The three face fluxes of cell (i, j, k), i, j, k in 0..n, into F (3 fields)
template <class TU, bool ANISO>
__global__ void k_tc_flux(KParams p, TcArgs t, const TU* __restrict__ u,
                          const double* __restrict__ w, double* __restrict__ F) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;  // 0..nx
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > p.nx || j > p.ny) return;
  const long long sy = p.pitch, sz = (long long)p.pitch * p.NY;
  const long long c = cell_index(p, i + NG - 1, j + NG - 1, k + NG - 1);
  const long long nb[3] = {c + 1, c + sy, c + sz};
  const double dd[3] = {p.dx, p.dy, p.dz};
  double out[3];
  if (!ANISO) {
#pragma unroll
    for (int a = 0; a < 3; ++a) out[a] = heatflux_iso(p, t, w, c, nb[a], dd[a]);
  } else {
    // :298-482 with the unit vector of B of this cell
    double bx = to_d(u[5 * p.fs + c]), by = to_d(u[6 * p.fs + c]), bz = to_d(u[7 * p.fs + c]);
    const double B2 = bx * bx + by * by + bz * bz;
    const double modB = sqrt(B2);
    bx = bx / modB;
    by = by / modB;
    bz = bz / modB;
    const double alpha = 5.0 * 0.3;
    double grad[3], kpar[3], kperp[3], csat[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const double Tc = w[2 * p.fs + c], Tn = w[2 * p.fs + nb[a]];
      if (fabs(Tc - Tn) < 1.0e-14) {
        grad[a] = 0.0;
        kpar[a] = 0.0;
        kperp[a] = 0.0;
        csat[a] = 0.0;
        continue;
      }
      const double meanDens = 0.5 * (w[c] + w[nb[a]]);
      const double meanTemp = 0.5 * (Tc + Tn);
      if (t.saturation) {
        const double meanPres = 0.5 * (w[p.fs + c] + w[p.fs + nb[a]]);
        double cs = sqrt(t.gamma * meanPres / meanDens);
        cs = tmin_(cs * t.vsc, kClight);
        csat[a] = alpha * meanDens * (cs * cs * cs);
      } else {
        csat[a] = 0.0;
      }
      grad[a] = (Tn - Tc) / (dd[a] * t.rsc);
      kpar[a] = ksp_parl(meanTemp);
      kperp[a] = ksp_perp(meanTemp, meanDens * t.rhosc, B2 * t.bsc2);
    }
    const double bgradT = bx * grad[0] + by * grad[1] + bz * grad[2];
    const double gpar[3] = {bgradT * bx, bgradT * by, bgradT * bz};
    const double gperp[3] = {grad[0] - gpar[0], grad[1] - gpar[1], grad[2] - gpar[2]};
    if (!t.saturation) {
#pragma unroll
      for (int a = 0; a < 3; ++a) out[a] = -kpar[a] * gpar[a] - kperp[a] * gperp[a];
    } else {
      const double gperp_n =
          sqrt(gperp[0] * gperp[0] + gperp[1] * gperp[1] + gperp[2] * gperp[2]);
#pragma unroll
      for (int a = 0; a < 3; ++a)
        out[a] = -1. / (1. / (kpar[a] + 1.e-14) + bgradT / (csat[a] + 1.e-14)) * gpar[a]
                 - 1. / (1. / (kperp[a] + 1.e-14) + gperp_n / (csat[a] + 1.e-14)) * gperp[a];
    }
  }
  F[c] = out[0];
  F[p.fs + c] = out[1];
  F[2 * p.fs + c] = out[2];
}

// :755-762 the energy update of the interior
template <class TU>
__global__ void k_tc_update(KParams p, double dts, const double* __restrict__ F,
                            TU* __restrict__ u) {
  const int ci = blockIdx.x * blockDim.x + threadIdx.x;
  const int cj = blockIdx.y * blockDim.y + threadIdx.y;
  const int ck = blockIdx.z;
  if (ci >= p.nx || cj >= p.ny) return;
  const long long sy = p.pitch, sz = (long long)p.pitch * p.NY;
  const long long c = cell_index(p, ci + NG, cj + NG, ck + NG);
  const double* G = F + p.fs;
  const double* H = F + 2 * p.fs;
  const double v = to_d(u[4 * p.fs + c]) -
                   dts * ((F[c] - F[c - 1]) / p.dx + (G[c] - G[c - sy]) / p.dy +
                          (H[c] - H[c - sz]) / p.dz);
  u[4 * p.fs + c] = from_d<TU>(v);
}

// thermal_bounds (:496-616), serial build, one pass per launch in the
// reference's order: pass 0-2 the periodic copies of x, y, z (whole
// transverse extent, when both walls of the axis are periodic), pass 3-5
// the outflow copies of x, y, z over 0..n+1, which the reference applies
// after the periodic ones on every wall.
template <class TU>
__global__ void k_tc_bounds(KParams p, TU* __restrict__ u, int pass) {
  const int axis = pass % 3;
  const bool periodic = pass < 3;
  const int t0 = blockIdx.x * blockDim.x + threadIdx.x;  // transverse fast
  const int t1 = blockIdx.y;                             // transverse slow
  int n, N0, N1;
  if (axis == 0) { n = p.nx; N0 = p.NY; N1 = p.NZ; }
  else if (axis == 1) { n = p.ny; N0 = p.NX; N1 = p.NZ; }
  else { n = p.nz; N0 = p.NX; N1 = p.NY; }
  int a0 = t0, a1 = t1;
  if (!periodic) {  // 0..n+1 of the transverse axes = array 1..N-2
    if (t0 >= N0 - 2 || t1 >= N1 - 2) return;
    a0 = t0 + NG - 1;
    a1 = t1 + NG - 1;
  } else if (t0 >= N0 || t1 >= N1) {
    return;
  }
  // ghost g <- source s on the low side, then the high side
  const int glo = NG - 1, ghi = NG + n;
  const int slo = periodic ? NG + n - 1 : NG, shi = periodic ? NG : NG + n - 1;
  auto at = [&](int g) -> long long {
    if (axis == 0) return cell_index(p, g, a0, a1);
    if (axis == 1) return cell_index(p, a0, g, a1);
    return cell_index(p, a0, a1, g);
  };
  TU* u5 = u + 4 * p.fs;
  u5[at(glo)] = u5[at(slo)];
  u5[at(ghi)] = u5[at(shi)];
}

template <class TU>
int tc_run_t(gch_domain* d, double dt_CFL) {
  const KParams& p = d->kp;
  const gch_params_t& hp = d->hp;
  cudaStream_t s = d->stream;
  TU* u = (TU*)d->u;
  double* w = d->tcw;                 // rho, p, T
  double* F = d->tcw + 3 * p.fs;      // F(5), G(5), H(5)
  const dim3 b(32, 8);
  const dim3 gall((p.NX + 31) / 32, (p.NY + 7) / 8, p.NZ);
  const dim3 gint((p.nx + 31) / 32, (p.ny + 7) / 8, p.nz);
  const dim3 gface((p.nx + 1 + 31) / 32, (p.ny + 1 + 7) / 8, p.nz + 1);
  auto prim = [&]() {
    with_neq(p.neq, [&](auto N) { k_tc_prim<TU, decltype(N)::value><<<gall, b, 0, s>>>(p, u, w); });
  };
  TcArgs t;
  t.rsc = hp.rsc;
  t.rhosc = hp.rhosc;
  t.vsc2 = hp.vsc2;
  t.vsc = std::sqrt(hp.vsc2);
  t.bsc2 = hp.bsc * hp.bsc;
  t.Psc = hp.Psc;
  t.gamma = hp.gamma;
  t.saturation = hp.tc_saturation;

  // the primitives and T of the state tstep left (its final calcprim)
  prim();
  k_tc_init<<<1, 1, 0, s>>>(d->tc_min);
  k_tc_dtcond<<<gint, b, 0, s>>>(p, w, d->tc_min);
  unsigned long long bits = 0;
  cudaError_t e = cudaMemcpyAsync(d->tc_min_host, d->tc_min, sizeof(bits),
                                  cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return GCH_ERR_CUDA;
  bits = *d->tc_min_host;
  double dtp;
  std::memcpy(&dtp, &bits, sizeof(dtp));

  // get_dt_cond tail, ST_steps and the substep sizes, on the host
  double ddx = std::min(hp.dx, hp.dy);
  ddx = std::min(ddx, hp.dz);
  const double x = ddx * hp.rsc;
  const double dt_cond = kRed * 0.5 * (x * x) * hp.cv * kRg * dtp * hp.rhosc / hp.mu;
  const double dt_hydro = dt_CFL * hp.tsc;
  int nsteps;
  double fstep;
  bool super = true;
  if (dt_cond < dt_hydro) {
    tc_st_steps(dt_hydro / dt_cond, &nsteps, &fstep);
  } else {
    super = false;
    fstep = dt_hydro / dt_cond;
    nsteps = 1;
  }
  d->tc_nsteps = nsteps;
  d->tc_dt_cond = dt_cond;
  const bool aniso = hp.th_cond == GCH_TC_ANISOTROPIC;
  const bool per[3] = {p.bc[0] == GCH_BC_PERIODIC && p.bc[1] == GCH_BC_PERIODIC,
                       p.bc[2] == GCH_BC_PERIODIC && p.bc[3] == GCH_BC_PERIODIC,
                       p.bc[4] == GCH_BC_PERIODIC && p.bc[5] == GCH_BC_PERIODIC};
  const int N0[3] = {p.NY, p.NX, p.NX}, N1[3] = {p.NZ, p.NZ, p.NY};
  for (int n = 1; n <= nsteps; ++n) {
    double dts;
    if (super)
      dts = dt_cond * fstep * tc_substep(n, nsteps, kNu) / hp.Psc / hp.rsc;
    else
      dts = dt_hydro / (double)nsteps / hp.Psc / hp.rsc;
    if (aniso) k_tc_flux<TU, true><<<gface, b, 0, s>>>(p, t, u, w, F);
    else k_tc_flux<TU, false><<<gface, b, 0, s>>>(p, t, u, w, F);
    k_tc_update<TU><<<gint, b, 0, s>>>(p, dts, F, u);
    for (int pass = 0; pass < 6; ++pass) {
      const int a = pass % 3;
      if (pass < 3 && !per[a]) continue;
      k_tc_bounds<TU><<<dim3((N0[a] + 127) / 128, N1[a]), 128, 0, s>>>(p, u, pass);
    }
    prim();
  }
  return cudaGetLastError() == cudaSuccess ? GCH_OK : GCH_ERR_CUDA;
}

}  // namespace

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
  if (d->mode == GCH_FP32_KAHAN) return tc_run_t<float2>(d, dt_CFL);
  return tc_run_t<double>(d, dt_CFL);
}

}  // namespace gch
