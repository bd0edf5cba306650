// gch_tc.cuh -- thermal conduction (src/thermal_cond.f90) on the device.
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
// per timestep.  The FP64 path computes in FP64 with the reference's
// expressions; its unit is compiled without multiply-add contraction, so
// only pow() (T^2.5) may round differently from the host's libm.  The FP32
// paths compute in FP32 (work type TW = float): the primitives come from the
// path's own conversion (FP64 or compensated pressure recovery), T^2.5 is
// T*T*sqrt(T), and the energy change of a substep is added to the FP64 or
// compensated u(5).  FP64 arithmetic on GB300 runs at 1/57 of the FP32 rate,
// and pow() in FP64 made a 256^3 substep take about 11 ms.
//
// The kernels and the per-timestep driver, templated on the precision
// policy; gch_tc.cu instantiates the FP64 path (no multiply-add
// contraction) and holds the host-side super-step arithmetic, gch_tc32.cu
// the FP32 paths (compiled like the other FP32 units).
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <type_traits>

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

// :142-178 Spitzer conductivities; T^2.5 by pow() in FP64, T*T*sqrt(T) in FP32
__device__ __forceinline__ double pow25(double T) { return pow(T, 2.5); }
__device__ __forceinline__ float pow25(float T) { return T * T * sqrtf(T); }
template <class TW>
__device__ __forceinline__ TW ksp(TW T) { return TW(6.e-7) * pow25(T); }
template <class TW>
__device__ __forceinline__ TW ksp_parl(TW T) { return TW(9.2181e-7) * pow25(T); }
template <class TW>
__device__ __forceinline__ TW ksp_perp(TW T, TW dens, TW B2) {
  return TW(0.30089e+33) * dens / (B2 * tsqrt(T)) * dens;
}

template <class TW>
struct TcArgs {
  TW rsc, rhosc, vsc, vsc2, bsc2, Psc, gamma;
  TW dd[3];  // dx, dy, dz
  int saturation;
};

// a stored value in the work type
template <class TW>
__device__ __forceinline__ TW to_w(double x) { return (TW)x; }
template <class TW>
__device__ __forceinline__ TW to_w(float2 x) { return (TW)x.x + (TW)x.y; }

// calcprim (src/hydro_core.f90:245-320) of every cell into w: rho, p, T.
// FP64: the reference's u2prim; FP32: the path's own conversion.
template <class Pol, int NEQ, class TW>
__global__ void k_tc_prim(KParams p, const typename Pol::TU* __restrict__ u, TW* __restrict__ w) {
  const int ax = blockIdx.x * blockDim.x + threadIdx.x;
  const int ay = blockIdx.y * blockDim.y + threadIdx.y;
  const int az = blockIdx.z;
  if (ax >= p.NX || ay >= p.NY) return;
  const long long c = cell_index(p, ax, ay, az);
  unsigned pfl = 0;
  if constexpr (sizeof(TW) == 8) {
    double uu[NEQ], pp[NEQ], T;
#pragma unroll
    for (int q = 0; q < NEQ; ++q) uu[q] = to_d(u[q * p.fs + c]);
    Ops<PolFP64>::u2prim<NEQ>(p, uu, pp, pfl, &T);
    w[c] = pp[0];
    w[p.fs + c] = pp[4];
    w[2 * p.fs + c] = T;
  } else {
    float pr[NEQ];
    Ops<Pol>::template load_prim<NEQ>(p, u, c, pr, pfl);
    float T;
    if (NEQ > kNeqDyn<NEQ> && p.eos == GCH_EOS_H_RATE)
      T = (pr[4] / tmax_(2.0f * pr[0] - pr[kNeqDyn<NEQ>], 1e-15f)) * p.f_Tempsc;
    else
      T = (pr[4] / pr[0]) * p.f_Tempsc;
    w[c] = pr[0];
    w[p.fs + c] = pr[4];
    w[2 * p.fs + c] = T;
  }
}

// get_dt_cond (:78-110): min over the interior of rho/Ksp(T) in the work
// type, one atomic per block on the bits of the (positive) FP64 value
template <class TW>
__global__ void k_tc_dtcond(KParams p, const TW* __restrict__ w,
                            unsigned long long* __restrict__ out) {
  const int ci = blockIdx.x * blockDim.x + threadIdx.x;
  const int cj = blockIdx.y * blockDim.y + threadIdx.y;
  const int ck = blockIdx.z;
  const TW huge = sizeof(TW) == 8 ? TW(1.7976931348623157e308) : TW(3.4028234663852886e38);
  TW v = huge;  // huge(1.)
  if (ci < p.nx && cj < p.ny) {
    const long long c = cell_index(p, ci + NG, cj + NG, ck + NG);
    v = w[c] / ksp(w[2 * p.fs + c]);
  }
  for (int o = 16; o > 0; o >>= 1) v = tmin_(v, __shfl_xor_sync(0xffffffffu, v, o));
  __shared__ TW red[8];
  const int t = threadIdx.y * blockDim.x + threadIdx.x;
  if ((t & 31) == 0) red[t >> 5] = v;
  __syncthreads();
  if (t == 0) {
    for (int i = 1; i < (int)(blockDim.x * blockDim.y) / 32; ++i) v = tmin_(v, red[i]);
    const double m = v < huge ? (double)v : 1.7976931348623157e308;
    atomicMin(out, (unsigned long long)__double_as_longlong(m));
  }
}

__global__ void k_tc_init(unsigned long long* out) { *out = 0x7FEFFFFFFFFFFFFFull; }

// One face of heatfluxes (:196-263): from cell a to its +1 neighbour b along
// an axis of spacing d
template <class TW>
__device__ __forceinline__ TW heatflux_iso(const KParams& p, const TcArgs<TW>& t, const TW* w,
                                           long long a, long long b, TW d) {
  const TW yhp = 1.0;
  const TW Ta = w[2 * p.fs + a], Tb = w[2 * p.fs + b];
  if (Ta == Tb) return 0.0;
  const TW meanP = TW(0.5) * (w[p.fs + a] + w[p.fs + b]);
  const TW meanDens = TW(0.5) * (w[a] + w[b]);
  const TW meanT = TW(0.5) * (Ta + Tb);
  const TW dT = (Tb - Ta) / (d * t.rsc);
  TW coef;
  if (t.saturation) {
    TW cs = tsqrt(t.gamma * meanP / meanDens);  // csound, src/hydro_core.f90:544-553
    cs = tmin_(cs * tsqrt(t.vsc2), TW(kClight));
    coef = tmin_(ksp(meanT), TW(5.) * TW(kPh) * cs * meanP * t.Psc / tabs(dT));
  } else {
    coef = ksp(meanT);
  }
  return -coef * dT * yhp;
}

// The three face fluxes of cell (i, j, k), i, j, k in 0..n, into F (3 fields)
template <class TU, class TW, bool ANISO>
__global__ void k_tc_flux(KParams p, TcArgs<TW> t, const TU* __restrict__ u,
                          const TW* __restrict__ w, TW* __restrict__ F) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;  // 0..nx
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > p.nx || j > p.ny) return;
  const long long sy = p.pitch, sz = (long long)p.pitch * p.NY;
  const long long c = cell_index(p, i + NG - 1, j + NG - 1, k + NG - 1);
  const long long nb[3] = {c + 1, c + sy, c + sz};
  TW out[3];
  if (!ANISO) {
#pragma unroll
    for (int a = 0; a < 3; ++a) out[a] = heatflux_iso<TW>(p, t, w, c, nb[a], t.dd[a]);
  } else {
    // :298-482 with the unit vector of B of this cell
    TW bx = to_w<TW>(u[5 * p.fs + c]), by = to_w<TW>(u[6 * p.fs + c]),
       bz = to_w<TW>(u[7 * p.fs + c]);
    const TW B2 = bx * bx + by * by + bz * bz;
    const TW modB = tsqrt(B2);
    bx = bx / modB;
    by = by / modB;
    bz = bz / modB;
    const TW alpha = TW(5.0 * 0.3);
    TW grad[3], kpar[3], kperp[3], csat[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const TW Tc = w[2 * p.fs + c], Tn = w[2 * p.fs + nb[a]];
      if (tabs(Tc - Tn) < TW(1.0e-14)) {
        grad[a] = 0.0;
        kpar[a] = 0.0;
        kperp[a] = 0.0;
        csat[a] = 0.0;
        continue;
      }
      const TW meanDens = TW(0.5) * (w[c] + w[nb[a]]);
      const TW meanTemp = TW(0.5) * (Tc + Tn);
      if (t.saturation) {
        const TW meanPres = TW(0.5) * (w[p.fs + c] + w[p.fs + nb[a]]);
        TW cs = tsqrt(t.gamma * meanPres / meanDens);
        cs = tmin_(cs * t.vsc, TW(kClight));
        csat[a] = alpha * meanDens * (cs * cs * cs);
      } else {
        csat[a] = 0.0;
      }
      grad[a] = (Tn - Tc) / (t.dd[a] * t.rsc);
      kpar[a] = ksp_parl(meanTemp);
      kperp[a] = ksp_perp(meanTemp, meanDens * t.rhosc, B2 * t.bsc2);
    }
    const TW bgradT = bx * grad[0] + by * grad[1] + bz * grad[2];
    const TW gpar[3] = {bgradT * bx, bgradT * by, bgradT * bz};
    const TW gperp[3] = {grad[0] - gpar[0], grad[1] - gpar[1], grad[2] - gpar[2]};
    if (!t.saturation) {
#pragma unroll
      for (int a = 0; a < 3; ++a) out[a] = -kpar[a] * gpar[a] - kperp[a] * gperp[a];
    } else {
      const TW gperp_n = tsqrt(gperp[0] * gperp[0] + gperp[1] * gperp[1] + gperp[2] * gperp[2]);
      const TW one = 1., eps = 1.e-14;
#pragma unroll
      for (int a = 0; a < 3; ++a)
        out[a] = -one / (one / (kpar[a] + eps) + bgradT / (csat[a] + eps)) * gpar[a]
                 - one / (one / (kperp[a] + eps) + gperp_n / (csat[a] + eps)) * gperp[a];
    }
  }
  F[c] = out[0];
  F[p.fs + c] = out[1];
  F[2 * p.fs + c] = out[2];
}

// :755-762 the energy update of the interior: FP64 as the reference; in
// FP32 the change of u(5) is formed in FP32 and added to the stored u(5)
template <class TU, class TW>
__global__ void k_tc_update(KParams p, double dts, TW dts_w, const TW* __restrict__ F,
                            TU* __restrict__ u) {
  const int ci = blockIdx.x * blockDim.x + threadIdx.x;
  const int cj = blockIdx.y * blockDim.y + threadIdx.y;
  const int ck = blockIdx.z;
  if (ci >= p.nx || cj >= p.ny) return;
  const long long sy = p.pitch, sz = (long long)p.pitch * p.NY;
  const long long c = cell_index(p, ci + NG, cj + NG, ck + NG);
  const TW* G = F + p.fs;
  const TW* H = F + 2 * p.fs;
  if constexpr (sizeof(TW) == 8) {
    const double v = to_d(u[4 * p.fs + c]) -
                     dts * ((F[c] - F[c - 1]) / p.dx + (G[c] - G[c - sy]) / p.dy +
                            (H[c] - H[c - sz]) / p.dz);
    u[4 * p.fs + c] = from_d<TU>(v);
  } else {
    const float du = dts_w * ((F[c] - F[c - 1]) / p.f_dx + (G[c] - G[c - sy]) / p.f_dy +
                              (H[c] - H[c - sz]) / p.f_dz);
    if constexpr (std::is_same<TU, float2>::value)
      u[4 * p.fs + c] = Ops<PolKahan>::addf(u[4 * p.fs + c], -du);
    else
      u[4 * p.fs + c] = u[4 * p.fs + c] - (double)du;
  }
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

template <class Pol>
int tc_run_t(gch_domain* d, double dt_CFL) {
  using TU = typename Pol::TU;
  using TW = typename std::conditional<std::is_same<Pol, PolFP64>::value, double, float>::type;
  const KParams& p = d->kp;
  const gch_params_t& hp = d->hp;
  cudaStream_t s = d->stream;
  TU* u = (TU*)d->u;
  TW* w = reinterpret_cast<TW*>(d->tcw);  // rho, p, T
  TW* F = w + 3 * p.fs;                   // F(5), G(5), H(5)
  const dim3 b(32, 8);
  const dim3 gall((p.NX + 31) / 32, (p.NY + 7) / 8, p.NZ);
  const dim3 gint((p.nx + 31) / 32, (p.ny + 7) / 8, p.nz);
  const dim3 gface((p.nx + 1 + 31) / 32, (p.ny + 1 + 7) / 8, p.nz + 1);
  auto prim = [&]() {
    with_neq(p.neq, [&](auto N) {
      k_tc_prim<Pol, decltype(N)::value, TW><<<gall, b, 0, s>>>(p, u, w);
    });
  };
  TcArgs<TW> t;
  t.rsc = (TW)hp.rsc;
  t.rhosc = (TW)hp.rhosc;
  t.vsc2 = (TW)hp.vsc2;
  t.vsc = (TW)std::sqrt(hp.vsc2);
  t.bsc2 = (TW)(hp.bsc * hp.bsc);
  t.Psc = (TW)hp.Psc;
  t.gamma = (TW)hp.gamma;
  t.dd[0] = (TW)p.dx;
  t.dd[1] = (TW)p.dy;
  t.dd[2] = (TW)p.dz;
  t.saturation = hp.tc_saturation;

  // the primitives and T of the state tstep left (its final calcprim)
  prim();
  k_tc_init<<<1, 1, 0, s>>>(d->tc_min);
  k_tc_dtcond<TW><<<gint, b, 0, s>>>(p, w, d->tc_min);
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
    if (aniso) k_tc_flux<TU, TW, true><<<gface, b, 0, s>>>(p, t, u, w, F);
    else k_tc_flux<TU, TW, false><<<gface, b, 0, s>>>(p, t, u, w, F);
    k_tc_update<TU, TW><<<gint, b, 0, s>>>(p, dts, (TW)dts, F, u);
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

}  // namespace gch
