// gch_policy.cuh -- precision-policy specific loads and updates.
//
//   load_prim : conserved -> primitive of one cell (src/hydro_core.f90:46-129)
//   update    : u - dtdx*dF - dtdy*dG - dtdz*dH (src/hydro_solver.f90:105-107,
//               src/flux_cd_module.f90:299-301)
//
// PolFP64 restates the reference expression by expression.  PolMixed keeps
// the pressure recovery and the accumulation into u in FP64 and everything
// else in FP32.
#pragma once

#include "gch_device.cuh"

namespace gch {

template <class Pol>
struct Ops;

// ---------------------------------------------------------------------------
template <>
struct Ops<PolFP64> {
  using TC = double;

  // src/hydro_core.f90:46-129 u2prim, on a cell of any stored type
  template <int NEQ, class TIn>
  __device__ __forceinline__ static void load_prim(const KParams& p, const TIn* src,
                                                   long long idx, TC* prim, unsigned& pfl) {
    double uu[NEQ];
#pragma unroll
    for (int q = 0; q < NEQ; ++q) uu[q] = (double)src[q * p.fs + idx];
    u2prim<NEQ>(p, uu, prim, pfl);
  }

  template <int NEQ>
  __device__ __forceinline__ static void u2prim(const KParams& p, const double* uu, double* prim,
                                                unsigned& pfl, double* T = nullptr) {
    double r = tmax_(uu[0], 1e-15);
    prim[0] = r;
    prim[1] = uu[1] / r;
    prim[2] = uu[2] / r;
    prim[3] = uu[3] / r;
    if (NEQ >= 8 && p.mhd) {
      prim[4] = (uu[4] - 0.5 * r * (prim[1] * prim[1] + prim[2] * prim[2] + prim[3] * prim[3])
                 - 0.5 * (uu[5] * uu[5] + uu[6] * uu[6] + uu[7] * uu[7])) / p.cv;
    } else {
      prim[4] = (uu[4] - 0.5 * r * (prim[1] * prim[1] + prim[2] * prim[2] + prim[3] * prim[3]))
                / p.cv;
    }
    if (!(prim[4] >= 1e-16)) ++pfl;
    prim[4] = tmax_(prim[4], 1e-16);
    if (NEQ >= 8) {
      prim[5] = uu[5];
      prim[6] = uu[6];
      prim[7] = uu[7];
    }
    if (p.eos == GCH_EOS_SINGLE_SPECIE) {
      double t = tmax_(1.0, (prim[4] / r) * p.Tempsc);
      prim[4] = r * t / p.Tempsc;
      if (T) *T = t;
    } else if (T) {
      *T = (prim[4] / r) * p.Tempsc;
    }
  }

  // Stored prim (primit array) -> prim
  template <int NEQ, class TIn>
  __device__ __forceinline__ static void load_stored_prim(const KParams& p, const TIn* src,
                                                          long long idx, TC* prim) {
#pragma unroll
    for (int q = 0; q < NEQ; ++q) prim[q] = (double)src[q * p.fs + idx];
  }

  // ((u - dtdx*(fr-fl)) - dtdy*(gr-gl)) - dtdz*(hr-hl)
  __device__ __forceinline__ static double update(double u, double dtdx, double dtdy, double dtdz,
                                                  double fl, double fr, double gl, double gr,
                                                  double hl, double hr) {
    return u - dtdx * (fr - fl) - dtdy * (gr - gl) - dtdz * (hr - hl);
  }

  // CT update of one B component, src/flux_cd_module.f90:311-321:
  // u - 0.5*dta*(a1 - a0) + 0.5*dtb*(b1 - b0), with signs sa, sb
  __device__ __forceinline__ static double ct(double u, double hdta, double a0, double a1,
                                              double hdtb, double b0, double b1, bool first_minus) {
    if (first_minus) return u - hdta * (a1 - a0) + hdtb * (b1 - b0);
    return u + hdta * (a1 - a0) - hdtb * (b1 - b0);
  }
};

// ---------------------------------------------------------------------------
template <>
struct Ops<PolMixed> {
  using TC = float;

  // u2prim with the pressure recovery in FP64; inputs promoted exactly.
  template <int NEQ, class TIn>
  __device__ __forceinline__ static void load_prim(const KParams& p, const TIn* src,
                                                   long long idx, TC* prim, unsigned& pfl) {
    double uu[NEQ];
#pragma unroll
    for (int q = 0; q < NEQ; ++q) uu[q] = (double)src[q * p.fs + idx];
    double r = tmax_(uu[0], 1e-15);
    double ir = 1.0 / r;
    double vx = uu[1] * ir, vy = uu[2] * ir, vz = uu[3] * ir;
    double pr = uu[4] - 0.5 * r * (vx * vx + vy * vy + vz * vz);
    if (NEQ >= 8 && p.mhd) pr = pr - 0.5 * (uu[5] * uu[5] + uu[6] * uu[6] + uu[7] * uu[7]);
    pr = pr / p.cv;
    if (!(pr >= 1e-16)) ++pfl;
    pr = tmax_(pr, 1e-16);
    if (p.eos == GCH_EOS_SINGLE_SPECIE) {
      double t = tmax_(1.0, (pr / r) * p.Tempsc);
      pr = r * t / p.Tempsc;
    }
    prim[0] = (float)r;
    prim[1] = (float)vx;
    prim[2] = (float)vy;
    prim[3] = (float)vz;
    prim[4] = (float)pr;
    if (NEQ >= 8) {
      prim[5] = (float)uu[5];
      prim[6] = (float)uu[6];
      prim[7] = (float)uu[7];
    }
  }

  template <int NEQ, class TIn>
  __device__ __forceinline__ static void load_stored_prim(const KParams& p, const TIn* src,
                                                          long long idx, TC* prim) {
#pragma unroll
    for (int q = 0; q < NEQ; ++q) prim[q] = (float)src[q * p.fs + idx];
  }

  // flux divergence in FP32, accumulated into u in FP64
  __device__ __forceinline__ static double update(double u, float dtdx, float dtdy, float dtdz,
                                                  float fl, float fr, float gl, float gr,
                                                  float hl, float hr) {
    float d = dtdx * (fr - fl) + dtdy * (gr - gl) + dtdz * (hr - hl);
    return u - (double)d;
  }

  __device__ __forceinline__ static double ct(double u, float hdta, float a0, float a1,
                                              float hdtb, float b0, float b1, bool first_minus) {
    float d = hdta * (a1 - a0) - hdtb * (b1 - b0);
    return first_minus ? u - (double)d : u + (double)d;
  }
};

}  // namespace gch
