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
  using R = double;  // accumulator of u updates
  __device__ __forceinline__ static double ld(double u) { return u; }
  // up + dt*s (src/hydro_solver.f90:119)
  __device__ __forceinline__ static double add(double u, double v) { return u + v; }

  // src/hydro_core.f90:46-129 u2prim, on a cell of any stored type
  template <int NEQ, class TIn>
  __device__ __forceinline__ static void load_prim(const KParams& p, const TIn* src,
                                                   long long idx, TC* prim, unsigned& pfl) {
    double uu[NEQ];
#pragma unroll
    for (int q = 0; q < NEQ; ++q) uu[q] = (double)src[q * p.fs + idx];
    u2prim<NEQ>(p, uu, prim, pfl);
  }
  // the same from values already in registers
  template <int NEQ>
  __device__ __forceinline__ static void prim_vals(const KParams& p, const double* uu, TC* prim,
                                                   unsigned& pfl) {
    u2prim<NEQ>(p, uu, prim, pfl);
  }

  template <int NEQ>
  __device__ __forceinline__ static void u2prim(const KParams& p, const double* uu, double* prim,
                                                unsigned& pfl, double* T = nullptr) {
    double r = tmax_(uu[0], 1e-15);
    prim[0] = r;
    prim[1] = tdiv(uu[1], r);
    prim[2] = tdiv(uu[2], r);
    prim[3] = tdiv(uu[3], r);
    if (NEQ >= 8 && p.mhd) {
      prim[4] = tdiv(uu[4] - 0.5 * r * (prim[1] * prim[1] + prim[2] * prim[2] + prim[3] * prim[3])
                         - 0.5 * (uu[5] * uu[5] + uu[6] * uu[6] + uu[7] * uu[7]),
                     p.cv);
    } else {
      prim[4] = tdiv(uu[4] - 0.5 * r * (prim[1] * prim[1] + prim[2] * prim[2] + prim[3] * prim[3]),
                     p.cv);
    }
    if (!(prim[4] >= 1e-16)) ++pfl;
    prim[4] = tmax_(prim[4], 1e-16);
    if (NEQ >= 8) {
      prim[5] = uu[5];
      prim[6] = uu[6];
      prim[7] = uu[7];
    }
#pragma unroll
    for (int q = kNeqDyn<NEQ>; q < NEQ; ++q) prim[q] = uu[q];  // passives (:86-89)
    if (p.eos == GCH_EOS_SINGLE_SPECIE) {
      double t = tmax_(1.0, (prim[4] / r) * p.Tempsc);
      prim[4] = r * t / p.Tempsc;
      if (T) *T = t;
    } else if (NEQ > kNeqDyn<NEQ> && p.eos == GCH_EOS_H_RATE) {
      // :106-111, n_HI in the first passive scalar
      double dentot = (2.0 * r - prim[kNeqDyn<NEQ>]);
      dentot = tmax_(dentot, 1e-15);
      const double t = tmax_(1.0, (prim[4] / dentot) * p.Tempsc);
      prim[4] = dentot * t / p.Tempsc;
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
// dt/dx (fr - fl) + dt/dy (gr - gl) + dt/dz (hr - hl) in FP32 with its
// roundings spelled out (one product, two fused multiply-adds), so that every
// kernel that inlines it rounds the same way whatever the compiler would
// contract: the deferred first stage and its update kernel agree bit for bit
// with the fused stage.
__device__ __forceinline__ float flux_sum(float dtdx, float dtdy, float dtdz, float fl, float fr,
                                          float gl, float gr, float hl, float hr) {
  return __fmaf_rn(dtdz, hr - hl, __fmaf_rn(dtdy, gr - gl, __fmul_rn(dtdx, fr - fl)));
}

// ---------------------------------------------------------------------------
// Error-free FP32 transformations (compensated "double-float" arithmetic).
// The FP32 units are compiled with multiply-add contraction, which could
// fuse a product into a following sum once these are inlined: every product
// that feeds a sum here is rounded on its own (__fmul_rn, never contracted)
// and the exact products use explicit fmaf.  That keeps the transformations
// exact, and it makes the pressure recovery round the same way in every
// kernel that inlines it (the one-box and the grouped CFL reductions agree
// bit for bit).
struct DF {
  float hi, lo;
};
__device__ __forceinline__ DF two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ DF fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = a + b;
  return {s, b - (s - a)};
}
__device__ __forceinline__ DF two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);  // rounded on its own: never fused into a later sum
  return {p, fmaf(a, b, -p)};
}
__device__ __forceinline__ DF df_add(DF x, DF y) {
  const DF s = two_sum(x.hi, y.hi);
  return fast_two_sum(s.hi, s.lo + (x.lo + y.lo));
}
// a^2 + b^2 + c^2 of exact FP32 inputs, to ~2^-44 relative
__device__ __forceinline__ DF df_sumsq(float a, float b, float c) {
  return df_add(df_add(two_prod(a, a), two_prod(b, b)), two_prod(c, c));
}

// u2prim from exact FP32 inputs with the pressure recovery in compensated
// FP32: m.m and B.B are formed exactly with FMA two-products, KE = m.m/rho is
// a pair quotient, and E - KE/2 - B.B/2 is taken in double-float, matching an
// FP64 evaluation to ~1e-13 relative of KE + B^2/2.
template <int NEQ>
__device__ __forceinline__ void prim_from_f32(const KParams& p, const float* uu, float* prim,
                                              unsigned& pfl) {
  const float r = tmax_(uu[0], 1e-15f);
  float ir = 1.0f / r;
  ir = ir * fmaf(-r, ir, 2.0f);
  const DF m2 = df_sumsq(uu[1], uu[2], uu[3]);
  const float q = __fmul_rn(m2.hi, ir);
  const float rem = fmaf(-q, r, m2.hi) + m2.lo;
  DF kb = fast_two_sum(q, __fmul_rn(rem, ir));
  if (NEQ >= 8 && p.mhd) kb = df_add(kb, df_sumsq(uu[5], uu[6], uu[7]));
  const DF d = two_sum(uu[4], __fmul_rn(-0.5f, kb.hi));
  float pr = (d.hi + (d.lo - __fmul_rn(0.5f, kb.lo))) * p.f_inv_cv;
  if (!(pr >= 1e-16f)) ++pfl;
  pr = tmax_(pr, 1e-16f);
  if (p.eos == GCH_EOS_SINGLE_SPECIE) {
    const float t = tmax_(1.0f, (pr * ir) * p.f_Tempsc);
    pr = r * t / p.f_Tempsc;
  } else if (NEQ > kNeqDyn<NEQ> && p.eos == GCH_EOS_H_RATE) {
    const float dentot = tmax_(2.0f * r - uu[kNeqDyn<NEQ>], 1e-15f);
    const float t = tmax_(1.0f, (pr / dentot) * p.f_Tempsc);
    pr = dentot * t / p.f_Tempsc;
  }
  prim[0] = r;
  prim[1] = uu[1] * ir;
  prim[2] = uu[2] * ir;
  prim[3] = uu[3] * ir;
  prim[4] = pr;
  if (NEQ >= 8) {
    prim[5] = uu[5];
    prim[6] = uu[6];
    prim[7] = uu[7];
  }
#pragma unroll
  for (int q = kNeqDyn<NEQ>; q < NEQ; ++q) prim[q] = uu[q];
}

// (h + l)^2 of a compensated pair, as a pair (the l^2 term is below 2^-48)
__device__ __forceinline__ DF df_sq(float2 x) {
  const DF p = two_prod(x.x, x.x);
  return fast_two_sum(p.hi, p.lo + __fmul_rn(2.0f * x.x, x.y));
}

// ---------------------------------------------------------------------------
template <>
struct Ops<PolMixed> {
  using TC = float;
  using R = double;
  __device__ __forceinline__ static double ld(double u) { return u; }
  __device__ __forceinline__ static double add(double u, double v) { return u + v; }

  // u2prim with the pressure recovery p = (E - m.m/(2 rho) - B.B/2)/cv
  // done at FP64-level accuracy:
  //  - FP64 source (u): FP64 arithmetic, one reciprocal (FP32 estimate and a
  //    Newton step in FP64 instead of an FP64 divide, which runs at 1/600 of
  //    the FP32 FMA rate on this part);
  //  - FP32 source (up): the inputs are exact FP32 numbers, so the products
  //    are formed exactly with FMA-based two-products and the cancellation
  //    E - KE - B^2/2 is taken in compensated FP32 ("double-float"), which
  //    matches an FP64 evaluation to ~1e-13 relative of KE + B^2/2.
  template <int NEQ, class TIn>
  __device__ __forceinline__ static void load_prim(const KParams& p, const TIn* src,
                                                   long long idx, TC* prim, unsigned& pfl) {
    if constexpr (sizeof(TIn) == 8) {
      double uu[NEQ];
#pragma unroll
      for (int q = 0; q < NEQ; ++q) uu[q] = (double)src[q * p.fs + idx];
      prim_vals<NEQ>(p, uu, prim, pfl);
    } else {
      float uu[NEQ];
#pragma unroll
      for (int q = 0; q < NEQ; ++q) uu[q] = (float)src[q * p.fs + idx];
      prim_from_f32<NEQ>(p, uu, prim, pfl);
    }
  }

  template <int NEQ>
  __device__ __forceinline__ static void prim_vals(const KParams& p, const double* uu, TC* prim,
                                                   unsigned& pfl) {
    {
      // the two floors compared on the integer pipes (ge_pos, the same
      // results as tmax_ and >=): three fewer FP64-pipe operations in a
      // recovery of about fourteen
      const double r = ge_pos(uu[0], 1e-15) ? uu[0] : 1e-15;
      const float rf = d2f_rn(r);
      const float irf = 1.0f / rf;
      double ir = f2d(irf);
      ir = ir * fma(-r, ir, 2.0);
      const double m2 = fma(uu[3], uu[3], fma(uu[2], uu[2], uu[1] * uu[1]));
      double kb = m2 * ir;
      if (NEQ >= 8 && p.mhd) kb = fma(uu[7], uu[7], fma(uu[6], uu[6], fma(uu[5], uu[5], kb)));
      double pr = fma(-0.5, kb, uu[4]) * p.inv_cv;
      const bool above = ge_pos(pr, 1e-16);
      if (!above) ++pfl;
      pr = above ? pr : 1e-16;
      if (p.eos == GCH_EOS_SINGLE_SPECIE) {
        const double t = tmax_(1.0, (pr * ir) * p.Tempsc);
        pr = r * t / p.Tempsc;
      } else if (NEQ > kNeqDyn<NEQ> && p.eos == GCH_EOS_H_RATE) {
        const double dentot = tmax_(2.0 * r - uu[kNeqDyn<NEQ>], 1e-15);
        const double t = tmax_(1.0, (pr / dentot) * p.Tempsc);
        pr = dentot * t / p.Tempsc;
      }
      prim[0] = rf;
      prim[1] = d2f_rn(uu[1]) * irf;
      prim[2] = d2f_rn(uu[2]) * irf;
      prim[3] = d2f_rn(uu[3]) * irf;
      prim[4] = d2f_rn(pr);
      if (NEQ >= 8) {
        prim[5] = d2f_rn(uu[5]);
        prim[6] = d2f_rn(uu[6]);
        prim[7] = d2f_rn(uu[7]);
      }
#pragma unroll
      for (int q = kNeqDyn<NEQ>; q < NEQ; ++q) prim[q] = d2f_rn(uu[q]);
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
    return u - f2d(flux_sum(dtdx, dtdy, dtdz, fl, fr, gl, gr, hl, hr));
  }
  // the same with a source term s: dt s joins the FP32 flux divergence in
  // one fused multiply-add (s = 0 leaves every bit as update() gives it)
  __device__ __forceinline__ static double update_src(double u, float dtdx, float dtdy,
                                                      float dtdz, float fl, float fr, float gl,
                                                      float gr, float hl, float hr, float dt,
                                                      float s) {
    return u - f2d(__fmaf_rn(-dt, s, flux_sum(dtdx, dtdy, dtdz, fl, fr, gl, gr, hl, hr)));
  }

  __device__ __forceinline__ static double ct(double u, float hdta, float a0, float a1,
                                              float hdtb, float b0, float b1, bool first_minus) {
    const float d = hdta * (a1 - a0) - hdtb * (b1 - b0);
    return first_minus ? u - f2d(d) : u + f2d(d);
  }
  // the same with a source term s (Powell's eight-wave terms): dt s joins
  // the FP32 difference in one fused multiply-add (s = 0 leaves every bit
  // as ct() gives it: u - (-x) is u + x)
  __device__ __forceinline__ static double ct_src(double u, float hdta, float a0, float a1,
                                                  float hdtb, float b0, float b1,
                                                  bool first_minus, float dt, float s) {
    const float d = hdta * (a1 - a0) - hdtb * (b1 - b0);
    return u - f2d(__fmaf_rn(-dt, s, first_minus ? d : -d));
  }
};


// ---------------------------------------------------------------------------
// FP32 with Kahan-compensated accumulation: u is a (hi, lo) FP32 pair per
// value; every per-cell operation is FP32 (no FP64 instruction on the step
// path), the pressure recovery is double-float.
template <>
struct Ops<PolKahan> {
  using TC = float;
  using R = float2;
  __device__ __forceinline__ static float2 ld(float2 u) { return u; }
  // pair + v: two-sum of the high parts, low parts folded in, renormalised
  __device__ __forceinline__ static float2 addf(float2 u, float v) {
    const DF s = two_sum(u.x, v);
    const DF r = fast_two_sum(s.hi, s.lo + u.y);
    return make_float2(r.hi, r.lo);
  }
  __device__ __forceinline__ static float2 add(float2 u, double v) { return addf(u, (float)v); }

  template <int NEQ, class TIn>
  __device__ __forceinline__ static void load_prim(const KParams& p, const TIn* src,
                                                   long long idx, TC* prim, unsigned& pfl) {
    if constexpr (sizeof(TIn) == 8) {
      float2 uu[NEQ];
#pragma unroll
      for (int q = 0; q < NEQ; ++q) uu[q] = src[q * p.fs + idx];
      prim_vals<NEQ>(p, uu, prim, pfl);
    } else {
      float uu[NEQ];
#pragma unroll
      for (int q = 0; q < NEQ; ++q) uu[q] = (float)src[q * p.fs + idx];
      prim_from_f32<NEQ>(p, uu, prim, pfl);
    }
  }

  template <int NEQ>
  __device__ __forceinline__ static void prim_vals(const KParams& p, const float2* uu, TC* prim,
                                                   unsigned& pfl) {
    {
      const float rh = tmax_(uu[0].x + uu[0].y, 1e-15f);
      const float rl = uu[0].x + uu[0].y == rh ? (uu[0].y - (rh - uu[0].x)) : 0.0f;
      float ir = 1.0f / rh;
      ir = ir * fmaf(-rh, ir, 2.0f);
      // m.m / rho as a pair quotient of pair operands
      const DF m2 = df_add(df_add(df_sq(uu[1]), df_sq(uu[2])), df_sq(uu[3]));
      const float q = __fmul_rn(m2.hi, ir);
      const float rem = (fmaf(-q, rh, m2.hi) - __fmul_rn(q, rl)) + m2.lo;
      DF kb = fast_two_sum(q, __fmul_rn(rem, ir));
      if (NEQ >= 8 && p.mhd)
        kb = df_add(kb, df_add(df_add(df_sq(uu[5]), df_sq(uu[6])), df_sq(uu[7])));
      const DF d = two_sum(uu[4].x, __fmul_rn(-0.5f, kb.hi));
      float pr = (d.hi + ((d.lo + uu[4].y) - __fmul_rn(0.5f, kb.lo))) * p.f_inv_cv;
      if (!(pr >= 1e-16f)) ++pfl;
      pr = tmax_(pr, 1e-16f);
      if (p.eos == GCH_EOS_SINGLE_SPECIE) {
        const float t = tmax_(1.0f, (pr * ir) * p.f_Tempsc);
        pr = rh * t / p.f_Tempsc;
      } else if (NEQ > kNeqDyn<NEQ> && p.eos == GCH_EOS_H_RATE) {
        const float dentot = tmax_(2.0f * rh - uu[kNeqDyn<NEQ>].x, 1e-15f);
        const float t = tmax_(1.0f, (pr / dentot) * p.f_Tempsc);
        pr = dentot * t / p.f_Tempsc;
      }
      prim[0] = rh;
      prim[1] = uu[1].x * ir;
      prim[2] = uu[2].x * ir;
      prim[3] = uu[3].x * ir;
      prim[4] = pr;
      if (NEQ >= 8) {
        prim[5] = uu[5].x;
        prim[6] = uu[6].x;
        prim[7] = uu[7].x;
      }
#pragma unroll
      for (int q = kNeqDyn<NEQ>; q < NEQ; ++q) prim[q] = uu[q].x;
    }
  }

  template <int NEQ, class TIn>
  __device__ __forceinline__ static void load_stored_prim(const KParams& p, const TIn* src,
                                                          long long idx, TC* prim) {
#pragma unroll
    for (int q = 0; q < NEQ; ++q) prim[q] = (float)src[q * p.fs + idx];
  }

  __device__ __forceinline__ static float2 update(float2 u, float dtdx, float dtdy, float dtdz,
                                                  float fl, float fr, float gl, float gr,
                                                  float hl, float hr) {
    return addf(u, -flux_sum(dtdx, dtdy, dtdz, fl, fr, gl, gr, hl, hr));
  }
  // the same with a source term s, as Ops<PolMixed>::update_src
  __device__ __forceinline__ static float2 update_src(float2 u, float dtdx, float dtdy,
                                                      float dtdz, float fl, float fr, float gl,
                                                      float gr, float hl, float hr, float dt,
                                                      float s) {
    return addf(u, -__fmaf_rn(-dt, s, flux_sum(dtdx, dtdy, dtdz, fl, fr, gl, gr, hl, hr)));
  }

  __device__ __forceinline__ static float2 ct(float2 u, float hdta, float a0, float a1,
                                              float hdtb, float b0, float b1, bool first_minus) {
    const float d = hdta * (a1 - a0) - hdtb * (b1 - b0);
    return addf(u, first_minus ? -d : d);
  }
  // the same with a source term s, as Ops<PolMixed>::ct_src
  __device__ __forceinline__ static float2 ct_src(float2 u, float hdta, float a0, float a1,
                                                  float hdtb, float b0, float b1,
                                                  bool first_minus, float dt, float s) {
    const float d = hdta * (a1 - a0) - hdtb * (b1 - b0);
    return addf(u, -__fmaf_rn(-dt, s, first_minus ? d : -d));
  }
};

}  // namespace gch
