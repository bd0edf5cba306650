// gch_device.cuh -- device-side building blocks of the GB300 timestep:
// precision policies, the kernel parameter block, array indexing, and the
// per-cell / per-interface physics of Guacho-3D restated for CUDA.
//
// Expression order follows the reference routine cited at each function
// (left to right, parentheses kept): compiled without FMA contraction
// (-fmad=false) the FP64 instantiation reproduces the reference's FP64 bits.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "guacho_gb300.h"
#include "gch_convert.h"
#include "gch_ddiv.h"
#include "gch_dsqrt.h"

namespace gch {

constexpr int NG = 2;            // ghost cells per side (OT/parameters.f90:193)
constexpr int kMaxNeq = 10;      // 8 dynamical equations + 2 passive scalars

// Equation counts (parameters.f90:131-135, 197-202): 5 dynamical equations
// (hydro) or 8 (with B), followed by npas = 0 or 2 passive scalars, so NEQ
// is one of 5, 7, 8, 10 and NEQ >= 8 exactly when B is carried.
template <int NEQ>
constexpr int kNeqDyn = NEQ >= 8 ? 8 : 5;

// Call f(std::integral_constant<int, NEQ>) for the runtime equation count
// (host side: selects the kernel instantiation).
template <class F>
inline void with_neq(int neq, F&& f) {
  switch (neq) {
    case 5: f(std::integral_constant<int, 5>()); break;
    case 7: f(std::integral_constant<int, 7>()); break;
    case 8: f(std::integral_constant<int, 8>()); break;
    case 10: f(std::integral_constant<int, 10>()); break;
    default: break;
  }
}
constexpr int TX = 32;           // stage-kernel tile width (one warp along x)
constexpr int TY = 8;            // stage-kernel tile height
constexpr int NT = TX * TY;

// ---------------------------------------------------------------------------
// Precision policies.
//   TU: storage of u (the conserved state carried between steps)
//   TS: storage of up / primit (stage state), E
//   TC: arithmetic of reconstruction, Riemann fluxes and E
struct PolFP64 {
  using TU = double;
  using TS = double;
  using TC = double;
  static constexpr int kMode = GCH_FP64;
  static constexpr int kMinBlocks = 1;   // stage kernels: blocks per SM hint
};
struct PolMixed {
  using TU = double;
  using TS = float;
  using TC = float;
  static constexpr int kMode = GCH_FP32_MIXED;
  static constexpr int kMinBlocks = 3;
};

struct PolKahan {
  using TU = float2;  // compensated (hi, lo) FP32 pair
  using TS = float;
  using TC = float;
  static constexpr int kMode = GCH_FP32_KAHAN;
  static constexpr int kMinBlocks = 3;
};

// Value conversions across the stored types: double, float, and the
// compensated pair (hi, lo) whose value is hi + lo.
__host__ __device__ __forceinline__ double to_d(double x) { return x; }
__host__ __device__ __forceinline__ double to_d(float x) { return (double)x; }
__host__ __device__ __forceinline__ double to_d(float2 x) { return (double)x.x + (double)x.y; }
template <class T>
__host__ __device__ __forceinline__ T from_d(double v);
template <>
__host__ __device__ __forceinline__ double from_d<double>(double v) { return v; }
template <>
__host__ __device__ __forceinline__ float from_d<float>(double v) { return (float)v; }
template <>
__host__ __device__ __forceinline__ float2 from_d<float2>(double v) {
  const float h = (float)v;
  return make_float2(h, (float)(v - (double)h));
}
__host__ __device__ __forceinline__ double neg(double x) { return -x; }
__host__ __device__ __forceinline__ float neg(float x) { return -x; }
__host__ __device__ __forceinline__ float2 neg(float2 x) { return make_float2(-x.x, -x.y); }
// store an accumulator value (double or pair) in a stage array type
template <class TD>
__device__ __forceinline__ TD store_as(double v) { return from_d<TD>(v); }
// FP64 u rounded to an FP32 stage state on the integer pipes (same bits)
template <>
__device__ __forceinline__ float store_as<float>(double v) { return d2f_rn(v); }
template <class TD>
__device__ __forceinline__ TD store_as(float2 v);
template <>
__device__ __forceinline__ float store_as<float>(float2 v) { return v.x + v.y; }
template <>
__device__ __forceinline__ float2 store_as<float2>(float2 v) { return v; }

// ---------------------------------------------------------------------------
// Kernel parameter block (by value; tables live in device memory).
struct KParams {
  int nx, ny, nz;             // interior cells
  int NX, NY, NZ;             // with ghosts
  int pitch;                  // elements per x row (>= NX, multiple of 4)
  long long fs;               // elements per field (pitch*NY*NZ)
  int neq;
  int mhd, pmhd;
  int solver, limiter, eos, cooling;
  int flux_cd, eight_wave, user_src;
  int bc[6];                  // left,right,bottom,top,out,in
  int bc_user;
  double dx, dy, dz;
  double cv, gamma, cfl, eta;
  double inv_cv;              // 1/cv for the mixed-precision paths
  double Tempsc, Psc, tsc;
  // cv, gamma, 1/cv, Tempsc and the cell widths rounded to FP32 once on the
  // host (round to nearest, the same value a device conversion gives): the
  // FP32 kernels read these from the parameter bank.  A conversion of the
  // FP64 value at every use would run on the FP64 pipe, and the compiler
  // re-forms such loop-invariant values per use under register pressure.
  float f_cv, f_gamma, f_inv_cv, f_Tempsc, f_dx, f_dy, f_dz;
  float f_Psc, f_tab_Tmin, f_tab_tail, f_tab_inv_dlog;
  // cooling table (device pointers)
  int ntab, tab_i0;
  double tab_inv_dlog, tab_tail, tab_Tmin;
  const double* tabT;
  const double* tabL;
  const float* tabTf;         // the same rows in FP32 (the FP32 paths)
  const float* tabLf;
  // user spheres and point masses (device pointers)
  int nsph, ngrav;
  const gch_sphere_t* sph;
  const double* grav;         // [4][ngrav]: GM, x, y, z
  const float* gravf;         // the same in FP32 (the FP32 paths)
  // TMA tensor maps of the stage sources (FP32 paths; device memory,
  // kTmaCount maps of 128 bytes, see gch_tma.cuh), null on the FP64 path
  const unsigned char* tmaps;
};

// Scalars shared by the kernels of one step, resident in device memory so a
// step can be captured in a CUDA graph without host round trips.
struct StepScalars {
  double dt;                  // dt_CFL of the step
  double time;                // simulated time
  double tprint;              // next output time
  double dtprint;
  double tmax;
  unsigned long long dtmin_bits;  // running min of the CFL reduction
  int iter;                   // currentIteration
  int n_iter;
  int dump;                   // dump flag of the last get_timestep
  int err;                    // GCH_ERR_* bits raised on the device
  int active;                 // loop condition of the device time loop
  // 1 while primit holds the primitives of the current u (interior and the
  // one-cell ghost shell), stored by get_timestep's CFL pass; cleared
  // when u changes (the end of tstep, an upload, a boundary fill)
  int prim_fresh;
  unsigned long long pfloor;  // pressure-floor hits (u2prim)
  // dt/dx, dt/dy, dt/dz of stage 1 (dtm = dt/2) and stage 2 (dt), computed
  // once per step exactly as src/hydro_solver.f90:91-93 does
  double dtd[2][3];
  // the same ratios and their halves rounded to FP32 (the FP32 kernels'
  // operands, converted once per step instead of once per thread)
  float dtdf[2][3];
  float hdtdf[2][3];
};

// Fill the per-stage ratios from sc->dt (one thread).
__device__ __forceinline__ void set_stage_ratios(StepScalars* sc, double dx, double dy,
                                                 double dz) {
  const double dtm = sc->dt / 2.0;  // src/hydro_solver.f90:152
  sc->dtd[0][0] = dtm / dx;
  sc->dtd[0][1] = dtm / dy;
  sc->dtd[0][2] = dtm / dz;
  sc->dtd[1][0] = sc->dt / dx;
  sc->dtd[1][1] = sc->dt / dy;
  sc->dtd[1][2] = sc->dt / dz;
  for (int s = 0; s < 2; ++s)
    for (int d = 0; d < 3; ++d) {
      sc->dtdf[s][d] = (float)sc->dtd[s][d];
      sc->hdtdf[s][d] = (float)(0.5 * sc->dtd[s][d]);
    }
}

__host__ __device__ inline long long cell_index(const KParams& p, int ax, int ay, int az) {
  return ((long long)az * p.NY + ay) * p.pitch + ax;
}

// ---------------------------------------------------------------------------
// Small helpers with the reference's semantics.
template <class T>
__device__ __forceinline__ T tmax_(T a, T b) { return a > b ? a : b; }
template <class T>
__device__ __forceinline__ T tmin_(T a, T b) { return a < b ? a : b; }
__device__ __forceinline__ double tcopysign(double a, double b) { return copysign(a, b); }
__device__ __forceinline__ float tcopysign(float a, float b) { return copysignf(a, b); }
// The FP64 stage kernels keep the hardware square root: the integer-pipe one
// (dsqrt_rn, same bits) made each of them about 7% slower at 256^3, its long
// dependent integer chain costing more than the FP64-pipe time it frees at
// one block per SM.  get_timestep's pass takes it (cfl_sqrt).
__device__ __forceinline__ double tsqrt(double a) { return sqrt(a); }
__device__ __forceinline__ float tsqrt(float a) { return sqrtf(a); }
__device__ __forceinline__ double tabs(double a) { return fabs(a); }
__device__ __forceinline__ float tabs(float a) { return fabsf(a); }
// Quotient with a denominator known to lie in [2^-126, 2^126]: the FP32
// paths use the hardware reciprocal (__fdividef, 2 ulp); FP64 divides
// exactly as the reference does.  The slope limiters use this one: their 24
// independent FP64 quotients per cell stay on the hardware division, since
// inlining ddiv_rn there made the latency-bound FP64 stage-2 kernel 17%
// slower (its code size and dependent integer chain), while ddiv_rn in HLLD,
// HLLC, the wave speeds and u2prim makes the FP64 step 7-11% faster.
__device__ __forceinline__ double tdiv_pos(double a, double b) { return a / b; }
__device__ __forceinline__ float tdiv_pos(float a, float b) { return __fdividef(a, b); }
// Any quotient: FP64 correctly rounded on the integer and FP32 pipes (the
// same bits as a / b); FP32 as the unit's division.
__device__ __forceinline__ double tdiv(double a, double b) { return ddiv_rn(a, b); }
__device__ __forceinline__ float tdiv(float a, float b) { return a / b; }

// The FP32 copies of the FP64 parameters (host, once per domain).
inline void set_f32_params(KParams& k) {
  k.f_cv = (float)k.cv;
  k.f_gamma = (float)k.gamma;
  k.f_inv_cv = (float)k.inv_cv;
  k.f_Tempsc = (float)k.Tempsc;
  k.f_dx = (float)k.dx;
  k.f_dy = (float)k.dy;
  k.f_dz = (float)k.dz;
  k.f_Psc = (float)k.Psc;
  k.f_tab_Tmin = (float)k.tab_Tmin;
  k.f_tab_tail = (float)k.tab_tail;
  k.f_tab_inv_dlog = (float)k.tab_inv_dlog;
}

// A parameter in the compute type T: the FP64 value, or its FP32 copy.
template <class T>
__device__ __forceinline__ T par(double d, float f) {
  if constexpr (sizeof(T) == 4) return f;
  else return d;
}

// src/hydro_core.f90:395-476  prim2f (x direction)
template <class T, int NEQ>
__device__ __forceinline__ void prim2f(const KParams& p, const T* prim, T* ff) {
  const T cv = par<T>(p.cv, p.f_cv);
  if (NEQ >= 8 && p.mhd) {
    T etot = T(0.5) * (prim[0] * (prim[1] * prim[1] + prim[2] * prim[2] + prim[3] * prim[3])
                       + prim[5] * prim[5] + prim[6] * prim[6] + prim[7] * prim[7])
             + cv * prim[4];
    ff[0] = prim[0] * prim[1];
    ff[1] = prim[0] * prim[1] * prim[1] + prim[4]
            + T(0.5) * (prim[6] * prim[6] + prim[7] * prim[7] - prim[5] * prim[5]);
    ff[2] = prim[0] * prim[1] * prim[2] - prim[5] * prim[6];
    ff[3] = prim[0] * prim[1] * prim[3] - prim[5] * prim[7];
    ff[4] = prim[1] * (etot + prim[4]
                       + T(0.5) * (prim[5] * prim[5] + prim[6] * prim[6] + prim[7] * prim[7]))
            - prim[5] * (prim[1] * prim[5] + prim[2] * prim[6] + prim[3] * prim[7]);
  } else {
    T etot = T(0.5) * prim[0] * (prim[1] * prim[1] + prim[2] * prim[2] + prim[3] * prim[3])
             + cv * prim[4];
    ff[0] = prim[0] * prim[1];
    ff[1] = prim[0] * prim[1] * prim[1] + prim[4];
    ff[2] = prim[0] * prim[1] * prim[2];
    ff[3] = prim[0] * prim[1] * prim[3];
    ff[4] = prim[1] * (etot + prim[4]);
  }
  if (NEQ >= 8) {
    ff[5] = T(0);
    ff[6] = prim[1] * prim[6] - prim[5] * prim[2];
    ff[7] = prim[1] * prim[7] - prim[5] * prim[3];
  }
#pragma unroll
  for (int q = kNeqDyn<NEQ>; q < NEQ; ++q) ff[q] = prim[q] * prim[1];  // passives, :471-473
}

// src/hydro_core.f90:331-383  prim2u
template <class T, int NEQ>
__device__ __forceinline__ void prim2u(const KParams& p, const T* prim, T* uu) {
  uu[0] = prim[0];
  uu[1] = prim[0] * prim[1];
  uu[2] = prim[0] * prim[2];
  uu[3] = prim[0] * prim[3];
  uu[4] = T(0.5) * prim[0] * (prim[1] * prim[1] + prim[2] * prim[2] + prim[3] * prim[3])
          + par<T>(p.cv, p.f_cv) * prim[4];
  if (NEQ >= 8) {
    if (p.mhd) uu[4] = uu[4] + T(0.5) * (prim[5] * prim[5] + prim[6] * prim[6] + prim[7] * prim[7]);
    uu[5] = prim[5];
    uu[6] = prim[6];
    uu[7] = prim[7];
  }
#pragma unroll
  for (int q = kNeqDyn<NEQ>; q < NEQ; ++q) uu[q] = prim[q];  // passives, :378-380
}

// src/hydro_core.f90:591-604  cfastX
template <class T>
__device__ __forceinline__ T cfastX(const KParams& p, const T* prim) {
  const T g = par<T>(p.gamma, p.f_gamma);
  T b2 = prim[5] * prim[5] + prim[6] * prim[6] + prim[7] * prim[7];
  T cs2va2 = tdiv(g * prim[4] + b2, prim[0]);
  T disc = cs2va2 * cs2va2
           - tdiv(tdiv(T(4.0) * g * prim[4] * (prim[5] * prim[5]), prim[0]), prim[0]);
  // >= 0 exactly; FP32 rounding can take it below zero where the sound
  // speed meets the normal Alfven speed (FP64 keeps the reference's value)
  if constexpr (sizeof(T) == 4) disc = tmax_(disc, T(0));
  return tsqrt(T(0.5) * (cs2va2 + tsqrt(disc)));
}

// src/hydro_core.f90:544-553  csound
template <class T>
__device__ __forceinline__ T csound(const KParams& p, T pr, T d) {
  return tsqrt(tdiv(par<T>(p.gamma, p.f_gamma) * pr, d));
}

// src/hydro_core.f90:735-796  average (slope limiter)
template <class T>
__device__ __forceinline__ T average(int lim, T a, T b) {
  T s, c, d, av, av1, av2;
  const T delta = T(1e-7);
  switch (lim) {
    case GCH_LIMITER_NO_AVERAGE: return T(0);
    case GCH_LIMITER_NO_LIMIT: return T(0.5) * (a + b);
    case GCH_LIMITER_MINMOD:
      s = tcopysign(T(1), a);
      return s * tmax_(T(0), tmin_(tabs(a), s * b));
    case GCH_LIMITER_VAN_LEER:
      // a*b > 0 (a normal number after FTZ) bounds a*a + b*b >= 2ab from
      // below; above, it is at most 2^126 while |a|, |b| < 6e18
      if (a * b <= T(0)) return T(0);
      return tdiv_pos(a * b * (a + b), a * a + b * b);
    case GCH_LIMITER_VAN_ALBADA:
      return tdiv_pos(a * (b * b + delta) + b * (a * a + delta), a * a + b * b + delta);
    case GCH_LIMITER_UMIST:
      s = tcopysign(T(1), a);
      c = T(0.25) * a + T(0.75) * b;
      d = T(0.75) * a + T(0.25) * b;
      av = tmin_(tmin_(tmin_(T(2) * tabs(a), T(2) * s * b), s * c), s * d);
      return s * tmax_(T(0), av);
    case GCH_LIMITER_WOODWARD:
      s = tcopysign(T(1), a);
      c = T(0.5) * (a + b);
      av = tmin_(tmin_(T(2) * tabs(a), T(2) * s * b), s * c);
      return s * tmax_(T(0), av);
    case GCH_LIMITER_SUPERBEE:
      s = tcopysign(T(1), b);
      av1 = tmin_(T(2) * tabs(b), s * a);
      av2 = tmin_(tabs(b), T(2) * s * a);
      return s * tmax_(tmax_(T(0), av1), av2);
  }
  return T(0);
}

// The limiter as a compile-time choice for the common ones; kLimRuntime
// dispatches on the runtime value.
constexpr int kLimRuntime = -99;
template <int LIM, class T>
__device__ __forceinline__ T average_t(int lim, T a, T b) {
  if constexpr (LIM == kLimRuntime) return average(lim, a, b);
  else return average(LIM, a, b);
}

// ---------------------------------------------------------------------------
// Riemann solvers, x direction.  `err` collects GCH_ERR_* bits.

// src/hlld.f90:48-319  prim2fhlld
template <class T, int NEQ>
__device__ __forceinline__ void hlld(const KParams& p, const T* pl, const T* pr, T* ff, int& err) {
  const T cv = par<T>(p.cv, p.f_cv);
  T csl = cfastX(p, pl);
  T csr = cfastX(p, pr);
  T sr = tmax_(pl[1] + csl, pr[1] + csr);
  T sl = tmin_(pl[1] - csl, pr[1] - csr);
  if (sl > T(0)) { prim2f<T, NEQ>(p, pl, ff); return; }
  if (sr < T(0)) { prim2f<T, NEQ>(p, pr, ff); return; }

  T bx = T(0.5) * (pl[5] + pr[5]);
  T signBx = tcopysign(T(1), bx);
  T pTL = pl[4] + T(0.5) * (bx * bx + pl[6] * pl[6] + pl[7] * pl[7]);
  T pTR = pr[4] + T(0.5) * (bx * bx + pr[6] * pr[6] + pr[7] * pr[7]);
  T slmul = sl - pl[1];
  T srmur = sr - pr[1];
  T rholul = pl[0] * pl[1];
  T rhorur = pr[0] * pr[1];
  T sM = tdiv(srmur * rhorur - slmul * rholul - pTR + pTL, srmur * pr[0] - slmul * pl[0]);
  T srmsM = sr - sM;
  T slmsM = sl - sM;
  T rhostl = tdiv(pl[0] * slmul, slmsM);
  T rhostr = tdiv(pr[0] * srmur, srmsM);
  T sstl = sM - tdiv(tabs(bx), tsqrt(rhostl));
  T sstr = sM + tdiv(tabs(bx), tsqrt(rhostr));
  T pst = tdiv(srmur * pr[0] * pTL - slmul * pl[0] * pTR
                   + pl[0] * pr[0] * srmur * slmul * (pr[1] - pl[1]),
               srmur * pr[0] - slmul * pl[0]);
  T vstl, wstl, bystl, bzstl, vstr, wstr, bystr, bzstr;

  if (sstl >= T(0)) {  // UL* region
    T el = T(0.5) * pl[0] * (pl[1] * pl[1] + pl[2] * pl[2] + pl[3] * pl[3]) + cv * pl[4]
           + T(0.5) * (bx * bx + pl[6] * pl[6] + pl[7] * pl[7]);
    T sMmul = sM - pl[1];
    T denl = pl[0] * slmul * slmsM - bx * bx;
    if (denl == T(0)) {
      vstl = pl[2]; wstl = pl[3]; bystl = T(0); bzstl = T(0);
    } else {
      vstl = pl[2] - tdiv(bx * pl[6] * sMmul, denl);
      wstl = pl[3] - tdiv(bx * pl[7] * sMmul, denl);
      bystl = tdiv(pl[6] * (pl[0] * (slmul * slmul) - bx * bx), denl);
      bzstl = tdiv(pl[7] * (pl[0] * (slmul * slmul) - bx * bx), denl);
    }
    T vdotbl = pl[1] * bx + pl[2] * pl[6] + pl[3] * pl[7];
    T vstdotbstl = sM * bx + vstl * bystl + wstl * bzstl;
    T estl = tdiv(slmul * el - pTL * pl[1] + pst * sM + bx * (vdotbl - vstdotbstl), slmsM);
    ff[0] = rhostl * sM;
    ff[1] = rhostl * (sM * sM) + pst - bx * bx;
    ff[2] = rhostl * sM * vstl - bx * bystl;
    ff[3] = rhostl * sM * wstl - bx * bzstl;
    ff[4] = sM * (estl + pst) - bx * (vstdotbstl);
    ff[5] = T(0);
    ff[6] = bystl * sM - bx * vstl;
    ff[7] = bzstl * sM - bx * wstl;
#pragma unroll
    for (int q = 8; q < NEQ; ++q) ff[q] = tdiv(sM * pl[q] * slmul, slmsM);  // :150-152
    return;
  }
  if (sstr <= T(0)) {  // UR* region
    T er = T(0.5) * pr[0] * (pr[1] * pr[1] + pr[2] * pr[2] + pr[3] * pr[3]) + cv * pr[4]
           + T(0.5) * (bx * bx + pr[6] * pr[6] + pr[7] * pr[7]);
    T sMmur = sM - pr[1];
    T denr = pr[0] * srmur * srmsM - bx * bx;
    if (denr == T(0)) {
      // the reference leaves the R star state uninitialised here
      // (src/hlld.f90:167-171); mirror the L fallback
      vstr = pr[2]; wstr = pr[3]; bystr = T(0); bzstr = T(0);
    } else {
      vstr = pr[2] - tdiv(bx * pr[6] * sMmur, denr);
      wstr = pr[3] - tdiv(bx * pr[7] * sMmur, denr);
      bystr = tdiv(pr[6] * (pr[0] * (srmur * srmur) - bx * bx), denr);
      bzstr = tdiv(pr[7] * (pr[0] * (srmur * srmur) - bx * bx), denr);
    }
    T vdotbr = pr[1] * bx + pr[2] * pr[6] + pr[3] * pr[7];
    T vstdotbstr = sM * bx + vstr * bystr + wstr * bzstr;
    T estr = tdiv(srmur * er - pTR * pr[1] + pst * sM + bx * (vdotbr - vstdotbstr), srmsM);
    ff[0] = rhostr * sM;
    ff[1] = rhostr * (sM * sM) + pst - bx * bx;
    ff[2] = rhostr * sM * vstr - bx * bystr;
    ff[3] = rhostr * sM * wstr - bx * bzstr;
    ff[4] = sM * (estr + pst) - bx * (vstdotbstr);
    ff[5] = T(0);
    ff[6] = bystr * sM - bx * vstr;
    ff[7] = bzstr * sM - bx * wstr;
#pragma unroll
    for (int q = 8; q < NEQ; ++q) ff[q] = tdiv(sM * pr[q] * srmur, srmsM);  // :198-200
    return;
  }
  T sMmul = sM - pl[1];
  T sMmur = sM - pr[1];
  T denl = pl[0] * slmul * slmsM - bx * bx;
  T denr = pr[0] * srmur * srmsM - bx * bx;
  if (denl == T(0)) {
    vstl = pl[2]; wstl = pl[3]; bystl = T(0); bzstl = T(0);
  } else {
    vstl = pl[2] - tdiv(bx * pl[6] * sMmul, denl);
    wstl = pl[3] - tdiv(bx * pl[7] * sMmul, denl);
    bystl = tdiv(pl[6] * (pl[0] * (slmul * slmul) - bx * bx), denl);
    bzstl = tdiv(pl[7] * (pl[0] * (slmul * slmul) - bx * bx), denl);
  }
  if (denr == T(0)) {
    vstr = pr[2]; wstr = pr[3]; bystr = T(0); bzstr = T(0);
  } else {
    vstr = pr[2] - tdiv(bx * pr[6] * sMmur, denr);
    wstr = pr[3] - tdiv(bx * pr[7] * sMmur, denr);
    bystr = tdiv(pr[6] * (pr[0] * (srmur * srmur) - bx * bx), denr);
    bzstr = tdiv(pr[7] * (pr[0] * (srmur * srmur) - bx * bx), denr);
  }
  T sql = tsqrt(rhostl), sqr = tsqrt(rhostr);
  T dd = sql + sqr;
  T vstst = tdiv(sql * vstl + sqr * vstr + (bystr - bystl) * signBx, dd);
  T wstst = tdiv(sql * wstl + sqr * wstr + (bzstr - bzstl) * signBx, dd);
  T sqlr = tsqrt(rhostl * rhostr);
  T bystst = tdiv(sql * bystr + sqr * bystl + sqlr * (vstr - vstl) * signBx, dd);
  T bzstst = tdiv(sql * bzstr + sqr * bzstl + sqlr * (wstr - wstl) * signBx, dd);
  T vststdotbstst = sM * bx + vstst * bystst + wstst * bzstst;
  if (sM >= T(0)) {  // UL** region
    T el = T(0.5) * pl[0] * (pl[1] * pl[1] + pl[2] * pl[2] + pl[3] * pl[3]) + cv * pl[4]
           + T(0.5) * (bx * bx + pl[6] * pl[6] + pl[7] * pl[7]);
    T vdotbl = pl[1] * bx + pl[2] * pl[6] + pl[3] * pl[7];
    T vstdotbstl = sM * bx + vstl * bystl + wstl * bzstl;
    T estl = tdiv(slmul * el - pTL * pl[1] + pst * sM + bx * (vdotbl - vstdotbstl), slmsM);
    T eststl = estl - sql * (vstdotbstl - vststdotbstst) * signBx;
    ff[0] = rhostl * sM;
    ff[1] = rhostl * (sM * sM) + pst - bx * bx;
    ff[2] = rhostl * sM * vstst - bx * bystst;
    ff[3] = rhostl * sM * wstst - bx * bzstst;
    ff[4] = sM * (eststl + pst) - bx * (vststdotbstst);
    ff[5] = T(0);
    ff[6] = bystst * sM - bx * vstst;
    ff[7] = bzstst * sM - bx * wstst;
#pragma unroll
    for (int q = 8; q < NEQ; ++q) ff[q] = tdiv(sM * pl[q] * slmul, slmsM);  // :277-279
    return;
  }
  if (sM <= T(0)) {  // UR** region
    T er = T(0.5) * pr[0] * (pr[1] * pr[1] + pr[2] * pr[2] + pr[3] * pr[3]) + cv * pr[4]
           + T(0.5) * (bx * bx + pr[6] * pr[6] + pr[7] * pr[7]);
    T vdotbr = pr[1] * bx + pr[2] * pr[6] + pr[3] * pr[7];
    T vstdotbstr = sM * bx + vstr * bystr + wstr * bzstr;
    T estr = tdiv(srmur * er - pTR * pr[1] + pst * sM + bx * (vdotbr - vstdotbstr), srmsM);
    T eststr = estr + sqr * (vstdotbstr - vststdotbstst) * signBx;
    ff[0] = rhostr * sM;
    ff[1] = rhostr * (sM * sM) + pst - bx * bx;
    ff[2] = rhostr * sM * vstst - bx * bystst;
    ff[3] = rhostr * sM * wstst - bx * bzstst;
    ff[4] = sM * (eststr + pst) - bx * (vststdotbstst);
    ff[5] = T(0);
    ff[6] = bystst * sM - bx * vstst;
    ff[7] = bzstst * sM - bx * wstst;
#pragma unroll
    for (int q = 8; q < NEQ; ++q) ff[q] = tdiv(sM * pr[q] * srmur, srmsM);  // :308-310
    return;
  }
  // src/hlld.f90:316-317 prints and stops here (sM not finite)
  for (int q = 0; q < NEQ; ++q) ff[q] = sM;
  err |= GCH_ERR_HLLD;
}

// Paired FP32 arithmetic: the left and right states of an interface in the
// two lanes of a float2, one paired FP32 operation (__fadd2_rn, __fmul2_rn,
// __ffma2_rn) for both.
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
  return __fadd2_rn(a, make_float2(-b.x, -b.y));
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// Limited linear reconstruction of one x or y face (src/hydro_core.f90:
// 712-733 limiter) for the FP32 paths with minmod or van Leer: the left
// state l + avg(l-ll, r-l)/2 and the right state r - avg(r-l, rr-r)/2 in the
// two lanes of float2 operations.  Both limiters are symmetric in their
// arguments, so the right slope is formed as avg(rr-r, r-l), the same
// expression as the left one with the outer difference first.
template <int LIM>
__device__ __forceinline__ float2 muscl_pair(float ll, float l, float r, float rr) {
  const float2 d = f2(l - ll, rr - r);  // outer differences
  const float2 m = f2(r - l);           // the centred difference, both lanes
  float2 s;
  if constexpr (LIM == GCH_LIMITER_VAN_LEER) {
    const float2 ab = mul2(d, m);
    const float2 num = mul2(ab, add2(d, m));
    const float2 den = fma2(d, d, mul2(m, m));
    s = f2(ab.x <= 0.0f ? 0.0f : __fdividef(num.x, den.x),
           ab.y <= 0.0f ? 0.0f : __fdividef(num.y, den.y));
  } else {  // minmod: sign(a) * max(0, min(|a|, sign(a) b))
    const float2 sg = f2(copysignf(1.0f, d.x), copysignf(1.0f, d.y));
    const float2 t = mul2(sg, m);
    s = mul2(sg, f2(tmax_(0.0f, tmin_(fabsf(d.x), t.x)), tmax_(0.0f, tmin_(fabsf(d.y), t.y))));
  }
  return fma2(f2(0.5f, -0.5f), s, f2(l, r));
}

// HLLD for the FP32 paths: the Miyoshi-Kusano states of hlld() above
// (src/hlld.f90:48-319), but
//  - the four star regions are selected by predicates instead of branches,
//    so a warp whose faces fall in different regions runs one instruction
//    stream: both single-star states and the double-star state are formed,
//    then the energy and the flux of the selected side, with the
//    reference's expressions;
//  - the left/right-symmetric work (fast speeds, total pressures, star
//    densities, single-star states) runs in the two lanes of float2
//    operations, one paired instruction for both sides (measured: 4-7%
//    fewer instructions in the stage kernels);
//  - quotients by the same denominator share one hardware reciprocal.
template <int NEQ>
__device__ __forceinline__ void hlld_pair(const KParams& p, const float* pl, const float* pr,
                                          float* ff, int& err) {
  const float cv = p.f_cv, g = p.f_gamma;
  const float2 rho = f2(pl[0], pr[0]), vx = f2(pl[1], pr[1]);
  const float2 vy = f2(pl[2], pr[2]), vz = f2(pl[3], pr[3]), pg = f2(pl[4], pr[4]);
  const float2 bn = f2(pl[5], pr[5]), by = f2(pl[6], pr[6]), bz = f2(pl[7], pr[7]);
  // cfastX of both states (src/hydro_core.f90:591-604)
  const float2 irho = f2(1.0f / pl[0], 1.0f / pr[0]);
  const float2 gp = mul2(f2(g), pg);
  const float2 btt = fma2(by, by, mul2(bz, bz));
  const float2 cs2va2 = mul2(add2(gp, fma2(bn, bn, btt)), irho);
  const float2 t4 = mul2(mul2(f2(4.0f), gp), mul2(mul2(bn, bn), mul2(irho, irho)));
  // (cs^2 + va^2)^2 - 4 cs^2 va_n^2 = (cs^2 - va_n^2)^2 + 4 cs^2 va_t^2 >= 0;
  // FP32 rounding can take it below zero where cs ~ va_n, so it is clamped
  const float2 disc = fma2(cs2va2, cs2va2, f2(-t4.x, -t4.y));
  const float2 h = mul2(f2(0.5f), add2(cs2va2, f2(sqrtf(fmaxf(disc.x, 0.0f)),
                                                  sqrtf(fmaxf(disc.y, 0.0f)))));
  const float2 cf = f2(sqrtf(h.x), sqrtf(h.y));
  const float2 lo = sub2(vx, cf), hi = add2(vx, cf);
  const float sl = tmin_(lo.x, lo.y), sr = tmax_(hi.x, hi.y);
  if (sl > 0.0f) { prim2f<float, NEQ>(p, pl, ff); return; }
  if (sr < 0.0f) { prim2f<float, NEQ>(p, pr, ff); return; }

  const float bx = 0.5f * (pl[5] + pr[5]);
  const float signBx = copysignf(1.0f, bx);
  const float bx2 = bx * bx;
  const float2 pT = fma2(f2(0.5f), add2(f2(bx2), btt), pg);  // total pressures
  const float2 sv = f2(sl, sr);
  const float2 smu = sub2(sv, vx);                           // S - u
  const float2 m = mul2(smu, rho);                           // rho (S - u)
  const float iden = 1.0f / (m.y - m.x);
  const float2 mv = mul2(m, vx);
  const float sM = (mv.y - mv.x - pT.y + pT.x) * iden;
  const float2 ssM = sub2(sv, f2(sM));                       // S - sM
  const float2 rhost = mul2(m, f2(1.0f / ssM.x, 1.0f / ssM.y));
  const float2 isq = f2(rsqrtf(rhost.x), rsqrtf(rhost.y));
  const float2 sq = mul2(rhost, isq);                        // sqrt(rho*)
  const float abx = fabsf(bx);
  const float sstl = sM - abx * isq.x, sstr = sM + abx * isq.y;
  const float pst = (m.y * pT.x - m.x * pT.y + m.x * m.y * (pr[1] - pl[1])) * iden;
  // single-star states with the reference's den == 0 fallbacks
  const float2 dlr = fma2(m, ssM, f2(-bx2));
  const float2 id = f2(dlr.x == 0.0f ? 0.0f : 1.0f / dlr.x, dlr.y == 0.0f ? 0.0f : 1.0f / dlr.y);
  const float2 sMmu = sub2(f2(sM), vx);
  const float2 fb = mul2(fma2(m, smu, f2(-bx2)), id);
  const float2 t1 = mul2(mul2(f2(bx), sMmu), id);
  const float2 vst = fma2(f2(-by.x, -by.y), t1, vy);
  const float2 wst = fma2(f2(-bz.x, -bz.y), t1, vz);
  const float2 byst = mul2(by, fb), bzst = mul2(bz, fb);
  // region: UL* | UR* | UL** | UR**
  const bool star_l = sstl >= 0.0f;
  const bool star_r = !star_l && sstr <= 0.0f;
  const bool dbl = !star_l && !star_r;
  const bool left = star_l || (dbl && sM >= 0.0f);
  if (dbl && !(sM >= 0.0f) && !(sM <= 0.0f)) {  // src/hlld.f90:316-317
#pragma unroll
    for (int q = 0; q < NEQ; ++q) ff[q] = sM;
    err |= GCH_ERR_HLLD;
    return;
  }
  // double-star state
  const float idd = 1.0f / (sq.x + sq.y);
  const float sqlr = sq.x * sq.y;
  const float2 av = mul2(sq, vst), aw = mul2(sq, wst);
  const float2 ab = mul2(sq, f2(byst.y, byst.x)), ac = mul2(sq, f2(bzst.y, bzst.x));
  const float vstst = (av.x + av.y + (byst.y - byst.x) * signBx) * idd;
  const float wstst = (aw.x + aw.y + (bzst.y - bzst.x) * signBx) * idd;
  const float bystst = (ab.x + ab.y + sqlr * (vst.y - vst.x) * signBx) * idd;
  const float bzstst = (ac.x + ac.y + sqlr * (wst.y - wst.x) * signBx) * idd;
  const float vststdotbstst = sM * bx + vstst * bystst + wstst * bzstst;
  // the selected side's single-star energy
  const float q0 = left ? pl[0] : pr[0], q1 = left ? pl[1] : pr[1];
  const float q2 = left ? pl[2] : pr[2], q3 = left ? pl[3] : pr[3];
  const float q4 = left ? pl[4] : pr[4], q6 = left ? pl[6] : pr[6], q7 = left ? pl[7] : pr[7];
  const float smu_s = left ? smu.x : smu.y, ssM_s = left ? ssM.x : ssM.y;
  const float pT_s = left ? pT.x : pT.y, rhos = left ? rhost.x : rhost.y;
  const float vst_s = left ? vst.x : vst.y, wst_s = left ? wst.x : wst.y;
  const float byst_s = left ? byst.x : byst.y, bzst_s = left ? bzst.x : bzst.y;
  const float e = 0.5f * q0 * (q1 * q1 + q2 * q2 + q3 * q3) + cv * q4
                  + 0.5f * (bx2 + q6 * q6 + q7 * q7);
  const float vdotb = q1 * bx + q2 * q6 + q3 * q7;
  const float vstdotbst = sM * bx + vst_s * byst_s + wst_s * bzst_s;
  const float est = (smu_s * e - pT_s * q1 + pst * sM + bx * (vdotb - vstdotbst)) / ssM_s;
  const float sqs = left ? -sq.x : sq.y;
  const float ex = dbl ? est + sqs * (vstdotbst - vststdotbstst) * signBx : est;
  const float vx_ = dbl ? vstst : vst_s, wx_ = dbl ? wstst : wst_s;
  const float byx = dbl ? bystst : byst_s, bzx = dbl ? bzstst : bzst_s;
  const float vbx = dbl ? vststdotbstst : vstdotbst;
  ff[0] = rhos * sM;
  ff[1] = rhos * (sM * sM) + pst - bx2;
  ff[2] = rhos * sM * vx_ - bx * byx;
  ff[3] = rhos * sM * wx_ - bx * bzx;
  ff[4] = sM * (ex + pst) - bx * vbx;
  ff[5] = 0.0f;
  ff[6] = byx * sM - bx * vx_;
  ff[7] = bzx * sM - bx * wx_;
  // passives: the star density of the side (src/hlld.f90:150-152, 198-200)
#pragma unroll
  for (int q = 8; q < NEQ; ++q) ff[q] = sM * (left ? pl[q] : pr[q]) * smu_s / ssM_s;
}

// src/hllc.f90:44-140  prim2fhllc (hydro, or passive B when NEQ == 8)
template <class T, int NEQ>
__device__ __forceinline__ void hllc(const KParams& p, const T* pl, const T* pr, T* ff, int& err) {
  const T cv = par<T>(p.cv, p.f_cv);
  T csl = csound(p, pl[4], pl[0]);
  T csr = csound(p, pr[4], pr[0]);
  T sr = tmax_(pl[1] + csl, pr[1] + csr);
  T sl = tmin_(pl[1] - csl, pr[1] - csr);
  if (sl > T(0)) { prim2f<T, NEQ>(p, pl, ff); return; }
  if (sr < T(0)) { prim2f<T, NEQ>(p, pr, ff); return; }
  T slmul = sl - pl[1];
  T srmur = sr - pr[1];
  T rholul = pl[0] * pl[1];
  T rhorur = pr[0] * pr[1];
  T sst = tdiv(srmur * rhorur - slmul * rholul - pr[4] + pl[4], srmur * pr[0] - slmul * pl[0]);
  T uu[NEQ], uuk[NEQ];
  if (sst >= T(0)) {
    T rhost = tdiv(pl[0] * (slmul), sl - sst);
    T ek = T(0.5) * pl[0] * (pl[1] * pl[1] + pl[2] * pl[2] + pl[3] * pl[3]) + cv * pl[4];
    uuk[0] = rhost;
    uuk[1] = rhost * sst;
    uuk[2] = rhost * pl[2];
    uuk[3] = rhost * pl[3];
    uuk[4] = rhost * (tdiv(ek, pl[0]) + (sst - pl[1]) * (sst + tdiv(pl[4], pl[0] * slmul)));
    if (NEQ >= 8) {
      uuk[5] = tdiv(rhost * pl[5], pl[0]);
      uuk[6] = tdiv(rhost * pl[6], pl[0]);
      uuk[7] = tdiv(rhost * pl[7], pl[0]);
    }
#pragma unroll
    for (int q = kNeqDyn<NEQ>; q < NEQ; ++q) uuk[q] = tdiv(rhost * pl[q], pl[0]);  // :95-97
    prim2f<T, NEQ>(p, pl, ff);
    prim2u<T, NEQ>(p, pl, uu);
#pragma unroll
    for (int q = 0; q < NEQ; ++q) ff[q] = ff[q] + sl * (uuk[q] - uu[q]);
    return;
  }
  if (sst <= T(0)) {
    T rhost = tdiv(pr[0] * (srmur), sr - sst);
    T ek = T(0.5) * pr[0] * (pr[1] * pr[1] + pr[2] * pr[2] + pr[3] * pr[3]) + cv * pr[4];
    uuk[0] = rhost;
    uuk[1] = rhost * sst;
    uuk[2] = rhost * pr[2];
    uuk[3] = rhost * pr[3];
    uuk[4] = rhost * (tdiv(ek, pr[0]) + (sst - pr[1]) * (sst + tdiv(pr[4], pr[0] * srmur)));
    if (NEQ >= 8) {
      uuk[5] = tdiv(rhost * pr[5], pr[0]);
      uuk[6] = tdiv(rhost * pr[6], pr[0]);
      uuk[7] = tdiv(rhost * pr[7], pr[0]);
    }
#pragma unroll
    for (int q = kNeqDyn<NEQ>; q < NEQ; ++q) uuk[q] = tdiv(rhost * pr[q], pr[0]);  // :124-126
    prim2f<T, NEQ>(p, pr, ff);
    prim2u<T, NEQ>(p, pr, uu);
#pragma unroll
    for (int q = 0; q < NEQ; ++q) ff[q] = ff[q] + sr * (uuk[q] - uu[q]);
    return;
  }
  // src/hllc.f90:135-138 prints and stops here
#pragma unroll
  for (int q = 0; q < NEQ; ++q) ff[q] = sst;
  err |= GCH_ERR_HLLC;
}

// src/hlle.f90:48-83 (FAST=true, MHD) and src/hll.f90:47-82 (FAST=false)
template <class T, int NEQ, bool FAST>
__device__ __forceinline__ void hll2(const KParams& p, const T* pl, const T* pr, T* ff) {
  T csl, csr;
  if (FAST) {
    csl = cfastX(p, pl);
    csr = cfastX(p, pr);
  } else {
    csl = csound(p, pl[4], pl[0]);
    csr = csound(p, pr[4], pr[0]);
  }
  T sr = tmax_(pl[1] + csl, pr[1] + csr);
  T sl = tmin_(pl[1] - csl, pr[1] - csr);
  if (sl > T(0)) { prim2f<T, NEQ>(p, pl, ff); return; }
  if (sr < T(0)) { prim2f<T, NEQ>(p, pr, ff); return; }
  T fL[NEQ], fR[NEQ], uL[NEQ], uR[NEQ];
  prim2f<T, NEQ>(p, pl, fL);
  prim2f<T, NEQ>(p, pr, fR);
  prim2u<T, NEQ>(p, pl, uL);
  prim2u<T, NEQ>(p, pr, uR);
#pragma unroll
  for (int q = 0; q < NEQ; ++q)
    ff[q] = (sr * fL[q] - sl * fR[q] + sl * sr * (uR[q] - uL[q])) / (sr - sl);
}

template <int SOLVER, int NEQ>
struct Riemann;
template <int NEQ>
struct Riemann<GCH_SOLVER_HLLD, NEQ> {
  static_assert(NEQ >= 8, "HLLD needs B");
  template <class T>
  __device__ __forceinline__ static void solve(const KParams& p, const T* l, const T* r, T* f,
                                               int& e) {
    if constexpr (sizeof(T) == 4)
      hlld_pair<NEQ>(p, l, r, f, e);  // FP32 paths: predicated regions, paired sides
    else
      hlld<T, NEQ>(p, l, r, f, e);    // FP64: the reference's branch order
  }
};
template <int NEQ>
struct Riemann<GCH_SOLVER_HLLC, NEQ> {
  template <class T>
  __device__ __forceinline__ static void solve(const KParams& p, const T* l, const T* r, T* f,
                                               int& e) {
    hllc<T, NEQ>(p, l, r, f, e);
  }
};
template <int NEQ>
struct Riemann<GCH_SOLVER_HLLE, NEQ> {
  static_assert(NEQ >= 8, "HLLE uses the fast magnetosonic speed");
  template <class T>
  __device__ __forceinline__ static void solve(const KParams& p, const T* l, const T* r, T* f,
                                               int&) {
    hll2<T, NEQ, true>(p, l, r, f);
  }
};
template <int NEQ>
struct Riemann<GCH_SOLVER_HLL, NEQ> {
  template <class T>
  __device__ __forceinline__ static void solve(const KParams& p, const T* l, const T* r, T* f,
                                               int&) {
    hll2<T, NEQ, false>(p, l, r, f);
  }
};

// ---------------------------------------------------------------------------
// Field permutations of swapy / swapz (src/hydro_core.f90:485-534):
// component q of the rotated state is component perm(q) of the original.
// Passive scalars are not permuted; B is only where it is carried.
template <int DIR, int NEQ>
__device__ __forceinline__ int perm(int q) {
  constexpr bool b = NEQ >= 8;
  if (DIR == 1) return q == 1 ? 2 : q == 2 ? 1 : (b && q == 5) ? 6 : (b && q == 6) ? 5 : q;
  if (DIR == 2) return q == 1 ? 3 : q == 3 ? 1 : (b && q == 5) ? 7 : (b && q == 7) ? 5 : q;
  return q;
}

// ---------------------------------------------------------------------------
// Ghost mapping.  For an array coordinate c (0..N-1, interior NG..NG+n-1)
// return the coordinate whose value a ghost cell holds after the boundary
// fill, and whether the normal component flips sign (closed walls).
// `layers` = 1 follows boundaryI (src/boundaries.f90:44-247), 2 boundaryII
// (:256-512), both equal for layer 1.
__device__ __forceinline__ int ghost_src(int c, int n, int bclo, int bchi, bool& flip) {
  flip = false;
  if (c < NG) {
    int l = NG - 1 - c;  // 0 for the first ghost layer
    if (bclo == GCH_BC_PERIODIC) return NG + n - 1 - l;
    if (bclo == GCH_BC_CLOSED) flip = true;
    return NG + l;
  }
  if (c >= NG + n) {
    int l = c - (NG + n);
    if (bchi == GCH_BC_PERIODIC) return NG + l;
    if (bchi == GCH_BC_CLOSED) flip = true;
    return NG + n - 1 - l;
  }
  return c;
}

// EXO/exoplanet.f90:156-158 cell position measured from the grid centre
__device__ __forceinline__ double cell_pos(int a, int n, double d) {
  int i = a - NG + 1;  // Fortran index
  return ((double)(i - n / 2) + 0.5) * d;
}

}  // namespace gch
