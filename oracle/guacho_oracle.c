/*
 * guacho_oracle.c -- CPU (FP64) restatement of Guacho-3D's per-timestep update.
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker for the CUDA path.  Only the
 * tests, the smoke check and the CPU-baseline leg of the benchmark load it.
 *
 * Every routine restates the reference routine cited beside it, in the same
 * loop order and with the same floating-point expression order (left to right,
 * parentheses kept), so that a build with -O2 -ffp-contract=off reproduces the
 * bits of gfortran -O3 -fdefault-real-8 on x86-64 (which has no FMA in its
 * baseline ISA).  Citations are file:line within the reference project.
 *
 * Deliberate deviations, each also recorded in the design notes:
 *  - HLLD, UR* region with denr == 0 (src/hlld.f90:167-171) assigns the L
 *    star variables and then reads the uninitialised R ones.  Here the R
 *    fallback mirrors the L one: vstr=primr(3), wstr=primr(4), bystr=bzstr=0.
 *  - The table lookup of the cooling curve (src/cooling_dmc.f90:98-102) reads
 *    one row past the table end when log10(T) rounds to exactly 8; the row
 *    index is clamped to the last interval here.
 *  - Ghost filling uses the serial (non-MPI) semantics of src/boundaries.f90
 *    (x, then y, then z faces).  The MPI build fills edge/corner ghosts in a
 *    different order; no interior result reads an edge or corner ghost.
 *  - The serial build of the E-field periodic branch does not compile in the
 *    reference (src/flux_cd_module.f90:120-128, unclosed if); the intended
 *    periodic copy is restated.
 */
#include "guacho_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NG 2

struct gor_state {
  gor_params_t p;
  int NX, NY, NZ;     /* with ghosts */
  size_t ncell;
  double *u, *up, *primit, *f, *g, *h, *e;
  double* primit0;    /* split solver background (src/globals.f90:42), else NULL */
  double* temp;       /* Temp (src/globals.f90), filled by calcprim */
  double time;
  int err;
};

/* cell index for 1-based interior coordinates i in [1-NG, n+NG] */
#define CID(s, i, j, k) \
  ((size_t)((k) + NG - 1) * (size_t)(s)->NY * (size_t)(s)->NX + \
   (size_t)((j) + NG - 1) * (size_t)(s)->NX + (size_t)((i) + NG - 1))
#define AT(s, arr, q, i, j, k) ((arr)[CID(s, i, j, k) * (size_t)(s)->p.neq + (q) - 1])
#define EAT(s, q, i, j, k) ((s)->e[CID(s, i, j, k) * 3 + (q) - 1])

static inline double dmax(double a, double b) { return a > b ? a : b; }
static inline double dmin(double a, double b) { return a < b ? a : b; }
static inline int neqdyn(const gor_params_t* p) { return p->neq - p->npas; }
static inline int bfield(const gor_params_t* p) { return neqdyn(p) >= 8; }

/* ---------------------------------------------------------------------- */
/* src/hydro_core.f90:46-129  u2prim                                        */
static void u2prim(const gor_params_t* p, const double* uu, double* prim, double* T) {
  double r = dmax(uu[0], 1e-15);
  prim[0] = r;
  prim[1] = uu[1] / r;
  prim[2] = uu[2] / r;
  prim[3] = uu[3] / r;
  if (p->mhd) {
    prim[4] = (uu[4] - 0.5 * r * (prim[1] * prim[1] + prim[2] * prim[2] + prim[3] * prim[3])
               - 0.5 * (uu[5] * uu[5] + uu[6] * uu[6] + uu[7] * uu[7])) / p->cv;
  } else {
    prim[4] = (uu[4] - 0.5 * r * (prim[1] * prim[1] + prim[2] * prim[2] + prim[3] * prim[3]))
              / p->cv;
  }
  prim[4] = dmax(prim[4], 1e-16);
  if (bfield(p) && (p->mhd || p->pmhd)) {
    prim[5] = uu[5];
    prim[6] = uu[6];
    prim[7] = uu[7];
  }
  const int nd = neqdyn(p);
  for (int q = nd; q < p->neq; ++q) prim[q] = uu[q];  /* passives (:86-89) */
  double t = 0.0;
  if (p->eq_of_state == GOR_EOS_ADIABATIC) t = (prim[4] / r) * p->Tempsc;
  if (p->eq_of_state == GOR_EOS_SINGLE_SPECIE) {
    r = dmax(r, 1e-15);
    t = dmax(1.0, (prim[4] / r) * p->Tempsc);
    prim[4] = r * t / p->Tempsc;
  }
  if (p->eq_of_state == GOR_EOS_H_RATE && p->npas > 0) {
    /* :106-111: n_HI + 2 n_HII = 2 rho - n_HI particles */
    double dentot = (2.0 * r - prim[nd]);
    dentot = dmax(dentot, 1e-15);
    t = dmax(1.0, (prim[4] / dentot) * p->Tempsc);
    prim[4] = dentot * t / p->Tempsc;
  }
  if (T) *T = t;
}

/* src/hydro_core.f90:331-383  prim2u (non-split branch) */
static void prim2u(const gor_params_t* p, const double* prim, double* uu) {
  uu[0] = prim[0];
  uu[1] = prim[0] * prim[1];
  uu[2] = prim[0] * prim[2];
  uu[3] = prim[0] * prim[3];
  uu[4] = 0.5 * prim[0] * (prim[1] * prim[1] + prim[2] * prim[2] + prim[3] * prim[3])
          + p->cv * prim[4];
  if (bfield(p) && p->mhd)
    uu[4] = uu[4] + 0.5 * (prim[5] * prim[5] + prim[6] * prim[6] + prim[7] * prim[7]);
  if (bfield(p) && (p->mhd || p->pmhd)) {
    uu[5] = prim[5];
    uu[6] = prim[6];
    uu[7] = prim[7];
  }
  for (int q = neqdyn(p); q < p->neq; ++q) uu[q] = prim[q];  /* :378-380 */
}

/* src/hydro_core.f90:395-476  prim2f (non-split branch) */
static void prim2f(const gor_params_t* p, const double* prim, double* ff) {
  if (p->mhd) {
    double etot = 0.5 * (prim[0] * (prim[1] * prim[1] + prim[2] * prim[2] + prim[3] * prim[3])
                         + prim[5] * prim[5] + prim[6] * prim[6] + prim[7] * prim[7])
                  + p->cv * prim[4];
    ff[0] = prim[0] * prim[1];
    ff[1] = prim[0] * prim[1] * prim[1] + prim[4]
            + 0.5 * (prim[6] * prim[6] + prim[7] * prim[7] - prim[5] * prim[5]);
    ff[2] = prim[0] * prim[1] * prim[2] - prim[5] * prim[6];
    ff[3] = prim[0] * prim[1] * prim[3] - prim[5] * prim[7];
    ff[4] = prim[1] * (etot + prim[4] + 0.5 * (prim[5] * prim[5] + prim[6] * prim[6]
                                               + prim[7] * prim[7]))
            - prim[5] * (prim[1] * prim[5] + prim[2] * prim[6] + prim[3] * prim[7]);
  } else {
    double etot = 0.5 * prim[0] * (prim[1] * prim[1] + prim[2] * prim[2] + prim[3] * prim[3])
                  + p->cv * prim[4];
    ff[0] = prim[0] * prim[1];
    ff[1] = prim[0] * prim[1] * prim[1] + prim[4];
    ff[2] = prim[0] * prim[1] * prim[2];
    ff[3] = prim[0] * prim[1] * prim[3];
    ff[4] = prim[1] * (etot + prim[4]);
  }
  if (bfield(p) && (p->mhd || p->pmhd)) {
    ff[5] = 0.0;
    ff[6] = prim[1] * prim[6] - prim[5] * prim[2];
    ff[7] = prim[1] * prim[7] - prim[5] * prim[3];
  }
  for (int q = neqdyn(p); q < p->neq; ++q) ff[q] = prim[q] * prim[1];  /* :471-473 */
}

/* src/hydro_core.f90:485-534  swapy / swapz */
static void swapy(const gor_params_t* p, double* v) {
  double a = v[1]; v[1] = v[2]; v[2] = a;
  if (bfield(p) && (p->mhd || p->pmhd)) { a = v[5]; v[5] = v[6]; v[6] = a; }
}
static void swapz(const gor_params_t* p, double* v) {
  double a = v[1]; v[1] = v[3]; v[3] = a;
  if (bfield(p) && (p->mhd || p->pmhd)) { a = v[5]; v[5] = v[7]; v[7] = a; }
}

/* src/hydro_core.f90:544-553  csound */
static inline double csound(const gor_params_t* p, double pr, double d) {
  return sqrt(p->gamma * pr / d);
}

/* src/hydro_core.f90:568-581  cfast */
static void cfast(const gor_params_t* p, double pr, double d, double bx, double by, double bz,
                  double* cfx, double* cfy, double* cfz) {
  double g = p->gamma;
  double b2 = bx * bx + by * by + bz * bz;
  double a = g * pr + b2;
  *cfx = sqrt(0.5 * (a + sqrt(a * a - 4.0 * g * pr * bx * bx)) / d);
  *cfy = sqrt(0.5 * (a + sqrt(a * a - 4.0 * g * pr * by * by)) / d);
  *cfz = sqrt(0.5 * (a + sqrt(a * a - 4.0 * g * pr * bz * bz)) / d);
}

/* src/hydro_core.f90:591-604  cfastX */
static inline double cfastX(const gor_params_t* p, const double* prim) {
  double g = p->gamma;
  double b2 = prim[5] * prim[5] + prim[6] * prim[6] + prim[7] * prim[7];
  double cs2va2 = (g * prim[4] + b2) / prim[0];
  return sqrt(0.5 * (cs2va2 + sqrt(cs2va2 * cs2va2
                                   - 4.0 * g * prim[4] * (prim[5] * prim[5]) / prim[0] / prim[0])));
}

/* src/hydro_core.f90:735-796  average (the slope limiter switch) */
static inline double average(int lim, double a, double b) {
  double s, c, d, av, av1, av2;
  const double delta = 1e-7;
  switch (lim) {
    case GOR_LIMITER_NO_AVERAGE: return 0.0;
    case GOR_LIMITER_NO_LIMIT: return 0.5 * (a + b);
    case GOR_LIMITER_MINMOD:
      s = copysign(1.0, a);
      return s * dmax(0.0, dmin(fabs(a), s * b));
    case GOR_LIMITER_VAN_LEER:
      if (a * b <= 0.0) return 0.0;
      return a * b * (a + b) / (a * a + b * b);
    case GOR_LIMITER_VAN_ALBADA:
      return (a * (b * b + delta) + b * (a * a + delta)) / (a * a + b * b + delta);
    case GOR_LIMITER_UMIST:
      s = copysign(1.0, a);
      c = 0.25 * a + 0.75 * b;
      d = 0.75 * a + 0.25 * b;
      av = dmin(dmin(dmin(2.0 * fabs(a), 2.0 * s * b), s * c), s * d);
      return s * dmax(0.0, av);
    case GOR_LIMITER_WOODWARD:
      s = copysign(1.0, a);
      c = 0.5 * (a + b);
      av = dmin(dmin(2.0 * fabs(a), 2.0 * s * b), s * c);
      return s * dmax(0.0, av);
    case GOR_LIMITER_SUPERBEE:
      s = copysign(1.0, b);
      av1 = dmin(2.0 * fabs(b), s * a);
      av2 = dmin(fabs(b), 2.0 * s * a);
      return s * dmax(dmax(0.0, av1), av2);
  }
  return 0.0;
}

/* src/hydro_core.f90:712-731  limiter */
static void limiter(const gor_params_t* p, const double* pll, double* pl, double* pr,
                    const double* prr) {
  for (int q = 0; q < p->neq; ++q) {
    double dl = pl[q] - pll[q];
    double dm = pr[q] - pl[q];
    double dr = prr[q] - pr[q];
    double al = average(p->slope_limiter, dl, dm);
    double ar = average(p->slope_limiter, dm, dr);
    pl[q] = pl[q] + al * 0.5;
    pr[q] = pr[q] - ar * 0.5;
  }
}

/* ---------------------------------------------------------------------- */
/* src/hlld.f90:48-319  prim2fhlld */
static void prim2fhlld(const gor_params_t* p, const double* pl, const double* pr, double* ff,
                       int* err) {
  const double cv = p->cv;
  double csl = cfastX(p, pl);
  double csr = cfastX(p, pr);
  double sr = dmax(pl[1] + csl, pr[1] + csr);
  double sl = dmin(pl[1] - csl, pr[1] - csr);
  if (sl > 0) { prim2f(p, pl, ff); return; }
  if (sr < 0) { prim2f(p, pr, ff); return; }

  double bx = 0.5 * (pl[5] + pr[5]);
  double signBx = copysign(1.0, bx);
  double pTL = pl[4] + 0.5 * (bx * bx + pl[6] * pl[6] + pl[7] * pl[7]);
  double pTR = pr[4] + 0.5 * (bx * bx + pr[6] * pr[6] + pr[7] * pr[7]);
  double slmul = sl - pl[1];
  double srmur = sr - pr[1];
  double rholul = pl[0] * pl[1];
  double rhorur = pr[0] * pr[1];
  double sM = (srmur * rhorur - slmul * rholul - pTR + pTL) / (srmur * pr[0] - slmul * pl[0]);
  double srmsM = sr - sM;
  double slmsM = sl - sM;
  double rhostl = pl[0] * slmul / slmsM;
  double rhostr = pr[0] * srmur / srmsM;
  double sstl = sM - fabs(bx) / sqrt(rhostl);
  double sstr = sM + fabs(bx) / sqrt(rhostr);
  double pst = (srmur * pr[0] * pTL - slmul * pl[0] * pTR
                + pl[0] * pr[0] * srmur * slmul * (pr[1] - pl[1]))
               / (srmur * pr[0] - slmul * pl[0]);
  double vstl, wstl, bystl, bzstl, vstr, wstr, bystr, bzstr;
  double el, er, denl, denr, sMmul, sMmur, vdotbl, vdotbr, vstdotbstl, vstdotbstr, estl, estr;

  /* UL* region */
  if (sstl >= 0) {
    el = 0.5 * pl[0] * (pl[1] * pl[1] + pl[2] * pl[2] + pl[3] * pl[3]) + cv * pl[4]
         + 0.5 * (bx * bx + pl[6] * pl[6] + pl[7] * pl[7]);
    sMmul = sM - pl[1];
    denl = pl[0] * slmul * slmsM - bx * bx;
    if (denl == 0) {
      vstl = pl[2]; wstl = pl[3]; bystl = 0.0; bzstl = 0.0;
    } else {
      vstl = pl[2] - bx * pl[6] * sMmul / denl;
      wstl = pl[3] - bx * pl[7] * sMmul / denl;
      bystl = pl[6] * (pl[0] * (slmul * slmul) - bx * bx) / denl;
      bzstl = pl[7] * (pl[0] * (slmul * slmul) - bx * bx) / denl;
    }
    vdotbl = pl[1] * bx + pl[2] * pl[6] + pl[3] * pl[7];
    vstdotbstl = sM * bx + vstl * bystl + wstl * bzstl;
    estl = (slmul * el - pTL * pl[1] + pst * sM + bx * (vdotbl - vstdotbstl)) / slmsM;
    ff[0] = rhostl * sM;
    ff[1] = rhostl * (sM * sM) + pst - bx * bx;
    ff[2] = rhostl * sM * vstl - bx * bystl;
    ff[3] = rhostl * sM * wstl - bx * bzstl;
    ff[4] = sM * (estl + pst) - bx * (vstdotbstl);
    ff[5] = 0.0;
    ff[6] = bystl * sM - bx * vstl;
    ff[7] = bzstl * sM - bx * wstl;
    for (int q = 8; q < p->neq; ++q) ff[q] = sM * pl[q] * slmul / slmsM;  /* :150-152 */
    return;
  }

  /* UR* region */
  if (sstr <= 0) {
    er = 0.5 * pr[0] * (pr[1] * pr[1] + pr[2] * pr[2] + pr[3] * pr[3]) + cv * pr[4]
         + 0.5 * (bx * bx + pr[6] * pr[6] + pr[7] * pr[7]);
    sMmur = sM - pr[1];
    denr = pr[0] * srmur * srmsM - bx * bx;
    if (denr == 0) {
      /* deviation: the reference leaves these uninitialised (hlld.f90:167-171) */
      vstr = pr[2]; wstr = pr[3]; bystr = 0.0; bzstr = 0.0;
    } else {
      vstr = pr[2] - bx * pr[6] * sMmur / denr;
      wstr = pr[3] - bx * pr[7] * sMmur / denr;
      bystr = pr[6] * (pr[0] * (srmur * srmur) - bx * bx) / denr;
      bzstr = pr[7] * (pr[0] * (srmur * srmur) - bx * bx) / denr;
    }
    vdotbr = pr[1] * bx + pr[2] * pr[6] + pr[3] * pr[7];
    vstdotbstr = sM * bx + vstr * bystr + wstr * bzstr;
    estr = (srmur * er - pTR * pr[1] + pst * sM + bx * (vdotbr - vstdotbstr)) / srmsM;
    ff[0] = rhostr * sM;
    ff[1] = rhostr * (sM * sM) + pst - bx * bx;
    ff[2] = rhostr * sM * vstr - bx * bystr;
    ff[3] = rhostr * sM * wstr - bx * bzstr;
    ff[4] = sM * (estr + pst) - bx * (vstdotbstr);
    ff[5] = 0.0;
    ff[6] = bystr * sM - bx * vstr;
    ff[7] = bzstr * sM - bx * wstr;
    for (int q = 8; q < p->neq; ++q) ff[q] = sM * pr[q] * srmur / srmsM;  /* :198-200 */
    return;
  }

  sMmul = sM - pl[1];
  sMmur = sM - pr[1];
  denl = pl[0] * slmul * slmsM - bx * bx;
  denr = pr[0] * srmur * srmsM - bx * bx;
  if (denl == 0) {
    vstl = pl[2]; wstl = pl[3]; bystl = 0.0; bzstl = 0.0;
  } else {
    vstl = pl[2] - bx * pl[6] * sMmul / denl;
    wstl = pl[3] - bx * pl[7] * sMmul / denl;
    bystl = pl[6] * (pl[0] * (slmul * slmul) - bx * bx) / denl;
    bzstl = pl[7] * (pl[0] * (slmul * slmul) - bx * bx) / denl;
  }
  if (denr == 0) {
    vstr = pr[2]; wstr = pr[3]; bystr = 0.0; bzstr = 0.0;
  } else {
    vstr = pr[2] - bx * pr[6] * sMmur / denr;
    wstr = pr[3] - bx * pr[7] * sMmur / denr;
    bystr = pr[6] * (pr[0] * (srmur * srmur) - bx * bx) / denr;
    bzstr = pr[7] * (pr[0] * (srmur * srmur) - bx * bx) / denr;
  }
  double dd = sqrt(rhostl) + sqrt(rhostr);
  double vstst = (sqrt(rhostl) * vstl + sqrt(rhostr) * vstr + (bystr - bystl) * signBx) / dd;
  double wstst = (sqrt(rhostl) * wstl + sqrt(rhostr) * wstr + (bzstr - bzstl) * signBx) / dd;
  double bystst = (sqrt(rhostl) * bystr + sqrt(rhostr) * bystl
                   + sqrt(rhostl * rhostr) * (vstr - vstl) * signBx) / dd;
  double bzstst = (sqrt(rhostl) * bzstr + sqrt(rhostr) * bzstl
                   + sqrt(rhostl * rhostr) * (wstr - wstl) * signBx) / dd;
  double vststdotbstst = sM * bx + vstst * bystst + wstst * bzstst;

  /* UL** region */
  if (sM >= 0) {
    el = 0.5 * pl[0] * (pl[1] * pl[1] + pl[2] * pl[2] + pl[3] * pl[3]) + cv * pl[4]
         + 0.5 * (bx * bx + pl[6] * pl[6] + pl[7] * pl[7]);
    vdotbl = pl[1] * bx + pl[2] * pl[6] + pl[3] * pl[7];
    vstdotbstl = sM * bx + vstl * bystl + wstl * bzstl;
    estl = (slmul * el - pTL * pl[1] + pst * sM + bx * (vdotbl - vstdotbstl)) / slmsM;
    double eststl = estl - sqrt(rhostl) * (vstdotbstl - vststdotbstst) * signBx;
    ff[0] = rhostl * sM;
    ff[1] = rhostl * (sM * sM) + pst - bx * bx;
    ff[2] = rhostl * sM * vstst - bx * bystst;
    ff[3] = rhostl * sM * wstst - bx * bzstst;
    ff[4] = sM * (eststl + pst) - bx * (vststdotbstst);
    ff[5] = 0.0;
    ff[6] = bystst * sM - bx * vstst;
    ff[7] = bzstst * sM - bx * wstst;
    for (int q = 8; q < p->neq; ++q) ff[q] = sM * pl[q] * slmul / slmsM;  /* :277-279 */
    return;
  }
  /* UR** region */
  if (sM <= 0) {
    er = 0.5 * pr[0] * (pr[1] * pr[1] + pr[2] * pr[2] + pr[3] * pr[3]) + cv * pr[4]
         + 0.5 * (bx * bx + pr[6] * pr[6] + pr[7] * pr[7]);
    vdotbr = pr[1] * bx + pr[2] * pr[6] + pr[3] * pr[7];
    vstdotbstr = sM * bx + vstr * bystr + wstr * bzstr;
    estr = (srmur * er - pTR * pr[1] + pst * sM + bx * (vdotbr - vstdotbstr)) / srmsM;
    double eststr = estr + sqrt(rhostr) * (vstdotbstr - vststdotbstst) * signBx;
    ff[0] = rhostr * sM;
    ff[1] = rhostr * (sM * sM) + pst - bx * bx;
    ff[2] = rhostr * sM * vstst - bx * bystst;
    ff[3] = rhostr * sM * wstst - bx * bzstst;
    ff[4] = sM * (eststr + pst) - bx * (vststdotbstst);
    ff[5] = 0.0;
    ff[6] = bystst * sM - bx * vstst;
    ff[7] = bzstst * sM - bx * wstst;
    for (int q = 8; q < p->neq; ++q) ff[q] = sM * pr[q] * srmur / srmsM;  /* :308-310 */
    return;
  }
  /* src/hlld.f90:316-317: print and stop */
  for (int q = 0; q < 8; ++q) ff[q] = NAN;
  *err |= GOR_ERR_HLLD_FALLTHROUGH;
}

/* src/hllc.f90:44-140  prim2fhllc */
static void prim2fhllc(const gor_params_t* p, const double* pl, const double* pr, double* ff,
                       int* err) {
  const int neq = p->neq;
  double uu[GOR_MAX_NEQ], uuk[GOR_MAX_NEQ];
  double csl = csound(p, pl[4], pl[0]);
  double csr = csound(p, pr[4], pr[0]);
  double sr = dmax(pl[1] + csl, pr[1] + csr);
  double sl = dmin(pl[1] - csl, pr[1] - csr);
  if (sl > 0) { prim2f(p, pl, ff); return; }
  if (sr < 0) { prim2f(p, pr, ff); return; }
  double slmul = sl - pl[1];
  double srmur = sr - pr[1];
  double rholul = pl[0] * pl[1];
  double rhorur = pr[0] * pr[1];
  double sst = (srmur * rhorur - slmul * rholul - pr[4] + pl[4]) / (srmur * pr[0] - slmul * pl[0]);
  if (sst >= 0.0) {
    double rhost = pl[0] * (slmul) / (sl - sst);
    double ek = 0.5 * pl[0] * (pl[1] * pl[1] + pl[2] * pl[2] + pl[3] * pl[3]) + p->cv * pl[4];
    uuk[0] = rhost;
    uuk[1] = rhost * sst;
    uuk[2] = rhost * pl[2];
    uuk[3] = rhost * pl[3];
    uuk[4] = rhost * (ek / pl[0] + (sst - pl[1]) * (sst + pl[4] / (pl[0] * slmul)));
    if (p->pmhd && bfield(p)) {
      uuk[5] = rhost * pl[5] / pl[0];
      uuk[6] = rhost * pl[6] / pl[0];
      uuk[7] = rhost * pl[7] / pl[0];
    } else if (bfield(p)) {
      /* uninitialised in the reference when neither pmhd nor passives;
       * HLLC is not used with full MHD */
      uuk[5] = uuk[6] = uuk[7] = 0.0;
    }
    for (int q = neqdyn(p); q < neq; ++q) uuk[q] = rhost * pl[q] / pl[0];  /* :95-97 */
    prim2f(p, pl, ff);
    prim2u(p, pl, uu);
    for (int q = 0; q < neq; ++q) ff[q] = ff[q] + sl * (uuk[q] - uu[q]);
    return;
  }
  if (sst <= 0.0) {
    double rhost = pr[0] * (srmur) / (sr - sst);
    double ek = 0.5 * pr[0] * (pr[1] * pr[1] + pr[2] * pr[2] + pr[3] * pr[3]) + p->cv * pr[4];
    uuk[0] = rhost;
    uuk[1] = rhost * sst;
    uuk[2] = rhost * pr[2];
    uuk[3] = rhost * pr[3];
    uuk[4] = rhost * (ek / pr[0] + (sst - pr[1]) * (sst + pr[4] / (pr[0] * srmur)));
    if (p->pmhd && bfield(p)) {
      uuk[5] = rhost * pr[5] / pr[0];
      uuk[6] = rhost * pr[6] / pr[0];
      uuk[7] = rhost * pr[7] / pr[0];
    } else if (bfield(p)) {
      uuk[5] = uuk[6] = uuk[7] = 0.0;
    }
    for (int q = neqdyn(p); q < neq; ++q) uuk[q] = rhost * pr[q] / pr[0];  /* :124-126 */
    prim2f(p, pr, ff);
    prim2u(p, pr, uu);
    for (int q = 0; q < neq; ++q) ff[q] = ff[q] + sr * (uuk[q] - uu[q]);
    return;
  }
  for (int q = 0; q < neq; ++q) ff[q] = NAN;
  *err |= GOR_ERR_HLLC_FALLTHROUGH;
}

/* src/hlle.f90:48-83 (prim2fhlle) and src/hll.f90:47-82 (prim2fhll):
 * the same two-wave formula with fast (HLLE) or sound (HLL) speeds. */
static void prim2fhll_common(const gor_params_t* p, const double* pl, const double* pr,
                             double* ff, int fast) {
  double fL[GOR_MAX_NEQ], fR[GOR_MAX_NEQ], uL[GOR_MAX_NEQ], uR[GOR_MAX_NEQ];
  double csl, csr;
  if (fast) {
    csl = cfastX(p, pl);
    csr = cfastX(p, pr);
  } else {
    csl = csound(p, pl[4], pl[0]);
    csr = csound(p, pr[4], pr[0]);
  }
  double sr = dmax(pl[1] + csl, pr[1] + csr);
  double sl = dmin(pl[1] - csl, pr[1] - csr);
  if (sl > 0) { prim2f(p, pl, ff); return; }
  if (sr < 0) { prim2f(p, pr, ff); return; }
  prim2f(p, pl, fL);
  prim2f(p, pr, fR);
  prim2u(p, pl, uL);
  prim2u(p, pr, uR);
  for (int q = 0; q < p->neq; ++q)
    ff[q] = (sr * fL[q] - sl * fR[q] + sl * sr * (uR[q] - uL[q])) / (sr - sl);
}

/* ---------------------------------------------------------------------- */
/* The split solver (SOLVER_HLLE_SPLIT_ALL): primitives are fluctuations over
 * a background state prim0, with the reference's expressions. */
static inline int split_all(const gor_params_t* p) {
  return p->riemann_solver == GOR_SOLVER_HLLE_SPLIT_ALL;
}

/* src/hydro_core.f90:143-229 u2primSplitAll (no density or pressure floor) */
static void u2prim_split(const gor_params_t* p, const double* uu, const double* p0,
                         double* prim, double* T) {
  prim[0] = uu[0];
  double r = prim[0] + p0[0];
  prim[1] = uu[1] / r;
  prim[2] = uu[2] / r;
  prim[3] = uu[3] / r;
  if (bfield(p) && (p->mhd || p->pmhd)) {
    prim[5] = uu[5];
    prim[6] = uu[6];
    prim[7] = uu[7];
  }
  if (p->mhd) {
    prim[4] = (uu[4] - 0.5 * r * (prim[1] * prim[1] + prim[2] * prim[2] + prim[3] * prim[3])
               - 0.5 * (uu[5] * uu[5] + uu[6] * uu[6] + uu[7] * uu[7])
               - p0[5] * uu[5] - p0[6] * uu[6] - p0[7] * uu[7]) / p->cv;
  } else {
    prim[4] = (uu[4] - 0.5 * r * (prim[1] * prim[1] + prim[2] * prim[2] + prim[3] * prim[3]))
              / p->cv;
  }
  const int nd = neqdyn(p);
  for (int q = nd; q < p->neq; ++q) prim[q] = uu[q];
  double t = 0.0;
  if (p->eq_of_state == GOR_EOS_ADIABATIC) t = ((prim[4] + p0[4]) / r) * p->Tempsc;
  if (p->eq_of_state == GOR_EOS_SINGLE_SPECIE) {
    r = dmax(r, 1e-15);
    t = dmax(1.0, ((prim[4] + p0[4]) / r) * p->Tempsc);
  }
  if (p->eq_of_state == GOR_EOS_H_RATE && p->npas > 0) {
    double dentot = (2.0 * r - prim[nd] - p0[nd]);
    dentot = dmax(dentot, 1e-15);
    t = dmax(1.0, ((prim[4] + p0[4]) / dentot) * p->Tempsc);
  }
  if (T) *T = t;
}

/* src/hydro_core.f90:331-383 prim2u with prim0 (split branch) */
static void prim2u_split(const gor_params_t* p, const double* prim, const double* p0,
                         double* uu) {
  uu[0] = prim[0];
  uu[1] = prim[1] * (prim[0] + p0[0]);
  uu[2] = prim[2] * (prim[0] + p0[0]);
  uu[3] = prim[3] * (prim[0] + p0[0]);
  const double v2 = prim[1] * prim[1] + prim[2] * prim[2] + prim[3] * prim[3];
  uu[4] = 0.5 * prim[0] * v2 + p->cv * prim[4];
  if (bfield(p) && p->mhd)
    uu[4] = uu[4] + 0.5 * (prim[5] * prim[5] + prim[6] * prim[6] + prim[7] * prim[7])
            + 0.5 * p0[0] * v2 + p0[5] * prim[5] + p0[6] * prim[6] + p0[7] * prim[7];
  if (bfield(p) && (p->mhd || p->pmhd)) {
    uu[5] = prim[5];
    uu[6] = prim[6];
    uu[7] = prim[7];
  }
  for (int q = neqdyn(p); q < p->neq; ++q) uu[q] = prim[q];
}

/* src/hydro_core.f90:395-476 prim2f with prim0 (split branch, MHD) */
static void prim2f_split(const gor_params_t* p, const double* prim, const double* p0,
                         double* ff) {
  const double rt = prim[0] + p0[0];
  const double b6 = prim[5], b7 = prim[6], b8 = prim[7];
  const double etot = 0.5 * (rt * (prim[1] * prim[1] + prim[2] * prim[2] + prim[3] * prim[3])
                             + b6 * b6 + b7 * b7 + b8 * b8)
                      + p->cv * prim[4] + p0[5] * b6 + p0[6] * b7 + p0[7] * b8;
  ff[0] = rt * prim[1];
  ff[1] = rt * prim[1] * prim[1] + prim[4] + 0.5 * (b7 * b7 + b8 * b8 - b6 * b6)
          - p0[5] * b6 + p0[6] * b7 + p0[7] * b8;
  ff[2] = rt * prim[1] * prim[2] - b6 * b7 - p0[6] * b6 - p0[5] * b7;
  ff[3] = rt * prim[1] * prim[3] - b6 * b8 - p0[7] * b6 - p0[5] * b8;
  const double t6 = b6 + p0[5], t7 = b7 + p0[6], t8 = b8 + p0[7];
  ff[4] = prim[1] * (etot + prim[4] + 0.5 * (t6 * t6 + t7 * t7 + t8 * t8) + p->cv * p0[4]
                     + p0[4] + 0.5 * (p0[5] * p0[5] + p0[6] * p0[6] + p0[7] * p0[7]))
          - t6 * (prim[1] * t6 + prim[2] * t7 + prim[3] * t8);
  ff[5] = 0.0;
  ff[6] = prim[1] * (p0[6] + b7) - prim[2] * (p0[5] + b6);
  ff[7] = prim[1] * (p0[7] + b8) - prim[3] * (p0[5] + b6);
  for (int q = neqdyn(p); q < p->neq; ++q) ff[q] = prim[q] * prim[1];
}

/* src/hlle_split_all.f90:51-84 prim2fhlleSplitAll */
static void prim2fhlle_split(const gor_params_t* p, const double* pl, const double* pr,
                             const double* p0l, const double* p0r, double* ff) {
  double tl[GOR_MAX_NEQ], tr[GOR_MAX_NEQ];
  for (int q = 0; q < p->neq; ++q) {
    tl[q] = pl[q] + p0l[q];
    tr[q] = pr[q] + p0r[q];
  }
  const double csl = cfastX(p, tl), csr = cfastX(p, tr);
  const double sr = dmax(pl[1] + p0l[1] + csl, pr[1] + p0r[1] + csr);
  const double sl = dmin(pl[1] + p0l[1] - csl, pr[1] + p0r[1] - csr);
  if (sl > 0) { prim2f_split(p, pl, p0l, ff); return; }
  if (sr < 0) { prim2f_split(p, pr, p0r, ff); return; }
  double fL[GOR_MAX_NEQ], fR[GOR_MAX_NEQ], uL[GOR_MAX_NEQ], uR[GOR_MAX_NEQ];
  prim2f_split(p, pl, p0l, fL);
  prim2f_split(p, pr, p0r, fR);
  prim2u_split(p, pl, p0l, uL);
  prim2u_split(p, pr, p0r, uR);
  for (int q = 0; q < p->neq; ++q)
    ff[q] = (sr * fL[q] - sl * fR[q] + sl * sr * (uR[q] - uL[q])) / (sr - sl);
}

void gor_riemann_split(const gor_params_t* p, const double* priml, const double* primr,
                       const double* prim0l, const double* prim0r, double* ff) {
  prim2fhlle_split(p, priml, primr, prim0l, prim0r, ff);
}

static void riemann(const gor_params_t* p, const double* pl, const double* pr, double* ff,
                    int* err) {
  switch (p->riemann_solver) {
    case GOR_SOLVER_HLLD: prim2fhlld(p, pl, pr, ff, err); break;
    case GOR_SOLVER_HLLC: prim2fhllc(p, pl, pr, ff, err); break;
    case GOR_SOLVER_HLLE: prim2fhll_common(p, pl, pr, ff, 1); break;
    case GOR_SOLVER_HLL: prim2fhll_common(p, pl, pr, ff, 0); break;
    default: *err |= GOR_ERR_BAD_PARAM;
  }
}

/* src/hlld.f90:331-432 (hlldfluxes) and its twins hllc.f90:152-253,
 * hlle.f90:95-196, hll.f90:93-194: fluxes at i+1/2, j+1/2, k+1/2 for
 * i,j,k in [0,n]. */
/* src/hlle_split_all.f90:96-241 hllEfluxesSplitAll: the fluctuations and the
 * background are read (and, in stage 2, limited) the same way, and solved
 * together; the faces of i, j, k in [0, n]. */
static void fluxes_split(gor_state_t* s, int choice) {
  const gor_params_t* p = &s->p;
  const int neq = p->neq, nx = p->nx, ny = p->ny, nz = p->nz;
  const double* P = s->primit;
  const double* P0 = s->primit0;
#pragma omp parallel for schedule(static)
  for (int k = 0; k <= nz; ++k) {
    double pl[GOR_MAX_NEQ], pr[GOR_MAX_NEQ], pll[GOR_MAX_NEQ], prr[GOR_MAX_NEQ];
    double ql[GOR_MAX_NEQ], qr[GOR_MAX_NEQ], qll[GOR_MAX_NEQ], qrr[GOR_MAX_NEQ];
    double ff[GOR_MAX_NEQ];
    for (int j = 0; j <= ny; ++j) {
      for (int i = 0; i <= nx; ++i) {
        for (int dir = 0; dir < 3; ++dir) {
          const int di = dir == 0, dj = dir == 1, dk = dir == 2;
          for (int q = 1; q <= neq; ++q) {
            pl[q - 1] = AT(s, P, q, i, j, k);
            pr[q - 1] = AT(s, P, q, i + di, j + dj, k + dk);
            ql[q - 1] = AT(s, P0, q, i, j, k);
            qr[q - 1] = AT(s, P0, q, i + di, j + dj, k + dk);
            if (choice == 2) {
              pll[q - 1] = AT(s, P, q, i - di, j - dj, k - dk);
              prr[q - 1] = AT(s, P, q, i + 2 * di, j + 2 * dj, k + 2 * dk);
              qll[q - 1] = AT(s, P0, q, i - di, j - dj, k - dk);
              qrr[q - 1] = AT(s, P0, q, i + 2 * di, j + 2 * dj, k + 2 * dk);
            }
          }
          void (*swap)(const gor_params_t*, double*) = dir == 1 ? swapy : swapz;
          if (dir != 0) {
            swap(p, pl); swap(p, pr); swap(p, ql); swap(p, qr);
            if (choice == 2) { swap(p, pll); swap(p, prr); swap(p, qll); swap(p, qrr); }
          }
          if (choice == 2) {
            limiter(p, pll, pl, pr, prr);
            limiter(p, qll, ql, qr, qrr);
          }
          prim2fhlle_split(p, pl, pr, ql, qr, ff);
          if (dir != 0) swap(p, ff);
          double* out = dir == 0 ? s->f : (dir == 1 ? s->g : s->h);
          for (int q = 1; q <= neq; ++q) AT(s, out, q, i, j, k) = ff[q - 1];
        }
      }
    }
  }
}

static void fluxes(gor_state_t* s, int choice) {
  const gor_params_t* p = &s->p;
  if (split_all(p)) {
    fluxes_split(s, choice);
    return;
  }
  const int neq = p->neq, nx = p->nx, ny = p->ny, nz = p->nz;
  int err = 0;
#pragma omp parallel for schedule(static) reduction(| : err)
  for (int k = 0; k <= nz; ++k) {
    double pl[GOR_MAX_NEQ], pr[GOR_MAX_NEQ], pll[GOR_MAX_NEQ], prr[GOR_MAX_NEQ], ff[GOR_MAX_NEQ];
    for (int j = 0; j <= ny; ++j) {
      for (int i = 0; i <= nx; ++i) {
        /* x direction */
        for (int q = 1; q <= neq; ++q) {
          pl[q - 1] = AT(s, s->primit, q, i, j, k);
          pr[q - 1] = AT(s, s->primit, q, i + 1, j, k);
        }
        if (choice == 2) {
          for (int q = 1; q <= neq; ++q) {
            pll[q - 1] = AT(s, s->primit, q, i - 1, j, k);
            prr[q - 1] = AT(s, s->primit, q, i + 2, j, k);
          }
          limiter(p, pll, pl, pr, prr);
        }
        riemann(p, pl, pr, ff, &err);
        for (int q = 1; q <= neq; ++q) AT(s, s->f, q, i, j, k) = ff[q - 1];

        /* y direction */
        for (int q = 1; q <= neq; ++q) {
          pl[q - 1] = AT(s, s->primit, q, i, j, k);
          pr[q - 1] = AT(s, s->primit, q, i, j + 1, k);
        }
        swapy(p, pl);
        swapy(p, pr);
        if (choice == 2) {
          for (int q = 1; q <= neq; ++q) {
            pll[q - 1] = AT(s, s->primit, q, i, j - 1, k);
            prr[q - 1] = AT(s, s->primit, q, i, j + 2, k);
          }
          swapy(p, pll);
          swapy(p, prr);
          limiter(p, pll, pl, pr, prr);
        }
        riemann(p, pl, pr, ff, &err);
        swapy(p, ff);
        for (int q = 1; q <= neq; ++q) AT(s, s->g, q, i, j, k) = ff[q - 1];

        /* z direction */
        for (int q = 1; q <= neq; ++q) {
          pl[q - 1] = AT(s, s->primit, q, i, j, k);
          pr[q - 1] = AT(s, s->primit, q, i, j, k + 1);
        }
        swapz(p, pl);
        swapz(p, pr);
        if (choice == 2) {
          for (int q = 1; q <= neq; ++q) {
            pll[q - 1] = AT(s, s->primit, q, i, j, k - 1);
            prr[q - 1] = AT(s, s->primit, q, i, j, k + 2);
          }
          swapz(p, pll);
          swapz(p, prr);
          limiter(p, pll, pl, pr, prr);
        }
        riemann(p, pl, pr, ff, &err);
        swapz(p, ff);
        for (int q = 1; q <= neq; ++q) AT(s, s->h, q, i, j, k) = ff[q - 1];
      }
    }
  }
  s->err |= err;
}

/* ---------------------------------------------------------------------- */
/* src/flux_cd_module.f90:45-237  boundaryI_ef (serial semantics) */
static void boundaryI_ef(gor_state_t* s) {
  const gor_params_t* p = &s->p;
  const int nx = p->nx, ny = p->ny, nz = p->nz;
  /* periodic */
  if (p->bc_left == GOR_BC_PERIODIC && p->bc_right == GOR_BC_PERIODIC)
    for (int k = 1 - NG; k <= nz + NG; ++k)
      for (int j = 1 - NG; j <= ny + NG; ++j)
        for (int q = 1; q <= 3; ++q) {
          EAT(s, q, 0, j, k) = EAT(s, q, nx, j, k);
          EAT(s, q, nx + 1, j, k) = EAT(s, q, 1, j, k);
        }
  if (p->bc_bottom == GOR_BC_PERIODIC && p->bc_top == GOR_BC_PERIODIC)
    for (int k = 1 - NG; k <= nz + NG; ++k)
      for (int i = 1 - NG; i <= nx + NG; ++i)
        for (int q = 1; q <= 3; ++q) {
          EAT(s, q, i, 0, k) = EAT(s, q, i, ny, k);
          EAT(s, q, i, ny + 1, k) = EAT(s, q, i, 1, k);
        }
  if (p->bc_out == GOR_BC_PERIODIC && p->bc_in == GOR_BC_PERIODIC)
    for (int j = 1 - NG; j <= ny + NG; ++j)
      for (int i = 1 - NG; i <= nx + NG; ++i)
        for (int q = 1; q <= 3; ++q) {
          EAT(s, q, i, j, 0) = EAT(s, q, i, j, nz);
          EAT(s, q, i, j, nz + 1) = EAT(s, q, i, j, 1);
        }
  /* closed (reflecting) */
  for (int k = 0; k <= nz + 1; ++k)
    for (int j = 0; j <= ny + 1; ++j) {
      if (p->bc_left == GOR_BC_CLOSED) {
        EAT(s, 1, 0, j, k) = -EAT(s, 1, 1, j, k);
        EAT(s, 2, 0, j, k) = EAT(s, 2, 1, j, k);
        EAT(s, 3, 0, j, k) = EAT(s, 3, 1, j, k);
      }
      if (p->bc_right == GOR_BC_CLOSED) {
        EAT(s, 1, nx + 1, j, k) = -EAT(s, 1, nx, j, k);
        EAT(s, 2, nx + 1, j, k) = EAT(s, 2, nx, j, k);
        EAT(s, 3, nx + 1, j, k) = EAT(s, 3, nx, j, k);
      }
    }
  for (int k = 0; k <= nz + 1; ++k)
    for (int i = 0; i <= nx + 1; ++i) {
      if (p->bc_bottom == GOR_BC_CLOSED) {
        EAT(s, 1, i, 0, k) = EAT(s, 1, i, 1, k);
        EAT(s, 2, i, 0, k) = -EAT(s, 2, i, 1, k);
        EAT(s, 3, i, 0, k) = EAT(s, 3, i, 1, k);
      }
      if (p->bc_top == GOR_BC_CLOSED) {
        EAT(s, 1, i, ny + 1, k) = EAT(s, 1, i, ny, k);
        EAT(s, 2, i, ny + 1, k) = -EAT(s, 2, i, ny, k);
        EAT(s, 3, i, ny + 1, k) = EAT(s, 3, i, ny, k);
      }
    }
  /* the z faces of the closed case copy all three components unchanged
   * (src/flux_cd_module.f90:179-192) */
  for (int j = 0; j <= ny + 1; ++j)
    for (int i = 0; i <= nx + 1; ++i)
      for (int q = 1; q <= 3; ++q) {
        if (p->bc_out == GOR_BC_CLOSED) EAT(s, q, i, j, 0) = EAT(s, q, i, j, 1);
        if (p->bc_in == GOR_BC_CLOSED) EAT(s, q, i, j, nz + 1) = EAT(s, q, i, j, nz);
      }
  /* outflow */
  for (int k = 0; k <= nz + 1; ++k)
    for (int j = 0; j <= ny + 1; ++j)
      for (int q = 1; q <= 3; ++q) {
        if (p->bc_left == GOR_BC_OUTFLOW) EAT(s, q, 0, j, k) = EAT(s, q, 1, j, k);
        if (p->bc_right == GOR_BC_OUTFLOW) EAT(s, q, nx + 1, j, k) = EAT(s, q, nx, j, k);
      }
  for (int k = 0; k <= nz + 1; ++k)
    for (int i = 0; i <= nx + 1; ++i)
      for (int q = 1; q <= 3; ++q) {
        if (p->bc_bottom == GOR_BC_OUTFLOW) EAT(s, q, i, 0, k) = EAT(s, q, i, 1, k);
        if (p->bc_top == GOR_BC_OUTFLOW) EAT(s, q, i, ny + 1, k) = EAT(s, q, i, ny, k);
      }
  for (int j = 0; j <= ny + 1; ++j)
    for (int i = 0; i <= nx + 1; ++i)
      for (int q = 1; q <= 3; ++q) {
        if (p->bc_out == GOR_BC_OUTFLOW) EAT(s, q, i, j, 0) = EAT(s, q, i, j, 1);
        if (p->bc_in == GOR_BC_OUTFLOW) EAT(s, q, i, j, nz + 1) = EAT(s, q, i, j, nz);
      }
}

/* src/flux_cd_module.f90:245-273  get_efield */
static void get_efield(gor_state_t* s) {
  const int nx = s->p.nx, ny = s->p.ny, nz = s->p.nz;
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        EAT(s, 1, i, j, k) = 0.25 * (-AT(s, s->g, 8, i, j - 1, k) - AT(s, s->g, 8, i, j, k)
                                     + AT(s, s->h, 7, i, j, k - 1) + AT(s, s->h, 7, i, j, k));
        EAT(s, 2, i, j, k) = 0.25 * (+AT(s, s->f, 8, i - 1, j, k) + AT(s, s->f, 8, i, j, k)
                                     - AT(s, s->h, 6, i, j, k - 1) - AT(s, s->h, 6, i, j, k));
        EAT(s, 3, i, j, k) = 0.25 * (-AT(s, s->f, 7, i - 1, j, k) - AT(s, s->f, 7, i, j, k)
                                     + AT(s, s->g, 6, i, j - 1, k) + AT(s, s->g, 6, i, j, k));
      }
  boundaryI_ef(s);
}

/* ---------------------------------------------------------------------- */
/* src/sources.f90:57-69 getpos is not needed: the user hook below computes
 * its own position (EXO/user_mod.f90:179-181). */

/* EXO/user_mod.f90:158-206  get_user_source_terms (point masses) */
static void user_source(const gor_params_t* p, const double* pp, double* sv, int i, int j,
                        int k) {
  double xc = ((double)(i - p->nx / 2) - 0.5) * p->dx;
  double yc = ((double)(j - p->ny / 2) - 0.5) * p->dy;
  double zc = ((double)(k - p->nz / 2) - 0.5) * p->dz;
  for (int l = 0; l < p->ngrav; ++l) {
    double x = xc - p->grav_x[l], y = yc - p->grav_y[l], z = zc - p->grav_z[l];
    double rad2 = x * x + y * y + z * z;
    double r15 = pow(rad2, 1.5);
    double GM = p->grav_GM[l];
    sv[1] = sv[1] - pp[0] * GM * x / r15;
    sv[2] = sv[2] - pp[0] * GM * y / r15;
    sv[3] = sv[3] - pp[0] * GM * z / r15;
    sv[4] = sv[4] - pp[0] * GM * (pp[1] * x + pp[2] * y + pp[3] * z) / r15;
  }
}

/* src/sources.f90:190-220 source, with divbcorr_8w_source :151-175 and
 * divergence_B :124-134 */
static void source(const gor_state_t* s, int i, int j, int k, const double* prim, double* sv) {
  const gor_params_t* p = &s->p;
  for (int q = 0; q < p->neq; ++q) sv[q] = 0.0;
  if (p->user_source_terms) user_source(p, prim, sv, i, j, k);
  if (p->eight_wave && bfield(p)) {
    double divB = (AT(s, s->primit, 6, i + 1, j, k) - AT(s, s->primit, 6, i - 1, j, k))
                      / (2.0 * p->dx)
                  + (AT(s, s->primit, 7, i, j + 1, k) - AT(s, s->primit, 7, i, j - 1, k))
                        / (2.0 * p->dy)
                  + (AT(s, s->primit, 8, i, j, k + 1) - AT(s, s->primit, 8, i, j, k - 1))
                        / (2.0 * p->dz);
    sv[1] = sv[1] - divB * prim[5];
    sv[2] = sv[2] - divB * prim[6];
    sv[3] = sv[3] - divB * prim[7];
    sv[4] = sv[4] - divB * (prim[1] * prim[5] + prim[2] * prim[6] + prim[3] * prim[7]);
    sv[5] = sv[5] - divB * prim[1];
    sv[6] = sv[6] - divB * prim[2];
    sv[7] = sv[7] - divB * prim[3];
  }
}

/* src/hydro_solver.f90:77-127  step (with flux_cd_update,
 * src/flux_cd_module.f90:285-323) */
static void step(gor_state_t* s, double dt) {
  const gor_params_t* p = &s->p;
  const int neq = p->neq, nx = p->nx, ny = p->ny, nz = p->nz;
  double dtdx = dt / p->dx, dtdy = dt / p->dy, dtdz = dt / p->dz;
  int ct = p->enable_flux_cd && bfield(p);
  if (ct) get_efield(s);
  int src = p->user_source_terms || p->eight_wave;
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= nz; ++k) {
    double sv[GOR_MAX_NEQ], prim[GOR_MAX_NEQ];
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        if (!ct) {
          for (int q = 1; q <= neq; ++q)
            AT(s, s->up, q, i, j, k) =
                AT(s, s->u, q, i, j, k)
                - dtdx * (AT(s, s->f, q, i, j, k) - AT(s, s->f, q, i - 1, j, k))
                - dtdy * (AT(s, s->g, q, i, j, k) - AT(s, s->g, q, i, j - 1, k))
                - dtdz * (AT(s, s->h, q, i, j, k) - AT(s, s->h, q, i, j, k - 1));
        } else {
          /* hydro (:299-301) and passives (:304-308) upwind, B by CT */
          for (int q = 1; q <= neq; ++q) {
            if (q >= 6 && q <= 8) continue;
            AT(s, s->up, q, i, j, k) =
                AT(s, s->u, q, i, j, k)
                - dtdx * (AT(s, s->f, q, i, j, k) - AT(s, s->f, q, i - 1, j, k))
                - dtdy * (AT(s, s->g, q, i, j, k) - AT(s, s->g, q, i, j - 1, k))
                - dtdz * (AT(s, s->h, q, i, j, k) - AT(s, s->h, q, i, j, k - 1));
          }
          AT(s, s->up, 6, i, j, k) = AT(s, s->u, 6, i, j, k)
                                     - 0.5 * dtdy * (EAT(s, 3, i, j + 1, k) - EAT(s, 3, i, j - 1, k))
                                     + 0.5 * dtdz * (EAT(s, 2, i, j, k + 1) - EAT(s, 2, i, j, k - 1));
          AT(s, s->up, 7, i, j, k) = AT(s, s->u, 7, i, j, k)
                                     + 0.5 * dtdx * (EAT(s, 3, i + 1, j, k) - EAT(s, 3, i - 1, j, k))
                                     - 0.5 * dtdz * (EAT(s, 1, i, j, k + 1) - EAT(s, 1, i, j, k - 1));
          AT(s, s->up, 8, i, j, k) = AT(s, s->u, 8, i, j, k)
                                     - 0.5 * dtdx * (EAT(s, 2, i + 1, j, k) - EAT(s, 2, i - 1, j, k))
                                     + 0.5 * dtdy * (EAT(s, 1, i, j + 1, k) - EAT(s, 1, i, j - 1, k));
        }
        if (src) {
          for (int q = 1; q <= neq; ++q) prim[q - 1] = AT(s, s->primit, q, i, j, k);
          source(s, i, j, k, prim, sv);
          for (int q = 1; q <= neq; ++q)
            AT(s, s->up, q, i, j, k) = AT(s, s->up, q, i, j, k) + dt * sv[q - 1];
        }
      }
  }
}

/* src/hydro_solver.f90:47-65  viscous_copy */
static void viscous_copy(gor_state_t* s) {
  const gor_params_t* p = &s->p;
  const int neq = p->neq, nx = p->nx, ny = p->ny, nz = p->nz;
  const double eta = p->eta;
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i)
        for (int q = 1; q <= neq; ++q)
          AT(s, s->u, q, i, j, k) =
              AT(s, s->up, q, i, j, k)
              + eta * (AT(s, s->up, q, i + 1, j, k) + AT(s, s->up, q, i - 1, j, k)
                       + AT(s, s->up, q, i, j + 1, k) + AT(s, s->up, q, i, j - 1, k)
                       + AT(s, s->up, q, i, j, k + 1) + AT(s, s->up, q, i, j, k - 1)
                       - 6.0 * AT(s, s->up, q, i, j, k));
}

/* ---------------------------------------------------------------------- */
/* Boundaries: src/boundaries.f90:44-247 (boundaryI, one ghost layer) and
 * :256-512 (boundaryII, two layers), serial semantics. */
static void copy_cell(const gor_state_t* s, double* a, int i, int j, int k, int si, int sj,
                      int sk, int flipq) {
  const int neq = s->p.neq;
  double* dst = &a[CID(s, i, j, k) * (size_t)neq];
  const double* src = &a[CID(s, si, sj, sk) * (size_t)neq];
  for (int q = 0; q < neq; ++q) dst[q] = (q + 1 == flipq) ? -src[q] : src[q];
}

static void impose_user_bc(gor_state_t* s, double* a);

static void boundary_fill(gor_state_t* s, double* a, int layers) {
  const gor_params_t* p = &s->p;
  const int nx = p->nx, ny = p->ny, nz = p->nz;
  /* range of the transverse indices: boundaryI covers 0..n+1, boundaryII the
   * whole array */
  const int lo = layers == 1 ? 0 : 1 - NG;
  const int hix = layers == 1 ? nx + 1 : nx + NG;
  const int hiy = layers == 1 ? ny + 1 : ny + NG;
  const int hiz = layers == 1 ? nz + 1 : nz + NG;
  /* periodic (full transverse planes in both cases) */
  if (p->bc_left == GOR_BC_PERIODIC && p->bc_right == GOR_BC_PERIODIC)
    for (int k = 1 - NG; k <= nz + NG; ++k)
      for (int j = 1 - NG; j <= ny + NG; ++j)
        for (int l = 0; l < layers; ++l) {
          copy_cell(s, a, -l, j, k, nx - l, j, k, 0);
          copy_cell(s, a, nx + 1 + l, j, k, 1 + l, j, k, 0);
        }
  if (p->bc_bottom == GOR_BC_PERIODIC && p->bc_top == GOR_BC_PERIODIC)
    for (int k = 1 - NG; k <= nz + NG; ++k)
      for (int i = 1 - NG; i <= nx + NG; ++i)
        for (int l = 0; l < layers; ++l) {
          copy_cell(s, a, i, -l, k, i, ny - l, k, 0);
          copy_cell(s, a, i, ny + 1 + l, k, i, 1 + l, k, 0);
        }
  if (p->bc_out == GOR_BC_PERIODIC && p->bc_in == GOR_BC_PERIODIC)
    for (int j = 1 - NG; j <= ny + NG; ++j)
      for (int i = 1 - NG; i <= nx + NG; ++i)
        for (int l = 0; l < layers; ++l) {
          copy_cell(s, a, i, j, -l, i, j, nz - l, 0);
          copy_cell(s, a, i, j, nz + 1 + l, i, j, 1 + l, 0);
        }
  /* closed, then outflow: the mirror source of ghost layer l is interior
   * layer l+1 counted from the face (j=nghost..1 in boundaryII; layer 1 only
   * in boundaryI) */
  for (int pass = 0; pass < 2; ++pass) {
    int bc = pass == 0 ? GOR_BC_CLOSED : GOR_BC_OUTFLOW;
    int fx = pass == 0 ? 2 : 0, fy = pass == 0 ? 3 : 0, fz = pass == 0 ? 4 : 0;
    for (int k = lo; k <= hiz; ++k)
      for (int j = lo; j <= hiy; ++j)
        for (int l = 0; l < layers; ++l) {
          if (p->bc_left == bc) copy_cell(s, a, -l, j, k, 1 + l, j, k, fx);
          if (p->bc_right == bc) copy_cell(s, a, nx + 1 + l, j, k, nx - l, j, k, fx);
        }
    for (int k = lo; k <= hiz; ++k)
      for (int i = lo; i <= hix; ++i)
        for (int l = 0; l < layers; ++l) {
          if (p->bc_bottom == bc) copy_cell(s, a, i, -l, k, i, 1 + l, k, fy);
          if (p->bc_top == bc) copy_cell(s, a, i, ny + 1 + l, k, i, ny - l, k, fy);
        }
    for (int j = lo; j <= hiy; ++j)
      for (int i = lo; i <= hix; ++i)
        for (int l = 0; l < layers; ++l) {
          if (p->bc_out == bc) copy_cell(s, a, i, j, -l, i, j, 1 + l, fz);
          if (p->bc_in == bc) copy_cell(s, a, i, j, nz + 1 + l, i, j, nz - l, fz);
        }
  }
  if (p->bc_user) impose_user_bc(s, a);
}

/* EXO/exoplanet.f90:125-266  impose_exo, generalised to a list of spheres
 * (the first sphere that contains a cell wins, as the if/else-if chain).
 * An orbiting sphere's centre and velocity at the state's time follow
 * EXO/exoplanet.f90:143-148. */
static void impose_user_bc(gor_state_t* s, double* a) {
  const gor_params_t* p = &s->p;
  const int neq = p->neq, nx = p->nx, ny = p->ny, nz = p->nz;
  gor_sphere_t now[GOR_MAX_SPHERES];
  for (int m = 0; m < p->nsph; ++m) {
    now[m] = p->sph[m];
    if (now[m].orbit_omega != 0.0) {
      const double th = now[m].orbit_omega * s->time + now[m].orbit_phase;
      now[m].xc = now[m].orbit_r * cos(th);
      now[m].zc = now[m].orbit_r * sin(th);
      now[m].vorb[0] = -now[m].orbit_omega * now[m].orbit_r * sin(th);
      now[m].vorb[1] = 0.0;
      now[m].vorb[2] = now[m].orbit_omega * now[m].orbit_r * cos(th);
    }
  }
  for (int k = 1 - NG; k <= nz + NG; ++k)
    for (int j = 1 - NG; j <= ny + NG; ++j)
      for (int i = 1 - NG; i <= nx + NG; ++i) {
        double x = ((double)(i - nx / 2) + 0.5) * p->dx;
        double y = ((double)(j - ny / 2) + 0.5) * p->dy;
        double z = ((double)(k - nz / 2) + 0.5) * p->dz;
        for (int m = 0; m < p->nsph; ++m) {
          const gor_sphere_t* sp = &now[m];
          double xs = x - sp->xc, ys = y - sp->yc, zs = z - sp->zc;
          double rads = sqrt(xs * xs + ys * ys + zs * zs);
          if (rads <= sp->radius) {
            if (rads == 0.0) rads = p->dx * 0.10;
            double velx = sp->vorb[0] + sp->vwind * xs / rads;
            double vely = sp->vorb[1] + sp->vwind * ys / rads;
            double velz = sp->vorb[2] + sp->vwind * zs / rads;
            double dens = sp->dens;
            double* c = &a[CID(s, i, j, k) * (size_t)neq];
            c[0] = dens;
            c[1] = dens * velx;
            c[2] = dens * vely;
            c[3] = dens * velz;
            double b2 = 0.0;
            if (bfield(p) && (p->mhd || p->pmhd)) {
              double rr = sp->radius / rads;
              double cpi = sp->bdip * (rr * rr * rr) / (2.0 * (rads * rads));
              c[5] = 3.0 * ys * xs * cpi;
              c[6] = (3.0 * (ys * ys) - rads * rads) * cpi;
              c[7] = 3.0 * ys * zs * cpi;
              b2 = c[5] * c[5] + c[6] * c[6] + c[7] * c[7];
            }
            c[4] = 0.5 * dens * (velx * velx + vely * vely + velz * velz) + p->cv * dens * sp->tfac;
            if (p->mhd) c[4] = c[4] + 0.5 * b2;
            break;
          }
        }
      }
}

void gor_boundaryI(gor_state_t* s) { boundary_fill(s, s->u, 1); }
static void boundaryII(gor_state_t* s) { boundary_fill(s, s->up, 2); }

/* ---------------------------------------------------------------------- */
/* src/hydro_core.f90:245-320  calcprim */
static void calcprim_arr(gor_state_t* s, const double* uarr, int only_ghost) {
  const gor_params_t* p = &s->p;
  const int neq = p->neq, nx = p->nx, ny = p->ny, nz = p->nz;
#define CP(i, j, k)                                                                          \
  (split_all(p) ? u2prim_split(p, &uarr[CID(s, i, j, k) * neq], &s->primit0[CID(s, i, j, k) * neq], \
                               &s->primit[CID(s, i, j, k) * neq], &s->temp[CID(s, i, j, k)])   \
                : u2prim(p, &uarr[CID(s, i, j, k) * neq], &s->primit[CID(s, i, j, k) * neq],   \
                         &s->temp[CID(s, i, j, k)]))
  if (only_ghost) {
    for (int j = 0; j <= ny + 1; ++j)
      for (int i = 0; i <= nx + 1; ++i) {
        CP(i, j, 0);
        CP(i, j, nz + 1);
      }
    for (int k = 0; k <= nz + 1; ++k)
      for (int i = 0; i <= nx + 1; ++i) {
        CP(i, 0, k);
        CP(i, ny + 1, k);
      }
    for (int k = 0; k <= nz + 1; ++k)
      for (int j = 0; j <= ny + 1; ++j) {
        CP(0, j, k);
        CP(nx + 1, j, k);
      }
    return;
  }
#undef CP
  const size_t n = s->ncell;
  if (split_all(p)) {  /* src/hydro_core.f90:307-309 */
#pragma omp parallel for schedule(static)
    for (size_t c = 0; c < n; ++c)
      u2prim_split(p, &uarr[c * neq], &s->primit0[c * neq], &s->primit[c * neq], &s->temp[c]);
    return;
  }
#pragma omp parallel for schedule(static)
  for (size_t c = 0; c < n; ++c) u2prim(p, &uarr[c * neq], &s->primit[c * neq], &s->temp[c]);
}

void gor_calcprim(gor_state_t* s, int only_ghost) { calcprim_arr(s, s->u, only_ghost); }

/* src/cooling_dmc.f90:89-106 cooldmc / src/cooling_chi.f90:87-105 coolchi,
 * with the row index int(log10(T)*10)-39 written for a table of any 1/dlog. */
static double cooltab(const gor_params_t* p, double T) {
  if (T > 1e8) return p->tab_tail * sqrt(T);
  int if1 = (int)(log10(T) * p->tab_inv_dlog) - p->tab_i0; /* 0-based row */
  if (if1 < 0) if1 = 0;
  if (if1 > p->ntab - 2) if1 = p->ntab - 2;
  double T0 = p->tab_T[if1], c0 = p->tab_L[if1];
  double T1 = p->tab_T[if1 + 1], c1 = p->tab_L[if1 + 1];
  return (c1 - c0) * (T - T0) / (T1 - T0) + c0;
}

/* src/cooling_dmc.f90:115-156 coolingdmc (coolingchi is identical) */
static void cooling_table(gor_state_t* s, double dt) {
  const gor_params_t* p = &s->p;
  const int neq = p->neq, nx = p->nx, ny = p->ny, nz = p->nz;
  const double dt_seconds = dt * p->tsc;
  const double Tmin = p->tab_Tmin;
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        double* uu = &s->u[CID(s, i, j, k) * neq];
        double* pp = &s->primit[CID(s, i, j, k) * neq];
        double T;
        u2prim(p, uu, pp, &T);
        if (T > Tmin) {
          double Eth0 = p->cv * pp[4];
          double aloss = cooltab(p, T);
          double dens = pp[0];
          double ce = (aloss * (dens * dens)) / (Eth0 * p->Psc);
          pp[4] = pp[4] * exp(-ce * dt_seconds);
          uu[4] = uu[4] - Eth0 + p->cv * pp[4];
        }
      }
}

/* src/cooling_h.f90: parametrised cooling with the non-equilibrium
 * ionisation of hydrogen (COOL_H); the first passive scalar is the neutral
 * hydrogen density.  All arithmetic FP64, as in the reference build. */
static double alpha_rec(double T) { return 2.55e-13 * pow(1.e4 / T, 0.79); } /* :75-84 */
static double colf(double T) { return 5.83e-11 * sqrt(T) * exp(-157828. / T); } /* :108-117 */
static double betah(double T) {                                               /* :125-136 */
  const double a = 157890. / T;
  return 1.133e-24 / sqrt(a) * (-0.0713 + 0.5 * log(a) + 0.640 * pow(a, -0.33333));
}

/* :155-242 ALOSS: energy loss rate of the cell */
static double aloss(double X1, double X2, double DT, double DEN, double DH0, double TE0) {
  const double XION = 2.179e-11, XO = 1.e-3;
  const double C0 = 0.5732, C1 = 1.8288e-5, C2 = -1.15822e-10, C3 = 9.4288e-16;
  const double D0 = 0.5856, D1 = 1.55083e-5, D2 = -9.669e-12, D3 = 5.716e-19;
  const double ENK = 118409., EN = 1.634E-11;
  (void)X2;
  (void)DT;
  const double TE = dmax(TE0, 10.);
  const double DH = DEN;
  const double DHP = (1. - X1) * DH;
  const double DE = DHP + 1.E-4 * DH;
  const double DOI = XO * DH0;
  const double DOII = XO * DHP;
  if (TE <= 1e4) return 0.;
  double OMEGA = 0.0;
  if (TE <= 55000.) OMEGA = C0 + TE * (C1 + TE * (C2 + TE * C3));
  if (TE >= 72000.) OMEGA = D0 + TE * (D1 + TE * (D2 + TE * D3));
  if (TE > 55000. && TE < 72000.) {
    const double OMEGAL = C0 + TE * (C1 + TE * (C2 + TE * C3));
    const double OMEGAH = D0 + TE * (D1 + TE * (D2 + TE * D3));
    const double FRAC = (TE - 55000.) / 17000.;
    OMEGA = (1. - FRAC) * OMEGAL + FRAC * OMEGAH;
  }
  const double QLA = 8.6287E-6 / (2. * sqrt(TE)) * OMEGA * exp(-ENK / TE);
  double ECOLL = DE * DH0 * QLA * EN;
  ECOLL = dmax(ECOLL, 0.);
  const double CION = 5.834E-11 * sqrt(TE) * exp(-1.579E5 / TE);
  const double EION = DE * DH0 * CION * XION;
  double EREC = DE * DHP * (betah(TE));
  EREC = dmax(EREC, 0.);
  const double TM = 1. / TE;
  const double T2 = TM * TM;
  double EOI = DE * DOI * pow(10., 1381465 * T2 - 12328.69 * TM - 19.82621);
  double EOII = DE * DOII * pow(10., -2061075. * T2 - 14596.24 * TM - 19.01402);
  EOI = dmax(EOI, 0.);
  EOII = dmax(EOII, 0.);
  const double BETAF = 1.3 * 1.42E-27 * pow(TE, 0.5);
  const double HIICOOL = DE * DHP * BETAF;
  const double EQUIL =
      (1.0455E-18 / pow(TE, 0.63)) * (1. - exp(-pow(TE * 1.E-5, 1.63))) * DE * DEN + HIICOOL;
  double FR = 0.0;
  if (TE <= 44770.) FR = 0.;
  if (TE >= 54770.) FR = 1.;
  if (TE > 44770. && TE < 54770.) {
    const double EX2 = exp(-2. * (TE - 49770.) / 500.);
    const double TANH = (1. - EX2) / (1. + EX2);
    FR = 0.5 * (1. + TANH);
  }
  return ECOLL + EION + (EREC + 7.033 * (EOI + EOII)) * (1. - FR) + EQUIL * FR;
}

/* :259-371 atomic (no diffuse radiation: radphi = 1, tprime = 10 K) */
static void atomic(const gor_params_t* p, double dt, double* uu) {
  const double xi = 1.e-4, boltzm = 1.3807e-16;
  const int nd = neqdyn(p);
  double prim[GOR_MAX_NEQ], T;
  u2prim(p, uu, prim, &T);
  const double col = colf(T);
  const double rec = alpha_rec(T);
  const double y0 = uu[nd] / uu[0];
  const double dh = uu[0];
  const double a = rec + col;
  const double b = -((2. + xi) * rec + (1. + xi) * col);
  const double c = (1. + xi) * rec;
  const double d = sqrt(b * b - 4. * a * c);
  const double g0 = (2. * a * y0 + b + d) / (2. * a * y0 + b - d);
  const double e = exp(-d * dh * dt);
  double y1 = (-b - d * (1. + g0 * e) / (1. - g0 * e)) / (2. * a);
  y1 = dmin(y1, 0.9999);
  y1 = dmax(y1, 0.);
  const double dh0 = uu[nd];
  const double al = aloss(y0, y1, dt, dh, dh0, T) / (dh * dh);
  const double tprime = 10.;
  const double ce = (2. * dh * al) / (3. * boltzm * T);
  double t1 = tprime + (T - tprime) * exp(-ce * dt);
  t1 = dmax(t1, 0.1 * T);
  t1 = dmin(t1, 10. * T);
  uu[nd] = y1 * uu[0];
  if (p->mhd)
    uu[4] = p->cv * (2. * uu[0] - uu[nd]) * t1 / p->Tempsc
            + 0.5 * prim[0] * (prim[1] * prim[1] + prim[2] * prim[2] + prim[3] * prim[3])
            + 0.5 * (prim[5] * prim[5] + prim[6] * prim[6] + prim[7] * prim[7]);
  else
    uu[4] = p->cv * (2. * uu[0] - uu[nd]) * t1 / p->Tempsc
            + 0.5 * prim[0] * (prim[1] * prim[1] + prim[2] * prim[2] + prim[3] * prim[3]);
}

/* :41-67 coolingh */
static void coolingh(gor_state_t* s, double dt_CFL) {
  const gor_params_t* p = &s->p;
  const int neq = p->neq;
  const double dt_seconds = dt_CFL * p->tsc;
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= p->nz; ++k)
    for (int j = 1; j <= p->ny; ++j)
      for (int i = 1; i <= p->nx; ++i) atomic(p, dt_seconds, &s->u[CID(s, i, j, k) * neq]);
}

/* src/hydro_core.f90:623-697  get_timestep */
void gor_get_timestep(gor_state_t* s, int iter, int n_iter, double t, double tprint,
                      double* dt, int* dump) {
  const gor_params_t* p = &s->p;
  s->time = t;  /* the step's time, read by the user boundary hook inside tstep */
  const int neq = p->neq, nx = p->nx, ny = p->ny, nz = p->nz;
  double dtp = 1e30;
#pragma omp parallel for schedule(static) reduction(min : dtp)
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        const double* pr = &s->primit[CID(s, i, j, k) * neq];
        if (p->mhd) {
          double cx, cy, cz;
          if (split_all(p)) {  /* :650-655: the total state's fast speeds */
            const double* p0 = &s->primit0[CID(s, i, j, k) * neq];
            cfast(p, pr[4] + p0[4], pr[0] + p0[0], pr[5] + p0[5], pr[6] + p0[6], pr[7] + p0[7],
                  &cx, &cy, &cz);
          } else {
            cfast(p, pr[4], pr[0], pr[5], pr[6], pr[7], &cx, &cy, &cz);
          }
          dtp = dmin(dtp, p->dx / (fabs(pr[1]) + cx));
          dtp = dmin(dtp, p->dy / (fabs(pr[2]) + cy));
          dtp = dmin(dtp, p->dz / (fabs(pr[3]) + cz));
        } else {
          double c = csound(p, pr[4], pr[0]);
          dtp = dmin(dtp, p->dx / (fabs(pr[1]) + c));
          dtp = dmin(dtp, p->dy / (fabs(pr[2]) + c));
          dtp = dmin(dtp, p->dz / (fabs(pr[3]) + c));
        }
      }
  if (iter <= n_iter)
    dtp = p->cfl * ldexp(1.0, -(n_iter + 1 - iter)) * dtp;
  else
    dtp = p->cfl * dtp;
  *dt = dtp;
  if ((t + *dt) >= tprint) {
    *dt = tprint - t;
    *dump = 1;
  }
}

/* ---------------------------------------------------------------------- */
/* src/thermal_cond.f90: Spitzer thermal conduction (isotropic, or split
 * along and across B), optionally saturated, advanced with Chebyshev super
 * time steps.  The heat fluxes live in component 5 of the face flux arrays
 * f, g, h, as in the reference. */
#define TC_RG 8.3145e7   /* gas constant, src/constants.f90:35 */
#define TC_PH 0.4        /* saturation parameter, thermal_cond.f90:36 */
#define TC_NU 0.01       /* super-step damping factor, :37 */
#define TC_RED 0.25      /* tstep_red_factor, :41 */
#define TC_CLIGHT 3.e10  /* :195, :281 */

/* real**integer with a variable exponent: gfortran evaluates it by binary
 * (square-and-multiply) exponentiation, which this restates */
static double powi_sq(double x, int m) {
  unsigned n = m < 0 ? 0u - (unsigned)m : (unsigned)m;
  double y = (n % 2u) ? x : 1.0;
  while (n >>= 1) {
    x = x * x;
    if (n % 2u) y = y * x;
  }
  return m < 0 ? 1.0 / y : y;
}

/* :625-636 superstep: length of a super step of N substeps */
double gor_superstep(int N, double snu) {
  const double a = powi_sq(1.0 + snu, 2 * N), b = powi_sq(1.0 - snu, 2 * N);
  return (double)N / (2.0 * snu) * (a - b) / (a + b);
}

/* :646-654 substep: size of substep j of N */
double gor_substep(int j, int N, double nu) {
  const double pi = acos(-1.0);
  return 1.0 / ((nu - 1.0) * cos(pi * (double)(2 * j - 1) / (2.0 * (double)N)) + nu + 1.0);
}

/* :664-681 ST_steps: the first N whose super step exceeds fs (200 when none
 * of 1..199 does, the value of the Fortran DO index after the loop) */
void gor_st_steps(double fs, int* Ns, double* fstep) {
  const double snu = sqrt(TC_NU);
  int j;
  for (j = 1; j <= 199; ++j)
    if (gor_superstep(j, snu) > fs) break;
  *Ns = j;
  *fstep = fs / gor_superstep(j, snu);
}

/* :142-178 Spitzer conductivities */
static double ksp(double T) { return 6.e-7 * pow(T, 2.5); }
static double ksp_parl(double T) { return 9.2181e-7 * pow(T, 2.5); }
static double ksp_perp(double T, double dens, double B2) {
  return 0.30089e+33 * dens / (B2 * sqrt(T)) * dens;
}

/* :78-110 get_dt_cond (seconds) */
static double get_dt_cond(gor_state_t* s) {
  const gor_params_t* p = &s->p;
  double dtp = 1.7976931348623157e308; /* huge(1.) */
  double ddx = dmin(p->dx, p->dy);
  ddx = dmin(ddx, p->dz);
  for (int k = 1; k <= p->nz; ++k)
    for (int j = 1; j <= p->ny; ++j)
      for (int i = 1; i <= p->nx; ++i)
        dtp = dmin(dtp, AT(s, s->primit, 1, i, j, k) / ksp(s->temp[CID(s, i, j, k)]));
  const double x = ddx * p->rsc;
  return TC_RED * 0.5 * (x * x) * p->cv * TC_RG * dtp * p->rhosc / p->mu;
}

/* One face of :189-267 heatfluxes: the flux from cell a to cell b (b = a + 1
 * along the face normal), spacing d */
static double heatflux_iso(const gor_state_t* s, size_t a, size_t b, double d) {
  const gor_params_t* p = &s->p;
  const int neq = p->neq;
  const double yhp = 1.0;
  const double Ta = s->temp[a], Tb = s->temp[b];
  if (Ta == Tb) return 0.0;
  const double meanP = 0.5 * (s->primit[a * neq + 4] + s->primit[b * neq + 4]);
  const double meanDens = 0.5 * (s->primit[a * neq] + s->primit[b * neq]);
  const double meanT = 0.5 * (Ta + Tb);
  const double dT = (Tb - Ta) / (d * p->rsc);
  double coef;
  if (p->tc_saturation) {
    double cs = csound(p, meanP, meanDens);
    cs = dmin(cs * sqrt(p->vsc2), TC_CLIGHT);
    coef = dmin(ksp(meanT), 5. * TC_PH * cs * meanP * p->Psc / fabs(dT));
  } else {
    coef = ksp(meanT);
  }
  return -coef * dT * yhp;
}

static void heatfluxes(gor_state_t* s) {
  const gor_params_t* p = &s->p;
  const int neq = p->neq;
#pragma omp parallel for schedule(static)
  for (int k = 0; k <= p->nz; ++k)
    for (int j = 0; j <= p->ny; ++j)
      for (int i = 0; i <= p->nx; ++i) {
        const size_t c = CID(s, i, j, k);
        s->f[c * neq + 4] = heatflux_iso(s, c, CID(s, i + 1, j, k), p->dx);
        s->g[c * neq + 4] = heatflux_iso(s, c, CID(s, i, j + 1, k), p->dy);
        s->h[c * neq + 4] = heatflux_iso(s, c, CID(s, i, j, k + 1), p->dz);
      }
}

/* :277-487 MHD_heatfluxes: conduction along and across the unit vector of B
 * of the cell on the left of the three faces */
static void mhd_heatfluxes(gor_state_t* s) {
  const gor_params_t* p = &s->p;
  const int neq = p->neq;
  const double phi = 0.3, alpha = 5.0 * phi;
  const double bsc2 = p->bsc * p->bsc;
  const double vsc = sqrt(p->vsc2);
#pragma omp parallel for schedule(static)
  for (int k = 0; k <= p->nz; ++k)
    for (int j = 0; j <= p->ny; ++j)
      for (int i = 0; i <= p->nx; ++i) {
        const size_t c = CID(s, i, j, k);
        const size_t nb[3] = {CID(s, i + 1, j, k), CID(s, i, j + 1, k), CID(s, i, j, k + 1)};
        const double dd[3] = {p->dx, p->dy, p->dz};
        double bx = s->primit[c * neq + 5], by = s->primit[c * neq + 6], bz = s->primit[c * neq + 7];
        const double B2 = bx * bx + by * by + bz * bz;
        const double modB = sqrt(B2);
        bx = bx / modB;
        by = by / modB;
        bz = bz / modB;
        double grad[3], kpar[3], kperp[3], csat[3];
        for (int a = 0; a < 3; ++a) {
          const double Tc = s->temp[c], Tn = s->temp[nb[a]];
          if (fabs(Tc - Tn) < 1.0e-14) {
            grad[a] = 0.0;
            kpar[a] = 0.0;
            kperp[a] = 0.0;
            csat[a] = 0.0;
            continue;
          }
          const double meanDens = 0.5 * (s->primit[c * neq] + s->primit[nb[a] * neq]);
          const double meanTemp = 0.5 * (Tc + Tn);
          if (p->tc_saturation) {
            const double meanPres = 0.5 * (s->primit[c * neq + 4] + s->primit[nb[a] * neq + 4]);
            double cs = csound(p, meanPres, meanDens);
            cs = dmin(cs * vsc, TC_CLIGHT);
            csat[a] = alpha * meanDens * (cs * cs * cs);
          } else {
            csat[a] = 0.0;
          }
          grad[a] = (Tn - Tc) / (dd[a] * p->rsc);
          kpar[a] = ksp_parl(meanTemp);
          kperp[a] = ksp_perp(meanTemp, meanDens * p->rhosc, B2 * bsc2);
        }
        const double bgradT = bx * grad[0] + by * grad[1] + bz * grad[2];
        const double gpar[3] = {bgradT * bx, bgradT * by, bgradT * bz};
        const double gperp[3] = {grad[0] - gpar[0], grad[1] - gpar[1], grad[2] - gpar[2]};
        double out[3];
        if (!p->tc_saturation) {
          for (int a = 0; a < 3; ++a) out[a] = -kpar[a] * gpar[a] - kperp[a] * gperp[a];
        } else {
          const double gpar_n = bgradT;
          const double gperp_n = sqrt(gperp[0] * gperp[0] + gperp[1] * gperp[1] + gperp[2] * gperp[2]);
          for (int a = 0; a < 3; ++a)
            out[a] = -1. / (1. / (kpar[a] + 1.e-14) + gpar_n / (csat[a] + 1.e-14)) * gpar[a]
                     - 1. / (1. / (kperp[a] + 1.e-14) + gperp_n / (csat[a] + 1.e-14)) * gperp[a];
        }
        s->f[c * neq + 4] = out[0];
        s->g[c * neq + 4] = out[1];
        s->h[c * neq + 4] = out[2];
      }
}

/* :496-616 thermal_bounds, serial build: the periodic copies of the first
 * ghost layer of u(5), then, unconditionally, the outflow copies of the
 * physical walls, which overwrite the periodic ones over 0:n+1 */
static void thermal_bounds(gor_state_t* s) {
  const gor_params_t* p = &s->p;
  const int neq = p->neq, nx = p->nx, ny = p->ny, nz = p->nz;
#define U5(i, j, k) s->u[CID(s, i, j, k) * neq + 4]
  if (p->bc_left == GOR_BC_PERIODIC && p->bc_right == GOR_BC_PERIODIC)
    for (int k = 1 - NG; k <= nz + NG; ++k)
      for (int j = 1 - NG; j <= ny + NG; ++j) {
        U5(0, j, k) = U5(nx, j, k);
        U5(nx + 1, j, k) = U5(1, j, k);
      }
  if (p->bc_bottom == GOR_BC_PERIODIC && p->bc_top == GOR_BC_PERIODIC)
    for (int k = 1 - NG; k <= nz + NG; ++k)
      for (int i = 1 - NG; i <= nx + NG; ++i) {
        U5(i, 0, k) = U5(i, ny, k);
        U5(i, ny + 1, k) = U5(i, 1, k);
      }
  if (p->bc_out == GOR_BC_PERIODIC && p->bc_in == GOR_BC_PERIODIC)
    for (int j = 1 - NG; j <= ny + NG; ++j)
      for (int i = 1 - NG; i <= nx + NG; ++i) {
        U5(i, j, 0) = U5(i, j, nz);
        U5(i, j, nz + 1) = U5(i, j, 1);
      }
  for (int k = 0; k <= nz + 1; ++k)
    for (int j = 0; j <= ny + 1; ++j) U5(0, j, k) = U5(1, j, k);
  for (int k = 0; k <= nz + 1; ++k)
    for (int j = 0; j <= ny + 1; ++j) U5(nx + 1, j, k) = U5(nx, j, k);
  for (int k = 0; k <= nz + 1; ++k)
    for (int i = 0; i <= nx + 1; ++i) U5(i, 0, k) = U5(i, 1, k);
  for (int k = 0; k <= nz + 1; ++k)
    for (int i = 0; i <= nx + 1; ++i) U5(i, ny + 1, k) = U5(i, ny, k);
  for (int j = 0; j <= ny + 1; ++j)
    for (int i = 0; i <= nx + 1; ++i) U5(i, j, 0) = U5(i, j, 1);
  for (int j = 0; j <= ny + 1; ++j)
    for (int i = 0; i <= nx + 1; ++i) U5(i, j, nz + 1) = U5(i, j, nz);
#undef U5
}

/* :690-768 thermal_conduction, from primit and Temp of the last calcprim */
void gor_thermal_conduction(gor_state_t* s, double dt_CFL, int* nsteps_out, double* dt_cond_out) {
  const gor_params_t* p = &s->p;
  const int neq = p->neq;
  const double dt_hydro = dt_CFL * p->tsc;
  const double dt_cond = get_dt_cond(s);
  int SuperStep = 1, Nsteps;
  double fstep;
  if (dt_cond < dt_hydro) {
    gor_st_steps(dt_hydro / dt_cond, &Nsteps, &fstep);
  } else {
    SuperStep = 0;
    fstep = dt_hydro / dt_cond;
    Nsteps = 1;
  }
  if (nsteps_out) *nsteps_out = Nsteps;
  if (dt_cond_out) *dt_cond_out = dt_cond;
  for (int n = 1; n <= Nsteps; ++n) {
    double dts;
    if (SuperStep)
      dts = dt_cond * fstep * gor_substep(n, Nsteps, TC_NU) / p->Psc / p->rsc;
    else
      dts = dt_hydro / (double)Nsteps / p->Psc / p->rsc;
    if (p->th_cond == 2) mhd_heatfluxes(s);
    if (p->th_cond == 1) heatfluxes(s);
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= p->nz; ++k)
      for (int j = 1; j <= p->ny; ++j)
        for (int i = 1; i <= p->nx; ++i) {
          const size_t c = CID(s, i, j, k);
          s->u[c * neq + 4] =
              s->u[c * neq + 4] -
              dts * ((s->f[c * neq + 4] - s->f[CID(s, i - 1, j, k) * neq + 4]) / p->dx +
                     (s->g[c * neq + 4] - s->g[CID(s, i, j - 1, k) * neq + 4]) / p->dy +
                     (s->h[c * neq + 4] - s->h[CID(s, i, j, k - 1) * neq + 4]) / p->dz);
        }
    thermal_bounds(s);
    calcprim_arr(s, s->u, 0);
  }
}

void gor_get_temp(const gor_state_t* s, double* temp) {
  memcpy(temp, s->temp, s->ncell * sizeof(double));
}

/* src/hydro_solver.f90:134-229  tstep */
void gor_tstep(gor_state_t* s, double dt_CFL) {
  const gor_params_t* p = &s->p;
  double dtm = dt_CFL / 2.0;
  fluxes(s, 1);
  step(s, dtm);
  boundaryII(s);
  calcprim_arr(s, s->up, 0);
  fluxes(s, 2);
  step(s, dt_CFL);
  viscous_copy(s);
  if (p->cooling == GOR_COOL_H) coolingh(s, dt_CFL);
  int table = p->cooling == GOR_COOL_DMC || p->cooling == GOR_COOL_CHI;
  if (table) cooling_table(s, dt_CFL);
  gor_boundaryI(s);
  calcprim_arr(s, s->u, table);
  if (p->th_cond != 0) gor_thermal_conduction(s, dt_CFL, NULL, NULL);
}

/* ---------------------------------------------------------------------- */
gor_state_t* gor_create(const gor_params_t* p) {
  if (p->nx < 1 || p->ny < 1 || p->nz < 1) return NULL;
  if (p->npas < 0 || p->npas > 2) return NULL;
  if (neqdyn(p) != 5 && neqdyn(p) != 8) return NULL;
  gor_state_t* s = (gor_state_t*)calloc(1, sizeof(gor_state_t));
  s->p = *p;
  s->NX = p->nx + 2 * NG;
  s->NY = p->ny + 2 * NG;
  s->NZ = p->nz + 2 * NG;
  s->ncell = (size_t)s->NX * s->NY * s->NZ;
  size_t nv = s->ncell * (size_t)p->neq;
  s->u = (double*)calloc(nv, sizeof(double));
  s->up = (double*)calloc(nv, sizeof(double));
  s->primit = (double*)calloc(nv, sizeof(double));
  s->f = (double*)calloc(nv, sizeof(double));
  s->g = (double*)calloc(nv, sizeof(double));
  s->h = (double*)calloc(nv, sizeof(double));
  s->e = (double*)calloc(s->ncell * 3, sizeof(double));
  s->temp = (double*)calloc(s->ncell, sizeof(double));
  if (split_all(p)) s->primit0 = (double*)calloc(nv, sizeof(double));
  if (!s->u || !s->up || !s->primit || !s->f || !s->g || !s->h || !s->e || !s->temp ||
      (split_all(p) && !s->primit0)) {
    gor_destroy(s);
    return NULL;
  }
  return s;
}

void gor_destroy(gor_state_t* s) {
  if (!s) return;
  free(s->u); free(s->up); free(s->primit);
  free(s->f); free(s->g); free(s->h); free(s->e); free(s->temp); free(s->primit0);
  free(s);
}

int gor_nthreads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

void gor_set_background(gor_state_t* s, const double* primit0) {
  if (s->primit0) memcpy(s->primit0, primit0, s->ncell * s->p.neq * sizeof(double));
}
void gor_set_u(gor_state_t* s, const double* u) {
  memcpy(s->u, u, s->ncell * s->p.neq * sizeof(double));
}
void gor_get_u(const gor_state_t* s, double* u) {
  memcpy(u, s->u, s->ncell * s->p.neq * sizeof(double));
}
void gor_get_primit(const gor_state_t* s, double* pr) {
  memcpy(pr, s->primit, s->ncell * s->p.neq * sizeof(double));
}
void gor_set_primit(gor_state_t* s, const double* pr) {
  memcpy(s->primit, pr, s->ncell * s->p.neq * sizeof(double));
}
double gor_time(const gor_state_t* s) { return s->time; }
void gor_set_time(gor_state_t* s, double t) { s->time = t; }
int gor_error(const gor_state_t* s) { return s->err; }

void gor_riemann(const gor_params_t* p, const double* pl, const double* pr, double* ff,
                 int* err) {
  riemann(p, pl, pr, ff, err);
}
void gor_prim2f(const gor_params_t* p, const double* prim, double* ff) { prim2f(p, prim, ff); }
void gor_u2prim(const gor_params_t* p, const double* uu, double* prim, double* T) {
  u2prim(p, uu, prim, T);
}
void gor_prim2u(const gor_params_t* p, const double* prim, double* uu) { prim2u(p, prim, uu); }
void gor_limiter(const gor_params_t* p, const double* pll, double* pl, double* pr,
                 const double* prr) {
  limiter(p, pll, pl, pr, prr);
}
double gor_cooltab(const gor_params_t* p, double T) { return cooltab(p, T); }

void gor_divb(const gor_state_t* s, double* divb) {
  const gor_params_t* p = &s->p;
  const int nx = p->nx, ny = p->ny, nz = p->nz;
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i)
        divb[((size_t)(k - 1) * ny + (j - 1)) * nx + (i - 1)] =
            (AT(s, s->u, 6, i + 1, j, k) - AT(s, s->u, 6, i - 1, j, k)) / (2.0 * p->dx)
            + (AT(s, s->u, 7, i, j + 1, k) - AT(s, s->u, 7, i, j - 1, k)) / (2.0 * p->dy)
            + (AT(s, s->u, 8, i, j, k + 1) - AT(s, s->u, 8, i, j, k - 1)) / (2.0 * p->dz);
}

/* src/main.f90:94-125 */
int gor_run(gor_state_t* s, double tmax, double dtprint, int max_steps, int n_iter, int* iter,
            double* tprint) {
  int steps = 0;
  while (s->time <= tmax && steps < max_steps) {
    double dt;
    int dump = 0;
    gor_get_timestep(s, *iter, n_iter, s->time, *tprint, &dt, &dump);
    gor_tstep(s, dt);
    s->time = s->time + dt;
    if (dump) *tprint = *tprint + dtprint;
    *iter = *iter + 1;
    ++steps;
    if (s->err) break;
  }
  return steps;
}
