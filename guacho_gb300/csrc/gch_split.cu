// gch_split.cu -- the split solver SOLVER_HLLE_SPLIT_ALL on the FP64 path.
//
// The state is a fluctuation over a background primit0 (src/globals.f90:42)
// that the caller sets with gch_set_background; the reference allocates it
// but never sets it, and here it is zero until set.  A step is the reference's
// tstep (src/hydro_solver.f90:134-229) with the split routines:
//   k_split_flux<1>   hllEfluxesSplitAll(1) (src/hlle_split_all.f90:96-153):
//                     the x, y and z face fluxes of cells 0..n into F
//   k_split_update<1> step(dt/2): up = u - dt/2 div F (hydro fields with
//                     flux-CD, all fields without) and the cell-centred E of
//                     get_efield (src/flux_cd_module.f90:254-269)
//   k_ct<1>           flux_cd_update of B (the kernel of the other solvers)
//   boundaryII on up, k_split_prim (calcprim with u2primSplitAll)
//   k_split_flux<2>, k_split_update<2>, k_ct<2>, [k_visc], boundaryI on u,
//   k_split_prim
// and get_timestep is k_split_cfl (the fast speeds of the total state,
// src/hydro_core.f90:650-655) + k_dtfin.  FP64 throughout, compiled without
// multiply-add contraction, with the reference's expression order: the
// oracle's restatement matches it bitwise.  Face fluxes go through global
// memory (3 x neq fields): the split solver is a rarely used option, and this
// keeps its code apart from the tiled stage kernels.
#include <cuda_runtime.h>

#include "gch_domain.h"
#include "gch_engine.cuh"

namespace gch {
namespace {

constexpr int kN = 8;  // MHD only (the split branches are written for B)

// src/hydro_core.f90:143-229 u2primSplitAll (no density or pressure floor)
__device__ __forceinline__ void u2prim_split(const KParams& p, const double* uu,
                                             const double* p0, double* prim) {
  prim[0] = uu[0];
  const double r = prim[0] + p0[0];
  prim[1] = uu[1] / r;
  prim[2] = uu[2] / r;
  prim[3] = uu[3] / r;
  prim[5] = uu[5];
  prim[6] = uu[6];
  prim[7] = uu[7];
  prim[4] = (uu[4] - 0.5 * r * (prim[1] * prim[1] + prim[2] * prim[2] + prim[3] * prim[3])
             - 0.5 * (uu[5] * uu[5] + uu[6] * uu[6] + uu[7] * uu[7])
             - p0[5] * uu[5] - p0[6] * uu[6] - p0[7] * uu[7]) / p.cv;
}

// src/hydro_core.f90:331-383 prim2u, split branch
__device__ __forceinline__ void prim2u_split(const KParams& p, const double* prim,
                                             const double* p0, double* uu) {
  uu[0] = prim[0];
  uu[1] = prim[1] * (prim[0] + p0[0]);
  uu[2] = prim[2] * (prim[0] + p0[0]);
  uu[3] = prim[3] * (prim[0] + p0[0]);
  const double v2 = prim[1] * prim[1] + prim[2] * prim[2] + prim[3] * prim[3];
  uu[4] = 0.5 * prim[0] * v2 + p.cv * prim[4];
  uu[4] = uu[4] + 0.5 * (prim[5] * prim[5] + prim[6] * prim[6] + prim[7] * prim[7])
          + 0.5 * p0[0] * v2 + p0[5] * prim[5] + p0[6] * prim[6] + p0[7] * prim[7];
  uu[5] = prim[5];
  uu[6] = prim[6];
  uu[7] = prim[7];
}

// src/hydro_core.f90:395-476 prim2f, split branch (x direction)
__device__ __forceinline__ void prim2f_split(const KParams& p, const double* prim,
                                             const double* p0, double* ff) {
  const double rt = prim[0] + p0[0];
  const double b6 = prim[5], b7 = prim[6], b8 = prim[7];
  const double etot = 0.5 * (rt * (prim[1] * prim[1] + prim[2] * prim[2] + prim[3] * prim[3])
                             + b6 * b6 + b7 * b7 + b8 * b8)
                      + p.cv * prim[4] + p0[5] * b6 + p0[6] * b7 + p0[7] * b8;
  ff[0] = rt * prim[1];
  ff[1] = rt * prim[1] * prim[1] + prim[4] + 0.5 * (b7 * b7 + b8 * b8 - b6 * b6)
          - p0[5] * b6 + p0[6] * b7 + p0[7] * b8;
  ff[2] = rt * prim[1] * prim[2] - b6 * b7 - p0[6] * b6 - p0[5] * b7;
  ff[3] = rt * prim[1] * prim[3] - b6 * b8 - p0[7] * b6 - p0[5] * b8;
  const double t6 = b6 + p0[5], t7 = b7 + p0[6], t8 = b8 + p0[7];
  ff[4] = prim[1] * (etot + prim[4] + 0.5 * (t6 * t6 + t7 * t7 + t8 * t8) + p.cv * p0[4]
                     + p0[4] + 0.5 * (p0[5] * p0[5] + p0[6] * p0[6] + p0[7] * p0[7]))
          - t6 * (prim[1] * t6 + prim[2] * t7 + prim[3] * t8);
  ff[5] = 0.0;
  ff[6] = prim[1] * (p0[6] + b7) - prim[2] * (p0[5] + b6);
  ff[7] = prim[1] * (p0[7] + b8) - prim[3] * (p0[5] + b6);
}

// src/hlle_split_all.f90:51-84 prim2fhlleSplitAll
__device__ __forceinline__ void hlle_split(const KParams& p, const double* pl, const double* pr,
                                           const double* ql, const double* qr, double* ff) {
  double tl[kN], tr[kN];
#pragma unroll
  for (int q = 0; q < kN; ++q) {
    tl[q] = pl[q] + ql[q];
    tr[q] = pr[q] + qr[q];
  }
  const double csl = cfastX(p, tl), csr = cfastX(p, tr);
  const double sr = tmax_(pl[1] + ql[1] + csl, pr[1] + qr[1] + csr);
  const double sl = tmin_(pl[1] + ql[1] - csl, pr[1] + qr[1] - csr);
  if (sl > 0.0) { prim2f_split(p, pl, ql, ff); return; }
  if (sr < 0.0) { prim2f_split(p, pr, qr, ff); return; }
  double fL[kN], fR[kN], uL[kN], uR[kN];
  prim2f_split(p, pl, ql, fL);
  prim2f_split(p, pr, qr, fR);
  prim2u_split(p, pl, ql, uL);
  prim2u_split(p, pr, qr, uR);
#pragma unroll
  for (int q = 0; q < kN; ++q)
    ff[q] = (sr * fL[q] - sl * fR[q] + sl * sr * (uR[q] - uL[q])) / (sr - sl);
}

// src/hydro_core.f90:485-534 swapy / swapz
__device__ __forceinline__ void swap_dir(int dir, double* v) {
  const int a = dir == 1 ? 2 : 3, b = dir == 1 ? 6 : 7;
  double t = v[1]; v[1] = v[a]; v[a] = t;
  t = v[5]; v[5] = v[b]; v[b] = t;
}

// calcprim of every cell with u2primSplitAll
__global__ void k_split_prim(KParams p, const double* __restrict__ u,
                             const double* __restrict__ prim0, double* __restrict__ primit,
                             const StepScalars* sc) {
  const int ax = blockIdx.x * blockDim.x + threadIdx.x;
  const int ay = blockIdx.y * blockDim.y + threadIdx.y;
  const int az = blockIdx.z;
  if (ax >= p.NX || ay >= p.NY || !sc->active) return;
  const long long c = cell_index(p, ax, ay, az);
  double uu[kN], q0[kN], pr[kN];
#pragma unroll
  for (int q = 0; q < kN; ++q) {
    uu[q] = u[q * p.fs + c];
    q0[q] = prim0[q * p.fs + c];
  }
  u2prim_split(p, uu, q0, pr);
#pragma unroll
  for (int q = 0; q < kN; ++q) primit[q * p.fs + c] = pr[q];
}

// The three face fluxes of cell (i, j, k), i, j, k in 0..n: F holds 3 x kN
// fields, direction-major; the flux through face i+1/2 is stored at cell i
template <int STAGE>
__global__ void k_split_flux(KParams p, const double* __restrict__ primit,
                             const double* __restrict__ prim0, double* __restrict__ F,
                             const StepScalars* sc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > p.nx || j > p.ny || !sc->active) return;
  const long long c = cell_index(p, i + NG - 1, j + NG - 1, k + NG - 1);
  const long long step[3] = {1, p.pitch, (long long)p.pitch * p.NY};
  for (int dir = 0; dir < 3; ++dir) {
    const long long s = step[dir];
    double pl[kN], pr[kN], ql[kN], qr[kN], ff[kN];
#pragma unroll
    for (int q = 0; q < kN; ++q) {
      pl[q] = primit[q * p.fs + c];
      pr[q] = primit[q * p.fs + c + s];
      ql[q] = prim0[q * p.fs + c];
      qr[q] = prim0[q * p.fs + c + s];
    }
    if (dir) {
      swap_dir(dir, pl); swap_dir(dir, pr); swap_dir(dir, ql); swap_dir(dir, qr);
    }
    if (STAGE == 2) {  // src/hydro_core.f90:712-733 limiter on both states
      double pll[kN], prr[kN], qll[kN], qrr[kN];
#pragma unroll
      for (int q = 0; q < kN; ++q) {
        pll[q] = primit[q * p.fs + c - s];
        prr[q] = primit[q * p.fs + c + 2 * s];
        qll[q] = prim0[q * p.fs + c - s];
        qrr[q] = prim0[q * p.fs + c + 2 * s];
      }
      if (dir) {
        swap_dir(dir, pll); swap_dir(dir, prr); swap_dir(dir, qll); swap_dir(dir, qrr);
      }
#pragma unroll
      for (int q = 0; q < kN; ++q) {
        const double al = average(p.limiter, pl[q] - pll[q], pr[q] - pl[q]);
        const double ar = average(p.limiter, pr[q] - pl[q], prr[q] - pr[q]);
        pl[q] = pl[q] + al * 0.5;
        pr[q] = pr[q] - ar * 0.5;
        const double bl = average(p.limiter, ql[q] - qll[q], qr[q] - ql[q]);
        const double br = average(p.limiter, qr[q] - ql[q], qrr[q] - qr[q]);
        ql[q] = ql[q] + bl * 0.5;
        qr[q] = qr[q] - br * 0.5;
      }
    }
    hlle_split(p, pl, pr, ql, qr, ff);
    if (dir) swap_dir(dir, ff);
#pragma unroll
    for (int q = 0; q < kN; ++q) F[(dir * kN + q) * p.fs + c] = ff[q];
  }
}

// step (src/hydro_solver.f90:77-127) from the stored face fluxes, and the
// cell-centred E of get_efield (src/flux_cd_module.f90:258-265)
template <int STAGE>
__global__ void k_split_update(KParams p, const double* __restrict__ src,
                               double* __restrict__ dst, const double* __restrict__ F,
                               double* __restrict__ E, const StepScalars* sc) {
  const int ci = blockIdx.x * blockDim.x + threadIdx.x;
  const int cj = blockIdx.y * blockDim.y + threadIdx.y;
  const int ck = blockIdx.z;
  if (ci >= p.nx || cj >= p.ny || !sc->active) return;
  const long long sy = p.pitch, sz = (long long)p.pitch * p.NY;
  const long long c = cell_index(p, ci + NG, cj + NG, ck + NG);
  const double dtdx = sc->dtd[STAGE - 1][0], dtdy = sc->dtd[STAGE - 1][1],
               dtdz = sc->dtd[STAGE - 1][2];
  const bool ct = p.flux_cd;
  const double* G = F + kN * p.fs;
  const double* H = F + 2 * kN * p.fs;
#pragma unroll
  for (int q = 0; q < kN; ++q) {
    if (ct && q >= 5) continue;  // B from flux_cd_update
    const long long o = q * p.fs + c;
    dst[o] = Ops<PolFP64>::update(src[o], dtdx, dtdy, dtdz, F[o - 1], F[o], G[o - sy], G[o],
                                  H[o - sz], H[o]);
  }
  if (ct) {
    E[c] = 0.25 * (-G[7 * p.fs + c - sy] - G[7 * p.fs + c] + H[6 * p.fs + c - sz]
                   + H[6 * p.fs + c]);
    E[p.fs + c] = 0.25 * (+F[7 * p.fs + c - 1] + F[7 * p.fs + c] - H[5 * p.fs + c - sz]
                          - H[5 * p.fs + c]);
    E[2 * p.fs + c] = 0.25 * (-F[6 * p.fs + c - 1] - F[6 * p.fs + c] + G[5 * p.fs + c - sy]
                              + G[5 * p.fs + c]);
  }
}

// get_timestep (src/hydro_core.f90:644-675, split branch): the fast speeds of
// the total state, the velocity of primit
__global__ void __launch_bounds__(256)
k_split_cfl(KParams p, const double* __restrict__ primit, const double* __restrict__ prim0,
            StepScalars* sc, int kz) {
  if (!sc->active) return;
  const int ci = blockIdx.x * 32 + threadIdx.x;
  const int cj = blockIdx.y * 8 + threadIdx.y;
  const int kb = blockIdx.z * kz;
  const int ke = min(p.nz, kb + kz);
  const CflConst<double> kc(p);
  double dtp = 1e30;
  int bad = 0;
  if (ci < p.nx && cj < p.ny) {
    for (int k = kb; k < ke; ++k) {
      const long long c = cell_index(p, ci + NG, cj + NG, k + NG);
      double pt[kN];
#pragma unroll
      for (int q = 0; q < kN; ++q) pt[q] = primit[q * p.fs + c];
      pt[0] = pt[0] + prim0[c];
      pt[4] = pt[4] + prim0[4 * p.fs + c];
      pt[5] = pt[5] + prim0[5 * p.fs + c];
      pt[6] = pt[6] + prim0[6 * p.fs + c];
      pt[7] = pt[7] + prim0[7 * p.fs + c];
      cfl_candidate<double, kN>(p, kc, pt, dtp, bad);
    }
  }
  cfl_block_reduce<double>(dtp, bad, sc);
}

__global__ void k_split_set_prim0(KParams p, const double* __restrict__ aos,
                                  double* __restrict__ prim0) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
       t < (long long)p.NX * p.NY * p.NZ; t += (long long)gridDim.x * blockDim.x) {
    const int ax = (int)(t % p.NX);
    const int ay = (int)((t / p.NX) % p.NY);
    const int az = (int)(t / ((long long)p.NX * p.NY));
    const long long c = cell_index(p, ax, ay, az);
    for (int q = 0; q < p.neq; ++q) prim0[q * p.fs + c] = aos[t * p.neq + q];
  }
}

using E64 = Engine<PolFP64>;

void prim_of(gch_domain* d, const double* a) {
  const KParams& p = d->kp;
  const dim3 b(32, 8), g((p.NX + 31) / 32, (p.NY + 7) / 8, p.NZ);
  k_split_prim<<<g, b, 0, d->stream>>>(p, a, d->prim0, (double*)d->primit, d->sc);
  gch_mark(d, "k_split_prim");
}

}  // namespace

int split_calcprim(gch_domain* d) {
  prim_of(d, (const double*)d->u);
  return cuda_status(cudaGetLastError());
}

int split_get_dt(gch_domain* d) {
  const KParams& p = d->kp;
  k_split_cfl<<<E64::column_grid(p), dim3(32, 8), 0, d->stream>>>(
      p, (const double*)d->primit, d->prim0, d->sc, E64::kzc);
  gch_mark(d, "k_split_cfl");
  k_dtfin<<<1, 1, 0, d->stream>>>(d->sc, p.cfl, p.dx, p.dy, p.dz);
  gch_mark(d, "k_dtfin");
  return cuda_status(cudaGetLastError());
}

int split_tstep(gch_domain* d) {
  const KParams& p = d->kp;
  cudaStream_t s = d->stream;
  d->launches = 0;
  const bool ct = p.flux_cd != 0;
  const dim3 b(32, 8);
  const dim3 gface((p.nx + 1 + 31) / 32, (p.ny + 1 + 7) / 8, p.nz + 1);
  const dim3 gint((p.nx + 31) / 32, (p.ny + 7) / 8, p.nz);
  double* u = (double*)d->u;
  double* up = (double*)d->up;
  double* E = (double*)d->E;
  // 1st half step from the primitives of u (the previous calcprim)
  k_split_flux<1><<<gface, b, 0, s>>>(p, (const double*)d->primit, d->prim0, d->split_f, d->sc);
  k_split_update<1><<<gint, b, 0, s>>>(p, u, up, d->split_f, E, d->sc);
  d->launches += 2;
  gch_mark(d, "k_split_stage1");
  if (ct) {
    k_ct<PolFP64, 1><<<E64::column_grid(p), b, 0, s>>>(p, u, up, E, nullptr, d->sc, E64::kzc);
    ++d->launches;
    gch_mark(d, "k_ct_stage1");
  }
  E64::ghost<double>(d, up, 2);
  prim_of(d, up);
  ++d->launches;
  // 2nd half step
  double* dst2 = p.eta != 0.0 ? (double*)d->w : u;
  k_split_flux<2><<<gface, b, 0, s>>>(p, (const double*)d->primit, d->prim0, d->split_f, d->sc);
  k_split_update<2><<<gint, b, 0, s>>>(p, u, dst2, d->split_f, E, d->sc);  // u - dt div F
  d->launches += 2;
  gch_mark(d, "k_split_stage2");
  if (ct) {
    k_ct<PolFP64, 2><<<E64::column_grid(p), b, 0, s>>>(p, u, dst2, E, nullptr, d->sc, E64::kzc);
    ++d->launches;
    gch_mark(d, "k_ct_stage2");
  }
  if (p.eta != 0.0) {
    k_visc<PolFP64, kN><<<gint, b, 0, s>>>(p, u, (const double*)d->w, up, d->sc);
    ++d->launches;
    gch_mark(d, "k_visc");
  }
  E64::ghost<double>(d, u, 1);
  prim_of(d, u);
  ++d->launches;
  return cuda_status(cudaGetLastError());
}

int split_set_background(gch_domain* d, const double* aos) {
  k_split_set_prim0<<<152 * 8, 256, 0, d->stream>>>(d->kp, aos, d->prim0);
  return cuda_status(cudaGetLastError());
}

int split_download_prim(gch_domain* d, double* aos) {
  k_soa_to_aos<double><<<E64::kLayoutGrid, kLayoutCells, 0, d->stream>>>(
      d->kp, (const double*)d->primit, aos, d->kp.neq);
  return cuda_status(cudaGetLastError());
}

}  // namespace gch
