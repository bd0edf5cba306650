// gch_api.cu -- the C ABI declared in include/guacho_gb300.h: parameter
// validation, device allocation, host<->device transfers, and the host-side
// sequencing of the per-precision engines.
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <new>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "gch_domain.h"

using gch::EngineOps;
using gch::KParams;
using gch::StepScalars;

namespace gch {

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library), looked up once.
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  }();
  return fn;
}

int encode_stage_map(unsigned char* map, const void* base, int es, const KParams& k, int box_x,
                     int box_rows) {
  static_assert(sizeof(CUtensorMap) == kTmaMapBytes, "tensor map size");
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc || (es != 4 && es != 8) || box_x * es % 16 != 0) return GCH_ERR_CUDA;
  // dims fastest first: x (the NX cells of a row with ghosts; the row
  // padding is never copied), field, y, z; strides in bytes of field, row,
  // plane (multiples of 16: rows are padded to 4 elements)
  const cuuint64_t dims[4] = {(cuuint64_t)k.NX, (cuuint64_t)k.neq, (cuuint64_t)k.NY,
                              (cuuint64_t)k.NZ};
  const cuuint64_t strides[3] = {(cuuint64_t)k.fs * es, (cuuint64_t)k.pitch * es,
                                 (cuuint64_t)k.pitch * k.NY * es};
  const cuuint32_t box[4] = {(cuuint32_t)box_x, (cuuint32_t)k.neq, (cuuint32_t)box_rows, 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  CUtensorMap* m = reinterpret_cast<CUtensorMap*>(map);
  const CUresult r = enc(m, es == 8 ? CU_TENSOR_MAP_DATA_TYPE_UINT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                         4, const_cast<void*>(base), dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? GCH_OK : GCH_ERR_CUDA;
}

}  // namespace gch

namespace {

const EngineOps& engine(const gch_domain* d) {
  if (d->mode == GCH_FP64) return gch::kEngineFP64;
  if (d->mode == GCH_FP32_KAHAN) return gch::kEngineKahan;
  return gch::kEngineMixed;
}

int cuda_ok(cudaError_t e) { return e == cudaSuccess ? GCH_OK : GCH_ERR_CUDA; }

bool valid_bc(int b) {
  return b == GCH_BC_OUTFLOW || b == GCH_BC_CLOSED || b == GCH_BC_PERIODIC || b == GCH_BC_OTHER;
}

// Device-side control writes: launched with by-value arguments so no host
// buffer must outlive the call.
__global__ void k_set_ctrl(StepScalars* sc, int iter, int n_iter, double time, double tprint,
                           double dtprint, double tmax, int active) {
  sc->iter = iter;
  sc->n_iter = n_iter;
  sc->time = time;
  sc->tprint = tprint;
  sc->dtprint = dtprint;
  sc->tmax = tmax;
  sc->active = active;
  sc->dump = 0;
}
__global__ void k_set_dt(StepScalars* sc, double dt, double dx, double dy, double dz) {
  sc->dt = dt;
  sc->active = 1;
  gch::set_stage_ratios(sc, dx, dy, dz);
}
__global__ void k_set_active(StepScalars* sc) { sc->active = 1; }
__global__ void k_restore_info(StepScalars* sc, int active, int err, unsigned long long pfloor) {
  sc->active = active;
  sc->err = err;
  sc->pfloor = pfloor;
}
__global__ void k_clear_info(StepScalars* sc) {
  sc->err = 0;
  sc->pfloor = 0;
}

// A host array in the reference's layout moves to and from the device
// either straight through the layout kernels, when the GPU can address it
// (page-locked memory mapped into the device address space: the kernels
// read or write it over the host link, which also does the transposition),
// or through a cudaMemcpy into the device staging buffer and the same
// kernels on that buffer (pageable memory).
const double* host_in(gch_domain* d, const double* h, int& st) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, h) == cudaSuccess && a.type == cudaMemoryTypeHost &&
      a.devicePointer)
    return (const double*)a.devicePointer;
  cudaGetLastError();  // an unregistered pointer is not an error here
  st |= cuda_ok(cudaMemcpyAsync(d->stage, h, d->ncell_host * d->kp.neq * sizeof(double),
                                cudaMemcpyHostToDevice, d->stream));
  return d->stage;
}
// whether the GPU addresses host array h directly (page-locked, mapped)
bool host_mapped(const double* h) {
  cudaPointerAttributes a;
  const bool m = cudaPointerGetAttributes(&a, h) == cudaSuccess && a.type == cudaMemoryTypeHost &&
                 a.devicePointer;
  cudaGetLastError();
  return m;
}
// the device view of a host output array, or the staging buffer (then
// host_out_finish copies it to the host)
double* host_out(gch_domain* d, double* h) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, h) == cudaSuccess && a.type == cudaMemoryTypeHost &&
      a.devicePointer)
    return (double*)a.devicePointer;
  cudaGetLastError();
  return d->stage;
}
int host_out_finish(gch_domain* d, double* h, const double* view) {
  if (view != d->stage) return GCH_OK;
  return cuda_ok(cudaMemcpyAsync(h, d->stage, d->ncell_host * d->kp.neq * sizeof(double),
                                 cudaMemcpyDeviceToHost, d->stream));
}

}  // namespace

bool gch::pipe_ok(const gch_domain* d) {
  const gch::KParams& k = d->kp;
  // the plain FP64 step is bound by its arithmetic (about 140 ms at 256^3
  // against 11 ms of copies), and its one-block-per-SM stage kernels lose
  // more to the partial waves of slab launches than the overlap saves
  // (measured: 172 ms per step overlapped)
  if (d->mode == GCH_FP64) return false;
  if (d->prim_in || d->hp.cooling == GCH_COOL_H || k.eta != 0.0 || d->hp.th_cond != GCH_TC_OFF)
    return false;
  if ((k.bc_user && k.nsph > 0) || k.solver == GCH_SOLVER_HLLE_SPLIT_ALL) return false;
  // the deferred first stage: no source terms, no passive scalars
  if (k.user_src || k.eight_wave || (k.neq != 5 && k.neq != 8)) return false;
  // every side at least one cell: the whole-shell fill of one layer
  return k.nx >= 1 && k.ny >= 1 && (k.nz + d->kz - 1) / d->kz >= 3;
}

namespace {
int fetch_scalars(gch_domain* d) {
  int st = cuda_ok(cudaMemcpyAsync(d->sc_host, d->sc, sizeof(StepScalars), cudaMemcpyDeviceToHost,
                                   d->stream));
  st |= cuda_ok(cudaStreamSynchronize(d->stream));
  return st;
}

}  // namespace

extern "C" {

void gch_params_default(gch_params_t* p, int nx, int ny, int nz) {
  memset(p, 0, sizeof(*p));
  p->abi_version = GCH_ABI_VERSION;
  p->precision = GCH_FP64;
  p->nx = nx;
  p->ny = ny;
  p->nz = nz;
  p->neq = 8;
  p->mhd = 1;
  p->pmhd = 0;
  p->riemann_solver = GCH_SOLVER_HLLD;
  p->slope_limiter = GCH_LIMITER_MINMOD;
  p->eq_of_state = GCH_EOS_ADIABATIC;
  p->cooling = GCH_COOL_NONE;
  p->enable_flux_cd = 1;
  p->eight_wave = 0;
  p->user_source_terms = 0;
  p->bc_left = p->bc_right = p->bc_bottom = p->bc_top = p->bc_out = p->bc_in = GCH_BC_PERIODIC;
  p->bc_user = 0;
  p->dx = 1.0 / nx;
  p->dy = 1.0 / ny;
  p->dz = 1.0 / nz;
  p->cv = 1.5;
  p->gamma = (p->cv + 1.0) / p->cv;
  p->cfl = 0.2;
  p->eta = 0.0;
  p->Tempsc = 1.0;
  p->Psc = 1.0;
  p->tsc = 1.0;
  p->tab_Tmin = 1e4;
  p->th_cond = GCH_TC_OFF;
  p->tc_saturation = 0;
  p->rsc = 1.0;
  p->rhosc = 1.0;
  p->vsc2 = 1.0;
  p->bsc = std::sqrt(4.0 * std::acos(-1.0));  // sqrt(4 pi Psc), Psc = 1
  p->mu = 1.0;
  p->npas = 0;
}

int gch_params_check(const gch_params_t* p) {
  if (!p || p->abi_version != GCH_ABI_VERSION) return GCH_ERR_PARAM;
  if (p->precision != GCH_FP64 && p->precision != GCH_FP32_MIXED &&
      p->precision != GCH_FP32_KAHAN)
    return GCH_ERR_PARAM;
  if (p->nx < 1 || p->ny < 1 || p->nz < 1) return GCH_ERR_PARAM;
  // 5 or 8 dynamical equations and 0 or 2 passive scalars
  if (p->npas != 0 && p->npas != 2) return GCH_ERR_PARAM;
  const int neqdyn = p->neq - p->npas;
  if (neqdyn != 5 && neqdyn != 8) return GCH_ERR_PARAM;
  const bool bfield = neqdyn == 8;
  if (p->mhd && !bfield) return GCH_ERR_PARAM;
  if (bfield && !(p->mhd || p->pmhd)) return GCH_ERR_PARAM;
  if (p->mhd && p->pmhd) return GCH_ERR_PARAM;
  switch (p->riemann_solver) {
    case GCH_SOLVER_HLLD:
    case GCH_SOLVER_HLLE:
      if (!p->mhd) return GCH_ERR_PARAM;  // both need the full MHD flux
      break;
    case GCH_SOLVER_HLLC:
    case GCH_SOLVER_HLL:
      if (p->mhd) return GCH_ERR_PARAM;   // hydro (or passive B) solvers
      break;
    case GCH_SOLVER_HLLE_SPLIT_ALL:
      // the split branches of the reference are written for MHD; built on
      // the FP64 path, without cooling, conduction, passives, sources or
      // user spheres
      if (!p->mhd || p->npas != 0 || p->precision != GCH_FP64 || p->cooling != GCH_COOL_NONE ||
          p->th_cond != GCH_TC_OFF || p->eight_wave || p->user_source_terms || p->bc_user)
        return GCH_ERR_PARAM;
      break;
    default:
      return GCH_ERR_PARAM;
  }
  if (p->slope_limiter < GCH_LIMITER_NO_AVERAGE || p->slope_limiter > GCH_LIMITER_SUPERBEE)
    return GCH_ERR_PARAM;
  if (p->eq_of_state != GCH_EOS_ADIABATIC && p->eq_of_state != GCH_EOS_SINGLE_SPECIE &&
      p->eq_of_state != GCH_EOS_H_RATE)
    return GCH_ERR_PARAM;
  if (p->cooling != GCH_COOL_NONE && p->cooling != GCH_COOL_H && p->cooling != GCH_COOL_DMC &&
      p->cooling != GCH_COOL_CHI)
    return GCH_ERR_PARAM;
  // the H-rate EOS and COOL_H read the neutral hydrogen density from the
  // first passive scalar (src/hydro_core.f90:106-111, src/cooling_h.f90:331)
  if ((p->eq_of_state == GCH_EOS_H_RATE || p->cooling == GCH_COOL_H) && p->npas < 1)
    return GCH_ERR_PARAM;
  // the user spheres set the dynamical fields only
  if (p->bc_user && p->npas != 0) return GCH_ERR_PARAM;
  if ((p->cooling == GCH_COOL_DMC || p->cooling == GCH_COOL_CHI) &&
      (p->ntab < 2 || p->ntab > GCH_MAX_TABLE || !(p->tab_inv_dlog > 0.0)))
    return GCH_ERR_PARAM;
  // flux-CD needs B (the reference's hydro build leaves up untouched then)
  if (p->enable_flux_cd && !bfield) return GCH_ERR_PARAM;
  if (p->eight_wave && !p->mhd) return GCH_ERR_PARAM;
  const int bcs[6] = {p->bc_left, p->bc_right, p->bc_bottom, p->bc_top, p->bc_out, p->bc_in};
  for (int i = 0; i < 6; ++i)
    if (!valid_bc(bcs[i])) return GCH_ERR_PARAM;
  for (int a = 0; a < 3; ++a)  // periodic walls come in pairs (src/boundaries.f90:111)
    if ((bcs[2 * a] == GCH_BC_PERIODIC) != (bcs[2 * a + 1] == GCH_BC_PERIODIC)) return GCH_ERR_PARAM;
  if (p->nsph < 0 || p->nsph > GCH_MAX_SPHERES || p->ngrav < 0 || p->ngrav > GCH_MAX_GRAV)
    return GCH_ERR_PARAM;
  if (p->bc_user && p->nsph == 0) return GCH_ERR_PARAM;
  if (p->user_source_terms && p->ngrav == 0) return GCH_ERR_PARAM;
  if (!(p->dx > 0 && p->dy > 0 && p->dz > 0 && p->cv > 0 && p->gamma > 0 && p->cfl > 0))
    return GCH_ERR_PARAM;
  if (!(p->eta >= 0.0)) return GCH_ERR_PARAM;
  if (p->th_cond != GCH_TC_OFF) {
    if (p->th_cond != GCH_TC_ISOTROPIC && p->th_cond != GCH_TC_ANISOTROPIC) return GCH_ERR_PARAM;
    if (p->th_cond == GCH_TC_ANISOTROPIC && !bfield) return GCH_ERR_PARAM;
    // with table cooling the reference's interior Temp is not refreshed
    // before conduction reads it
    if (p->cooling == GCH_COOL_DMC || p->cooling == GCH_COOL_CHI) return GCH_ERR_PARAM;
    if (!(p->rsc > 0 && p->rhosc > 0 && p->vsc2 > 0 && p->bsc > 0 && p->mu > 0 && p->Psc > 0 &&
          p->tsc > 0))
      return GCH_ERR_PARAM;
  }
  return GCH_OK;
}

int gch_destroy(gch_domain_t* d) {
  if (!d) return GCH_OK;
  if (d->graph) cudaGraphExecDestroy(d->graph);
  for (int i = 0; i < gch_domain::kPipeEv; ++i)
    if (d->pipe_ev[i]) cudaEventDestroy(d->pipe_ev[i]);
  if (d->cstream) cudaStreamDestroy(d->cstream);
  for (int i = 0; i < 64; ++i)
    if (d->prof_ev[i]) cudaEventDestroy(d->prof_ev[i]);
  cudaFree(d->u);
  cudaFree(d->up);
  cudaFree(d->w);
  cudaFree(d->E);
  cudaFree(d->s678);
  cudaFree(d->primit);
  cudaFree(d->prim0);
  cudaFree(d->split_f);
  cudaFree(d->tab);
  cudaFree(d->sph);
  cudaFree(d->grav);
  cudaFree(d->sc);
  cudaFree(d->tmaps);
  cudaFree(d->stage);
  cudaFree(d->dif);
  cudaFree(d->tcw);
  cudaFree(d->tc_min);
  if (d->tc_min_host) cudaFreeHost(d->tc_min_host);
  if (d->sc_host) cudaFreeHost(d->sc_host);
  if (d->stream && d->own_stream) cudaStreamDestroy(d->stream);
  delete d;
  return GCH_OK;
}

int gch_create(const gch_params_t* p, void* stream, gch_domain_t** out) {
  if (!out) return GCH_ERR_PARAM;
  *out = nullptr;
  int st = gch_params_check(p);
  if (st) return st;
  int dev = 0, ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return GCH_ERR_NO_DEVICE;
  if (cudaGetDevice(&dev) != cudaSuccess) return GCH_ERR_NO_DEVICE;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return GCH_ERR_NO_DEVICE;
  if (prop.major != 10) return GCH_ERR_NO_DEVICE;  // built for sm_103a only

  gch_domain* d = new (std::nothrow) gch_domain();
  if (!d) return GCH_ERR_CUDA;
  d->hp = *p;
  d->mode = p->precision;
  d->prim_in = p->cooling == GCH_COOL_DMC || p->cooling == GCH_COOL_CHI;
  // FP32 with FP64 u: get_timestep stores the primitives it recovers (in
  // FP64 arithmetic) for the first stage, which otherwise recovers them
  // again in one FP64-bound burst per plane.  (On the pair path the store
  // costs more than the first stage saves.)
  d->prim_pre = !d->prim_in && p->precision == GCH_FP32_MIXED;
  d->tu_size = 8;
  d->ts_size = d->mode == GCH_FP64 ? 8 : 4;

  KParams& k = d->kp;
  memset(&k, 0, sizeof(k));
  k.nx = p->nx; k.ny = p->ny; k.nz = p->nz;
  k.NX = p->nx + 2 * gch::NG; k.NY = p->ny + 2 * gch::NG; k.NZ = p->nz + 2 * gch::NG;
  k.pitch = (k.NX + 3) & ~3;
  k.fs = (long long)k.pitch * k.NY * k.NZ;
  k.neq = p->neq;
  k.mhd = p->mhd; k.pmhd = p->pmhd;
  k.solver = p->riemann_solver; k.limiter = p->slope_limiter;
  k.eos = p->eq_of_state; k.cooling = p->cooling;
  k.flux_cd = p->enable_flux_cd; k.eight_wave = p->eight_wave; k.user_src = p->user_source_terms;
  k.bc[0] = p->bc_left; k.bc[1] = p->bc_right; k.bc[2] = p->bc_bottom;
  k.bc[3] = p->bc_top; k.bc[4] = p->bc_out; k.bc[5] = p->bc_in;
  k.bc_user = p->bc_user;
  k.dx = p->dx; k.dy = p->dy; k.dz = p->dz;
  k.cv = p->cv; k.gamma = p->gamma; k.cfl = p->cfl; k.eta = p->eta;
  k.inv_cv = 1.0 / p->cv;
  k.Tempsc = p->Tempsc; k.Psc = p->Psc; k.tsc = p->tsc;
  k.ntab = p->ntab; k.tab_i0 = p->tab_i0;
  k.tab_inv_dlog = p->tab_inv_dlog; k.tab_tail = p->tab_tail; k.tab_Tmin = p->tab_Tmin;
  gch::set_f32_params(k);
  k.nsph = p->bc_user ? p->nsph : 0;
  k.ngrav = p->user_source_terms ? p->ngrav : 0;

  // z planes per block: enough blocks to fill the 152 SMs several times
  {
    const long long tiles = (long long)((k.nx + gch::TX - 1) / gch::TX) * ((k.ny + gch::TY - 1) / gch::TY);
    int kz = 16;
    while (kz > 2 && tiles * ((k.nz + kz - 1) / kz) < 8 * 152) kz /= 2;
    d->kz = std::min(kz, k.nz);
  }

  cudaStream_t s = (cudaStream_t)stream;
  if (!s) {
    // graph capture needs a stream other than the legacy default stream
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
      delete d;
      return GCH_ERR_CUDA;
    }
    d->own_stream = true;
  }
  d->stream = s;

  const size_t fs = (size_t)k.fs;
  cudaError_t e = cudaSuccess;
  auto alloc = [&](void** ptr, size_t bytes) {
    if (e == cudaSuccess) e = cudaMalloc(ptr, bytes);
    if (e == cudaSuccess) e = cudaMemsetAsync(*ptr, 0, bytes, s);
  };
  alloc(&d->u, fs * k.neq * d->tu_size);
  alloc(&d->up, fs * k.neq * d->ts_size);
  if (p->eta != 0.0) alloc(&d->w, fs * k.neq * d->tu_size);
  if (k.neq >= 8 && p->enable_flux_cd) alloc(&d->E, fs * 3 * d->ts_size);
  if (p->eight_wave) alloc(&d->s678, fs * 3 * d->ts_size);
  if (d->prim_in || d->prim_pre) alloc(&d->primit, fs * k.neq * d->ts_size);
  d->ncell_host = (size_t)k.NX * k.NY * k.NZ;
  alloc((void**)&d->stage, d->ncell_host * k.neq * sizeof(double));
  alloc((void**)&d->sc, sizeof(StepScalars));
  if (p->riemann_solver == GCH_SOLVER_HLLE_SPLIT_ALL) {
    alloc((void**)&d->prim0, fs * k.neq * sizeof(double));
    alloc(&d->primit, fs * k.neq * sizeof(double));
    alloc((void**)&d->split_f, fs * 3 * k.neq * sizeof(double));
  }
  if (p->th_cond != GCH_TC_OFF) {
    alloc((void**)&d->tcw, fs * 6 * sizeof(double));
    alloc((void**)&d->tc_min, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMallocHost((void**)&d->tc_min_host, sizeof(unsigned long long));
  }
  if (e == cudaSuccess && d->prim_in) {  // the tabulated cooling curve, FP64 and FP32 rows
    const int nt = p->ntab;
    e = cudaMalloc((void**)&d->tab, 2 * nt * (sizeof(double) + sizeof(float)));
    if (e == cudaSuccess) e = cudaMemcpy(d->tab, p->tab_T, nt * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
      e = cudaMemcpy(d->tab + nt, p->tab_L, nt * sizeof(double), cudaMemcpyHostToDevice);
    float f[2 * GCH_MAX_TABLE];
    for (int i = 0; i < nt; ++i) {
      f[i] = (float)p->tab_T[i];
      f[nt + i] = (float)p->tab_L[i];
    }
    float* tf = reinterpret_cast<float*>(d->tab + 2 * nt);
    if (e == cudaSuccess) e = cudaMemcpy(tf, f, 2 * nt * sizeof(float), cudaMemcpyHostToDevice);
    k.tabT = d->tab;
    k.tabL = d->tab + nt;
    k.tabTf = tf;
    k.tabLf = tf + nt;
  }
  if (e == cudaSuccess && k.nsph > 0) {
    e = cudaMalloc((void**)&d->sph, k.nsph * sizeof(gch_sphere_t));
    if (e == cudaSuccess) e = cudaMemcpy(d->sph, p->sph, k.nsph * sizeof(gch_sphere_t), cudaMemcpyHostToDevice);
    k.sph = d->sph;
  }
  if (e == cudaSuccess && k.ngrav > 0) {
    double g[4 * GCH_MAX_GRAV];
    for (int l = 0; l < k.ngrav; ++l) {
      g[l] = p->grav_GM[l];
      g[k.ngrav + l] = p->grav_x[l];
      g[2 * k.ngrav + l] = p->grav_y[l];
      g[3 * k.ngrav + l] = p->grav_z[l];
    }
    float gf[4 * GCH_MAX_GRAV];
    for (int i = 0; i < 4 * k.ngrav; ++i) gf[i] = (float)g[i];
    e = cudaMalloc((void**)&d->grav, 4 * k.ngrav * (sizeof(double) + sizeof(float)));
    if (e == cudaSuccess) e = cudaMemcpy(d->grav, g, 4 * k.ngrav * sizeof(double), cudaMemcpyHostToDevice);
    float* gfd = reinterpret_cast<float*>(d->grav + 4 * k.ngrav);
    if (e == cudaSuccess) e = cudaMemcpy(gfd, gf, 4 * k.ngrav * sizeof(float), cudaMemcpyHostToDevice);
    k.grav = d->grav;
    k.gravf = gfd;
  }
  if (e == cudaSuccess && d->mode != GCH_FP64 && p->riemann_solver != GCH_SOLVER_HLLE_SPLIT_ALL) {
    // TMA tensor maps of the FP32 stage kernels' sources: stage 1 from u
    // (8-byte FP64 or pair values) and, when the domain keeps them (table
    // cooling, or the primitives get_timestep stores), from primit (FP32);
    // stage 2 from up (FP32).  Maps of an array the domain does not have
    // stay zero and are never used.
    e = cudaMalloc((void**)&d->tmaps, gch::kTmaCount * gch::kTmaMapBytes);
    if (e == cudaSuccess) {
      alignas(64) unsigned char maps[gch::kTmaCount * gch::kTmaMapBytes];
      memset(maps, 0, sizeof(maps));
      const int esu = (int)d->tu_size, ess = (int)d->ts_size;
      int r = gch::encode_stage_map(maps + gch::kTmaS1Rows * gch::kTmaMapBytes, d->u, esu, k, 36, 1);
      r |= gch::encode_stage_map(maps + gch::kTmaS1Sides * gch::kTmaMapBytes, d->u, esu, k,
                                 16 / esu, gch::TY);
      if (d->primit) {
        r |= gch::encode_stage_map(maps + gch::kTmaS1PRows * gch::kTmaMapBytes, d->primit, ess, k,
                                   36, 1);
        r |= gch::encode_stage_map(maps + gch::kTmaS1PSides * gch::kTmaMapBytes, d->primit, ess,
                                   k, 16 / ess, gch::TY);
      }
      r |= gch::encode_stage_map(maps + gch::kTmaS2Rows * gch::kTmaMapBytes, d->up, ess, k, 36, 1);
      r |= gch::encode_stage_map(maps + gch::kTmaS2Sides * gch::kTmaMapBytes, d->up, ess, k,
                                 16 / ess, gch::TY);
      if (r != GCH_OK) e = cudaErrorInvalidValue;
      if (e == cudaSuccess) e = cudaMemcpy(d->tmaps, maps, sizeof(maps), cudaMemcpyHostToDevice);
      k.tmaps = d->tmaps;
    }
  }
  if (e == cudaSuccess) e = cudaMallocHost((void**)&d->sc_host, sizeof(StepScalars));
  if (e == cudaSuccess) {
    StepScalars init;
    memset(&init, 0, sizeof(init));
    init.dtmin_bits = 0x7FF0000000000000ull;
    init.active = 1;
    init.n_iter = 10;
    init.iter = 1;
    *d->sc_host = init;
    e = cudaMemcpyAsync(d->sc, d->sc_host, sizeof(StepScalars), cudaMemcpyHostToDevice, s);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    gch_destroy(d);
    return GCH_ERR_CUDA;
  }
  *out = d;
  return GCH_OK;
}

int gch_upload(gch_domain_t* d, const double* u) {
  if (!d || !u) return GCH_ERR_PARAM;
  int st = GCH_OK;
  const double* src = host_in(d, u, st);
  st |= engine(d).upload(d, src);
  st |= cuda_ok(cudaStreamSynchronize(d->stream));
  return st;
}

int gch_set_background(gch_domain_t* d, const double* primit0) {
  if (!d || !primit0 || !d->prim0) return GCH_ERR_PARAM;
  int st = GCH_OK;
  const double* src = host_in(d, primit0, st);
  st |= gch::split_set_background(d, src);
  st |= cuda_ok(cudaStreamSynchronize(d->stream));
  return st;
}

int gch_download(gch_domain_t* d, double* u, double* primit) {
  if (!d) return GCH_ERR_PARAM;
  int st = GCH_OK;
  if (u) {
    double* dst = host_out(d, u);
    st |= engine(d).download_u(d, dst);
    st |= host_out_finish(d, u, dst);
  }
  if (primit) {
    double* dst = host_out(d, primit);
    st |= engine(d).download_prim(d, dst);
    st |= host_out_finish(d, primit, dst);
  }
  st |= cuda_ok(cudaStreamSynchronize(d->stream));
  return st;
}

int gch_boundaryI(gch_domain_t* d) {
  if (!d) return GCH_ERR_PARAM;
  k_set_active<<<1, 1, 0, d->stream>>>(d->sc);
  return engine(d).boundaryI(d);
}

int gch_calcprim(gch_domain_t* d) {
  if (!d) return GCH_ERR_PARAM;
  k_set_active<<<1, 1, 0, d->stream>>>(d->sc);
  return engine(d).calcprim(d);
}

int gch_get_timestep(gch_domain_t* d, int current_iter, int n_iter, double current_time,
                     double tprint, double* dt, int* dump_flag) {
  if (!d || !dt || !dump_flag) return GCH_ERR_PARAM;
  k_set_ctrl<<<1, 1, 0, d->stream>>>(d->sc, current_iter, n_iter, current_time, tprint, 0.0, 0.0, 1);
  int st = engine(d).get_dt(d);
  st |= fetch_scalars(d);
  *dt = d->sc_host->dt;
  if (d->sc_host->dump) *dump_flag = 1;
  st |= d->sc_host->err;
  return st;
}

int gch_tstep(gch_domain_t* d, double dt) {
  if (!d) return GCH_ERR_PARAM;
  if (!(dt > 0.0) || !std::isfinite(dt)) return GCH_ERR_DT;
  k_set_dt<<<1, 1, 0, d->stream>>>(d->sc, dt, d->kp.dx, d->kp.dy, d->kp.dz);
  int st = engine(d).tstep(d);
  if (d->hp.th_cond != GCH_TC_OFF && st == GCH_OK) st |= gch::tc_run(d, dt);
  return st;
}

int gch_tc_info(gch_domain_t* d, int* nsteps, double* dt_cond) {
  if (!d) return GCH_ERR_PARAM;
  if (nsteps) *nsteps = d->tc_nsteps;
  if (dt_cond) *dt_cond = d->tc_dt_cond;
  return GCH_OK;
}

int gch_step_host_overlaps(const gch_domain_t* d) { return d && gch::pipe_ok(d) ? 1 : 0; }

int gch_step_host(gch_domain_t* d, double* u, int current_iter, int n_iter, double current_time,
                  double tprint, double* dt, int* dump_flag) {
  if (!d || !u || !dt || !dump_flag) return GCH_ERR_PARAM;
  int st = GCH_OK;
  if (gch::pipe_ok(d) && !host_mapped(u)) {
    // a pageable array: the copy-engine copies of u in and out overlap the
    // step.  (A page-locked array keeps the serial order below: the layout
    // kernels move it over the link themselves, which never stalled, while
    // copy-engine DMA on this system took 40-540 ms for a step now and then,
    // with or without the overlap.)
    k_set_ctrl<<<1, 1, 0, d->stream>>>(d->sc, current_iter, n_iter, current_time, tprint, 0.0,
                                       0.0, 1);
    st |= engine(d).step_host(d, u);
  } else {
    const double* src = host_in(d, u, st);
    st |= engine(d).upload(d, src);
    if (d->prim_in) st |= engine(d).calcprim(d);
    k_set_ctrl<<<1, 1, 0, d->stream>>>(d->sc, current_iter, n_iter, current_time, tprint, 0.0,
                                       0.0, 1);
    st |= engine(d).get_dt(d);
    st |= engine(d).tstep(d);
    if (d->hp.th_cond != GCH_TC_OFF && st == GCH_OK) {
      st |= fetch_scalars(d);  // the conduction substeps need dt on the host
      st |= gch::tc_run(d, d->sc_host->dt);
    }
    double* dst = host_out(d, u);
    st |= engine(d).download_u(d, dst);
    st |= host_out_finish(d, u, dst);
  }
  st |= fetch_scalars(d);
  *dt = d->sc_host->dt;
  if (d->sc_host->dump) *dump_flag = 1;
  st |= d->sc_host->err;
  return st;
}

}  // extern "C"

namespace {
// The time loop of src/main.f90:94-125 driven from the host, for domains
// whose step needs the host (thermal conduction); leaves the loop state in
// the device scalars as the device loop's tail does.
int host_loop(gch_domain* d, int max_steps, double tmax, double dtprint, int n_iter,
              double time, int iter, double tprint) {
  int st = GCH_OK;
  for (int n = 0; n < max_steps && time <= tmax && st == GCH_OK; ++n) {
    double dt = 0.0;
    int dump = 0;
    st |= gch_get_timestep(d, iter, n_iter, time, tprint, &dt, &dump);
    if (st) break;
    st |= gch_tstep(d, dt);
    time = time + dt;
    if (dump) tprint = tprint + dtprint;
    iter = iter + 1;
  }
  k_set_ctrl<<<1, 1, 0, d->stream>>>(d->sc, iter, n_iter, time, tprint, dtprint, tmax,
                                     time <= tmax ? 1 : 0);
  return st | cuda_ok(cudaGetLastError());
}
}  // namespace

// Enqueue up to max_steps device-resident iterations (no host sync; with
// thermal conduction the steps run from the host before this returns).
int gch_advance_enqueue(gch_domain* d, int max_steps, double tmax, double dtprint, int n_iter,
                        double time, int iter, double tprint) {
  if (d->hp.th_cond != GCH_TC_OFF)
    return host_loop(d, max_steps, tmax, dtprint, n_iter, time, iter, tprint);
  k_set_ctrl<<<1, 1, 0, d->stream>>>(d->sc, iter, n_iter, time, tprint, dtprint, tmax,
                                     time <= tmax ? 1 : 0);
  int st = cuda_ok(cudaGetLastError());
  if (!d->graph) {
    // capture one device-resident iteration of src/main.f90:94-125
    cudaGraph_t g = nullptr;
    st |= cuda_ok(cudaStreamBeginCapture(d->stream, cudaStreamCaptureModeThreadLocal));
    st |= engine(d).get_dt(d);
    st |= engine(d).tstep(d);
    st |= engine(d).loopfin(d);
    st |= cuda_ok(cudaStreamEndCapture(d->stream, &g));
    if (st == GCH_OK) st |= cuda_ok(cudaGraphInstantiate(&d->graph, g, 0));
    if (g) cudaGraphDestroy(g);
    if (st) return st;
  }
  for (int n = 0; n < max_steps; ++n) st |= cuda_ok(cudaGraphLaunch(d->graph, d->stream));
  return st;
}

// Wait for the enqueued iterations and read the loop state back.
int gch_advance_finish(gch_domain* d, double* time, int* iter, double* tprint) {
  int st = fetch_scalars(d);
  if (time) *time = d->sc_host->time;
  if (iter) *iter = d->sc_host->iter;
  if (tprint) *tprint = d->sc_host->tprint;
  st |= d->sc_host->err;
  return st;
}

extern "C" {

int gch_advance(gch_domain_t* d, int max_steps, double tmax, double dtprint, int n_iter,
                double* time, int* iter, double* tprint, int* steps_done) {
  if (!d || !time || !iter || !tprint || max_steps < 0) return GCH_ERR_PARAM;
  const int iter0 = *iter;
  if (d->hp.th_cond != GCH_TC_OFF) {
    int st = host_loop(d, max_steps, tmax, dtprint, n_iter, *time, *iter, *tprint);
    st |= gch_advance_finish(d, time, iter, tprint);
    if (steps_done) *steps_done = *iter - iter0;
    return st;
  }
  // Launch the step graph in chunks and stop as soon as the device loop
  // condition (time <= tmax, no error) turns false: the host never queues
  // more than one chunk of steps past the end of the run.
  int st = gch_advance_enqueue(d, 0, tmax, dtprint, n_iter, *time, *iter, *tprint);
  int left = max_steps;
  int chunk = 8;
  while (st == GCH_OK && left > 0) {
    const int k = std::min(chunk, left);
    for (int n = 0; n < k; ++n) st |= cuda_ok(cudaGraphLaunch(d->graph, d->stream));
    left -= k;
    st |= fetch_scalars(d);
    if (!d->sc_host->active || d->sc_host->err) break;
    chunk = std::min(chunk * 2, 256);
  }
  st |= gch_advance_finish(d, time, iter, tprint);
  if (steps_done) *steps_done = *iter - iter0;
  return st;
}

int gch_last_step_info(gch_domain_t* d, long long* pfloor_hits, int* err_bits) {
  if (!d) return GCH_ERR_PARAM;
  int st = fetch_scalars(d);
  if (pfloor_hits) *pfloor_hits = (long long)d->sc_host->pfloor;
  if (err_bits) *err_bits = d->sc_host->err;
  k_clear_info<<<1, 1, 0, d->stream>>>(d->sc);
  return st;
}

int gch_advance_timed(gch_domain_t* d, int steps, int n_iter, float* ms) {
  if (!d || !ms || steps < 0) return GCH_ERR_PARAM;
  const double inf = 1e300;
  int st = fetch_scalars(d);
  const double t0 = d->sc_host->time;
  const int it0 = d->sc_host->iter > 0 ? d->sc_host->iter : 1;
  cudaEvent_t a, b;
  st |= cuda_ok(cudaEventCreate(&a));
  st |= cuda_ok(cudaEventCreate(&b));
  k_set_ctrl<<<1, 1, 0, d->stream>>>(d->sc, it0, n_iter, t0, inf, inf, inf, 1);
  if (d->hp.th_cond != GCH_TC_OFF) {  // host-driven steps
    st |= cuda_ok(cudaEventRecord(a, d->stream));
    st |= host_loop(d, steps, inf, inf, n_iter, t0, it0, inf);
  } else {
    st |= gch_advance_enqueue(d, 0, inf, inf, n_iter, t0, it0, inf);  // capture only
    st |= cuda_ok(cudaEventRecord(a, d->stream));
    for (int n = 0; n < steps; ++n) st |= cuda_ok(cudaGraphLaunch(d->graph, d->stream));
  }
  st |= cuda_ok(cudaEventRecord(b, d->stream));
  st |= cuda_ok(cudaEventSynchronize(b));
  st |= cuda_ok(cudaEventElapsedTime(ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  st |= fetch_scalars(d);
  st |= d->sc_host->err;
  return st;
}

int gch_profile_step(gch_domain_t* d, int cap, float* ms, char* names, int name_len, int* n) {
  if (!d || !ms || !names || !n || cap < 1 || name_len < 2) return GCH_ERR_PARAM;
  int st = fetch_scalars(d);
  const double inf = 1e300;
  const int it0 = d->sc_host->iter > 0 ? d->sc_host->iter : 1;
  for (int i = 0; i < 64; ++i)
    if (!d->prof_ev[i]) st |= cuda_ok(cudaEventCreate(&d->prof_ev[i]));
  k_set_ctrl<<<1, 1, 0, d->stream>>>(d->sc, it0, 10, d->sc_host->time, inf, inf, inf, 1);
  d->prof_on = true;
  d->prof_n = 0;
  st |= cuda_ok(cudaEventRecord(d->prof_ev[0], d->stream));
  st |= engine(d).get_dt(d);
  st |= engine(d).tstep(d);
  d->prof_on = false;
  st |= cuda_ok(cudaStreamSynchronize(d->stream));
  const int m = std::min(cap, d->prof_n);
  for (int i = 0; i < m; ++i) {
    st |= cuda_ok(cudaEventElapsedTime(&ms[i], d->prof_ev[i], d->prof_ev[i + 1]));
    strncpy(names + (size_t)i * name_len, d->prof_name[i], name_len - 1);
    names[(size_t)i * name_len + name_len - 1] = 0;
  }
  *n = m;
  return st;
}

int gch_launches_per_step(gch_domain_t* d) {
  if (!d) return -1;
  return d->launches + 2;  // + k_cfl and k_dtfin of get_timestep
}

int gch_get_kz(gch_domain_t* d) { return d ? d->kz : -1; }

int gch_set_kz(gch_domain_t* d, int kz) {
  if (!d || kz < 1 || kz > d->kp.nz) return GCH_ERR_PARAM;
  int st = cuda_ok(cudaStreamSynchronize(d->stream));
  if (d->graph) {  // the captured step holds the old grid
    cudaGraphExecDestroy(d->graph);
    d->graph = nullptr;
  }
  d->kz = kz;
  return st;
}

int gch_autotune(gch_domain_t* d, int cap, int* cand_kz, float* cand_ms, int* ncand) {
  if (!d) return GCH_ERR_PARAM;
  int st = fetch_scalars(d);
  const StepScalars keep = *d->sc_host;
  k_set_active<<<1, 1, 0, d->stream>>>(d->sc);
  cudaEvent_t e0, e1;
  st |= cuda_ok(cudaEventCreate(&e0));
  st |= cuda_ok(cudaEventCreate(&e1));
  int best_kz = d->kz, n = 0;
  float best = 0.f;
  for (int kz : {1, 2, 4, 8, 12, 16, 20, 24, 32}) {
    if (kz > d->kp.nz || st) break;
    d->kz = kz;
    st |= engine(d).probe(d);  // warm-up
    st |= cuda_ok(cudaEventRecord(e0, d->stream));
    for (int r = 0; r < 3; ++r) st |= engine(d).probe(d);
    st |= cuda_ok(cudaEventRecord(e1, d->stream));
    st |= cuda_ok(cudaEventSynchronize(e1));
    float ms = 0.f;
    st |= cuda_ok(cudaEventElapsedTime(&ms, e0, e1));
    ms /= 3;
    if (n < cap) {
      if (cand_kz) cand_kz[n] = kz;
      if (cand_ms) cand_ms[n] = ms;
    }
    if (n == 0 || ms < best) {
      best = ms;
      best_kz = kz;
    }
    ++n;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (ncand) *ncand = std::min(n, cap);
  // the probes counted the pressure floors of the stage-1 states: put the
  // step information back as it was
  k_restore_info<<<1, 1, 0, d->stream>>>(d->sc, keep.active, keep.err, keep.pfloor);
  st |= cuda_ok(cudaGetLastError());
  st |= gch_set_kz(d, best_kz);
  return st;
}

}  // extern "C"
