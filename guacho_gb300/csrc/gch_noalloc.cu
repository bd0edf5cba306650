// gch_noalloc.cu -- get_timestep for callers that cannot allocate device
// memory.
//
// Some host codes cannot call cudaMalloc at the moment they need a
// timestep.  A Fortran or C driver that hands the GPU library a fixed,
// pre-sized memory budget (for example one sized at start-up by a job
// scheduler's memory limit) forbids hidden allocations, because a late
// allocation can fail or fragment memory in the middle of a run; a code that
// owns every device buffer through its own pool allocator has no way to
// return library-made buffers to that pool.  gch_get_timestep_noalloc serves
// them: the caller passes the state and the output slots in device memory it
// owns, and the only other memory the reduction needs -- one partial minimum
// per thread block plus a completion counter -- lives in a fixed array
// compiled into the library.
//
// Limits and sharing rules:
//  - the array holds kNoAllocMaxBlocks partial minima (512 KiB); a box needs
//    ceil(nx/32)*ceil(ny/8)*ceil(nz/8) of them, so up to 512^3 cells.  A
//    larger box is refused with GCH_ERR_TOO_LARGE before any launch;
//  - every GPU that loads the library keeps the array until the process
//    exits, whether or not this entry point is used;
//  - all calls share the one array, and each call starts by clearing its
//    completion counter: calls that may overlap on the GPU (different
//    streams without ordering between them) race and must not be issued;
//    calls on one stream are ordered and safe;
//  - the first call on a device (and the first call after that device's
//    context was destroyed and created again, e.g. by cudaDeviceReset) looks
//    up the array's device address with cudaGetSymbolAddress, with that
//    device current; make that first call before any stream capture begins.
//    Later calls only clear the counter and launch.
#include <cuda_runtime.h>

#include <mutex>

#include "gch_device.cuh"
#include "guacho_gb300.h"

namespace {

constexpr int kNoAllocMaxBlocks = 65536;
constexpr int kMaxDevices = 64;

// [0, kNoAllocMaxBlocks): per-block minima (bits of a positive double)
// [kNoAllocMaxBlocks]:     number of blocks that finished
static __device__ __align__(256) unsigned long long g_cfl_scratch[kNoAllocMaxBlocks + 32];

std::mutex g_setup_mutex;
unsigned long long* g_scratch_ptr[kMaxDevices] = {};
void* g_scratch_ctx[kMaxDevices] = {};  // the context the address belongs to

// cuCtxGetCurrent through the runtime's driver entry point (no link against
// the driver library): the identity of the current context, so that an
// address looked up in a context that has since been destroyed is not reused.
using CtxGetCurrentFn = int (*)(void**);
CtxGetCurrentFn ctx_get_current() {
  static CtxGetCurrentFn fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<CtxGetCurrentFn>(f);
  }();
  return fn;
}

// The device address of g_cfl_scratch on the current device, looked up once
// per device and context.  In host code the symbol is only a stand-in, never
// a device address.
int scratch_for_current_device(unsigned long long** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return GCH_ERR_CUDA;
  CtxGetCurrentFn get = ctx_get_current();
  if (!get) return GCH_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  void* ctx = nullptr;
  if (get(&ctx) != 0) return GCH_ERR_CUDA;
  if (!ctx || !g_scratch_ptr[dev] || g_scratch_ctx[dev] != ctx) {
    // the lookup also makes the device's primary context current if no
    // runtime call on this thread has done so yet
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_cfl_scratch) != cudaSuccess || !ptr) return GCH_ERR_CUDA;
    if (!ctx && (get(&ctx) != 0 || !ctx)) return GCH_ERR_CUDA;
    g_scratch_ptr[dev] = static_cast<unsigned long long*>(ptr);
    g_scratch_ctx[dev] = ctx;
  }
  *out = g_scratch_ptr[dev];
  return GCH_OK;
}

// One kernel: CFL candidate of every interior cell read straight from u in
// the reference's host layout (u(neq, 1-2:nx+2, ...), FP64, in device
// memory), a block minimum into the scratch array, and -- in the last block
// to finish -- the minimum over blocks, the ramp and the output clip of
// src/hydro_core.f90:644-694.  FP64 arithmetic as the plain drop-in.
__global__ void __launch_bounds__(256)
k_cfl_noalloc(gch::KParams p, const double* __restrict__ u, unsigned long long* scratch,
              int iter, int n_iter, double time, double tprint, double* dt_out,
              int* dump_out) {
  using namespace gch;
  const int nblocks = gridDim.x * gridDim.y * gridDim.z;
  const int bid = (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
  const int ci = blockIdx.x * 32 + threadIdx.x;
  const int cj = blockIdx.y * 8 + threadIdx.y;
  const int kb = blockIdx.z * 8;
  const int ke = min(p.nz, kb + 8);
  double dtp = 1e30;
  if (ci < p.nx && cj < p.ny) {
    for (int k = kb; k < ke; ++k) {
      const long long cell =
          ((long long)(k + NG) * p.NY + (cj + NG)) * p.NX + (ci + NG);  // no row padding
      double uu[8], pr[8];
      for (int q = 0; q < p.neq; ++q) uu[q] = u[cell * p.neq + q];
      for (int q = p.neq; q < 8; ++q) uu[q] = 0.0;
      // src/hydro_core.f90:46-129 u2prim (FP64, the reference's order)
      const double r = tmax_(uu[0], 1e-15);
      pr[0] = r;
      pr[1] = uu[1] / r;
      pr[2] = uu[2] / r;
      pr[3] = uu[3] / r;
      if (p.mhd)
        pr[4] = (uu[4] - 0.5 * r * (pr[1] * pr[1] + pr[2] * pr[2] + pr[3] * pr[3])
                 - 0.5 * (uu[5] * uu[5] + uu[6] * uu[6] + uu[7] * uu[7])) / p.cv;
      else
        pr[4] = (uu[4] - 0.5 * r * (pr[1] * pr[1] + pr[2] * pr[2] + pr[3] * pr[3])) / p.cv;
      pr[4] = tmax_(pr[4], 1e-16);
      if (p.eos == GCH_EOS_SINGLE_SPECIE) {
        const double t = tmax_(1.0, (pr[4] / r) * p.Tempsc);
        pr[4] = r * t / p.Tempsc;
      }
      pr[5] = uu[5];
      pr[6] = uu[6];
      pr[7] = uu[7];
      double cx, cy, cz;
      if (p.mhd) {  // src/hydro_core.f90:568-581 cfast
        const double g = p.gamma;
        const double b2 = pr[5] * pr[5] + pr[6] * pr[6] + pr[7] * pr[7];
        const double a = g * pr[4] + b2;
        cx = sqrt(0.5 * (a + sqrt(a * a - 4.0 * g * pr[4] * pr[5] * pr[5])) / pr[0]);
        cy = sqrt(0.5 * (a + sqrt(a * a - 4.0 * g * pr[4] * pr[6] * pr[6])) / pr[0]);
        cz = sqrt(0.5 * (a + sqrt(a * a - 4.0 * g * pr[4] * pr[7] * pr[7])) / pr[0]);
      } else {  // src/hydro_core.f90:544-553 csound
        cx = cy = cz = sqrt(p.gamma * pr[4] / pr[0]);
      }
      dtp = tmin_(dtp, p.dx / (fabs(pr[1]) + cx));
      dtp = tmin_(dtp, p.dy / (fabs(pr[2]) + cy));
      dtp = tmin_(dtp, p.dz / (fabs(pr[3]) + cz));
    }
  }
  // block minimum
  for (int o = 16; o > 0; o >>= 1) dtp = tmin_(dtp, __shfl_xor_sync(0xffffffffu, dtp, o));
  __shared__ double red[8];
  __shared__ bool last;
  const int t = threadIdx.y * 32 + threadIdx.x;
  if ((t & 31) == 0) red[t >> 5] = dtp;
  __syncthreads();
  if (t == 0) {
    double v = red[0];
    for (int w = 1; w < 8; ++w) v = tmin_(v, red[w]);
    scratch[bid] = (unsigned long long)__double_as_longlong(v);
    __threadfence();  // the partial is visible before the count
    const unsigned int done = atomicAdd((unsigned int*)&scratch[kNoAllocMaxBlocks], 1u);
    last = done == (unsigned int)(nblocks - 1);
  }
  __syncthreads();
  if (!last) return;
  // the last block: minimum over all partial minima
  __threadfence();
  double v = 1e30;
  for (int b = t; b < nblocks; b += 256)
    v = tmin_(v, __longlong_as_double((long long)((volatile unsigned long long*)scratch)[b]));
  for (int o = 16; o > 0; o >>= 1) v = tmin_(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((t & 31) == 0) red[t >> 5] = v;
  __syncthreads();
  if (t == 0) {
    double m = red[0];
    for (int w = 1; w < 8; ++w) m = tmin_(m, red[w]);
    // src/hydro_core.f90:677-694
    if (iter <= n_iter)
      m = p.cfl * ldexp(1.0, -(n_iter + 1 - iter)) * m;
    else
      m = p.cfl * m;
    int dump = 0;
    if ((time + m) >= tprint) {
      m = tprint - time;
      dump = 1;
    }
    *dt_out = m;
    *dump_out = dump;
    scratch[kNoAllocMaxBlocks] = 0ull;  // counter ready for the next call
  }
}

}  // namespace

extern "C" int gch_get_timestep_noalloc(const gch_params_t* p, const double* u_dev,
                                        int current_iter, int n_iter, double current_time,
                                        double tprint, double* dt_dev, int* dump_dev,
                                        void* stream) {
  if (!p || !u_dev || !dt_dev || !dump_dev) return GCH_ERR_PARAM;
  int st = gch_params_check(p);
  if (st) return st;
  // the reduction reads u; with table cooling the reference takes dt from
  // the stored (cooled) primitives instead
  if (p->cooling != GCH_COOL_NONE) return GCH_ERR_PARAM;
  // the one-cell state of the kernel holds the 8 dynamical equations only
  if (p->npas != 0) return GCH_ERR_PARAM;
  // the split solver's timestep needs the background state of a domain
  if (p->riemann_solver == GCH_SOLVER_HLLE_SPLIT_ALL) return GCH_ERR_PARAM;
  const long long gx = (p->nx + 31) / 32, gy = (p->ny + 7) / 8, gz = (p->nz + 7) / 8;
  if (gx * gy * gz > kNoAllocMaxBlocks || gy > 65535 || gz > 65535) return GCH_ERR_TOO_LARGE;
  unsigned long long* scratch = nullptr;
  st = scratch_for_current_device(&scratch);
  if (st) return st;
  gch::KParams k = {};
  k.nx = p->nx; k.ny = p->ny; k.nz = p->nz;
  k.NX = p->nx + 2 * gch::NG; k.NY = p->ny + 2 * gch::NG; k.NZ = p->nz + 2 * gch::NG;
  k.neq = p->neq;
  k.mhd = p->mhd;
  k.eos = p->eq_of_state;
  k.dx = p->dx; k.dy = p->dy; k.dz = p->dz;
  k.cv = p->cv; k.gamma = p->gamma; k.cfl = p->cfl;
  k.Tempsc = p->Tempsc;
  gch::set_f32_params(k);
  cudaStream_t s = (cudaStream_t)stream;
  // the completion counter must start at zero (a call cut short earlier
  // could have left it set); clearing it is a memset, not an allocation
  if (cudaMemsetAsync(scratch + kNoAllocMaxBlocks, 0, sizeof(unsigned long long), s) !=
      cudaSuccess)
    return GCH_ERR_CUDA;
  k_cfl_noalloc<<<dim3((unsigned)gx, (unsigned)gy, (unsigned)gz), dim3(32, 8), 0, s>>>(
      k, u_dev, scratch, current_iter, n_iter, current_time, tprint, dt_dev, dump_dev);
  return cudaGetLastError() == cudaSuccess ? GCH_OK : GCH_ERR_CUDA;
}
