// gch_batch.cu -- many independent boxes of uneven size, each with its own
// CFL dt, advanced together.
//
// Grouped mode (FP32 policies; no COOL_H, conduction, resistivity or
// passive scalars; table cooling and user spheres are carried): one step of
// all boxes is one CUDA graph of grouped launches,
// one launch per kernel of the step for up to 64 boxes (gch_group.cuh).  The
// two stage kernels work (box, tile, z chunk) items, either one block per
// item or as a persistent grid whose blocks pull items from a device
// counter.  The autotuner picks the z-march depth of an item and the launch
// form (one block per item, or 1, 2 or 3 resident blocks per SM) by timing
// the stage-1 flux kernel over the whole batch for every pair (it runs once, before the first step; that kernel only
// writes the stage arrays up and E, so timing it leaves the state
// untouched).  The tile of a work item stays 32 x 8 cells: the stage
// kernel's shared-memory layout and its TMA boxes are built for it.  The
// loop state of every box is gathered into one array and read back with one
// copy.
//
// Otherwise (FP64, or physics the grouped step does not carry) every box
// runs its own captured step graph on its own stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <new>
#include <vector>

#include "gch_domain.h"

namespace {

using gch::StepScalars;

// the loop controls of a batched advance: no output clip, no tmax
__global__ void k_batch_begin(StepScalars* const* sc, int n, int n_iter) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n) return;
  StepScalars* s = sc[b];
  s->n_iter = n_iter;
  s->tprint = 1e300;
  s->dtprint = 1e300;
  s->tmax = 1e300;
  s->dump = 0;
  s->active = s->err == 0;
}

__global__ void k_batch_gather(StepScalars* const* sc, int n, StepScalars* out) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < n) out[b] = *sc[b];
}

__global__ void k_batch_clear_info(StepScalars* const* sc, int n) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n) return;
  sc[b]->err = 0;
  sc[b]->pfloor = 0;
}

int cuda_ok(cudaError_t e) { return e == cudaSuccess ? GCH_OK : GCH_ERR_CUDA; }

}  // namespace

struct gch_batch {
  std::vector<gch_domain*> boxes;
  std::vector<double> time;
  std::vector<int> iter;
  // grouped mode
  const gch::GroupOps* gops = nullptr;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int kz = 0;                                // 0 until the autotuner ran
  int bps = 0;                               // stage kernels: persistent blocks per SM (0: one per item)
  std::vector<int> tune_kz;                  // candidates and their times
  std::vector<int> tune_bps;
  std::vector<float> tune_ms;
  int* queue = nullptr;                      // device work counter of the stage kernels
  cudaGraphExec_t graph = nullptr;
  StepScalars** sc_list = nullptr;           // device: the boxes' scalar blocks
  StepScalars* sc_all = nullptr;             // device gather buffer
  StepScalars* sc_all_host = nullptr;        // pinned
};

namespace {

// FP32 boxes without resistivity, COOL_H, thermal conduction or passive
// scalars; table cooling and user spheres run grouped too
bool groupable(const gch_params_t& p) {
  const bool table = p.cooling == GCH_COOL_DMC || p.cooling == GCH_COOL_CHI;
  return p.precision != GCH_FP64 && p.eta == 0.0 && p.th_cond == GCH_TC_OFF &&
         (p.cooling == GCH_COOL_NONE || table) && p.npas == 0;
}

int grid_of(int n) { return (n + 127) / 128; }

// Time the stage-1 flux kernel of all boxes for each candidate pair of
// z-march depth and resident blocks per SM, and keep the fastest.
int autotune(gch_batch* b) {
  const int n = (int)b->boxes.size();
  int nzmax = 1;
  for (gch_domain* d : b->boxes) nzmax = std::max(nzmax, d->kp.nz);
  cudaEvent_t e0, e1;
  int st = cuda_ok(cudaEventCreate(&e0));
  st |= cuda_ok(cudaEventCreate(&e1));
  b->tune_kz.clear();
  b->tune_bps.clear();
  b->tune_ms.clear();
  float best = 0.f;
  int best_kz = std::min(8, nzmax), best_bps = 3;
  st |= b->gops->prep(b->boxes.data(), n, b->stream);
  for (int kz : {2, 4, 8, 12, 16, 20, 24, 32}) {
    if (kz > nzmax && kz != 2) break;
    for (int bps : {0, 1, 2, 3}) {
      st |= b->gops->probe(b->boxes.data(), n, kz, bps, b->queue, b->stream);  // warm-up
      st |= cuda_ok(cudaEventRecord(e0, b->stream));
      for (int r = 0; r < 3; ++r)
        st |= b->gops->probe(b->boxes.data(), n, kz, bps, b->queue, b->stream);
      st |= cuda_ok(cudaEventRecord(e1, b->stream));
      st |= cuda_ok(cudaEventSynchronize(e1));
      float ms = 0.f;
      st |= cuda_ok(cudaEventElapsedTime(&ms, e0, e1));
      if (st) break;
      b->tune_kz.push_back(kz);
      b->tune_bps.push_back(bps);
      b->tune_ms.push_back(ms / 3);
      if (b->tune_kz.size() == 1 || ms < best) {
        best = ms;
        best_kz = kz;
        best_bps = bps;
      }
    }
    if (st) break;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  // the probes (and the CFL pass before them) counted pressure floors: clear them
  k_batch_clear_info<<<grid_of(n), 128, 0, b->stream>>>(b->sc_list, n);
  st |= cuda_ok(cudaGetLastError());
  b->kz = best_kz;
  b->bps = best_bps;
  return st;
}

int grouped_advance(gch_batch* b, int steps, int n_iter) {
  const int n = (int)b->boxes.size();
  int st = GCH_OK;
  k_batch_begin<<<grid_of(n), 128, 0, b->stream>>>(b->sc_list, n, n_iter);
  st |= cuda_ok(cudaGetLastError());
  if (!b->kz) st |= autotune(b);
  if (!b->graph && !st) {
    cudaGraph_t g = nullptr;
    st |= cuda_ok(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    st |= b->gops->step(b->boxes.data(), n, b->kz, b->bps, b->queue, b->stream);
    st |= cuda_ok(cudaStreamEndCapture(b->stream, &g));
    if (st == GCH_OK) st |= cuda_ok(cudaGraphInstantiate(&b->graph, g, 0));
    if (g) cudaGraphDestroy(g);
  }
  if (st) return st;
  for (int s = 0; s < steps; ++s) st |= cuda_ok(cudaGraphLaunch(b->graph, b->stream));
  k_batch_gather<<<grid_of(n), 128, 0, b->stream>>>(b->sc_list, n, b->sc_all);
  st |= cuda_ok(cudaMemcpyAsync(b->sc_all_host, b->sc_all, n * sizeof(StepScalars),
                                cudaMemcpyDeviceToHost, b->stream));
  st |= cuda_ok(cudaStreamSynchronize(b->stream));
  for (int i = 0; i < n; ++i) {
    b->time[i] = b->sc_all_host[i].time;
    b->iter[i] = b->sc_all_host[i].iter;
    st |= b->sc_all_host[i].err;
  }
  return st;
}

}  // namespace

extern "C" {

int gch_batch_destroy(gch_batch_t* b) {
  if (!b) return GCH_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  cudaFree(b->sc_list);
  cudaFree(b->sc_all);
  cudaFree(b->queue);
  if (b->sc_all_host) cudaFreeHost(b->sc_all_host);
  if (b->stream && b->own_stream) cudaStreamDestroy(b->stream);
  for (gch_domain* d : b->boxes) gch_destroy(d);
  delete b;
  return GCH_OK;
}

int gch_batch_create(int n, const gch_params_t* params, void* stream, gch_batch_t** out) {
  if (!out || n < 1 || !params) return GCH_ERR_PARAM;
  *out = nullptr;
  bool grouped = groupable(params[0]);
  for (int i = 1; i < n; ++i) {
    const gch_params_t& a = params[0];
    const gch_params_t& c = params[i];
    if (c.precision != a.precision || c.neq != a.neq || c.mhd != a.mhd ||
        c.riemann_solver != a.riemann_solver || c.slope_limiter != a.slope_limiter ||
        c.enable_flux_cd != a.enable_flux_cd || c.cooling != a.cooling)
      return GCH_ERR_PARAM;
    grouped = grouped && groupable(c);
  }
  gch_batch* b = new (std::nothrow) gch_batch();
  if (!b) return GCH_ERR_CUDA;
  for (int i = 0; i < n; ++i) {
    gch_domain* d = nullptr;
    int st = gch_create(&params[i], nullptr, &d);
    if (st) {
      gch_batch_destroy(b);
      return st;
    }
    b->boxes.push_back(d);
    b->time.push_back(0.0);
    b->iter.push_back(1);
  }
  if (grouped) {
    b->gops = params[0].precision == GCH_FP32_KAHAN ? &gch::kGroupKahan : &gch::kGroupMixed;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaSuccess;
    if (!s) {  // capture needs a stream other than the legacy default stream
      e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
      b->own_stream = e == cudaSuccess;
    }
    b->stream = s;
    std::vector<StepScalars*> sc(n);
    for (int i = 0; i < n; ++i) sc[i] = b->boxes[i]->sc;
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->sc_list, n * sizeof(StepScalars*));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->sc_all, n * sizeof(StepScalars));
    if (e == cudaSuccess) e = cudaMallocHost((void**)&b->sc_all_host, n * sizeof(StepScalars));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->queue, sizeof(int));
    if (e == cudaSuccess)
      e = cudaMemcpy(b->sc_list, sc.data(), n * sizeof(StepScalars*), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      gch_batch_destroy(b);
      return GCH_ERR_CUDA;
    }
  }
  *out = b;
  return GCH_OK;
}

int gch_batch_upload(gch_batch_t* b, int box, const double* u) {
  if (!b || box < 0 || box >= (int)b->boxes.size()) return GCH_ERR_PARAM;
  if (b->stream) cudaStreamSynchronize(b->stream);
  int st = gch_upload(b->boxes[box], u);
  st |= gch_boundaryI(b->boxes[box]);
  st |= gch_calcprim(b->boxes[box]);
  st |= cuda_ok(cudaStreamSynchronize(b->boxes[box]->stream));
  return st;
}

int gch_batch_download(gch_batch_t* b, int box, double* u) {
  if (!b || box < 0 || box >= (int)b->boxes.size()) return GCH_ERR_PARAM;
  if (b->stream) cudaStreamSynchronize(b->stream);
  return gch_download(b->boxes[box], u, nullptr);
}

int gch_batch_advance(gch_batch_t* b, int steps, int n_iter) {
  if (!b || steps < 0) return GCH_ERR_PARAM;
  if (b->gops) return grouped_advance(b, steps, n_iter);
  int st = GCH_OK;
  const double inf = 1e300;
  for (size_t i = 0; i < b->boxes.size(); ++i)
    st |= gch_advance_enqueue(b->boxes[i], steps, inf, inf, n_iter, b->time[i], b->iter[i], inf);
  for (size_t i = 0; i < b->boxes.size(); ++i) {
    double tp;
    st |= gch_advance_finish(b->boxes[i], &b->time[i], &b->iter[i], &tp);
  }
  return st;
}

int gch_batch_time(gch_batch_t* b, double* times, int* iters) {
  if (!b) return GCH_ERR_PARAM;
  for (size_t i = 0; i < b->boxes.size(); ++i) {
    if (times) times[i] = b->time[i];
    if (iters) iters[i] = b->iter[i];
  }
  return GCH_OK;
}

int gch_batch_tuning(gch_batch_t* b, int* grouped, int* kz, int cap, int* cand_kz,
                     float* cand_ms, int* ncand) {
  if (!b) return GCH_ERR_PARAM;
  if (grouped) *grouped = b->gops != nullptr;
  if (kz) *kz = b->gops ? b->kz : -1;
  // the candidates timed with the chosen blocks per SM
  int m = 0;
  for (size_t i = 0; i < b->tune_kz.size() && m < cap; ++i) {
    if (b->tune_bps[i] != b->bps) continue;
    if (cand_kz) cand_kz[m] = b->tune_kz[i];
    if (cand_ms) cand_ms[m] = b->tune_ms[i];
    ++m;
  }
  if (ncand) *ncand = m;
  return GCH_OK;
}

int gch_batch_tuning_grid(gch_batch_t* b, int* grouped, int* kz, int* bps, int cap,
                          int* cand_kz, int* cand_bps, float* cand_ms, int* ncand) {
  if (!b) return GCH_ERR_PARAM;
  if (grouped) *grouped = b->gops != nullptr;
  if (kz) *kz = b->gops ? b->kz : -1;
  if (bps) *bps = b->gops ? b->bps : -1;
  const int m = std::min(cap, (int)b->tune_kz.size());
  for (int i = 0; i < m; ++i) {
    if (cand_kz) cand_kz[i] = b->tune_kz[i];
    if (cand_bps) cand_bps[i] = b->tune_bps[i];
    if (cand_ms) cand_ms[i] = b->tune_ms[i];
  }
  if (ncand) *ncand = m;
  return GCH_OK;
}

}  // extern "C"
