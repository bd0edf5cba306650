// gch_batch.cu -- many independent boxes of uneven size, each with its own
// CFL dt, advanced together.  Each box runs its captured step graph on its
// own stream so that small boxes overlap on the 152 SMs.
#include <cuda_runtime.h>

#include <new>
#include <vector>

#include "gch_domain.h"

struct gch_batch {
  std::vector<gch_domain*> boxes;
  std::vector<double> time;
  std::vector<int> iter;
};

extern "C" {

int gch_batch_destroy(gch_batch_t* b) {
  if (!b) return GCH_OK;
  for (gch_domain* d : b->boxes) gch_destroy(d);
  delete b;
  return GCH_OK;
}

int gch_batch_create(int n, const gch_params_t* params, void* stream, gch_batch_t** out) {
  (void)stream;  // every box gets its own stream
  if (!out || n < 1 || !params) return GCH_ERR_PARAM;
  *out = nullptr;
  for (int i = 1; i < n; ++i) {
    const gch_params_t& a = params[0];
    const gch_params_t& c = params[i];
    if (c.precision != a.precision || c.neq != a.neq || c.mhd != a.mhd ||
        c.riemann_solver != a.riemann_solver || c.slope_limiter != a.slope_limiter ||
        c.enable_flux_cd != a.enable_flux_cd || c.cooling != a.cooling)
      return GCH_ERR_PARAM;
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
  *out = b;
  return GCH_OK;
}

int gch_batch_upload(gch_batch_t* b, int box, const double* u) {
  if (!b || box < 0 || box >= (int)b->boxes.size()) return GCH_ERR_PARAM;
  int st = gch_upload(b->boxes[box], u);
  st |= gch_boundaryI(b->boxes[box]);
  st |= gch_calcprim(b->boxes[box]);
  return st;
}

int gch_batch_download(gch_batch_t* b, int box, double* u) {
  if (!b || box < 0 || box >= (int)b->boxes.size()) return GCH_ERR_PARAM;
  return gch_download(b->boxes[box], u, nullptr);
}

int gch_batch_advance(gch_batch_t* b, int steps, int n_iter) {
  if (!b || steps < 0) return GCH_ERR_PARAM;
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

}  // extern "C"
