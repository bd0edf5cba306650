// gch_domain.h -- host-side state of one domain and the per-precision engine
// table.  Shared by the C-ABI layer (gch_api.cu) and the kernel instantiation
// units (gch_fp64.cu, gch_fp32.cu).
#pragma once

#include <cuda_runtime.h>

#include "gch_device.cuh"
#include "gch_tma.cuh"
#include "guacho_gb300.h"

struct gch_domain {
  gch_params_t hp;              // parameters as given
  gch::KParams kp;              // kernel parameter block
  cudaStream_t stream = nullptr;
  bool own_stream = false;      // created here (destroyed with the domain)
  int mode = GCH_FP64;
  bool prim_in = false;         // tabulated cooling keeps a primit array
  // FP32 paths otherwise: get_timestep's CFL pass stores the primitives of u
  // in primit for the first stage of the same step (StepScalars::prim_fresh)
  bool prim_pre = false;
  size_t tu_size = 8, ts_size = 8;
  // device arrays
  void* u = nullptr;            // neq fields, TU
  void* up = nullptr;           // neq fields, TS
  void* w = nullptr;            // neq fields, TU (stage-2 result when eta != 0)
  void* E = nullptr;            // 3 fields, TS
  void* s678 = nullptr;         // 3 fields, TS (eight-wave sources)
  void* primit = nullptr;       // neq fields, TS (tabulated cooling; FP64 with the split solver)
  double* prim0 = nullptr;      // split solver: the background primit0, neq fields
  double* split_f = nullptr;    // split solver: x, y, z face fluxes, 3 x neq fields
  double* tab = nullptr;        // [2][ntab]
  gch_sphere_t* sph = nullptr;
  double* grav = nullptr;       // [4][ngrav]
  unsigned char* tmaps = nullptr;       // TMA tensor maps of the stage sources (FP32 paths)
  gch::StepScalars* sc = nullptr;       // device
  gch::StepScalars* sc_host = nullptr;  // pinned mirror
  double* stage = nullptr;      // device staging buffer, host layout (FP64 AoS)
  size_t ncell_host = 0;        // NX*NY*NZ
  int kz = 8;                   // z planes per block of the stage kernels
  // the z chunks [zc0, zc0 + zcn) of kz planes that the next stage launch
  // covers (all of them when zcn == 0): a slab of the pipelined second stage
  int zc0 = 0, zcn = 0;
  // the next first-stage launch defers its update: it writes the flux
  // differences to `dif` (3 x neq fields of the stage type, allocated on
  // first use) for k_s1_apply
  bool defer = false;
  void* dif = nullptr;
  // gch_step_host's download behind the second stage: the copy stream and
  // one event per copied slab plus one for the last copy
  cudaStream_t cstream = nullptr;
  static constexpr int kPipeEv = 24;
  cudaEvent_t pipe_ev[kPipeEv] = {};
  int launches = 0;             // kernel launches of the last tstep
  // thermal conduction (th_cond != 0): rho, p, T and the three face fluxes
  // (6 fields, FP64), the device min of the conduction timescale and its
  // pinned copy, and the substep count / timescale of the last tstep
  double* tcw = nullptr;
  unsigned long long* tc_min = nullptr;
  unsigned long long* tc_min_host = nullptr;
  int tc_nsteps = 0;
  double tc_dt_cond = 0.0;
  // CUDA graph of one device-resident step (get_timestep + tstep + loop tail)
  cudaGraphExec_t graph = nullptr;
  // per-launch profiling: when prof_on, an event is recorded after every
  // launch with the kernel's name (gch_profile_step)
  bool prof_on = false;
  int prof_n = 0;
  cudaEvent_t prof_ev[64] = {};
  const char* prof_name[64] = {};
};

// Record the end of the launch just issued (no-op unless profiling).
inline void gch_mark(gch_domain* d, const char* name) {
  if (!d->prof_on || d->prof_n >= 63) return;
  d->prof_name[d->prof_n] = name;
  cudaEventRecord(d->prof_ev[d->prof_n + 1], d->stream);
  ++d->prof_n;
}

namespace gch {

struct EngineOps {
  int (*get_dt)(gch_domain*);         // k_cfl + k_dtfin
  int (*tstep)(gch_domain*);          // both stages + boundaries
  int (*boundaryI)(gch_domain*);      // ghost layer of u + user spheres
  int (*calcprim)(gch_domain*);       // primit from u (tabulated cooling)
  // host layout (staging buffer or mapped host memory) <-> u / primit
  int (*upload)(gch_domain*, const double*);
  int (*download_u)(gch_domain*, double*);
  int (*download_prim)(gch_domain*, double*);
  int (*loopfin)(gch_domain*);        // device time-loop tail
  int (*probe)(gch_domain*);          // stage-1 fluxes alone (autotuner)
  // gch_step_host's upload, get_timestep and tstep with the copies in and
  // out of the host array `host` (reference layout) overlapped with the
  // step; only for domains pipe_ok accepts (the step's controls are set)
  int (*step_host)(gch_domain*, double* host);
};

// Whether gch_step_host can overlap the download of u with the second
// stage: the boundary fill of u is the plain shell fill (no user spheres,
// table cooling, COOL_H, resistivity, conduction or split solver) and the
// box has at least three z chunks.
bool pipe_ok(const gch_domain* d);

extern const EngineOps kEngineFP64;
extern const EngineOps kEngineMixed;
extern const EngineOps kEngineKahan;

// Grouped launches over many boxes of one precision (gch_group.cuh).  The
// boxes share solver, neq, limiter and flux-CD, have no table cooling,
// resistivity or user spheres, and are advanced on one stream.
struct GroupOps {
  // one device-resident iteration of every box: k_cfl, k_dtfin, both
  // stages with their CT and ghost fills, k_loopfin.  The stage kernels are
  // persistent: `bps` blocks per SM pull (box, tile, z chunk) work items of
  // `kz` planes from the device counter `queue` (cleared before each launch)
  int (*step)(gch_domain* const* boxes, int n, int kz, int bps, int* queue, cudaStream_t s);
  // the stage-1 flux kernel alone (writes up and E, leaves u): the
  // autotuner's timing probe
  int (*probe)(gch_domain* const* boxes, int n, int kz, int bps, int* queue, cudaStream_t s);
  // before the probes: the stored primitives the first stage reads on the
  // FP32 + FP64-u path (the CFL pass of the current u; leaves u)
  int (*prep)(gch_domain* const* boxes, int n, cudaStream_t s);
};
extern const GroupOps kGroupMixed;
extern const GroupOps kGroupKahan;

// Encode the 4-D TMA tensor map (x, field, y, z) of a stage source array
// (es-byte elements, the domain's padded layout) with a box of `box_x`
// cells x every field x `box_rows` rows x 1 plane into `map` (128 bytes);
// GCH_OK or GCH_ERR_CUDA (gch_api.cu).
int encode_stage_map(unsigned char* map, const void* base, int es, const KParams& k, int box_x,
                     int box_rows);

// Thermal conduction after a tstep of dt_CFL (gch_tc.cu): synchronises once.
int tc_run(gch_domain* d, double dt_CFL);
// the split solver SOLVER_HLLE_SPLIT_ALL on the FP64 path (gch_split.cu)
int split_calcprim(gch_domain* d);
int split_get_dt(gch_domain* d);
int split_tstep(gch_domain* d);
int split_set_background(gch_domain* d, const double* aos);
int split_download_prim(gch_domain* d, double* aos);
int tc_run_kahan(gch_domain* d, double dt_CFL);  // the FP32 paths (gch_tc32.cu)
int tc_run_mixed(gch_domain* d, double dt_CFL);
// The super-time-stepping scalars of src/thermal_cond.f90:625-681.
double tc_superstep(int N, double snu);
double tc_substep(int j, int N, double nu);
void tc_st_steps(double fs, int* Ns, double* fstep);

}  // namespace gch

// Device-resident time loop split in its asynchronous and waiting halves
// (used by the batched driver to overlap boxes on their own streams).
int gch_advance_enqueue(gch_domain* d, int max_steps, double tmax, double dtprint, int n_iter,
                        double time, int iter, double tprint);
int gch_advance_finish(gch_domain* d, double* time, int* iter, double* tprint);
