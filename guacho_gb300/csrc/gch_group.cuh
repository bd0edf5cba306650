// gch_group.cuh -- grouped launches: one kernel launch advances a stage of
// many independent boxes of uneven size.
//
// Every box keeps its own arrays, parameters and StepScalars (its own CFL
// dt).  A grouped launch carries the per-box parameter blocks in its kernel
// parameter space (__grid_constant__, up to kGroupMax boxes, 22 KB) and a
// one-dimensional grid: block b belongs to the box whose first block blk0
// is the largest one <= b, and is decoded to that box's tile coordinates.
// The per-box bodies are the ones of the one-box kernels, so a box computes
// exactly what it computes alone.
#pragma once

#include "gch_kernels.cuh"

namespace gch {

constexpr int kGroupMax = 64;  // boxes per grouped launch

struct GroupBox {
  KParams p;
  const void* a0;  // kernel-specific arrays (see GroupEngine)
  const void* a1;
  void* a2;
  void* a3;
  void* a4;
  StepScalars* sc;
  int blk0;        // first linear block of this box in the launch
  int gx, gy;      // blocks along the two fastest grid axes of the box
  int kz;          // z planes per block (stage and CT kernels)
};

struct GroupArgs {
  int nbox;
  int i0, i1;      // kernel-specific integers (ghost fill: axis, layers)
  GroupBox box[kGroupMax];
};
static_assert(sizeof(GroupArgs) <= 32000, "grouped launch exceeds the kernel parameter limit");

// the box owning linear block `blk` (binary search over blk0)
__device__ __forceinline__ int group_box(const GroupArgs& g, int blk) {
  int lo = 0, hi = g.nbox - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (g.box[mid].blk0 <= blk) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// The stage kernel of many boxes (a0 = stage source: u, or primit with
// table cooling, in stage 1 and up in stage 2; a1 = u, a2 = stage
// destination, a3 = E, a4 = s678).  Work item b -- one (box, tile, z chunk),
// numbered box by box from the box's blk0 on as the blocks of a one-box
// grid -- is worked by one block.  Two launch forms:
//  - k_flux_grp: one block per work item (the hardware hands out blocks);
//  - k_flux_pst: a persistent grid of a few blocks per SM, each block taking
//    the next item from the device counter `queue` (zero at launch) until
//    all `total` items are done.  The block fetches its following item while
//    it works the current one, so the counter's latency stays hidden.
//    Blocks never wait on one another: a grid larger than what the SMs hold
//    at once only starts its last blocks later.
template <class Pol, int SOLVER, int NEQ, int STAGE, int LIM, bool PRIM_IN>
__device__ __forceinline__ void flux_item(const GroupArgs& g, int item) {
  using TIn = typename Src<Pol, NEQ, STAGE, PRIM_IN>::TIn;
  using TD = typename std::conditional<STAGE == 1, typename Pol::TS, typename Pol::TU>::type;
  const GroupBox& x = g.box[group_box(g, item)];
  const int l = item - x.blk0;
  flux_body<Pol, SOLVER, NEQ, STAGE, PRIM_IN, LIM>(
      x.p, (const TIn*)x.a0, (const typename Pol::TU*)x.a1, (TD*)x.a2, (typename Pol::TS*)x.a3,
      (typename Pol::TS*)x.a4, x.sc, x.kz, l % x.gx, (l / x.gx) % x.gy, l / (x.gx * x.gy));
}
template <class Pol, int SOLVER, int NEQ, int STAGE, int LIM, bool PRIM_IN>
__global__ void __launch_bounds__(NT, Pol::kMinBlocks) k_flux_grp(const __grid_constant__ GroupArgs g) {
  flux_item<Pol, SOLVER, NEQ, STAGE, LIM, PRIM_IN>(g, blockIdx.x);
}
template <class Pol, int SOLVER, int NEQ, int STAGE, int LIM, bool PRIM_IN>
__global__ void __launch_bounds__(NT, Pol::kMinBlocks)
    k_flux_pst(const __grid_constant__ GroupArgs g, int* queue, int total) {
  __shared__ int s_item[2];
  const bool lead = threadIdx.x == 0 && threadIdx.y == 0;
  if (lead) s_item[0] = atomicAdd(queue, 1);
  __syncthreads();
  for (int slot = 0;; slot ^= 1) {
    const int item = s_item[slot];
    if (item >= total) break;
    int next = 0;
    if (lead) next = atomicAdd(queue, 1);  // its result is needed only after the item
    flux_item<Pol, SOLVER, NEQ, STAGE, LIM, PRIM_IN>(g, item);
    if (lead) s_item[slot ^ 1] = next;
    __syncthreads();  // the item is finished with shared memory; the next index is set
  }
}

// a1 = u, a2 = destination of B, a3 = E, a4 = s678
// Six blocks per SM: the register cap of four blocks made the compiler
// spill in this kernel (measured on 64 boxes of 32^3..96^3: the grouped
// step 4.27 ms with four, 4.05 ms with six).
template <class Pol, int STAGE>
__global__ void __launch_bounds__(256, 6) k_ct_grp(const __grid_constant__ GroupArgs g) {
  using TD = typename std::conditional<STAGE == 1, typename Pol::TS, typename Pol::TU>::type;
  const GroupBox& x = g.box[group_box(g, blockIdx.x)];
  const int l = blockIdx.x - x.blk0;
  ct_body<Pol, STAGE>(x.p, (const typename Pol::TU*)x.a1, (TD*)x.a2,
                           (const typename Pol::TS*)x.a3, (const typename Pol::TS*)x.a4, x.sc,
                           x.kz, l % x.gx, (l / x.gx) % x.gy, l / (x.gx * x.gy));
}

// a2 = the array to fill; i1 = layers; 256 cells of one box per block
template <class T>
__global__ void __launch_bounds__(256) k_ghost_all_grp(const __grid_constant__ GroupArgs g) {
  const GroupBox& x = g.box[group_box(g, blockIdx.x)];
  if (!x.sc->active) return;
  const long long t = (long long)(blockIdx.x - x.blk0) * 256 + threadIdx.x;
  if (t < ghost_all_count(x.p, g.i1)) ghost_all_cell<T>(x.p, (T*)x.a2, x.p.neq, g.i1, t);
}

// a2 = the array to fill; i0 = axis, i1 = layers
template <class T>
__global__ void __launch_bounds__(128) k_ghost_grp(const __grid_constant__ GroupArgs g) {
  const GroupBox& x = g.box[group_box(g, blockIdx.x)];
  const int l = blockIdx.x - x.blk0;
  ghost_body<T>(x.p, (T*)x.a2, x.p.neq, g.i0, g.i1, x.sc, l % x.gx, (l / x.gx) % x.gy,
                l / (x.gx * x.gy));
}

// a1 = u, or primit with table cooling (PRIM_IN); a2 = where the primitives
// recovered from u are stored for the first stage (null: not stored)
template <class Pol, int NEQ, bool PRIM_IN>
__global__ void __launch_bounds__(256) k_cfl_grp(const __grid_constant__ GroupArgs g) {
  using TSrc = typename std::conditional<PRIM_IN, typename Pol::TS, typename Pol::TU>::type;
  const GroupBox& x = g.box[group_box(g, blockIdx.x)];
  const int l = blockIdx.x - x.blk0;
  cfl_body<Pol, NEQ, PRIM_IN>(x.p, (const TSrc*)x.a1, x.sc, x.kz, l % x.gx, (l / x.gx) % x.gy,
                              l / (x.gx * x.gy), (typename Pol::TS*)x.a2);
}

// The user boundary spheres of the boxes that have them: a2 = the array to
// fill, i0 = blocks per sphere; a box's blocks are its spheres x i0
template <class T>
__global__ void __launch_bounds__(256) k_user_bc_grp(const __grid_constant__ GroupArgs g) {
  const GroupBox& x = g.box[group_box(g, blockIdx.x)];
  const int l = blockIdx.x - x.blk0;
  user_bc_body<T>(x.p, (T*)x.a2, x.p.neq, x.sc, l / g.i0, l % g.i0, g.i0);
}

// Table cooling: a1 = u, a2 = primit; block (32, 8), one block per 32 x 8
// tile of each interior plane
template <class Pol, int NEQ>
__global__ void __launch_bounds__(256) k_cool_grp(const __grid_constant__ GroupArgs g) {
  const GroupBox& x = g.box[group_box(g, blockIdx.x)];
  const int l = blockIdx.x - x.blk0;
  cool_body<Pol, NEQ>(x.p, (typename Pol::TU*)x.a1, (typename Pol::TS*)x.a2, x.sc,
                      (l % x.gx) * 32 + threadIdx.x, ((l / x.gx) % x.gy) * 8 + threadIdx.y,
                      l / (x.gx * x.gy));
}

// calcprim of the ghost shell after boundaryI: a1 = u, a2 = primit,
// i0 = blocks per box (grid-stride over the box's shell).  OWN: the shell
// of the primitives get_timestep's CFL pass stored (k_prim_shell_own)
template <class Pol, int NEQ, bool OWN = false>
__global__ void __launch_bounds__(256) k_calcprim_shell_grp(const __grid_constant__ GroupArgs g) {
  const GroupBox& x = g.box[group_box(g, blockIdx.x)];
  calcprim_shell_body<Pol, NEQ, OWN>(x.p, (const typename Pol::TU*)x.a1,
                                     (typename Pol::TS*)x.a2, x.sc, blockIdx.x - x.blk0, g.i0);
}

// one thread per box
static __global__ void k_dtfin_grp(const __grid_constant__ GroupArgs g) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= g.nbox) return;
  const KParams& p = g.box[b].p;
  dtfin_body(g.box[b].sc, p.cfl, p.dx, p.dy, p.dz);
}
static __global__ void k_loopfin_grp(const __grid_constant__ GroupArgs g) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < g.nbox) loopfin_body(g.box[b].sc);
}

}  // namespace gch
