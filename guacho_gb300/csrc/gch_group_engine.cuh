// gch_group_engine.cuh -- launch orchestration of one timestep of many boxes
// with grouped kernels (gch_group.cuh): one launch per kernel of the step
// for up to kGroupMax boxes, whatever their sizes.  Included by exactly one
// translation unit per FP32 policy, which defines that policy's GroupOps.
#pragma once

#include <algorithm>
#include <climits>
#include <cstring>
#include <memory>

#include "gch_engine.cuh"
#include "gch_group.cuh"

namespace gch {

template <class Pol>
struct GroupEngine {
  using TU = typename Pol::TU;
  using TS = typename Pol::TS;
  using TC = typename Ops<Pol>::TC;
  static constexpr int kzc = Engine<Pol>::kzc;

  // Fill the argument block of each chunk of <= kGroupMax boxes and launch
  // it: setup(GroupBox&, box) fills the kernel-specific fields and returns
  // the box's block count; launch(GroupArgs&, total blocks) issues the kernel.
  template <class Setup, class Launch>
  static int chunks(gch_domain* const* boxes, int n, Setup setup, Launch launch) {
    std::unique_ptr<GroupArgs> g(new GroupArgs);
    for (int c0 = 0; c0 < n; c0 += kGroupMax) {
      const int m = std::min(kGroupMax, n - c0);
      std::memset(g.get(), 0, sizeof(GroupArgs));
      g->nbox = m;
      long long blocks = 0;
      for (int i = 0; i < m; ++i) {
        GroupBox& x = g->box[i];
        gch_domain* d = boxes[c0 + i];
        x.p = d->kp;
        x.sc = d->sc;
        x.blk0 = (int)blocks;
        blocks += setup(x, d);
        if (blocks > INT_MAX) return GCH_ERR_TOO_LARGE;
      }
      launch(*g, (unsigned)blocks);
    }
    return cuda_status(cudaGetLastError());
  }

  // ---- stage kernels ---------------------------------------------------------
  // `blocks` work items: with bps = 0 one block per item, otherwise a
  // persistent grid of min(blocks, bps x SMs) blocks pulling them from
  // `queue`, which is cleared on the stream first.
  static int sm_count() {
    static int n = [] {
      int dev = 0, v = 0;
      if (cudaGetDevice(&dev) != cudaSuccess ||
          cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        v = 152;
      return v > 0 ? v : 152;
    }();
    return n;
  }
  template <int SOLVER, int NEQ, int STAGE, int LIM, bool PRIM_IN>
  static void flux_lim(GroupArgs& g, unsigned blocks, int bps, int* queue, cudaStream_t s) {
    constexpr size_t smem = FluxLayout<Pol, NEQ, STAGE, PRIM_IN>::kBytes;
    static bool attr = false;  // once per instantiation
    if (!attr) {
      cudaFuncSetAttribute(k_flux_grp<Pol, SOLVER, NEQ, STAGE, LIM, PRIM_IN>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      cudaFuncSetAttribute(k_flux_pst<Pol, SOLVER, NEQ, STAGE, LIM, PRIM_IN>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      attr = true;
    }
    if (!blocks) return;
    if (bps <= 0) {
      k_flux_grp<Pol, SOLVER, NEQ, STAGE, LIM, PRIM_IN><<<blocks, dim3(TX, TY), smem, s>>>(g);
      return;
    }
    const unsigned grid = std::min<unsigned>(blocks, (unsigned)(bps * sm_count()));
    cudaMemsetAsync(queue, 0, sizeof(int), s);
    k_flux_pst<Pol, SOLVER, NEQ, STAGE, LIM, PRIM_IN><<<grid, dim3(TX, TY), smem, s>>>(
        g, queue, (int)blocks);
  }
  // stage 1 reads u, or primit with table cooling (prim_in); stage 2 reads
  // up and specialises minmod and van Leer
  template <int SOLVER, int NEQ, int STAGE>
  static void flux_solver(GroupArgs& g, unsigned blocks, int bps, int* queue, cudaStream_t s,
                          int lim, bool prim_in) {
    if constexpr (STAGE == 1) {
      if (prim_in) flux_lim<SOLVER, NEQ, STAGE, kLimRuntime, true>(g, blocks, bps, queue, s);
      else flux_lim<SOLVER, NEQ, STAGE, kLimRuntime, false>(g, blocks, bps, queue, s);
    } else if (lim == GCH_LIMITER_MINMOD) {
      flux_lim<SOLVER, NEQ, STAGE, GCH_LIMITER_MINMOD, false>(g, blocks, bps, queue, s);
    } else if (lim == GCH_LIMITER_VAN_LEER) {
      flux_lim<SOLVER, NEQ, STAGE, GCH_LIMITER_VAN_LEER, false>(g, blocks, bps, queue, s);
    } else {
      flux_lim<SOLVER, NEQ, STAGE, kLimRuntime, false>(g, blocks, bps, queue, s);
    }
  }
  template <int STAGE>
  static int flux(gch_domain* const* boxes, int n, int kz, int bps, int* queue, cudaStream_t s) {
    const KParams& p0 = boxes[0]->kp;
    const int sv = p0.solver, neq = p0.neq, lim = p0.limiter;
    // the first stage reads stored primitives with table cooling and on the
    // FP32 + FP64-u path (stored by the CFL pass of the same step)
    const bool prim_in = boxes[0]->prim_in || boxes[0]->prim_pre;
    auto setup = [&](GroupBox& x, gch_domain* d) -> long long {
      const KParams& p = d->kp;
      // stage source: u (or primit) for the first half step, up for the second
      x.a0 = STAGE == 1 ? (prim_in ? d->primit : d->u) : d->up;
      x.a1 = d->u;
      x.a2 = STAGE == 1 ? d->up : d->u;
      x.a3 = d->E;
      x.a4 = d->s678;
      x.kz = std::max(1, std::min(kz, p.nz));
      x.gx = (p.nx + TX - 1) / TX;
      x.gy = (p.ny + TY - 1) / TY;
      return (long long)x.gx * x.gy * ((p.nz + x.kz - 1) / x.kz);
    };
    auto go = [&](auto launch) { return chunks(boxes, n, setup, launch); };
#define GCH_GRP_FLUX(SV, NQ)                                                               \
    if (sv == SV && neq == NQ)                                                             \
      return go([&](GroupArgs& g, unsigned b) {                                            \
        flux_solver<SV, NQ, STAGE>(g, b, bps, queue, s, lim, prim_in);                     \
      });
    GCH_GRP_FLUX(GCH_SOLVER_HLLD, 8)
    GCH_GRP_FLUX(GCH_SOLVER_HLLC, 5)
    GCH_GRP_FLUX(GCH_SOLVER_HLLC, 8)
    GCH_GRP_FLUX(GCH_SOLVER_HLLE, 8)
    GCH_GRP_FLUX(GCH_SOLVER_HLL, 5)
    GCH_GRP_FLUX(GCH_SOLVER_HLL, 8)
#undef GCH_GRP_FLUX
    return GCH_ERR_PARAM;
  }

  // column-marching cell kernels: tile 32 x 8, kzc planes per block
  static long long column_setup(GroupBox& x, const KParams& p) {
    x.kz = kzc;
    x.gx = (p.nx + 31) / 32;
    x.gy = (p.ny + 7) / 8;
    return (long long)x.gx * x.gy * ((p.nz + kzc - 1) / kzc);
  }

  template <int STAGE>
  static int ct(gch_domain* const* boxes, int n, cudaStream_t s) {
    return chunks(
        boxes, n,
        [&](GroupBox& x, gch_domain* d) {
          x.a1 = d->u;
          x.a2 = STAGE == 1 ? d->up : d->u;
          x.a3 = d->E;
          x.a4 = d->s678;
          return column_setup(x, d->kp);
        },
        [&](GroupArgs& g, unsigned b) {
          if (b) k_ct_grp<Pol, STAGE><<<b, dim3(32, 8), 0, s>>>(g);
        });
  }

  // the user spheres of the boxes that have them, after a ghost fill
  // (Engine<Pol>::ghost): blocks per sphere as the one-box launch's 4 x 152
  // split over the boxes, at least 8
  template <class T>
  static int user_bc(gch_domain* const* boxes, int n, bool on_up, cudaStream_t s) {
    bool any = false;
    for (int i = 0; i < n; ++i) any = any || (boxes[i]->kp.bc_user && boxes[i]->kp.nsph > 0);
    if (!any) return GCH_OK;
    const int per = std::max(8, 4 * 152 / n);
    return chunks(
        boxes, n,
        [&](GroupBox& x, gch_domain* d) -> long long {
          const KParams& p = d->kp;
          x.a2 = on_up ? d->up : d->u;
          return (p.bc_user && p.nsph > 0) ? (long long)p.nsph * per : 0;
        },
        [&](GroupArgs& g, unsigned b) {
          g.i0 = per;
          if (b) k_user_bc_grp<T><<<b, 256, 0, s>>>(g);
        });
  }

  template <class T>
  static int ghost(gch_domain* const* boxes, int n, bool on_up, int layers, cudaStream_t s) {
    return ghost_fill<T>(boxes, n, on_up, layers, s) | user_bc<T>(boxes, n, on_up, s);
  }

  template <class T>
  static int ghost_fill(gch_domain* const* boxes, int n, bool on_up, int layers, cudaStream_t s) {
    bool all = true;
    for (int i = 0; i < n; ++i) all = all && ghost_all_ok(boxes[i]->kp, layers);
    if (all) {  // the whole shell of every box in one launch
      return chunks(
          boxes, n,
          [&](GroupBox& x, gch_domain* d) -> long long {
            x.a2 = on_up ? d->up : d->u;
            return (ghost_all_count(d->kp, layers) + 255) / 256;
          },
          [&](GroupArgs& g, unsigned b) {
            g.i1 = layers;
            if (b) k_ghost_all_grp<T><<<b, 256, 0, s>>>(g);
          });
    }
    int st = GCH_OK;  // a box with a side shorter than the fill: axis by axis
    for (int axis = 0; axis < 3; ++axis) {
      st |= chunks(
          boxes, n,
          [&](GroupBox& x, gch_domain* d) -> long long {
            const KParams& p = d->kp;
            x.a2 = on_up ? d->up : d->u;
            const int N0 = axis == 0 ? p.NY : p.NX;
            const int N1 = axis == 2 ? p.NY : p.NZ;
            x.gx = (N0 + 127) / 128;
            x.gy = N1;
            return (long long)x.gx * N1 * 2 * layers;
          },
          [&](GroupArgs& g, unsigned b) {
            g.i0 = axis;
            g.i1 = layers;
            if (b) k_ghost_grp<T><<<b, 128, 0, s>>>(g);
          });
    }
    return st;
  }

  // get_timestep's CFL pass: from u, or from primit with table cooling (the
  // reference takes dt from the stored, cooled primitives).  On the FP32 +
  // FP64-u path it stores the primitives it recovers from u for the first
  // stage, and the ghost shell's follow (prim_shell).
  static int cfl(gch_domain* const* boxes, int n, int, cudaStream_t s) {
    const int neq = boxes[0]->kp.neq;
    const bool prim_in = boxes[0]->prim_in;
    int st = chunks(
        boxes, n,
        [&](GroupBox& x, gch_domain* d) {
          x.a1 = prim_in ? d->primit : d->u;
          x.a2 = d->prim_pre ? d->primit : nullptr;
          return column_setup(x, d->kp);
        },
        [&](GroupArgs& g, unsigned b) {
          if (!b) return;
          if (neq == 8 && prim_in) k_cfl_grp<Pol, 8, true><<<b, dim3(32, 8), 0, s>>>(g);
          else if (neq == 8) k_cfl_grp<Pol, 8, false><<<b, dim3(32, 8), 0, s>>>(g);
          else if (prim_in) k_cfl_grp<Pol, 5, true><<<b, dim3(32, 8), 0, s>>>(g);
          else k_cfl_grp<Pol, 5, false><<<b, dim3(32, 8), 0, s>>>(g);
        });
    if (boxes[0]->prim_pre) st |= prim_shell(boxes, n, true, s);
    return st;
  }

  // table cooling of every box (updates u(5) and primit), one block per
  // 32 x 8 tile of every interior plane
  static int cool(gch_domain* const* boxes, int n, cudaStream_t s) {
    const int neq = boxes[0]->kp.neq;
    return chunks(
        boxes, n,
        [&](GroupBox& x, gch_domain* d) -> long long {
          const KParams& p = d->kp;
          x.a1 = d->u;
          x.a2 = d->primit;
          x.gx = (p.nx + 31) / 32;
          x.gy = (p.ny + 7) / 8;
          return (long long)x.gx * x.gy * p.nz;
        },
        [&](GroupArgs& g, unsigned b) {
          if (!b) return;
          if (neq == 8) k_cool_grp<Pol, 8><<<b, dim3(32, 8), 0, s>>>(g);
          else k_cool_grp<Pol, 5><<<b, dim3(32, 8), 0, s>>>(g);
        });
  }

  // primitives of every box's ghost shell after boundaryI (table cooling)
  static int calcprim_shell(gch_domain* const* boxes, int n, cudaStream_t s) {
    return prim_shell(boxes, n, false, s);
  }
  // own: the shell of the primitives the CFL pass stored (FP32 + FP64 u)
  static int prim_shell(gch_domain* const* boxes, int n, bool own, cudaStream_t s) {
    const int neq = boxes[0]->kp.neq;
    const int per = std::max(4, 152 * 16 / n);
    return chunks(
        boxes, n,
        [&](GroupBox& x, gch_domain* d) -> long long {
          x.a1 = d->u;
          x.a2 = d->primit;
          return per;
        },
        [&](GroupArgs& g, unsigned b) {
          if (!b) return;
          g.i0 = per;
          if (own && neq == 8) k_calcprim_shell_grp<Pol, 8, true><<<b, 256, 0, s>>>(g);
          else if (own) k_calcprim_shell_grp<Pol, 5, true><<<b, 256, 0, s>>>(g);
          else if (neq == 8) k_calcprim_shell_grp<Pol, 8><<<b, 256, 0, s>>>(g);
          else k_calcprim_shell_grp<Pol, 5><<<b, 256, 0, s>>>(g);
        });
  }

  static int scalar_tail(gch_domain* const* boxes, int n, bool loop_tail, cudaStream_t s) {
    return chunks(
        boxes, n, [](GroupBox&, gch_domain*) { return 0LL; },
        [&](GroupArgs& g, unsigned) {
          if (loop_tail) k_loopfin_grp<<<1, kGroupMax, 0, s>>>(g);
          else k_dtfin_grp<<<1, kGroupMax, 0, s>>>(g);
        });
  }

  // get_timestep + tstep + the loop tail of every box (Engine<Pol>::get_dt,
  // tstep and loopfin without resistivity, COOL_H or conduction): the
  // stage-1 fluxes from primit and the cooling with the ghost-shell
  // primitives after boundaryI when the boxes cool by table, the user
  // spheres of each box after each ghost fill
  static int step(gch_domain* const* boxes, int n, int kz, int bps, int* queue, cudaStream_t s) {
    const KParams& p0 = boxes[0]->kp;
    const bool ctp = p0.neq >= 8 && p0.flux_cd;
    const bool prim_in = boxes[0]->prim_in;
    int st = GCH_OK;
    st |= cfl(boxes, n, kz, s);
    st |= scalar_tail(boxes, n, false, s);
    st |= flux<1>(boxes, n, kz, bps, queue, s);
    if (ctp) st |= ct<1>(boxes, n, s);
    st |= ghost<TS>(boxes, n, true, 2, s);
    st |= flux<2>(boxes, n, kz, bps, queue, s);
    if (ctp) st |= ct<2>(boxes, n, s);
    if (prim_in) st |= cool(boxes, n, s);
    st |= ghost<TU>(boxes, n, false, 1, s);
    if (prim_in) st |= calcprim_shell(boxes, n, s);
    st |= scalar_tail(boxes, n, true, s);
    return st;
  }

  static int probe(gch_domain* const* boxes, int n, int kz, int bps, int* queue,
                   cudaStream_t s) {
    return flux<1>(boxes, n, kz, bps, queue, s);
  }

  static int prep(gch_domain* const* boxes, int n, cudaStream_t s) {
    return boxes[0]->prim_pre ? cfl(boxes, n, 0, s) : GCH_OK;
  }

  static constexpr GroupOps ops() { return GroupOps{&step, &probe, &prep}; }
};

}  // namespace gch
