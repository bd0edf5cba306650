// gch_engine.cuh -- launch orchestration of one timestep for a precision
// policy.  Included by exactly one translation unit per policy, which also
// defines that policy's EngineOps table.
#pragma once

#include "gch_domain.h"
#include "gch_kernels.cuh"

namespace gch {

inline int cuda_status(cudaError_t e) { return e == cudaSuccess ? GCH_OK : GCH_ERR_CUDA; }

template <class Pol>
struct Engine {
  using TU = typename Pol::TU;
  using TS = typename Pol::TS;

  static dim3 cell_grid(const KParams& p) {
    return dim3((p.nx + 31) / 32, (p.ny + 7) / 8, p.nz);
  }
  // cell kernels that march over kzc planes per block (fewer blocks: one
  // reduction atomic per block)
  static constexpr int kzc = 8;
  static dim3 column_grid(const KParams& p) {
    return dim3((p.nx + 31) / 32, (p.ny + 7) / 8, (p.nz + kzc - 1) / kzc);
  }

  // ---- stage kernels, dispatched on solver and neq ----------------------
  template <int SOLVER, int NEQ, int STAGE, bool PRIM_IN, int LIM>
  static void flux_launch_lim(gch_domain* d, const void* src, void* dst) {
    const KParams& p = d->kp;
    dim3 grid((p.nx + TX - 1) / TX, (p.ny + TY - 1) / TY,
              d->zcn > 0 ? d->zcn : (p.nz + d->kz - 1) / d->kz);
    dim3 block(TX, TY);
    using TIn = typename Src<Pol, NEQ, STAGE, PRIM_IN>::TIn;
    using TD = typename std::conditional<STAGE == 1, TS, TU>::type;
    using TC = typename Ops<Pol>::TC;
    constexpr size_t smem = FluxLayout<Pol, NEQ, STAGE, PRIM_IN>::kBytes;
    // (the FP32 policies only: the FP64 step keeps the serial order)
    if constexpr (STAGE == 1 && !PRIM_IN && (NEQ == 5 || NEQ == 8) &&
                  !std::is_same<Pol, PolFP64>::value) {
      if (d->defer) {  // the flux differences into dif, no update
        static bool attr_d = false;
        if (!attr_d) {
          cudaFuncSetAttribute(k_flux<Pol, SOLVER, NEQ, STAGE, PRIM_IN, LIM, true>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
          attr_d = true;
        }
        k_flux<Pol, SOLVER, NEQ, STAGE, PRIM_IN, LIM, true><<<grid, block, smem, d->stream>>>(
            p, (const TIn*)src, (const TU*)d->u, (TD*)d->dif, (TS*)d->E, (TS*)d->s678, d->sc,
            d->kz, d->zc0);
        return;
      }
    }
    static bool attr = false;  // once per instantiation
    if (!attr) {
      cudaFuncSetAttribute(k_flux<Pol, SOLVER, NEQ, STAGE, PRIM_IN, LIM>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      attr = true;
    }
    k_flux<Pol, SOLVER, NEQ, STAGE, PRIM_IN, LIM><<<grid, block, smem, d->stream>>>(
        p, (const TIn*)src, (const TU*)d->u, (TD*)dst, (TS*)d->E, (TS*)d->s678, d->sc, d->kz,
        d->zc0);
  }

  // stage 1 has no limiter; stage 2 specialises minmod and van Leer
  template <int SOLVER, int NEQ, int STAGE, bool PRIM_IN>
  static void flux_launch(gch_domain* d, const void* src, void* dst) {
    if constexpr (STAGE == 1)
      flux_launch_lim<SOLVER, NEQ, STAGE, PRIM_IN, kLimRuntime>(d, src, dst);
    else if (d->kp.limiter == GCH_LIMITER_MINMOD)
      flux_launch_lim<SOLVER, NEQ, STAGE, PRIM_IN, GCH_LIMITER_MINMOD>(d, src, dst);
    else if (d->kp.limiter == GCH_LIMITER_VAN_LEER)
      flux_launch_lim<SOLVER, NEQ, STAGE, PRIM_IN, GCH_LIMITER_VAN_LEER>(d, src, dst);
    else
      flux_launch_lim<SOLVER, NEQ, STAGE, PRIM_IN, kLimRuntime>(d, src, dst);
  }

  // the stage kernels of one equation count, dispatched on the solver
  // (the passive-scalar counts are instantiated in their own translation
  // units, see GCH_PASSIVE_FLUX below)
  template <int NEQ, int STAGE, bool PRIM_IN>
  static int flux_n(gch_domain* d, const void* src, void* dst);  // defined below

  template <int STAGE, bool PRIM_IN>
  static int flux(gch_domain* d, const void* src, void* dst) {
    switch (d->kp.neq) {
      case 5: return flux_n<5, STAGE, PRIM_IN>(d, src, dst);
      case 7: return flux_n<7, STAGE, PRIM_IN>(d, src, dst);
      case 8: return flux_n<8, STAGE, PRIM_IN>(d, src, dst);
      case 10: return flux_n<10, STAGE, PRIM_IN>(d, src, dst);
    }
    return GCH_ERR_PARAM;
  }

  template <class T>
  static void ghost(gch_domain* d, T* a, int layers) {
    const KParams& p = d->kp;
    if (ghost_all_ok(p, layers)) {  // the whole shell in one launch
      const long long n = ghost_all_count(p, layers);
      const unsigned g = (unsigned)std::min<long long>((n + 255) / 256, 152 * 16);
      k_ghost_all<T><<<g, 256, 0, d->stream>>>(p, a, p.neq, layers, d->sc);
      ++d->launches;
      gch_mark(d, "k_ghost");
    } else {  // a side shorter than the fill: the axes one after the other
      for (int axis = 0; axis < 3; ++axis) {
        int N0, N1;
        if (axis == 0) { N0 = p.NY; N1 = p.NZ; }
        else if (axis == 1) { N0 = p.NX; N1 = p.NZ; }
        else { N0 = p.NX; N1 = p.NY; }
        dim3 grid((N0 + 127) / 128, N1, 2 * layers);
        k_ghost<T><<<grid, 128, 0, d->stream>>>(p, a, p.neq, axis, layers, d->sc);
        ++d->launches;
        gch_mark(d, "k_ghost");
      }
    }
    if (p.bc_user && p.nsph > 0) {
      // grid-stride over each sphere's bounding box; 4 blocks per SM per sphere
      k_user_bc<T><<<dim3(4 * 152, p.nsph), 256, 0, d->stream>>>(p, a, p.neq, d->sc);
      ++d->launches;
      gch_mark(d, "k_user_bc");
    }
  }

  // grid-stride launches over the one-cell ghost shell
  static unsigned shell_grid(const KParams& p) {
    const long long ns = (long long)(p.nx + 2) * (p.ny + 2) * (p.nz + 2) -
                         (long long)p.nx * p.ny * p.nz;
    return (unsigned)std::min<long long>((ns + 255) / 256, 152 * 16);
  }

  // ---- get_timestep --------------------------------------------------------
  // the CFL min over the interior (k_cfl), then dt from it (k_dtfin)
  static int get_dt(gch_domain* d) {
    const KParams& p = d->kp;
    if constexpr (std::is_same<Pol, PolFP64>::value)
      if (p.solver == GCH_SOLVER_HLLE_SPLIT_ALL) return split_get_dt(d);
    dim3 cgrid = column_grid(p), block(32, 8);
    if (d->prim_in) {
      with_neq(p.neq, [&](auto N) {
        k_cfl<Pol, decltype(N)::value, true><<<cgrid, block, 0, d->stream>>>(p, (const TS*)d->primit, d->sc, kzc);
      });
    } else {
      with_neq(p.neq, [&](auto N) {
        k_cfl<Pol, decltype(N)::value, false><<<cgrid, block, 0, d->stream>>>(
            p, (const TU*)d->u, d->sc, kzc, d->prim_pre ? (TS*)d->primit : nullptr);
      });
    }
    gch_mark(d, "k_cfl");
    if (d->prim_pre) {  // the ghost shell's primitives too; then they are fresh
      with_neq(p.neq, [&](auto N) {
        k_prim_shell_own<Pol, decltype(N)::value><<<shell_grid(p), 256, 0, d->stream>>>(
            p, (const TU*)d->u, (TS*)d->primit, d->sc);
      });
      gch_mark(d, "k_prim_shell");
    }
    k_dtfin<<<1, 1, 0, d->stream>>>(d->sc, p.cfl, p.dx, p.dy, p.dz);
    gch_mark(d, "k_dtfin");
    return cuda_status(cudaGetLastError());
  }

  // ---- tstep (src/hydro_solver.f90:134-229) ---------------------------------
  static int tstep(gch_domain* d) {
    const KParams& p = d->kp;
    if constexpr (std::is_same<Pol, PolFP64>::value)
      if (p.solver == GCH_SOLVER_HLLE_SPLIT_ALL) return split_tstep(d);
    d->launches = 0;
    return stage1(d) | stage2(d);
  }

  // the first half step and boundaryII on up
  static int stage1(gch_domain* d) {
    const KParams& p = d->kp;
    int st = GCH_OK;
    const bool ct = p.neq >= 8 && p.flux_cd;
    const dim3 cblock(32, 8);
    // 1st half step: first-order fluxes, up = u - dtm*divF (from the stored
    // primitives with table cooling, or those get_timestep stored for this u)
    if (d->prim_pre) {
      with_neq(p.neq, [&](auto N) {
        k_prim_refresh<Pol, decltype(N)::value><<<152 * 4, 256, 0, d->stream>>>(
            p, (const TU*)d->u, (TS*)d->primit, d->sc);
      });
      ++d->launches;
      gch_mark(d, "k_prim_refresh");
    }
    if (d->prim_in || d->prim_pre) st |= flux<1, true>(d, d->primit, d->up);
    else st |= flux<1, false>(d, d->u, d->up);
    ++d->launches;
    gch_mark(d, "k_flux_stage1");
    if (ct) {
      k_ct<Pol, 1><<<column_grid(p), cblock, 0, d->stream>>>(
          p, (const TU*)d->u, (TS*)d->up, (const TS*)d->E, (const TS*)d->s678, d->sc, kzc);
      ++d->launches;
      gch_mark(d, "k_ct_stage1");
    }
    // boundaryII on up (+ user spheres)
    ghost<TS>(d, (TS*)d->up, 2);
    return st | cuda_status(cudaGetLastError());
  }

  // the second half step, the sources after it and boundaryI on u
  static int stage2(gch_domain* d) {
    const KParams& p = d->kp;
    int st = GCH_OK;
    const bool ct = p.neq >= 8 && p.flux_cd;
    const dim3 cgrid = cell_grid(p), cblock(32, 8);
    // 2nd half step: limited reconstruction, u(+w) = u - dt*divF
    void* dst2 = p.eta != 0.0 ? d->w : d->u;
    st |= flux<2, false>(d, d->up, dst2);
    ++d->launches;
    gch_mark(d, "k_flux_stage2");
    if (ct) {
      k_ct<Pol, 2><<<column_grid(p), cblock, 0, d->stream>>>(
          p, (const TU*)d->u, (TU*)dst2, (const TS*)d->E, (const TS*)d->s678, d->sc, kzc);
      ++d->launches;
      gch_mark(d, "k_ct_stage2");
    }
    if (p.eta != 0.0) {
      with_neq(p.neq, [&](auto N) {
        k_visc<Pol, decltype(N)::value><<<cgrid, cblock, 0, d->stream>>>(p, (TU*)d->u, (const TU*)d->w, (const TS*)d->up, d->sc);
      });
      ++d->launches;
      gch_mark(d, "k_visc");
    }
    if (p.cooling == GCH_COOL_H) {  // ionisation of H and its cooling (u(5), n_HI)
      with_neq(p.neq, [&](auto N) {
        constexpr int n = decltype(N)::value;
        if constexpr (n > kNeqDyn<n>)
          k_cool_h<Pol, n><<<cgrid, cblock, 0, d->stream>>>(p, (TU*)d->u, d->sc);
      });
      ++d->launches;
      gch_mark(d, "k_cool_h");
    }
    if (d->prim_in) {  // tabulated cooling (updates primit and u(5))
      with_neq(p.neq, [&](auto N) {
        k_cool<Pol, decltype(N)::value><<<cgrid, cblock, 0, d->stream>>>(p, (TU*)d->u, (TS*)d->primit, d->sc);
      });
      ++d->launches;
      gch_mark(d, "k_cool");
    }
    // boundaryI on u (+ user spheres), then primitives of the ghost shell
    ghost<TU>(d, (TU*)d->u, 1);
    if (d->prim_pre) clear_prim_fresh(d);  // u has changed
    if (d->prim_in) {  // primitives of the ghost shell (interior ones come from k_cool)
      const long long ns = (long long)(p.nx + 2) * (p.ny + 2) * (p.nz + 2) -
                           (long long)p.nx * p.ny * p.nz;
      const unsigned g = (unsigned)std::min<long long>((ns + 255) / 256, 152 * 16);
      with_neq(p.neq, [&](auto N) {
        k_calcprim_shell<Pol, decltype(N)::value><<<g, 256, 0, d->stream>>>(
            p, (const TU*)d->u, (TS*)d->primit, d->sc);
      });
      ++d->launches;
      gch_mark(d, "k_calcprim");
    }
    st |= cuda_status(cudaGetLastError());
    return st;
  }

  // ---- gch_step_host with the copies overlapped (pageable host arrays) ------
  // Upload: the host array goes up in slabs of z chunks (copy-engine copies
  // into the staging buffer on the copy stream); each slab is transposed into
  // u as it lands, its CFL candidates are reduced, and the first stage's
  // fluxes of the slab below it (which needs one plane of this one) run
  // deferred: they do not depend on dt, so they write their flux differences
  // and k_s1_apply finishes the update once k_dtfin has dt.  Download: the
  // second stage, its CT and the x/y ghost ring run slab by slab; each
  // finished slab is transposed into the staging buffer and copied to the
  // host while the next slabs compute.  The last chunk's second-stage
  // fluxes go first: under periodic walls its E is the z neighbour of the
  // first slab's CT.  Each slab's CT follows the fluxes of the slab after it
  // (its E at the slab's top plane).  The z ghost planes follow the
  // whole-shell fill at the end (it writes the rings again with the same
  // values).  The kernels' per-plane results do not depend on where a chunk
  // or slab begins, and the deferred update rounds as the fused one, so the
  // host array ends bit for bit as with upload, get_timestep, tstep and
  // download in turn.
  static constexpr int kUpEv = 0, kDownEv = 10;  // event slots of the two phases
  // Slabs of z chunks covering chunks [c0, c0 + n): two single-chunk slabs at
  // the end where the pipeline waits on them (`small_first`: the start), the
  // rest in at most 8 slabs of equal depth; at most 10 slabs.  out[i] =
  // {first chunk, chunks}; returns the count.
  static int slab_plan(int c0, int n, bool small_first, int (*out)[2]) {
    int ns = 0;
    if (n <= 4) {
      for (int i = 0; i < n; ++i) out[ns][0] = c0 + i, out[ns++][1] = 1;
      return ns;
    }
    const int r = n - 2, m = (r + 7) / 8;
    int c = c0;
    if (small_first)
      for (int i = 0; i < 2; ++i) out[ns][0] = c++, out[ns++][1] = 1;
    for (int left = r; left > 0; left -= m) {
      out[ns][0] = c;
      out[ns++][1] = std::min(m, left);
      c += std::min(m, left);
    }
    if (!small_first)
      for (int i = 0; i < 2; ++i) out[ns][0] = c++, out[ns++][1] = 1;
    return ns;
  }
  static int step_host(gch_domain* d, double* host) {
    // the FP64 step keeps the serial order (pipe_ok); no deferred stage there
    if constexpr (std::is_same<Pol, PolFP64>::value) return GCH_ERR_PARAM;
    const KParams& p = d->kp;
    int st = GCH_OK;
    d->launches = 0;
    if (!d->cstream) {
      st |= cuda_status(cudaStreamCreateWithFlags(&d->cstream, cudaStreamNonBlocking));
      for (int i = 0; i < gch_domain::kPipeEv && st == GCH_OK; ++i)
        st |= cuda_status(cudaEventCreateWithFlags(&d->pipe_ev[i], cudaEventDisableTiming));
      if (st) return st;
    }
    if (!d->dif) {
      st |= cuda_status(cudaMalloc(&d->dif, (size_t)3 * p.neq * p.fs * sizeof(TS)));
      if (st) return st;
    }
    if (d->prim_pre) clear_prim_fresh(d);  // the first stage recovers from u here
    const int kz = d->kz, C = (p.nz + kz - 1) / kz;
    const long long plane = (long long)p.NX * p.NY;
    const size_t rowb = (size_t)p.neq * sizeof(double);
    const dim3 cblock(32, 8);
    int ne = kUpEv;
    // array planes [az0, az1) from the host into u
    auto up_slab = [&](int az0, int az1) {
      const long long c0 = az0 * plane, c1 = az1 * plane;
      st |= cuda_status(cudaMemcpyAsync(d->stage + c0 * p.neq, host + c0 * p.neq,
                                        (size_t)(c1 - c0) * rowb, cudaMemcpyHostToDevice,
                                        d->cstream));
      st |= cuda_status(cudaEventRecord(d->pipe_ev[ne], d->cstream));
      st |= cuda_status(cudaStreamWaitEvent(d->stream, d->pipe_ev[ne++], 0));
      k_aos_to_soa<TU><<<kLayoutGrid, kLayoutCells, 0, d->stream>>>(p, d->stage, (TU*)d->u,
                                                                     p.neq, c0, c1);
      ++d->launches;
      gch_mark(d, "k_aos_to_soa");
    };
    auto cfl_slab = [&](int c0, int nc) {
      const dim3 g((p.nx + 31) / 32, (p.ny + 7) / 8, nc);
      with_neq(p.neq, [&](auto N) {
        k_cfl<Pol, decltype(N)::value, false><<<g, cblock, 0, d->stream>>>(
            p, (const TU*)d->u, d->sc, kz, nullptr, c0);
      });
      ++d->launches;
      gch_mark(d, "k_cfl");
    };
    auto flux1_deferred = [&](int c0, int nc) {
      d->zc0 = c0;
      d->zcn = nc;
      d->defer = true;
      st |= flux<1, false>(d, d->u, d->up);
      d->defer = false;
      d->zc0 = d->zcn = 0;
      ++d->launches;
      gch_mark(d, "k_flux_stage1");
    };
    // the last slabs are single chunks: only their fluxes remain once the
    // last copy has landed
    int plan[10][2];
    const int ns = slab_plan(0, C, false, plan);
    for (int i = 0; i < ns; ++i) {
      const int c = plan[i][0], nc = plan[i][1];
      const int az0 = c == 0 ? 0 : NG + c * kz;
      const int az1 = c + nc == C ? p.NZ : NG + std::min(p.nz, (c + nc) * kz);
      up_slab(az0, az1);
      cfl_slab(c, nc);
      if (i > 0) flux1_deferred(plan[i - 1][0], plan[i - 1][1]);
    }
    flux1_deferred(plan[ns - 1][0], plan[ns - 1][1]);
    k_dtfin<<<1, 1, 0, d->stream>>>(d->sc, p.cfl, p.dx, p.dy, p.dz);
    ++d->launches;
    gch_mark(d, "k_dtfin");
    // the first stage's update, its CT and boundaryII on up
    with_neq(p.neq, [&](auto N) {
      constexpr int n = decltype(N)::value;
      if constexpr ((n == 5 || n == 8) && !std::is_same<Pol, PolFP64>::value)
        k_s1_apply<Pol, n><<<cell_grid(p), cblock, 0, d->stream>>>(p, (const TU*)d->u, (TS*)d->up,
                                                                    (const TS*)d->dif, d->sc);
    });
    ++d->launches;
    gch_mark(d, "k_s1_apply");
    if (p.neq >= 8 && p.flux_cd) {
      k_ct<Pol, 1><<<column_grid(p), cblock, 0, d->stream>>>(
          p, (const TU*)d->u, (TS*)d->up, (const TS*)d->E, (const TS*)d->s678, d->sc, kzc);
      ++d->launches;
      gch_mark(d, "k_ct_stage1");
    }
    ghost<TS>(d, (TS*)d->up, 2);
    return st | stage2_dl(d, host);
  }

  static int stage2_dl(gch_domain* d, double* host) {
    const KParams& p = d->kp;
    int st = GCH_OK;
    const bool ct = p.neq >= 8 && p.flux_cd;
    const int kz = d->kz, C = (p.nz + kz - 1) / kz;
    const long long plane = (long long)p.NX * p.NY;
    long long cut[gch_domain::kPipeEv][2];
    int np = 0;
    auto flux2 = [&](int c0, int nc) {
      d->zc0 = c0;
      d->zcn = nc;
      st |= flux<2, false>(d, d->up, d->u);
      d->zc0 = d->zcn = 0;
      ++d->launches;
      gch_mark(d, "k_flux_stage2");
    };
    // planes [az0, az1) of u (array coordinates) into the staging buffer, for
    // a copy queued below
    auto layout_out = [&](int az0, int az1) {
      cut[np][0] = az0 * plane;
      cut[np][1] = az1 * plane;
      k_soa_to_aos<TU><<<kLayoutGrid, kLayoutCells, 0, d->stream>>>(
          p, (const TU*)d->u, d->stage, p.neq, cut[np][0], cut[np][1]);
      ++d->launches;
      gch_mark(d, "k_soa_to_aos");
      cudaEventRecord(d->pipe_ev[kDownEv + np++], d->stream);
    };
    auto finish = [&](int c0, int nc) {
      const int z0 = c0 * kz, z1 = std::min(p.nz, (c0 + nc) * kz);
      if (ct) {
        const dim3 g((p.nx + 31) / 32, (p.ny + 7) / 8, nc);
        k_ct<Pol, 2><<<g, dim3(32, 8), 0, d->stream>>>(p, (const TU*)d->u, (TU*)d->u,
                                                       (const TS*)d->E, (const TS*)d->s678,
                                                       d->sc, kz, c0);
        ++d->launches;
        gch_mark(d, "k_ct_stage2");
      }
      const long long n = (2LL * p.NX + 2LL * (p.NY - 2)) * (z1 - z0);
      const unsigned g = (unsigned)std::min<long long>((n + 255) / 256, 152 * 16);
      k_ghost_ring<TU><<<g, 256, 0, d->stream>>>(p, (TU*)d->u, p.neq, 1, NG + z0, NG + z1, d->sc);
      ++d->launches;
      gch_mark(d, "k_ghost_ring");
      layout_out(NG + z0, NG + z1);
    };
    // the first slabs are single chunks: the first copy starts early
    int plan[10][2];
    const int ns = slab_plan(0, C - 1, true, plan);
    flux2(C - 1, 1);
    for (int i = 0; i < ns; ++i) {
      flux2(plan[i][0], plan[i][1]);
      if (i > 0) finish(plan[i - 1][0], plan[i - 1][1]);
    }
    finish(plan[ns - 1][0], plan[ns - 1][1]);
    finish(C - 1, 1);
    // the rest of the whole-shell fill: the z ghost planes, and the rings of
    // the outermost planes
    {
      const long long n = 2LL * p.NX * p.NY;
      const unsigned g = (unsigned)std::min<long long>((n + 255) / 256, 152 * 16);
      k_ghost_all<TU><<<g, 256, 0, d->stream>>>(p, (TU*)d->u, p.neq, 1, d->sc, 1);
      const long long nr = 2LL * p.NX + 2LL * (p.NY - 2);
      const unsigned gr = (unsigned)std::min<long long>((nr + 255) / 256, 152 * 16);
      k_ghost_ring<TU><<<gr, 256, 0, d->stream>>>(p, (TU*)d->u, p.neq, 1, 0, 1, d->sc);
      k_ghost_ring<TU><<<gr, 256, 0, d->stream>>>(p, (TU*)d->u, p.neq, 1, p.NZ - 1, p.NZ, d->sc);
      d->launches += 3;
      gch_mark(d, "k_ghost");
    }
    if (d->prim_pre) clear_prim_fresh(d);
    layout_out(0, NG);
    layout_out(NG + p.nz, p.NZ);
    st |= cuda_status(cudaGetLastError());
    // the copies, queued after every launch (a copy into pageable memory
    // returns only when it is done)
    for (int i = 0; i < np && st == GCH_OK; ++i) {
      st |= cuda_status(cudaStreamWaitEvent(d->cstream, d->pipe_ev[kDownEv + i], 0));
      st |= cuda_status(cudaMemcpyAsync(host + cut[i][0] * p.neq, d->stage + cut[i][0] * p.neq,
                                        (cut[i][1] - cut[i][0]) * p.neq * sizeof(double),
                                        cudaMemcpyDeviceToHost, d->cstream));
    }
    st |= cuda_status(cudaEventRecord(d->pipe_ev[gch_domain::kPipeEv - 1], d->cstream));
    st |= cuda_status(cudaStreamWaitEvent(d->stream, d->pipe_ev[gch_domain::kPipeEv - 1], 0));
    return st;
  }

  static void clear_prim_fresh(gch_domain* d) {
    cudaMemsetAsync(&d->sc->prim_fresh, 0, sizeof(int), d->stream);
  }

  static int boundaryI(gch_domain* d) {
    ghost<TU>(d, (TU*)d->u, 1);
    if (d->prim_pre) clear_prim_fresh(d);
    return cuda_status(cudaGetLastError());
  }

  static int calcprim(gch_domain* d) {
    if constexpr (std::is_same<Pol, PolFP64>::value)
      if (d->kp.solver == GCH_SOLVER_HLLE_SPLIT_ALL) return split_calcprim(d);
    if (!d->prim_in) return GCH_OK;  // primitives are formed on the fly
    const KParams& p = d->kp;
    dim3 g((p.NX + 31) / 32, (p.NY + 7) / 8, p.NZ), b(32, 8);
    with_neq(p.neq, [&](auto N) {
      k_calcprim<Pol, decltype(N)::value><<<g, b, 0, d->stream>>>(p, (const TU*)d->u, (TS*)d->primit, d->sc);
    });
    return cuda_status(cudaGetLastError());
  }

  // host layout <-> u: `aos` is the staging buffer or mapped host memory
  static constexpr int kLayoutGrid = 152 * 8;
  static int upload(gch_domain* d, const double* aos) {
    if (d->prim_pre) clear_prim_fresh(d);
    k_aos_to_soa<TU><<<kLayoutGrid, kLayoutCells, 0, d->stream>>>(d->kp, aos, (TU*)d->u, d->kp.neq);
    return cuda_status(cudaGetLastError());
  }
  static int download_u(gch_domain* d, double* aos) {
    k_soa_to_aos<TU><<<kLayoutGrid, kLayoutCells, 0, d->stream>>>(d->kp, (const TU*)d->u, aos,
                                                                   d->kp.neq);
    return cuda_status(cudaGetLastError());
  }
  static int download_prim(gch_domain* d, double* aos) {
    const KParams& p = d->kp;
    if constexpr (std::is_same<Pol, PolFP64>::value)
      if (p.solver == GCH_SOLVER_HLLE_SPLIT_ALL) return split_download_prim(d, aos);
    if (d->prim_in) {
      k_soa_to_aos<TS><<<kLayoutGrid, kLayoutCells, 0, d->stream>>>(p, (const TS*)d->primit, aos, p.neq);
    } else {
      with_neq(p.neq, [&](auto N) {
        k_prim_to_aos<Pol, decltype(N)::value><<<kLayoutGrid, kLayoutCells, 0, d->stream>>>(
            p, (const TU*)d->u, aos);
      });
    }
    return cuda_status(cudaGetLastError());
  }
  static int loopfin(gch_domain* d) {
    k_loopfin<<<1, 1, 0, d->stream>>>(d->sc);
    return cuda_status(cudaGetLastError());
  }

  // the stage-1 flux kernel alone: it writes the stage arrays up and E and
  // leaves u and primit unchanged (the autotuner times it)
  static int probe(gch_domain* d) {
    int st = (d->prim_in || d->prim_pre) ? flux<1, true>(d, d->primit, d->up)
                                         : flux<1, false>(d, d->u, d->up);
    return st | cuda_status(cudaGetLastError());
  }

  static constexpr EngineOps ops() {
    return EngineOps{&get_dt,   &tstep,      &boundaryI, &calcprim, &upload,
                     &download_u, &download_prim, &loopfin, &probe,  &step_host};
  }
};

// Not inline, so that an explicit instantiation declaration keeps the
// passive-scalar instantiations out of the policy's main translation unit.
template <class Pol>
template <int NEQ, int STAGE, bool PRIM_IN>
int Engine<Pol>::flux_n(gch_domain* d, const void* src, void* dst) {
  const int s = d->kp.solver;
  if constexpr (NEQ >= 8) {  // with B: all four solvers (HLLC/HLL carry it passively)
    if (s == GCH_SOLVER_HLLD) flux_launch<GCH_SOLVER_HLLD, NEQ, STAGE, PRIM_IN>(d, src, dst);
    else if (s == GCH_SOLVER_HLLE) flux_launch<GCH_SOLVER_HLLE, NEQ, STAGE, PRIM_IN>(d, src, dst);
    else if (s == GCH_SOLVER_HLLC) flux_launch<GCH_SOLVER_HLLC, NEQ, STAGE, PRIM_IN>(d, src, dst);
    else if (s == GCH_SOLVER_HLL) flux_launch<GCH_SOLVER_HLL, NEQ, STAGE, PRIM_IN>(d, src, dst);
    else return GCH_ERR_PARAM;
  } else {  // hydro
    if (s == GCH_SOLVER_HLLC) flux_launch<GCH_SOLVER_HLLC, NEQ, STAGE, PRIM_IN>(d, src, dst);
    else if (s == GCH_SOLVER_HLL) flux_launch<GCH_SOLVER_HLL, NEQ, STAGE, PRIM_IN>(d, src, dst);
    else return GCH_ERR_PARAM;
  }
  return GCH_OK;
}

// The stage kernels with passive scalars (7 and 10 equations) of policy POL,
// declared `extern` in the policy's main translation unit and instantiated
// in a second one, so the two compile in parallel.
#define GCH_PASSIVE_FLUX(EXTERN, POL)                                                 \
  EXTERN template int Engine<POL>::flux_n<7, 1, false>(gch_domain*, const void*, void*); \
  EXTERN template int Engine<POL>::flux_n<7, 1, true>(gch_domain*, const void*, void*);  \
  EXTERN template int Engine<POL>::flux_n<7, 2, false>(gch_domain*, const void*, void*); \
  EXTERN template int Engine<POL>::flux_n<10, 1, false>(gch_domain*, const void*, void*); \
  EXTERN template int Engine<POL>::flux_n<10, 1, true>(gch_domain*, const void*, void*);  \
  EXTERN template int Engine<POL>::flux_n<10, 2, false>(gch_domain*, const void*, void*);

}  // namespace gch
