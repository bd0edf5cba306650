// gch_kernels.cuh -- kernels of one Guacho timestep on sm_103a.
//
// A step is (src/hydro_solver.f90:134-229):
//   k_flux<STAGE 1>   u (or primit) -> first-order HLL*-family fluxes on the
//                     faces of an x-y tile marching along z; hydro update of
//                     up(1:5) and the cell-centred E of flux-CD, fused
//   k_ct<1>           up(6:8) from E (src/flux_cd_module.f90:311-321)
//   k_ghost_all       boundaryII on up (2 layers) [+ k_user_bc]
//   k_flux<STAGE 2>   up -> limited linear reconstruction + fluxes; u(1:5)
//   k_ct<2>           u(6:8)
//   [k_visc] [k_cool] k_ghost_all (boundaryI, 1 layer) [+ k_user_bc]
//   [k_prim_ghost]
// and get_timestep is k_cfl (block min -> one atomic per block) + k_dtfin.
//
// Memory layout: structure of arrays, one 3-D array per field with the
// reference's two ghost cells per side, x fastest, rows padded to a multiple
// of 4 elements (16-byte aligned rows in FP32 and FP64).
#pragma once

#include <type_traits>

#include "gch_policy.cuh"
#include "gch_tma.cuh"

namespace gch {


__device__ __forceinline__ void raise_err(int* errp, int bits) {
  if (bits) atomicOr(errp, bits);
}

// u + dt * s for a source term s as a separate accumulation (the FP64 stage
// update, in the reference's order, and the CT kernels' eight-wave terms):
// FP64 on the FP64 and FP64-u paths; on the pair path the FP32 product dt*s
// is added to the pair (no FP64 instruction)
template <class Pol, class R, class T>
__device__ __forceinline__ R add_source(R u, double dt, float dtf, T s) {
  if constexpr (std::is_same<Pol, PolKahan>::value) return Ops<PolKahan>::addf(u, dtf * s);
  else return Ops<Pol>::add(u, dt * (double)s);
}

// ---------------------------------------------------------------------------
// Per-cell prim load from the stage source.
template <class Pol, int NEQ, int STAGE, bool PRIM_IN>
struct Src {
  using TC = typename Ops<Pol>::TC;
  // STAGE 1: u (TU) or primit (TS, PRIM_IN); STAGE 2: up (TS)
  using TIn = typename std::conditional<(STAGE == 1 && !PRIM_IN), typename Pol::TU,
                                        typename Pol::TS>::type;
  __device__ __forceinline__ static void load(const KParams& p, const TIn* src, long long idx,
                                              TC* prim, unsigned& pfl) {
    if constexpr (PRIM_IN)
      Ops<Pol>::template load_stored_prim<NEQ>(p, src, idx, prim);
    else
      Ops<Pol>::template load_prim<NEQ>(p, src, idx, prim, pfl);
  }
  // the same in two halves: the stored values of a cell into registers
  // (issued early, so their latency overlaps other work), then the
  // conversion, with the arithmetic of load()
  __device__ __forceinline__ static void fetch(const KParams& p, const TIn* src, long long idx,
                                               TIn* raw) {
#pragma unroll
    for (int q = 0; q < NEQ; ++q) raw[q] = src[q * p.fs + idx];
  }
  __device__ __forceinline__ static void convert(const KParams& p, const TIn* raw, TC* prim,
                                                 unsigned& pfl) {
    if constexpr (PRIM_IN) {
#pragma unroll
      for (int q = 0; q < NEQ; ++q) prim[q] = (TC)raw[q];
    } else if constexpr (std::is_same<TIn, float>::value) {
      prim_from_f32<NEQ>(p, raw, prim, pfl);  // FP32 stage state (up)
    } else {
      Ops<Pol>::template prim_vals<NEQ>(p, raw, prim, pfl);  // u: FP64 or pairs
    }
  }
};

// FP32 x/y-face reconstruction with minmod or van Leer runs paired
// (muscl_pair); FP64 and the other limiters take the scalar expressions.
template <class TC, int LIM>
constexpr bool kPairedMuscl = sizeof(TC) == 4 &&
                              (LIM == GCH_LIMITER_VAN_LEER || LIM == GCH_LIMITER_MINMOD);

// Shared memory of the stage kernel (dynamic: up to 72 KB in FP32).  The
// staged primitive plane P has two layouts:
//  - field-major [q][y][x] (the FP64 path, staged by per-thread loads);
//  - row-major [y][q][x] with a 128-byte multiple row stride (the FP32
//    paths): a TMA box of one halo row of every field lands in one row of P,
//    and each row starts 128-byte aligned as a TMA destination must.
template <class TC, int NEQ, int STAGE, bool TMA>
struct FluxSmem {
  static constexpr int H = STAGE == 1 ? 1 : 2;
  static constexpr int NQ = STAGE == 1 ? 1 : 3;
  static constexpr int PW = TX + 2 * H;                       // staged row width
  static constexpr int PH = TY + 2 * H;                       // staged rows
  static constexpr int RS = (NEQ * PW * (int)sizeof(TC) + 127) / 128 * 128 / (int)sizeof(TC);
  static constexpr int kP = TMA ? PH * RS : NEQ * PH * PW;
  __device__ __forceinline__ static int pidx(int q, int y, int x) {
    if constexpr (TMA) return y * RS + q * PW + x;
    else return (q * PH + y) * PW + x;
  }
  TC P[kP];
  TC F[NEQ][TY][TX + 1];
  TC G[NEQ][TY + 1][TX];
  TC Hz[2][NEQ][TY][TX];
  TC Q[NQ][NEQ][TY][TX];
};

// Stored values on their way into the stage kernel's shared memory.
//  TmaRows / TmaSides: the halo ring of a plane copied by TMA (FP32 paths).
//  Rows: the whole halo row(s) below and above the tile, 36 cells wide (the
//  box starts at the tile's x origin, 16-byte aligned), every field; the
//  second stage lands its rows in P directly, the first stage (whose stored
//  type differs from the compute type) in TmaRows.  Sides: the H columns left
//  and right of the tile in a box 16 bytes wide, every field, TY rows.
//  ColBuf: the next column value of each thread, copied by cp.async where
//  there is room.
template <class TIn, int NEQ, int H>
struct TmaRows {
  static constexpr int kRow = (NEQ * (TX + 4) * (int)sizeof(TIn) + 127) / 128 * 128;
  unsigned char raw[2 * H][kRow];
  __device__ __forceinline__ TIn& at(int strip_row, int q, int x) {
    return reinterpret_cast<TIn*>(raw[strip_row])[q * (TX + 4) + x];
  }
};
template <class TIn, int NEQ>
struct TmaSides {
  static constexpr int SW = 16 / (int)sizeof(TIn);  // cells per 16-byte box row
  static constexpr int kSide = (TY * NEQ * 16 + 127) / 128 * 128;
  unsigned char raw[2][kSide];
  __device__ __forceinline__ TIn& at(int side, int y, int q, int c) {
    return reinterpret_cast<TIn*>(raw[side])[(y * NEQ + q) * SW + c];
  }
};
template <class TIn, int NEQ>
struct ColBuf {
  TIn col[NEQ][TY][TX];
};

// The stage kernel's dynamic shared memory.  The FP32 paths stage the halo
// ring of every plane by TMA (the copies of plane k+1 are in flight while
// plane k is worked on: the first stage's raw rows and both stages' side
// columns have their own buffer; the second stage's rows land in P once the
// faces of the previous plane are done).  A block stays within 75 KB so that
// three blocks fit on an SM; the first stage also copies the next column
// value of each thread with cp.async where the block stays within 64 KB
// (hydro), which leaves L1 room for the halo reuse.
template <class Pol, int NEQ, int STAGE, bool PRIM_IN>
struct FluxLayout {
  using TC = typename Ops<Pol>::TC;
  using TIn = typename Src<Pol, NEQ, STAGE, PRIM_IN>::TIn;
  static constexpr int H = STAGE == 1 ? 1 : 2;
  static constexpr bool kTma = sizeof(TC) == 4;
  using SM = FluxSmem<TC, NEQ, STAGE, kTma>;
  static constexpr size_t kMain = (sizeof(SM) + 127) / 128 * 128;
  static constexpr size_t kRows = (kTma && STAGE == 1) ? sizeof(TmaRows<TIn, NEQ, H>) : 0;
  static constexpr size_t kSides = kTma ? sizeof(TmaSides<TIn, NEQ>) : 0;
  static constexpr size_t kBar = kTma ? 128 : 0;  // mbarrier + abort flag
  static constexpr size_t kCol = sizeof(ColBuf<TIn, NEQ>);
  static constexpr size_t kLimit = 64 * 1024;
  static constexpr bool kAsyncCol =
      STAGE == 1 && sizeof(TC) == 4 && kMain + kRows + kSides + kBar + kCol <= kLimit;
  static constexpr size_t kBytes = kMain + kRows + kSides + kBar + (kAsyncCol ? kCol : 0);
  // bytes of one plane's halo copies (full boxes, out-of-range cells filled)
  static constexpr unsigned kTmaBytes =
      (unsigned)(2 * H * NEQ * (TX + 4) * sizeof(TIn) + 2 * TY * NEQ * 16);
  // (with passive scalars, NEQ = 10, the second stage holds two blocks per SM
  // with or without the TMA buffers)
  static_assert(!kTma || NEQ > 8 || kBytes <= 75 * 1024, "three blocks per SM");
};

// cp.async of one 4-, 8- or 16-byte value from global into shared memory,
// and the waits of the issuing thread for its own copies.
template <class T>
__device__ __forceinline__ void cp_async(T* s, const T* g) {
  static_assert(sizeof(T) == 4 || sizeof(T) == 8 || sizeof(T) == 16, "cp.async size");
  const unsigned sa = (unsigned)__cvta_generic_to_shared(s);
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(sa), "l"(g), "n"(sizeof(T))
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// ---------------------------------------------------------------------------
// Stage kernel.  Block = TX x TY cells of one x-y tile; the block marches
// over planes [kb, ke) of z.  Per plane k:
//   1. the primitive plane k with an H-cell halo (H = 1 first order, 2
//      limited) is staged in shared memory: centre cells from the column
//      ring (each thread owns one column), halo cells formed from global
//      memory;
//   2. one work loop solves every face the tile needs, through a single
//      Riemann call site: first the z face k+1/2 of each thread's own
//      column, then the tile's x faces and y faces; fluxes go to shared
//      memory;
//   3. each cell: hydro update (+ sources) and E from its six faces.
// Column state (the next planes, z slopes, z fluxes) lives in shared
// memory slots owned by one thread, which keeps registers for the solver.
// Fluxes are never written to global memory.
// The body takes the block's tile coordinates (bx, by) and z chunk (bz) as
// arguments: the one-box kernel passes blockIdx, the grouped kernel of many
// boxes passes the coordinates decoded from its linear block index.
// DEFER (first stage only): instead of the update, write the three flux
// differences (fr - fl, gr - gl, hr - hl) of every updated field q to fields
// 3q, 3q+1, 3q+2 of `dst`: the fluxes do not depend on dt, so they can be
// computed before get_timestep has it (k_s1_apply finishes the update).
template <class Pol, int SOLVER, int NEQ, int STAGE, bool PRIM_IN, int LIM, bool DEFER = false>
__device__ __forceinline__ void
flux_body(const KParams& p, const typename Src<Pol, NEQ, STAGE, PRIM_IN>::TIn* __restrict__ src,
          const typename Pol::TU* u,
          typename std::conditional<STAGE == 1, typename Pol::TS, typename Pol::TU>::type* dst,
          typename Pol::TS* __restrict__ E, typename Pol::TS* __restrict__ s678,
          StepScalars* sc, int kz, int bx, int by, int bz) {
  using TC = typename Ops<Pol>::TC;
  using TD = typename std::conditional<STAGE == 1, typename Pol::TS, typename Pol::TU>::type;
  using S = Src<Pol, NEQ, STAGE, PRIM_IN>;
  using TIn = typename S::TIn;
  if (!sc->active) return;
  constexpr int H = STAGE == 1 ? 1 : 2;
  constexpr int NRING = 2 * H * (TX + TY);
  using LAY = FluxLayout<Pol, NEQ, STAGE, PRIM_IN>;
  using SM = typename LAY::SM;
  constexpr bool TMA = LAY::kTma, ACOL = LAY::kAsyncCol;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  SM& sm = *reinterpret_cast<SM*>(smem_raw);
  auto& trows = *reinterpret_cast<TmaRows<TIn, NEQ, H>*>(smem_raw + LAY::kMain);
  auto& tsides = *reinterpret_cast<TmaSides<TIn, NEQ>*>(smem_raw + LAY::kMain + LAY::kRows);
  uint64_t* tbar = reinterpret_cast<uint64_t*>(smem_raw + LAY::kMain + LAY::kRows + LAY::kSides);
  int* tabort = reinterpret_cast<int*>(tbar + 1);
  auto& sbc = *reinterpret_cast<ColBuf<TIn, NEQ>*>(smem_raw + LAY::kMain + LAY::kRows +
                                                   LAY::kSides + LAY::kBar);
  // primitive plane k with halo: component q of the cell (x, y) of the
  // staged plane, x and y counted from the halo's corner
  auto sP = [&](int q, int y, int x) -> TC& { return sm.P[SM::pidx(q, y, x)]; };
  auto& sF = sm.F;    // x-face fluxes
  auto& sG = sm.G;    // y-face fluxes
  auto& sH = sm.Hz;   // z-face fluxes, slot (face+1/2)&1
  auto& sQ = sm.Q;    // column ring: [0] p(k+1), [1] p(k+2), [2] z slope of p(k)

  const int tx = threadIdx.x, ty = threadIdx.y;
  const int tid = ty * TX + tx;
  const int i0 = bx * TX, j0 = by * TY;
  const int kb = bz * kz;
  const int ke = min(p.nz, kb + kz);
  const int ci = i0 + tx, cj = j0 + ty;
  const bool active = ci < p.nx && cj < p.ny;
  const bool ct = NEQ >= 8 && p.flux_cd;
  const int lim = p.limiter;

  const double dt = STAGE == 1 ? sc->dt / 2.0 : sc->dt;  // dtm = dt_CFL/2.
  const float dtf = (float)dt;
  const TC dtdx = par<TC>(sc->dtd[STAGE - 1][0], sc->dtdf[STAGE - 1][0]);
  const TC dtdy = par<TC>(sc->dtd[STAGE - 1][1], sc->dtdf[STAGE - 1][1]);
  const TC dtdz = par<TC>(sc->dtd[STAGE - 1][2], sc->dtdf[STAGE - 1][2]);

  int err = 0;
  unsigned pfl = 0;

  // clamp a global coordinate into the array (inactive lanes of partial
  // tiles read valid memory; their values are never used)
  auto gidx = [&](int ax, int ay, int az) -> long long {
    ax = min(max(ax, 0), p.NX - 1);
    ay = min(max(ay, 0), p.NY - 1);
    az = min(max(az, 0), p.NZ - 1);
    return cell_index(p, ax, ay, az);
  };
  const int axc = ci + NG, ayc = cj + NG;
  TC bzm = 0;  // Bz at k-1 of this column (eight-wave div B)

  // The march starts before kb so that every plane's column values, z
  // slopes and z faces come from the same code as in the body of the march
  // (one inlined instance each): the results of a plane do not depend on
  // where a z chunk begins.  Iteration k loads p(k+H) into the column ring;
  // stage 2 forms the z slope of p(k+1) from k >= kb-2 on; the z face k+1/2
  // is solved from k >= kb-1 on; planes k >= kb are staged and updated.
  const int k0 = kb - (STAGE == 1 ? 2 : 4);
  const int nfx = (TX + 1) * TY;
  const int nfy = TX * (TY + 1);

  // The halo ring of a plane has fewer cells than the block has threads:
  // thread tid < NRING owns halo cell (hx, hy) of every plane.
  static_assert(NRING <= NT, "one halo cell per thread");
  const bool has_halo = tid < NRING;
  int hx = 0, hy = 0;
  if (tid < 2 * H * TX) {  // rows below / above the tile
    const int row = tid / TX;
    hx = tid % TX;
    hy = row < H ? row - H : TY + (row - H);
  } else {  // columns left / right
    const int rr = tid - 2 * H * TX;
    const int col = rr / TY;
    hy = rr % TY;
    hx = col < H ? col - H : TX + (col - H);
  }

  // TMA staging of the halo ring (FP32 paths).  Warp 0 issues the copies of
  // a plane: 2H rows of 36 cells (x from the tile origin i0, every field) and
  // the left and right column boxes (16 bytes wide, TY rows); they complete
  // on the mbarrier *tbar, whose phase flips once per plane.  Stage 1 copies
  // into its raw buffers, which are free once the plane's halo is
  // converted, so the copies of plane k+1 are issued right after plane k is
  // staged.  Stage 2 copies its rows into P itself, free once the faces of
  // the plane before are solved (or, when the update reads P's halo rows
  // for the eight-wave div B, once that update is done).
  // the right column box starts at the last 16-byte boundary at or before
  // the tile's first right-halo cell
  constexpr int XR = NG + TX + H - 1 - ((NG + TX + H - 1) % TmaSides<TIn, NEQ>::SW);
  auto early2 = [&]() { return !(NEQ >= 8 && p.eight_wave); };
  auto tma_issue = [&](int kk) {
    if constexpr (TMA) {
      if (tid < 32) {
        constexpr int kRowsMap = STAGE == 2 ? kTmaS2Rows : (PRIM_IN ? kTmaS1PRows : kTmaS1Rows);
        static_assert(kRowsMap + 1 == (STAGE == 2 ? kTmaS2Sides
                                                  : (PRIM_IN ? kTmaS1PSides : kTmaS1Sides)),
                      "a source's side map follows its row map");
        const unsigned char* maps = p.tmaps + kRowsMap * kTmaMapBytes;
        if (tid == 0) mbar_arrive_expect_tx(tbar, LAY::kTmaBytes);
        __syncwarp();
        const int az = kk + NG;
        if (tid < 2 * H) {  // halo row `tid` (0..H-1 below, H..2H-1 above)
          const int ay = tid < H ? j0 + NG - H + tid : j0 + NG + TY + (tid - H);
          void* dst;
          if constexpr (STAGE == 1) dst = trows.raw[tid];
          else dst = &sm.P[SM::pidx(0, tid < H ? tid : TY + tid, 0)];
          tma_load_4d(dst, maps, tbar, i0, 0, ay, az);
        } else if (tid < 2 * H + 2) {  // left / right columns
          const int sd = tid - 2 * H;
          tma_load_4d(tsides.raw[sd], maps + kTmaMapBytes, tbar, sd == 0 ? i0 : i0 + XR, 0, j0 + NG,
                      az);
        }
      }
    }
  };
  if constexpr (TMA) {
    if (tid == 0) {
      // a TMA destination must be 128-byte aligned: refuse to copy otherwise
      *tabort = (smem_addr(smem_raw) & 127u) != 0;
      if (!*tabort) {
        mbar_init(tbar, 1);
        mbar_init_fence();
      }
    }
    __syncthreads();
    if (*tabort) {
      if (tid == 0) atomicOr(&sc->err, GCH_ERR_TIMEOUT);
      return;
    }
    if (kb < ke) tma_issue(kb);
  }
  // the halo cell of this thread from the TMA copies, converted; stage 2 row
  // cells are converted in place in P
  auto halo_from_tma = [&]() {
    TIn hv[NEQ];
    const int c = hx + 2;  // column in a 36-wide row box (box origin i0 = tile x - 2)
    if (hy < 0 || hy >= TY) {
      const int r = hy < 0 ? hy + H : H + (hy - TY);  // strip row 0..2H-1
      if constexpr (STAGE == 1) {
#pragma unroll
        for (int q = 0; q < NEQ; ++q) hv[q] = trows.at(r, q, c);
      } else {
#pragma unroll
        for (int q = 0; q < NEQ; ++q) hv[q] = sP(q, hy + H, hx + H);
      }
    } else {
      const int sd = hx < 0 ? 0 : 1;
      const int cc = hx < 0 ? hx + 2 : NG + hx - XR;
#pragma unroll
      for (int q = 0; q < NEQ; ++q) hv[q] = tsides.at(sd, hy, q, cc);
    }
    TC pr[NEQ];
    S::convert(p, hv, pr, pfl);
#pragma unroll
    for (int q = 0; q < NEQ; ++q) sP(q, hy + H, hx + H) = pr[q];
  };

  // Stored values are fetched into registers before they are needed: the
  // next column value after the faces of a plane are solved (converted at
  // the start of the next iteration), and this plane's u before the barrier
  // that precedes the update.  Their load latency overlaps the barrier wait
  // and the update instead of stalling the start of a plane.  With ACOL the
  // next column value goes to shared memory by cp.async instead; each thread
  // reads back only what it copied, after its own wait.
  TIn colr[NEQ];
  auto fetch_col = [&](int az_) {
    const long long cc = gidx(axc, ayc, az_);
    if constexpr (ACOL) {
#pragma unroll
      for (int q = 0; q < NEQ; ++q) cp_async(&sbc.col[q][ty][tx], src + q * p.fs + cc);
      cp_async_commit();
    } else {
      S::fetch(p, src, cc, colr);
    }
  };
  fetch_col(k0 + NG + H);
  auto prefetch_next = [&](int k) {
    if (k + 1 < ke) fetch_col(k + 1 + NG + H);
  };

  // Whether a plane starts with a barrier.  The update of the plane before
  // reads the face fluxes, which the next faces overwrite only after the
  // barrier that precedes them, and its own cell of P; the staging of the
  // next plane writes this thread's cell, its column ring and halo cells,
  // which nothing reads before that barrier.  So without source terms no
  // thread can overwrite what another still reads, and the barrier is left
  // out.  With source terms the update reads neighbouring cells of P (the
  // eight-wave div B), and the TMA rows of stage 2 wait for that update.
  // (The FP64 kernels, one block per SM and latency-bound, keep the barrier
  // and the single face call site below: both changes made them slower.)
  constexpr bool kEarlyZ = sizeof(TC) == 4;
  const bool plane_sync = !kEarlyZ || p.user_src || (NEQ >= 8 && p.eight_wave);
  for (int k = k0; k < ke; ++k) {
    const bool plane = k >= kb;
    const bool zface = k >= kb - 1;
    const bool zwork = STAGE == 1 ? zface : k >= kb - 2;
    const int az = k + NG;
    const int hslot = (k + 1) & 1;  // face k+1/2
    // one face: 0 = the z face k+1/2 of this thread's column (its own
    // shared-memory cells only), 1 = x face (fx, fy), 2 = y face (fx, fy)
    auto face = [&](int kind, int fx, int fy) {
      TC l[NEQ], r[NEQ], f[NEQ];
      if (kind == 0) {
        if (STAGE == 1) {
#pragma unroll
          for (int q = 0; q < NEQ; ++q) {
            l[q] = sP(perm<2, NEQ>(q), ty + H, tx + H);
            r[q] = sQ[0][perm<2, NEQ>(q)][ty][tx];
          }
        } else {
          // the slope of p(k) comes from the ring (formed by the previous
          // iteration); the slope of p(k+1) from p(k..k+2) is formed here
          // once and kept for face k+3/2
#pragma unroll
          for (int q = 0; q < NEQ; ++q) {
            const int s = perm<2, NEQ>(q);
            const TC al = sQ[2][s][ty][tx], rr = sQ[1][s][ty][tx];
            l[q] = sP(s, ty + H, tx + H);
            r[q] = sQ[0][s][ty][tx];
            const TC dm = r[q] - l[q], dr = rr - r[q];
            const TC ar = average_t<LIM>(lim, dm, dr);
            sQ[2][s][ty][tx] = ar;
            l[q] = l[q] + al * TC(0.5);
            r[q] = r[q] - ar * TC(0.5);
          }
          if (!zface) return;  // slope of p(kb-1) only
        }
      } else if (kind == 1) {
        const int cy = fy + H, cl = fx - 1 + H;
#pragma unroll
        for (int q = 0; q < NEQ; ++q) {
          l[q] = sP(q, cy, cl);
          r[q] = sP(q, cy, cl + 1);
          if (STAGE == 2) {
            const TC ll = sP(q, cy, cl - 1), rr = sP(q, cy, cl + 2);
            if constexpr (kPairedMuscl<TC, LIM>) {
              const float2 o = muscl_pair<LIM>(ll, l[q], r[q], rr);
              l[q] = o.x;
              r[q] = o.y;
            } else {
              const TC dl = l[q] - ll, dm = r[q] - l[q], dr = rr - r[q];
              const TC al = average_t<LIM>(lim, dl, dm), ar = average_t<LIM>(lim, dm, dr);
              l[q] = l[q] + al * TC(0.5);
              r[q] = r[q] - ar * TC(0.5);
            }
          }
        }
      } else {
        const int cx = fx + H, cl = fy - 1 + H;
#pragma unroll
        for (int q = 0; q < NEQ; ++q) {
          const int s = perm<1, NEQ>(q);
          l[q] = sP(s, cl, cx);
          r[q] = sP(s, cl + 1, cx);
          if (STAGE == 2) {
            const TC ll = sP(s, cl - 1, cx), rr = sP(s, cl + 2, cx);
            if constexpr (kPairedMuscl<TC, LIM>) {
              const float2 o = muscl_pair<LIM>(ll, l[q], r[q], rr);
              l[q] = o.x;
              r[q] = o.y;
            } else {
              const TC dl = l[q] - ll, dm = r[q] - l[q], dr = rr - r[q];
              const TC al = average_t<LIM>(lim, dl, dm), ar = average_t<LIM>(lim, dm, dr);
              l[q] = l[q] + al * TC(0.5);
              r[q] = r[q] - ar * TC(0.5);
            }
          }
        }
      }
      Riemann<SOLVER, NEQ>::solve(p, l, r, f, err);
      if (kind == 0) {
#pragma unroll
        for (int q = 0; q < NEQ; ++q) sH[hslot][perm<2, NEQ>(q)][ty][tx] = f[q];
      } else if (kind == 1) {
#pragma unroll
        for (int q = 0; q < NEQ; ++q) sF[q][fy][fx] = f[q];
      } else {
#pragma unroll
        for (int q = 0; q < NEQ; ++q) sG[perm<1, NEQ>(q)][fy][fx] = f[q];
      }
    };
    if (plane && plane_sync) {
      if constexpr (TMA && STAGE == 2) fence_proxy_async_smem();
      __syncthreads();  // readers of the previous plane are done
      if constexpr (TMA && STAGE == 2)
        if (!early2() && k > kb) tma_issue(k);
    }
    // 1. the column ring shifts (centre <- p(k), p(k+1) <- p(k+2)) and the
    //    next plane of the column is formed from the fetched values
    {
      if constexpr (ACOL) {
        cp_async_wait_all();  // this thread's copies
#pragma unroll
        for (int q = 0; q < NEQ; ++q) colr[q] = sbc.col[q][ty][tx];
      }
      TC nx_[NEQ];
      S::convert(p, colr, nx_, pfl);
#pragma unroll
      for (int q = 0; q < NEQ; ++q) {
        sP(q, ty + H, tx + H) = sQ[0][q][ty][tx];
        if (STAGE == 1) {
          sQ[0][q][ty][tx] = nx_[q];
        } else {
          sQ[0][q][ty][tx] = sQ[1][q][ty][tx];
          sQ[1][q][ty][tx] = nx_[q];
        }
      }
    }
    if (plane) {
      //  the halo of plane k
      if constexpr (TMA) {
        const unsigned parity = (unsigned)(k - kb) & 1u;  // one phase per plane
        if (has_halo) {
          if (mbar_wait(tbar, parity)) halo_from_tma();
          else *tabort = 1;
        } else {
          if constexpr (kEarlyZ)
            if (active) face(0, tx, ty);  // this column's z face while the halo is converted
        }
        fence_proxy_async_smem();  // the raw buffers are read: the next copy may overwrite
        __syncthreads();
        if (*tabort) {  // a copy did not arrive: report, drain, leave together
          if (tid == 0) {
            atomicOr(&sc->err, GCH_ERR_TIMEOUT);
            mbar_wait(tbar, parity);
          }
          return;
        }
        if constexpr (STAGE == 1)
          if (k + 1 < ke) tma_issue(k + 1);
      } else {
        if (has_halo) {
          TC pr[NEQ];
          S::load(p, src, gidx(i0 + hx + NG, j0 + hy + NG, az), pr, pfl);
#pragma unroll
          for (int q = 0; q < NEQ; ++q) sP(q, hy + H, hx + H) = pr[q];
        } else {
          if constexpr (kEarlyZ)
            if (active) face(0, tx, ty);  // this column's z face while the halo is loaded
        }
        __syncthreads();
      }
    }

    // 2. all faces through one Riemann call site.  In a plane, the threads
    //    without a halo cell have already solved their column's z face
    //    while the halo was converted (below the column shift): the loop takes
    //    the other NRING z faces and the x and y faces, so a plane needs at
    //    most three rounds of 256 solves instead of four.
    const int nzw = plane && kEarlyZ ? NRING : NT;
    const int nwork = plane ? nzw + nfx + nfy : (zwork ? NT : 0);
    for (int w = tid; w < nwork; w += NT) {
      int kind;  // 0 = z (own column), 1 = x, 2 = y
      int fx, fy;
      bool need;
      if (w < nzw) {
        kind = 0; fx = tx; fy = ty; need = active;
      } else if (w - nzw < nfx) {
        kind = 1;
        fx = (w - nzw) % (TX + 1);
        fy = (w - nzw) / (TX + 1);
        need = j0 + fy < p.ny && i0 + fx - 1 < p.nx;
      } else {
        kind = 2;
        fx = (w - nzw - nfx) % TX;
        fy = (w - nzw - nfx) / TX;
        need = i0 + fx < p.nx && j0 + fy - 1 < p.ny;
      }
      if (need) face(kind, fx, fy);
    }
    if (!plane) {  // column-private work only: no barrier
      if (NEQ >= 8) bzm = sP(7, ty + H, tx + H);
      prefetch_next(k);
      continue;
    }
    // with flux-CD, B comes from the CT kernel: the flux update covers the
    // hydro fields and the passives (src/flux_cd_module.f90:299-308)
    auto upd = [&](int q) { return !ct || q < 5 || q >= 8; };
    const long long c = cell_index(p, axc, ayc, az);
    typename Pol::TU uq[NEQ];
    if (active && !DEFER) {
#pragma unroll
      for (int q = 0; q < NEQ; ++q)
        if (upd(q)) uq[q] = u[q * p.fs + c];
    }
    if constexpr (TMA && STAGE == 2) fence_proxy_async_smem();  // P read by the faces
    __syncthreads();
    if constexpr (TMA && STAGE == 2)
      if (early2() && k + 1 < ke) tma_issue(k + 1);  // P's halo rows are free now
    prefetch_next(k);

    // 3. cell update and E
    if (active) {
      const int hp = k & 1, hn = (k + 1) & 1;  // faces k-1/2, k+1/2
      TC sv[NEQ];
#pragma unroll
      for (int q = 0; q < NEQ; ++q) sv[q] = TC(0);
      // (a deferred first stage runs only without source terms)
      const bool src_terms = !DEFER && (p.user_src || (NEQ >= 8 && p.eight_wave));
      if (src_terms) {
        TC pcen[NEQ];
#pragma unroll
        for (int q = 0; q < NEQ; ++q) pcen[q] = sP(q, ty + H, tx + H);
        // src/sources.f90:190-220 with the cell's stage primitives
        if (p.user_src && sizeof(TC) == 4) {
          // EXO/user_mod.f90:158-206 point masses, FP32 paths: positions,
          // the FP32 copy of the masses and r^3 as r^2 sqrt(r^2)
          const float xc = ((float)(ci + 1 - p.nx / 2) - 0.5f) * p.f_dx;
          const float yc = ((float)(cj + 1 - p.ny / 2) - 0.5f) * p.f_dy;
          const float zc = ((float)(k + 1 - p.nz / 2) - 0.5f) * p.f_dz;
          for (int l = 0; l < p.ngrav; ++l) {
            const float x = xc - p.gravf[p.ngrav + l];
            const float y = yc - p.gravf[2 * p.ngrav + l];
            const float z = zc - p.gravf[3 * p.ngrav + l];
            const float GM = p.gravf[l];
            const float rad2 = x * x + y * y + z * z;
            const float r15 = rad2 * sqrtf(rad2);
            sv[1] = sv[1] - pcen[0] * GM * x / r15;
            sv[2] = sv[2] - pcen[0] * GM * y / r15;
            sv[3] = sv[3] - pcen[0] * GM * z / r15;
            sv[4] = sv[4] - pcen[0] * GM * (pcen[1] * x + pcen[2] * y + pcen[3] * z) / r15;
          }
        } else if (p.user_src) {
          // EXO/user_mod.f90:158-206 point masses
          const double xc = ((double)(ci + 1 - p.nx / 2) - 0.5) * p.dx;
          const double yc = ((double)(cj + 1 - p.ny / 2) - 0.5) * p.dy;
          const double zc = ((double)(k + 1 - p.nz / 2) - 0.5) * p.dz;
          for (int l = 0; l < p.ngrav; ++l) {
            const TC x = (TC)(xc - p.grav[p.ngrav + l]);
            const TC y = (TC)(yc - p.grav[2 * p.ngrav + l]);
            const TC z = (TC)(zc - p.grav[3 * p.ngrav + l]);
            const TC GM = (TC)p.grav[l];
            const TC rad2 = x * x + y * y + z * z;
            const TC r15 = (TC)pow((double)rad2, 1.5);
            sv[1] = sv[1] - pcen[0] * GM * x / r15;
            sv[2] = sv[2] - pcen[0] * GM * y / r15;
            sv[3] = sv[3] - pcen[0] * GM * z / r15;
            sv[4] = sv[4] - pcen[0] * GM * (pcen[1] * x + pcen[2] * y + pcen[3] * z) / r15;
          }
        }
        if (NEQ >= 8 && p.eight_wave) {
          // src/sources.f90:124-175
          const TC bzp = sQ[0][7][ty][tx];
          // 2 dx in the compute type (doubling is exact in either type)
          const TC dx2 = TC(2) * par<TC>(p.dx, p.f_dx), dy2 = TC(2) * par<TC>(p.dy, p.f_dy),
                   dz2 = TC(2) * par<TC>(p.dz, p.f_dz);
          const TC divB = (sP(5, ty + H, tx + H + 1) - sP(5, ty + H, tx + H - 1)) / dx2
                          + (sP(6, ty + H + 1, tx + H) - sP(6, ty + H - 1, tx + H)) / dy2
                          + (bzp - bzm) / dz2;
          sv[1] = sv[1] - divB * pcen[5];
          sv[2] = sv[2] - divB * pcen[6];
          sv[3] = sv[3] - divB * pcen[7];
          sv[4] = sv[4] - divB * (pcen[1] * pcen[5] + pcen[2] * pcen[6] + pcen[3] * pcen[7]);
          sv[5] = sv[5] - divB * pcen[1];
          sv[6] = sv[6] - divB * pcen[2];
          sv[7] = sv[7] - divB * pcen[3];
        }
      }
#pragma unroll
      for (int q = 0; q < NEQ; ++q) {
        if constexpr (DEFER) {
          if (upd(q)) {
            dst[(3 * q) * p.fs + c] = sF[q][ty][tx + 1] - sF[q][ty][tx];
            dst[(3 * q + 1) * p.fs + c] = sG[q][ty + 1][tx] - sG[q][ty][tx];
            dst[(3 * q + 2) * p.fs + c] = sH[hn][q][ty][tx] - sH[hp][q][ty][tx];
          }
        } else if (upd(q)) {
          if constexpr (sizeof(TC) == 4) {
            // FP32 paths: dt s joins the FP32 flux divergence (sv is zero
            // without source terms).  A second accumulation under
            // `if (src_terms)` was evaluated for every cell and selected:
            // 5 FP64 multiply-adds and 4 conversions per cell on the
            // FP32 + FP64 u path, two-sums on the pair path.
            dst[q * p.fs + c] = store_as<TD>(Ops<Pol>::update_src(
                Ops<Pol>::ld(uq[q]), dtdx, dtdy, dtdz, sF[q][ty][tx], sF[q][ty][tx + 1],
                sG[q][ty][tx], sG[q][ty + 1][tx], sH[hp][q][ty][tx], sH[hn][q][ty][tx], dtf,
                sv[q]));
          } else {
            auto unew = Ops<Pol>::update(Ops<Pol>::ld(uq[q]), dtdx, dtdy, dtdz,
                                         sF[q][ty][tx], sF[q][ty][tx + 1], sG[q][ty][tx],
                                         sG[q][ty + 1][tx], sH[hp][q][ty][tx], sH[hn][q][ty][tx]);
            if (src_terms) unew = add_source<Pol>(unew, dt, dtf, sv[q]);
            dst[q * p.fs + c] = store_as<TD>(unew);
          }
        }
      }
      if (ct) {
        // src/flux_cd_module.f90:258-265
        const TC e1 = TC(0.25) * (-sG[7][ty][tx] - sG[7][ty + 1][tx] + sH[hp][6][ty][tx]
                                  + sH[hn][6][ty][tx]);
        const TC e2 = TC(0.25) * (+sF[7][ty][tx] + sF[7][ty][tx + 1] - sH[hp][5][ty][tx]
                                  - sH[hn][5][ty][tx]);
        const TC e3 = TC(0.25) * (-sF[6][ty][tx] - sF[6][ty][tx + 1] + sG[5][ty][tx]
                                  + sG[5][ty + 1][tx]);
        E[c] = e1;
        E[p.fs + c] = e2;
        E[2 * p.fs + c] = e3;
        if (p.eight_wave) {
          s678[c] = sv[5];
          s678[p.fs + c] = sv[6];
          s678[2 * p.fs + c] = sv[7];
        }
      }
    }
    if (NEQ >= 8) bzm = sP(7, ty + H, tx + H);
  }
  raise_err(&sc->err, err);
}

// grid (ceil(nx/TX), ceil(ny/TY), z chunks); block z works chunk bz0 + z
// (kz planes each), so a launch can cover a slab of chunks
template <class Pol, int SOLVER, int NEQ, int STAGE, bool PRIM_IN, int LIM, bool DEFER = false>
__global__ void __launch_bounds__(NT, Pol::kMinBlocks)
k_flux(KParams p, const typename Src<Pol, NEQ, STAGE, PRIM_IN>::TIn* __restrict__ src,
       const typename Pol::TU* u,
       typename std::conditional<STAGE == 1, typename Pol::TS, typename Pol::TU>::type* dst,
       typename Pol::TS* __restrict__ E, typename Pol::TS* __restrict__ s678,
       StepScalars* sc, int kz, int bz0 = 0) {
  static_assert(!DEFER || (STAGE == 1 && !PRIM_IN), "only the first stage from u defers");
  flux_body<Pol, SOLVER, NEQ, STAGE, PRIM_IN, LIM, DEFER>(p, src, u, dst, E, s678, sc, kz,
                                                          blockIdx.x, blockIdx.y, blockIdx.z + bz0);
}

// The first stage's update of a deferred first stage (DEFER above), once dt
// is known: up = u - dt/2 * divF from the stored flux differences, through
// the same Ops::update as the fused stage (a difference minus a zero left
// flux is the difference itself), so up ends the same bit for bit.
// block (32, 8); grid (ceil(nx/32), ceil(ny/8), nz)
template <class Pol, int NEQ>
__global__ void __launch_bounds__(256)
k_s1_apply(KParams p, const typename Pol::TU* __restrict__ u, typename Pol::TS* __restrict__ up,
           const typename Pol::TS* __restrict__ dif, const StepScalars* sc) {
  using TC = typename Ops<Pol>::TC;
  if (!sc->active) return;
  const int ci = blockIdx.x * 32 + threadIdx.x, cj = blockIdx.y * 8 + threadIdx.y;
  if (ci >= p.nx || cj >= p.ny) return;
  const TC dtdx = par<TC>(sc->dtd[0][0], sc->dtdf[0][0]);
  const TC dtdy = par<TC>(sc->dtd[0][1], sc->dtdf[0][1]);
  const TC dtdz = par<TC>(sc->dtd[0][2], sc->dtdf[0][2]);
  const bool ct = NEQ >= 8 && p.flux_cd;
  const long long c = cell_index(p, ci + NG, cj + NG, (int)blockIdx.z + NG);
#pragma unroll
  for (int q = 0; q < NEQ; ++q) {
    if (ct && q >= 5 && q < 8) continue;
    const TC a = (TC)dif[(3 * q) * p.fs + c], b = (TC)dif[(3 * q + 1) * p.fs + c],
             h = (TC)dif[(3 * q + 2) * p.fs + c];
    up[q * p.fs + c] = store_as<typename Pol::TS>(
        Ops<Pol>::update(Ops<Pol>::ld(u[q * p.fs + c]), dtdx, dtdy, dtdz, TC(0), a, TC(0), b,
                         TC(0), h));
  }
}
// Products rounded on their own (never fused into a following sum), so the
// CFL candidate rounds the same way in every kernel that inlines it (the
// one-box and the grouped CFL reduction).
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }

// get_timestep's square roots and quotients.  In FP64 they run on the integer
// and FP32 pipes, correctly rounded (the same bits as sqrt and /): the CFL
// pass is bound by the FP64 pipe and has the issue slots to spare.  FP32 as
// the unit's operations.
__device__ __forceinline__ double cfl_sqrt(double a) { return dsqrt_rn(a); }
__device__ __forceinline__ float cfl_sqrt(float a) { return sqrtf(a); }
__device__ __forceinline__ double cfl_div(double a, double b) { return ddiv_rn(a, b); }
__device__ __forceinline__ float cfl_div(float a, float b) { return a / b; }

// The cell widths and gamma in the compute type, converted once per thread.
template <class TC>
struct CflConst {
  TC h[3], g;
  __device__ __forceinline__ explicit CflConst(const KParams& p)
      : h{par<TC>(p.dx, p.f_dx), par<TC>(p.dy, p.f_dy), par<TC>(p.dz, p.f_dz)},
        g(par<TC>(p.gamma, p.f_gamma)) {}
};

// min(dx/(|vx|+cfx), dy/(|vy|+cfy), dz/(|vz|+cfz)) of one cell into dtp.
// The running min stays in the compute type: a float converts to double
// exactly and in order, so the FP32 paths take the min of the same values
// as a min over their FP64 images, with no FP64 instruction per cell.
template <class TC, int NEQ>
__device__ __forceinline__ void cfl_candidate(const KParams& p, const CflConst<TC>& k,
                                              const TC* pr, TC& dtp, int& bad) {
  TC cand[3];
  if (NEQ >= 8 && p.mhd) {
    // src/hydro_core.f90:568-581 cfast
    const TC g = k.g;
    const TC bx = pr[5], by = pr[6], bz = pr[7];
    const TC b2 = mul_rn(bx, bx) + mul_rn(by, by) + mul_rn(bz, bz);
    const TC gp = mul_rn(g, pr[4]);
    const TC a = gp + b2;
    const TC a2 = mul_rn(a, a), g4 = mul_rn(TC(4.0), gp);
    // a^2 - 4 g p b_n^2 >= 0 exactly; in FP32 rounding can take it below
    // zero where the sound speed meets the normal Alfven speed (clamped);
    // FP64 keeps the reference's expression
    auto disc = [&](TC bn) {
      const TC d = a2 - mul_rn(mul_rn(g4, bn), bn);
      return sizeof(TC) == 4 ? tmax_(d, TC(0)) : d;
    };
    const TC cx = cfl_sqrt(cfl_div(mul_rn(TC(0.5), a + cfl_sqrt(disc(bx))), pr[0]));
    const TC cy = cfl_sqrt(cfl_div(mul_rn(TC(0.5), a + cfl_sqrt(disc(by))), pr[0]));
    const TC cz = cfl_sqrt(cfl_div(mul_rn(TC(0.5), a + cfl_sqrt(disc(bz))), pr[0]));
    cand[0] = cfl_div(k.h[0], tabs(pr[1]) + cx);
    cand[1] = cfl_div(k.h[1], tabs(pr[2]) + cy);
    cand[2] = cfl_div(k.h[2], tabs(pr[3]) + cz);
  } else {
    // src/hydro_core.f90:544-553 csound
    const TC c0 = cfl_sqrt(tdiv(k.g * pr[4], pr[0]));
    cand[0] = cfl_div(k.h[0], tabs(pr[1]) + c0);
    cand[1] = cfl_div(k.h[1], tabs(pr[2]) + c0);
    cand[2] = cfl_div(k.h[2], tabs(pr[3]) + c0);
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (cand[d] == cand[d]) dtp = tmin_(dtp, cand[d]);
    else bad = 1;
  }
}

// Block-wide min of dtp into sc->dtmin_bits; every thread of the block calls.
// The min is taken in the compute type T and converted to FP64 once per
// block (exact and order-preserving for a float); T(1e30) is the sentinel of
// a thread without cells and becomes the FP64 1e30 on every path.
template <class T>
__device__ __forceinline__ void cfl_block_reduce(T dtp, int bad, StepScalars* sc) {
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(&sc->err, GCH_ERR_DT);
  for (int o = 16; o > 0; o >>= 1) dtp = tmin_(dtp, __shfl_xor_sync(0xffffffffu, dtp, o));
  __shared__ T red[32];
  const int t = threadIdx.y * blockDim.x + threadIdx.x;
  const int lane = t & 31, wid = t >> 5;
  if (lane == 0) red[wid] = dtp;
  __syncthreads();
  if (wid == 0) {
    const int nw = (blockDim.x * blockDim.y) >> 5;
    T v = lane < nw ? red[lane] : T(1e30);
    for (int o = 16; o > 0; o >>= 1) v = tmin_(v, __shfl_xor_sync(0xffffffffu, v, o));
    const double m = v < T(1e30) ? (double)v : 1e30;
    // positive doubles order like their bit patterns
    if (lane == 0) atomicMin(&sc->dtmin_bits, (unsigned long long)__double_as_longlong(m));
  }
}

// ---------------------------------------------------------------------------
// Constrained transport of B (src/flux_cd_module.f90:311-321) with the E
// ghost layer of boundaryI_ef (:45-237) applied as an index map.
template <class Pol, int STAGE>
__device__ __forceinline__ void
ct_body(const KParams& p, const typename Pol::TU* u,
        typename std::conditional<STAGE == 1, typename Pol::TS, typename Pol::TU>::type* dst,
        const typename Pol::TS* __restrict__ E, const typename Pol::TS* __restrict__ s678,
        StepScalars* sc, int kz, int bx, int by, int bz) {
  using TC = typename Ops<Pol>::TC;
  using TD = typename std::conditional<STAGE == 1, typename Pol::TS, typename Pol::TU>::type;
  if (!sc->active) return;
  const int ci = bx * 32 + threadIdx.x;
  const int cj = by * 8 + threadIdx.y;
  const int kb = bz * kz;
  const int ke = min(p.nz, kb + kz);
  const bool active = ci < p.nx && cj < p.ny;
  if (!active) return;
  const int ax = ci + NG, ay = cj + NG;
  const double dt = STAGE == 1 ? sc->dt / 2.0 : sc->dt;
  const float dtf = (float)dt;
  const TC hx = par<TC>(0.5 * sc->dtd[STAGE - 1][0], sc->hdtdf[STAGE - 1][0]);
  const TC hy = par<TC>(0.5 * sc->dtd[STAGE - 1][1], sc->hdtdf[STAGE - 1][1]);
  const TC hz = par<TC>(0.5 * sc->dtd[STAGE - 1][2], sc->hdtdf[STAGE - 1][2]);

  // E at the face neighbours of this column.  The ghost layer follows
  // boundaryI_ef (src/flux_cd_module.f90:45-237): periodic copy, outflow
  // copy, closed copy with the normal component of the x/y walls negated and
  // nothing negated on z walls.  The CT reads E1 only at y and z neighbours,
  // E2 only at x and z neighbours and E3 only in the plane, so a neighbour
  // beyond a wall is its source cell with no sign change, and every
  // neighbour is a fixed offset from the cell: the x/y offsets are mapped
  // once per column, the z ones at the box's bottom and top planes.
  // 32-bit cell offsets: a padded field is below 2^31 cells (larger boxes are
  // refused at creation).
  bool f_;
  const int pitch = p.pitch, plane = p.pitch * p.NY;
  const int oxm = ghost_src(ax - 1, p.nx, p.bc[0], p.bc[1], f_) - ax;
  const int oxp = ghost_src(ax + 1, p.nx, p.bc[0], p.bc[1], f_) - ax;
  const int oym = (ghost_src(ay - 1, p.ny, p.bc[2], p.bc[3], f_) - ay) * pitch;
  const int oyp = (ghost_src(ay + 1, p.ny, p.bc[2], p.bc[3], f_) - ay) * pitch;
  const int ozb = (ghost_src(kb + NG - 1, p.nz, p.bc[4], p.bc[5], f_) - (kb + NG)) * plane;
  const int ozt = (ghost_src(p.nz + NG, p.nz, p.bc[4], p.bc[5], f_) - (p.nz + NG - 1)) * plane;
  const long long fs = p.fs;
  const typename Pol::TS* __restrict__ E1 = E;
  const typename Pol::TS* __restrict__ E2 = E + fs;
  const typename Pol::TS* __restrict__ E3 = E + 2 * fs;
  const typename Pol::TU* U6 = u + 5 * fs;
  const typename Pol::TU* U7 = u + 6 * fs;
  const typename Pol::TU* U8 = u + 7 * fs;
  TD* D6 = dst + 5 * fs;
  TD* D7 = dst + 6 * fs;
  TD* D8 = dst + 7 * fs;
  int c = (int)cell_index(p, ax, ay, kb + NG);

  // E1 and E2 of this column at planes k-1 and k: the z neighbours march
  // with the column, so each plane loads only its k+1 values
  TC e1m = (TC)E1[c + ozb], e2m = (TC)E2[c + ozb];
  TC e1c = (TC)E1[c], e2c = (TC)E2[c];
  for (int k = kb; k < ke; ++k, c += plane) {
    if (k + 1 < ke) {  // next plane's B and E into L2 (no registers held)
      asm volatile("prefetch.global.L2 [%0];" ::"l"(U6 + c + plane));
      asm volatile("prefetch.global.L2 [%0];" ::"l"(U7 + c + plane));
      asm volatile("prefetch.global.L2 [%0];" ::"l"(U8 + c + plane));
      asm volatile("prefetch.global.L2 [%0];" ::"l"(E3 + c + plane));
      if (k + 2 < p.nz) {
        asm volatile("prefetch.global.L2 [%0];" ::"l"(E1 + c + 2 * plane));
        asm volatile("prefetch.global.L2 [%0];" ::"l"(E2 + c + 2 * plane));
      }
    }
    const int oz = k + 1 < p.nz ? plane : ozt;  // the plane above, or its source
    const TC e1p = (TC)E1[c + oz], e2p = (TC)E2[c + oz];
    const TC e2zm = e2m, e2zp = e2p, e1zm = e1m, e1zp = e1p;
    e1m = e1c; e2m = e2c; e1c = e1p; e2c = e2p;
    const TC e3ym = (TC)E3[c + oym], e3yp = (TC)E3[c + oyp];
    const TC e3xm = (TC)E3[c + oxm], e3xp = (TC)E3[c + oxp];
    const TC e2xm = (TC)E2[c + oxm], e2xp = (TC)E2[c + oxp];
    const TC e1ym = (TC)E1[c + oym], e1yp = (TC)E1[c + oyp];
    const auto u6 = Ops<Pol>::ld(U6[c]);
    const auto u7 = Ops<Pol>::ld(U7[c]);
    const auto u8 = Ops<Pol>::ld(U8[c]);
    // src/flux_cd_module.f90:311-321
    if constexpr (sizeof(TC) == 4) {
      // FP32 paths: the eight-wave terms join the FP32 differences (zero
      // without them).  Added after the CT under `if (p.eight_wave)`, the
      // grouped kernel evaluated them for every cell and selected.
      TC s6 = TC(0), s7 = TC(0), s8 = TC(0);
      if (p.eight_wave) {
        s6 = (TC)s678[c];
        s7 = (TC)s678[fs + c];
        s8 = (TC)s678[2 * fs + c];
      }
      D6[c] = store_as<TD>(Ops<Pol>::ct_src(u6, hy, e3ym, e3yp, hz, e2zm, e2zp, true, dtf, s6));
      D7[c] = store_as<TD>(Ops<Pol>::ct_src(u7, hx, e3xm, e3xp, hz, e1zm, e1zp, false, dtf, s7));
      D8[c] = store_as<TD>(Ops<Pol>::ct_src(u8, hx, e2xm, e2xp, hy, e1ym, e1yp, true, dtf, s8));
    } else {
      auto b6 = Ops<Pol>::ct(u6, hy, e3ym, e3yp, hz, e2zm, e2zp, true);
      auto b7 = Ops<Pol>::ct(u7, hx, e3xm, e3xp, hz, e1zm, e1zp, false);
      auto b8 = Ops<Pol>::ct(u8, hx, e2xm, e2xp, hy, e1ym, e1yp, true);
      if (p.eight_wave) {
        b6 = add_source<Pol>(b6, dt, dtf, s678[c]);
        b7 = add_source<Pol>(b7, dt, dtf, s678[fs + c]);
        b8 = add_source<Pol>(b8, dt, dtf, s678[2 * fs + c]);
      }
      D6[c] = store_as<TD>(b6);
      D7[c] = store_as<TD>(b7);
      D8[c] = store_as<TD>(b8);
    }
  }
}

// block (32, 8); grid (ceil(nx/32), ceil(ny/8), z chunks of kz planes from
// chunk bz0).  Enough blocks per SM to keep loads in flight for this bandwidth-bound update: four for
// stage 1, six for stage 2 (measured on the 256^3 turbulence box: stage 2
// 0.202 -> 0.184 ms with six; stage 1 0.180 -> 0.184 ms, so it keeps four).
template <class Pol, int STAGE>
__global__ void __launch_bounds__(256, STAGE == 2 ? 6 : 4)
k_ct(KParams p, const typename Pol::TU* u,
     typename std::conditional<STAGE == 1, typename Pol::TS, typename Pol::TU>::type* dst,
     const typename Pol::TS* __restrict__ E, const typename Pol::TS* __restrict__ s678,
     StepScalars* sc, int kz, int bz0 = 0) {
  ct_body<Pol, STAGE>(p, u, dst, E, s678, sc, kz, blockIdx.x, blockIdx.y, blockIdx.z + bz0);
}

// ---------------------------------------------------------------------------
// Ghost fill of one axis (src/boundaries.f90:44-512): `layers` ghost layers
// on both sides of `axis`, over the whole transverse extent.
template <class T>
__device__ __forceinline__ void ghost_body(const KParams& p, T* a, int neq, int axis, int layers,
                                           const StepScalars* sc, int bx, int by, int bz) {
  if (!sc->active) return;
  const int t0 = bx * 128 + threadIdx.x;  // transverse fast index
  const int t1 = by;                      // transverse slow index
  const int side_layer = bz;              // 2*layers entries
  const int side = side_layer & 1;
  const int l = side_layer >> 1;
  int n, N0, N1, blo, bhi;
  if (axis == 0) { n = p.nx; N0 = p.NY; N1 = p.NZ; blo = p.bc[0]; bhi = p.bc[1]; }
  else if (axis == 1) { n = p.ny; N0 = p.NX; N1 = p.NZ; blo = p.bc[2]; bhi = p.bc[3]; }
  else { n = p.nz; N0 = p.NX; N1 = p.NY; blo = p.bc[4]; bhi = p.bc[5]; }
  if (t0 >= N0 || t1 >= N1 || l >= layers) return;
  const int bc = side ? bhi : blo;
  if (bc == GCH_BC_OTHER) return;
  const int g = side ? NG + n + l : NG - 1 - l;
  bool flip;
  const int s = ghost_src(g, n, blo, bhi, flip);
  int dx, dy, dz, sx, sy, sz;
  if (axis == 0) { dx = g; sx = s; dy = sy = t0; dz = sz = t1; }
  else if (axis == 1) { dy = g; sy = s; dx = sx = t0; dz = sz = t1; }
  else { dz = g; sz = s; dx = sx = t0; dy = sy = t1; }
  const long long di = cell_index(p, dx, dy, dz), si = cell_index(p, sx, sy, sz);
  for (int q = 0; q < neq; ++q) {
    T v = a[q * p.fs + si];
    if (flip && q == axis + 1) v = neg(v);
    a[q * p.fs + di] = v;
  }
}

// ---------------------------------------------------------------------------
// All ghost layers of one fill in one launch.  The x, y and z fills of
// src/boundaries.f90 run one after the other and each copies whole planes,
// the other axes' ghosts included, so every ghost cell ends up with the value
// of one interior cell: per axis, a coordinate in a filled layer of a wall
// with a rule maps to its source (periodic wrap or mirror), any other
// coordinate stays, and each closed wall crossed negates its normal momentum
// once.  When every side is at least `layers` cells long no source is a cell
// that this launch writes, so the cells can be filled in any order.
//
// Cell t in [0, ghost_all_count) enumerates the z band (all x, y), then the
// y band outside it (all x), then the x band outside both.
__host__ __device__ inline long long ghost_all_count(const KParams& p, int L) {
  const long long b = 2 * L;
  return b * p.NX * p.NY + (p.NZ - b) * b * p.NX + (p.NZ - b) * (p.NY - b) * b;
}
__host__ __device__ inline bool ghost_all_ok(const KParams& p, int L) {
  return p.nx >= L && p.ny >= L && p.nz >= L;
}
// layer b of the band: 0..L-1 below the interior, L..2L-1 above it
__device__ __forceinline__ int ghost_band(int b, int L, int n) {
  return b < L ? NG - 1 - b : NG + n + (b - L);
}
// the i-th coordinate outside the band
__device__ __forceinline__ int ghost_rest(int i, int L, int n) {
  return i < NG - L ? i : (i < NG - L + n ? i + L : i + 2 * L);
}
// source coordinate of c along one axis, or c itself
__device__ __forceinline__ int ghost_map(int c, int n, int L, int blo, int bhi, bool& flip) {
  flip = false;
  const bool lo = c < NG && c >= NG - L, hi = c >= NG + n && c < NG + n + L;
  if (!lo && !hi) return c;
  if ((lo ? blo : bhi) == GCH_BC_OTHER) return c;
  return ghost_src(c, n, blo, bhi, flip);
}
// the ghost cell (ax, ay, az) from its interior source
template <class T>
__device__ __forceinline__ void ghost_fill_at(const KParams& p, T* a, int neq, int L, int ax,
                                              int ay, int az) {
  bool fx, fy, fz;
  const int sx = ghost_map(ax, p.nx, L, p.bc[0], p.bc[1], fx);
  const int sy = ghost_map(ay, p.ny, L, p.bc[2], p.bc[3], fy);
  const int sz = ghost_map(az, p.nz, L, p.bc[4], p.bc[5], fz);
  if (sx == ax && sy == ay && sz == az) return;  // only walls without a rule
  const long long di = cell_index(p, ax, ay, az), si = cell_index(p, sx, sy, sz);
  for (int q = 0; q < neq; ++q) {
    T v = a[q * p.fs + si];
    if ((fx && q == 1) || (fy && q == 2) || (fz && q == 3)) v = neg(v);
    a[q * p.fs + di] = v;
  }
}
template <class T>
__device__ __forceinline__ void ghost_all_cell(const KParams& p, T* a, int neq, int L,
                                               long long t) {
  const long long b = 2 * L;
  const long long cz = b * p.NX * p.NY, cy = (p.NZ - b) * b * p.NX;
  int ax, ay, az;
  if (t < cz) {
    ax = (int)(t % p.NX);
    const long long r = t / p.NX;
    ay = (int)(r % p.NY);
    az = ghost_band((int)(r / p.NY), L, p.nz);
  } else if (t < cz + cy) {
    t -= cz;
    ax = (int)(t % p.NX);
    const long long r = t / p.NX;
    ay = ghost_band((int)(r % b), L, p.ny);
    az = ghost_rest((int)(r / b), L, p.nz);
  } else {
    t -= cz + cy;
    ax = ghost_band((int)(t % b), L, p.nx);
    const long long r = t / b;
    ay = ghost_rest((int)(r % (p.NY - b)), L, p.ny);
    az = ghost_rest((int)(r / (p.NY - b)), L, p.nz);
  }
  ghost_fill_at<T>(p, a, neq, L, ax, ay, az);
}

// block 256; grid-stride over ghost_all_count cells (with zband_only, the z
// band alone: the ghost planes of z, which come first in that order)
template <class T>
__global__ void __launch_bounds__(256) k_ghost_all(KParams p, T* a, int neq, int layers,
                                                   const StepScalars* sc, int zband_only = 0) {
  if (!sc->active) return;
  const long long n = zband_only ? 2LL * layers * p.NX * p.NY : ghost_all_count(p, layers);
  for (long long t = blockIdx.x * 256LL + threadIdx.x; t < n; t += (long long)gridDim.x * 256)
    ghost_all_cell<T>(p, a, neq, layers, t);
}

// The x and y ghost cells of the interior planes az in [az0, az1) (array
// coordinates), the cells of those planes that the whole-shell fill writes:
// per plane the y band over every x, then the x band over the other rows.
// Their sources lie in the same plane, so a slab of planes can be filled as
// soon as its interior cells are final.  block 256; grid-stride.
template <class T>
__global__ void __launch_bounds__(256) k_ghost_ring(KParams p, T* a, int neq, int L, int az0,
                                                    int az1, const StepScalars* sc) {
  if (!sc->active) return;
  const long long b = 2 * L;
  const long long per = b * p.NX + (p.NY - b) * b;
  const long long n = per * (az1 - az0);
  for (long long t = blockIdx.x * 256LL + threadIdx.x; t < n; t += (long long)gridDim.x * 256) {
    const int az = az0 + (int)(t / per);
    long long r = t % per;
    int ax, ay;
    if (r < b * p.NX) {
      ax = (int)(r % p.NX);
      ay = ghost_band((int)(r / p.NX), L, p.ny);
    } else {
      r -= b * p.NX;
      ax = ghost_band((int)(r % b), L, p.nx);
      ay = ghost_rest((int)(r / b), L, p.ny);
    }
    ghost_fill_at<T>(p, a, neq, L, ax, ay, az);
  }
}

// block 128; grid (ceil(N0/128), N1, 2*layers) over the transverse extent
template <class T>
__global__ void k_ghost(KParams p, T* a, int neq, int axis, int layers, const StepScalars* sc) {
  ghost_body<T>(p, a, neq, axis, layers, sc, blockIdx.x, blockIdx.y, blockIdx.z);
}

// A sphere at time t: as given, or moved along its circular orbit in the
// x-z plane (EXO/exoplanet.f90:143-148: XP = Rorb cos(omegap t + phi),
// ZP = Rorb sin(omegap t + phi), and the orbital velocity).
__device__ __forceinline__ gch_sphere_t sphere_at(const gch_sphere_t& s0, double t) {
  gch_sphere_t s = s0;
  if (s.orbit_omega != 0.0) {
    double sn, cs;
    sincos(__dadd_rn(__dmul_rn(s.orbit_omega, t), s.orbit_phase), &sn, &cs);
    s.xc = __dmul_rn(s.orbit_r, cs);
    s.zc = __dmul_rn(s.orbit_r, sn);
    s.vorb[0] = __dmul_rn(__dmul_rn(-s.orbit_omega, s.orbit_r), sn);
    s.vorb[1] = 0.0;
    s.vorb[2] = __dmul_rn(__dmul_rn(s.orbit_omega, s.orbit_r), cs);
  }
  return s;
}

// User boundary spheres (EXO/exoplanet.f90:125-266 pattern) over the box
// [lo, hi) of array coordinates of sphere `m`; the first sphere containing a
// cell wins.
// Body for block `blk` of the `nblk` blocks given to sphere `m`.
template <class T>
__device__ __forceinline__ void user_bc_body(const KParams& p, T* a, int neq,
                                             const StepScalars* sc, int m, int blk, int nblk) {
  if (!sc->active) return;
  const double t = sc->time;
  const gch_sphere_t sp = sphere_at(p.sph[m], t);
  // bounding box of the sphere in array coordinates, clipped to the array
  auto lo_hi = [&](double c, double r, double d, int n, int N, int& lo, int& hi) {
    // cell centre of array coordinate a: ((a-NG+1 - n/2) + 0.5)*d
    double amin = (c - r) / d - 0.5 + n / 2 + NG - 1;
    double amax = (c + r) / d - 0.5 + n / 2 + NG - 1;
    lo = max(0, (int)floor(amin) - 1);
    hi = min(N, (int)ceil(amax) + 2);
  };
  // the box once per block (FP64 divides), shared with the block's threads
  __shared__ int box[6];
  if (threadIdx.x == 0) {
    lo_hi(sp.xc, sp.radius, p.dx, p.nx, p.NX, box[0], box[1]);
    lo_hi(sp.yc, sp.radius, p.dy, p.ny, p.NY, box[2], box[3]);
    lo_hi(sp.zc, sp.radius, p.dz, p.nz, p.NZ, box[4], box[5]);
  }
  __syncthreads();
  const int xl = box[0], xh = box[1], yl = box[2], yh = box[3], zl = box[4], zh = box[5];
  const long long wx = xh - xl, wy = yh - yl, wz = zh - zl;
  if (wx <= 0 || wy <= 0 || wz <= 0) return;
  const long long total = wx * wy * wz;
  for (long long t = blk * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)nblk * blockDim.x) {
    const int ax = xl + (int)(t % wx);
    const int ay = yl + (int)((t / wx) % wy);
    const int az = zl + (int)(t / (wx * wy));
    const double x = cell_pos(ax, p.nx, p.dx);
    const double y = cell_pos(ay, p.ny, p.dy);
    const double z = cell_pos(az, p.nz, p.dz);
    bool earlier = false;
    for (int e = 0; e < m; ++e) {
      const gch_sphere_t q = sphere_at(p.sph[e], t);
      const double xs = x - q.xc, ys = y - q.yc, zs = z - q.zc;
      if (sqrt(xs * xs + ys * ys + zs * zs) <= q.radius) { earlier = true; break; }
    }
    if (earlier) continue;
    const double xs = x - sp.xc, ys = y - sp.yc, zs = z - sp.zc;
    double rads = sqrt(xs * xs + ys * ys + zs * zs);
    if (!(rads <= sp.radius)) continue;
    if (rads == 0.0) rads = p.dx * 0.10;
    const double velx = sp.vorb[0] + sp.vwind * xs / rads;
    const double vely = sp.vorb[1] + sp.vwind * ys / rads;
    const double velz = sp.vorb[2] + sp.vwind * zs / rads;
    const double dens = sp.dens;
    const long long c = cell_index(p, ax, ay, az);
    a[c] = from_d<T>(dens);
    a[p.fs + c] = from_d<T>(dens * velx);
    a[2 * p.fs + c] = from_d<T>(dens * vely);
    a[3 * p.fs + c] = from_d<T>(dens * velz);
    double b2 = 0.0;
    if (neq >= 8) {
      const double rr = sp.radius / rads;
      const double cpi = sp.bdip * (rr * rr * rr) / (2.0 * (rads * rads));
      const double b5 = 3.0 * ys * xs * cpi;
      const double b6 = (3.0 * (ys * ys) - rads * rads) * cpi;
      const double b7 = 3.0 * ys * zs * cpi;
      a[5 * p.fs + c] = from_d<T>(b5);
      a[6 * p.fs + c] = from_d<T>(b6);
      a[7 * p.fs + c] = from_d<T>(b7);
      b2 = b5 * b5 + b6 * b6 + b7 * b7;
    }
    double e = 0.5 * dens * (velx * velx + vely * vely + velz * velz) + p.cv * dens * sp.tfac;
    if (p.mhd) e = e + 0.5 * b2;
    a[4 * p.fs + c] = from_d<T>(e);
  }
}
// grid (blocks per sphere, nsph)
template <class T>
__global__ void k_user_bc(KParams p, T* a, int neq, const StepScalars* sc) {
  user_bc_body<T>(p, a, neq, sc, blockIdx.y, blockIdx.x, gridDim.x);
}

// ---------------------------------------------------------------------------
// CFL reduction (src/hydro_core.f90:644-675): per-cell candidate, warp
// shuffle min, one atomicMin per block on the bits of the positive double.

// With `store` (u as the source) every interior cell's primitives are also
// written to `store` in the stage type: the first stage of the same step
// then reads them instead of recovering them again.
template <class Pol, int NEQ, bool PRIM_IN>
__device__ __forceinline__ void
cfl_body(const KParams& p,
         const typename std::conditional<PRIM_IN, typename Pol::TS, typename Pol::TU>::type* src,
         StepScalars* sc, int kz, int bx, int by, int bz, typename Pol::TS* store = nullptr) {
  using TC = typename Ops<Pol>::TC;
  if (!sc->active) return;
  const int ci = bx * 32 + threadIdx.x;
  const int cj = by * 8 + threadIdx.y;
  const int kb = bz * kz;
  const int ke = min(p.nz, kb + kz);
  const CflConst<TC> kc(p);
  TC dtp = TC(1e30);
  int bad = 0;
  if (ci < p.nx && cj < p.ny) {
    unsigned pfl = 0;
    for (int k = kb; k < ke; ++k) {
      const long long c = cell_index(p, ci + NG, cj + NG, k + NG);
      TC pr[NEQ];
      if constexpr (PRIM_IN)
        Ops<Pol>::template load_stored_prim<NEQ>(p, src, c, pr);
      else
        Ops<Pol>::template load_prim<NEQ>(p, src, c, pr, pfl);
      if (!PRIM_IN && store) {
#pragma unroll
        for (int q = 0; q < NEQ; ++q) store[q * p.fs + c] = (typename Pol::TS)pr[q];
      }
      cfl_candidate<TC, NEQ>(p, kc, pr, dtp, bad);
    }
    if (pfl) atomicAdd(&sc->pfloor, (unsigned long long)pfl);
  }
  cfl_block_reduce<TC>(dtp, bad, sc);
}

// block (32, 8); grid (ceil(nx/32), ceil(ny/8), z chunks of kz planes from
// chunk bz0)
template <class Pol, int NEQ, bool PRIM_IN>
__global__ void __launch_bounds__(256)
k_cfl(KParams p, const typename std::conditional<PRIM_IN, typename Pol::TS, typename Pol::TU>::type* src,
      StepScalars* sc, int kz, typename Pol::TS* store = nullptr, int bz0 = 0) {
  cfl_body<Pol, NEQ, PRIM_IN>(p, src, sc, kz, blockIdx.x, blockIdx.y, blockIdx.z + bz0, store);
}

// get_timestep's scalar tail (src/hydro_core.f90:677-694) and the bookkeeping
// of the device time loop (src/main.f90:94-125).
__device__ __forceinline__ void dtfin_body(StepScalars* sc, double cfl, double dx, double dy,
                                           double dz) {
  if (!sc->active) return;
  double dtp = __longlong_as_double((long long)sc->dtmin_bits);
  sc->dtmin_bits = 0x7FF0000000000000ull;  // +inf for the next reduction
  if (sc->iter <= sc->n_iter)
    dtp = cfl * ldexp(1.0, -(sc->n_iter + 1 - sc->iter)) * dtp;
  else
    dtp = cfl * dtp;
  double dt = dtp;
  int dump = 0;
  if ((sc->time + dt) >= sc->tprint) {
    dt = sc->tprint - sc->time;
    dump = 1;
  }
  if (!(dt > 0.0) || !(dt < 1e300)) sc->err |= GCH_ERR_DT;
  sc->dt = dt;
  sc->dump = dump;
  set_stage_ratios(sc, dx, dy, dz);
}
static __global__ void k_dtfin(StepScalars* sc, double cfl, double dx, double dy, double dz) {
  dtfin_body(sc, cfl, dx, dy, dz);
}

// Time-loop tail after a tstep (src/main.f90:108-123): device-resident loop.
__device__ __forceinline__ void loopfin_body(StepScalars* sc) {
  if (!sc->active) return;
  sc->time = sc->time + sc->dt;
  if (sc->dump) {
    sc->tprint = sc->tprint + sc->dtprint;
    sc->dump = 0;
  }
  sc->iter = sc->iter + 1;
  sc->active = (sc->time <= sc->tmax) && sc->err == 0;
}
static __global__ void k_loopfin(StepScalars* sc) { loopfin_body(sc); }

// Table cooling on the FP32 paths: the primitives from the path's own
// conversion (FP64 or compensated pressure recovery) and the update of
// src/cooling_dmc.f90:136-150 in FP32, from the FP32 rows of the table.  The
// energy change is taken as Eth0 * expm1(-Ce dt tsc), which equals the
// reference's -Eth0 + cv p exp(-Ce dt tsc) but keeps a loss below the FP32
// rounding of exp(); it is added to the FP64 or compensated u(5).
template <class Pol, int NEQ>
__device__ __forceinline__ void cool_f32(const KParams& p, typename Pol::TU* u,
                                         typename Pol::TS* primit, const StepScalars* sc,
                                         long long c) {
  float pr[NEQ];
  unsigned pfl = 0;
  Ops<Pol>::template load_prim<NEQ>(p, (const typename Pol::TU*)u, c, pr, pfl);
  const float r = pr[0];
  float T;
  if (NEQ > kNeqDyn<NEQ> && p.eos == GCH_EOS_H_RATE)
    T = (pr[4] / tmax_(2.0f * r - pr[kNeqDyn<NEQ>], 1e-15f)) * p.f_Tempsc;
  else
    T = (pr[4] / r) * p.f_Tempsc;
  if (T > p.f_tab_Tmin) {
    const float Eth0 = p.f_cv * pr[4];
    float aloss;
    if (T > 1e8f) {
      aloss = p.f_tab_tail * sqrtf(T);
    } else {
      int if1 = (int)(log10f(T) * p.f_tab_inv_dlog) - p.tab_i0;
      if1 = max(0, min(if1, p.ntab - 2));
      const float T0 = p.tabTf[if1], c0 = p.tabLf[if1];
      const float T1 = p.tabTf[if1 + 1], c1 = p.tabLf[if1 + 1];
      aloss = (c1 - c0) * (T - T0) / (T1 - T0) + c0;
    }
    const float ce = (aloss * (r * r)) / (Eth0 * p.f_Psc);
    const float em1 = expm1f(-ce * (float)(sc->dt * p.tsc));
    const float dE = Eth0 * em1;
    if constexpr (std::is_same<Pol, PolKahan>::value)
      u[4 * p.fs + c] = Ops<PolKahan>::addf(u[4 * p.fs + c], dE);
    else
      u[4 * p.fs + c] = u[4 * p.fs + c] + (double)dE;
    pr[4] = fmaf(pr[4], em1, pr[4]);
  }
#pragma unroll
  for (int q = 0; q < NEQ; ++q) primit[q * p.fs + c] = pr[q];
}

// ---------------------------------------------------------------------------
// Tabulated cooling (src/cooling_dmc.f90:115-156, src/cooling_chi.f90:114-154).
// The FP64 path computes in FP64 throughout, as the reference (Lambda in
// real(8)); the FP32 paths use cool_f32.  Writes primit of every interior
// cell and u(5) of the cooled ones.
template <class Pol, int NEQ>
__device__ __forceinline__ void cool_body(const KParams& p, typename Pol::TU* u,
                                          typename Pol::TS* primit, StepScalars* sc, int ci,
                                          int cj, int ck) {
  if (ci >= p.nx || cj >= p.ny || !sc->active) return;
  const long long c = cell_index(p, ci + NG, cj + NG, ck + NG);
  if constexpr (!std::is_same<Pol, PolFP64>::value) {
    cool_f32<Pol, NEQ>(p, u, primit, sc, c);
  } else {
    double uu[NEQ], pp[NEQ];
#pragma unroll
    for (int q = 0; q < NEQ; ++q) uu[q] = to_d(u[q * p.fs + c]);
    unsigned pfl = 0;
    double T;
    Ops<PolFP64>::u2prim<NEQ>(p, uu, pp, pfl, &T);
    if (T > p.tab_Tmin) {
      const double Eth0 = p.cv * pp[4];
      double aloss;
      if (T > 1e8) {
        aloss = p.tab_tail * sqrt(T);
      } else {
        int if1 = (int)(log10(T) * p.tab_inv_dlog) - p.tab_i0;
        if1 = max(0, min(if1, p.ntab - 2));
        const double T0 = p.tabT[if1], c0 = p.tabL[if1];
        const double T1 = p.tabT[if1 + 1], c1 = p.tabL[if1 + 1];
        aloss = (c1 - c0) * (T - T0) / (T1 - T0) + c0;
      }
      const double dens = pp[0];
      const double ce = (aloss * (dens * dens)) / (Eth0 * p.Psc);
      pp[4] = pp[4] * exp(-ce * (sc->dt * p.tsc));
      u[4 * p.fs + c] = from_d<typename Pol::TU>(uu[4] - Eth0 + p.cv * pp[4]);
    }
#pragma unroll
    for (int q = 0; q < NEQ; ++q) primit[q * p.fs + c] = (typename Pol::TS)pp[q];
  }
}
// block (32, 8); grid (ceil(nx/32), ceil(ny/8), nz)
template <class Pol, int NEQ>
__global__ void k_cool(KParams p, typename Pol::TU* u, typename Pol::TS* primit,
                       StepScalars* sc) {
  cool_body<Pol, NEQ>(p, u, primit, sc, blockIdx.x * blockDim.x + threadIdx.x,
                      blockIdx.y * blockDim.y + threadIdx.y, blockIdx.z);
}

// COOL_H (src/cooling_h.f90): non-equilibrium ionisation of hydrogen and
// the parametrised cooling tied to it, per interior cell, FP64 (the
// reference computes it in real(8)).  The first passive scalar is the
// neutral hydrogen density.
namespace coolh {
// T is double on the FP64 path (the reference's expressions) and float on
// the FP32 paths
template <class T>
__device__ __forceinline__ T tpow(T x, T y) { return pow(x, y); }
template <>
__device__ __forceinline__ float tpow(float x, float y) { return powf(x, y); }
template <class T>
__device__ __forceinline__ T texp(T x) { return exp(x); }
template <>
__device__ __forceinline__ float texp(float x) { return expf(x); }
template <class T>
__device__ __forceinline__ T tlog(T x) { return log(x); }
template <>
__device__ __forceinline__ float tlog(float x) { return logf(x); }

template <class T>
__device__ __forceinline__ T alpha(T t) { return T(2.55e-13) * tpow(T(1.e4) / t, T(0.79)); }
template <class T>
__device__ __forceinline__ T colf(T t) {
  return T(5.83e-11) * tsqrt(t) * texp(T(-157828.) / t);
}
template <class T>
__device__ __forceinline__ T betah(T t) {
  const T a = T(157890.) / t;
  return T(1.133e-24) / tsqrt(a) * (T(-0.0713) + T(0.5) * tlog(a) + T(0.640) * tpow(a, T(-0.33333)));
}
// :155-242 ALOSS (X2 and DT enter only a quantity the reference does not use)
template <class T>
__device__ __forceinline__ T aloss(T X1, T DEN, T DH0, T TE0) {
  const T XION = 2.179e-11, XO = 1.e-3;
  const T C0 = 0.5732, C1 = 1.8288e-5, C2 = -1.15822e-10, C3 = 9.4288e-16;
  const T D0 = 0.5856, D1 = 1.55083e-5, D2 = -9.669e-12, D3 = 5.716e-19;
  const T ENK = 118409., EN = 1.634E-11;
  const T one = 1.;
  const T TE = tmax_(TE0, T(10.));
  const T DH = DEN;
  const T DHP = (one - X1) * DH;
  const T DE = DHP + T(1.E-4) * DH;
  const T DOI = XO * DH0;
  const T DOII = XO * DHP;
  if (TE <= T(1e4)) return 0.;
  T OMEGA = 0.0;
  if (TE <= T(55000.)) OMEGA = C0 + TE * (C1 + TE * (C2 + TE * C3));
  if (TE >= T(72000.)) OMEGA = D0 + TE * (D1 + TE * (D2 + TE * D3));
  if (TE > T(55000.) && TE < T(72000.)) {
    const T OMEGAL = C0 + TE * (C1 + TE * (C2 + TE * C3));
    const T OMEGAH = D0 + TE * (D1 + TE * (D2 + TE * D3));
    const T FRAC = (TE - T(55000.)) / T(17000.);
    OMEGA = (one - FRAC) * OMEGAL + FRAC * OMEGAH;
  }
  const T QLA = T(8.6287E-6) / (T(2.) * tsqrt(TE)) * OMEGA * texp(-ENK / TE);
  const T ECOLL = tmax_(DE * DH0 * QLA * EN, T(0.));
  const T CION = T(5.834E-11) * tsqrt(TE) * texp(T(-1.579E5) / TE);
  const T EION = DE * DH0 * CION * XION;
  const T EREC = tmax_(DE * DHP * (betah(TE)), T(0.));
  const T TM = one / TE;
  const T T2 = TM * TM;
  const T EOI =
      tmax_(DE * DOI * tpow(T(10.), T(1381465) * T2 - T(12328.69) * TM - T(19.82621)), T(0.));
  const T EOII =
      tmax_(DE * DOII * tpow(T(10.), T(-2061075.) * T2 - T(14596.24) * TM - T(19.01402)), T(0.));
  const T BETAF = T(1.3 * 1.42E-27) * tpow(TE, T(0.5));
  const T HIICOOL = DE * DHP * BETAF;
  const T EQUIL = (T(1.0455E-18) / tpow(TE, T(0.63))) *
                      (one - texp(-tpow(TE * T(1.E-5), T(1.63)))) * DE * DEN +
                  HIICOOL;
  T FR = 0.0;
  if (TE >= T(54770.)) FR = 1.;
  if (TE > T(44770.) && TE < T(54770.)) {
    const T EX2 = texp(T(-2.) * (TE - T(49770.)) / T(500.));
    const T TANH = (one - EX2) / (one + EX2);
    FR = T(0.5) * (one + TANH);
  }
  return ECOLL + EION + (EREC + T(7.033) * (EOI + EOII)) * (one - FR) + EQUIL * FR;
}
}  // namespace coolh

// COOL_H on the FP32 paths: the same update in FP32 from the path's own
// primitives.  Two changes keep it accurate in FP32:
//  - the discriminant of the ionisation quadratic, b^2 - 4ac, cancels to
//    about 1e-8 of its terms; it equals (xi*rec + (1 + xi)*col)^2 exactly,
//    and d is taken as that sum;
//  - the new total energy differs from the stored one only by the thermal
//    part, cv*((2 rho - n_HI') T' - (2 rho - n_HI) T)/Tempsc, which is added
//    to the FP64 or compensated u(5).  Where the pressure floor or the 1 K
//    clamp acted, the stored energy is not cv p + KE + B^2/2 and the
//    reference's value is stored instead.
template <class Pol, int NEQ>
__device__ __forceinline__ void cool_h_f32(const KParams& p, typename Pol::TU* u,
                                           const StepScalars* sc, long long c) {
  constexpr int ND = kNeqDyn<NEQ>;
  float pr[NEQ];
  unsigned pfl = 0;
  Ops<Pol>::template load_prim<NEQ>(p, (const typename Pol::TU*)u, c, pr, pfl);
  const float rho = pr[0], nhi = pr[ND];
  const float dent0 = p.eos == GCH_EOS_H_RATE ? tmax_(2.0f * rho - nhi, 1e-15f) : rho;
  const float T = (pr[4] / dent0) * p.f_Tempsc;
  const bool clamped = pfl != 0 || (p.eos != GCH_EOS_ADIABATIC && !(T > 1.001f));
  const float dt = (float)(sc->dt * p.tsc);
  const float xi = 1.e-4f, boltzm = 1.3807e-16f;
  const float col = coolh::colf(T);
  const float rec = coolh::alpha(T);
  const float y0 = nhi / rho;
  const float dh = rho;
  const float a = rec + col;
  const float b = -((2.f + xi) * rec + (1.f + xi) * col);
  const float d = xi * rec + (1.f + xi) * col;
  const float g0 = (2.f * a * y0 + b + d) / (2.f * a * y0 + b - d);
  const float e = expf(-d * dh * dt);
  float y1 = (-b - d * (1.f + g0 * e) / (1.f - g0 * e)) / (2.f * a);
  y1 = tmin_(y1, 0.9999f);
  y1 = tmax_(y1, 0.f);
  const float al = coolh::aloss(y0, dh, nhi, T) / (dh * dh);
  const float tprime = 10.f;
  const float ce = (2.f * dh * al) / (3.f * boltzm * T);
  float t1 = tprime + (T - tprime) * expf(-ce * dt);
  t1 = tmax_(t1, 0.1f * T);
  t1 = tmin_(t1, 10.f * T);
  const float nhi1 = y1 * rho;
  const float eth1 = p.f_cv * (2.f * rho - nhi1) * t1 / p.f_Tempsc;
  if constexpr (std::is_same<Pol, PolKahan>::value) {
    u[ND * p.fs + c] = make_float2(nhi1, 0.f);
    if (clamped) {
      float e5 = eth1 + 0.5f * rho * (pr[1] * pr[1] + pr[2] * pr[2] + pr[3] * pr[3]);
      if (NEQ >= 8 && p.mhd) e5 = e5 + 0.5f * (pr[5] * pr[5] + pr[6] * pr[6] + pr[7] * pr[7]);
      u[4 * p.fs + c] = make_float2(e5, 0.f);
    } else {
      u[4 * p.fs + c] = Ops<PolKahan>::addf(u[4 * p.fs + c], eth1 - p.f_cv * pr[4]);
    }
  } else {
    u[ND * p.fs + c] = (double)nhi1;
    if (clamped) {
      float e5 = eth1 + 0.5f * rho * (pr[1] * pr[1] + pr[2] * pr[2] + pr[3] * pr[3]);
      if (NEQ >= 8 && p.mhd) e5 = e5 + 0.5f * (pr[5] * pr[5] + pr[6] * pr[6] + pr[7] * pr[7]);
      u[4 * p.fs + c] = (double)e5;
    } else {
      u[4 * p.fs + c] = u[4 * p.fs + c] + (double)(eth1 - p.f_cv * pr[4]);
    }
  }
}

template <class Pol, int NEQ>
__global__ void k_cool_h(KParams p, typename Pol::TU* u, const StepScalars* sc) {
  static_assert(NEQ > kNeqDyn<NEQ>, "COOL_H needs the neutral hydrogen passive");
  constexpr int ND = kNeqDyn<NEQ>;
  const int ci = blockIdx.x * blockDim.x + threadIdx.x;
  const int cj = blockIdx.y * blockDim.y + threadIdx.y;
  const int ck = blockIdx.z;
  if (ci >= p.nx || cj >= p.ny || !sc->active) return;
  const long long c = cell_index(p, ci + NG, cj + NG, ck + NG);
  if constexpr (!std::is_same<Pol, PolFP64>::value) {
    cool_h_f32<Pol, NEQ>(p, u, sc, c);
    return;
  }
  // :259-371 atomic, without diffuse radiation (radphi = 1, tprime = 10 K)
  const double dt = sc->dt * p.tsc;
  const double xi = 1.e-4, boltzm = 1.3807e-16;
  double uu[NEQ], prim[NEQ], T;
#pragma unroll
  for (int q = 0; q < NEQ; ++q) uu[q] = to_d(u[q * p.fs + c]);
  unsigned pfl = 0;
  Ops<PolFP64>::u2prim<NEQ>(p, uu, prim, pfl, &T);
  const double col = coolh::colf(T);
  const double rec = coolh::alpha(T);
  const double y0 = uu[ND] / uu[0];
  const double dh = uu[0];
  const double a = rec + col;
  const double b = -((2. + xi) * rec + (1. + xi) * col);
  const double cc = (1. + xi) * rec;
  const double d = sqrt(b * b - 4. * a * cc);
  const double g0 = (2. * a * y0 + b + d) / (2. * a * y0 + b - d);
  const double e = exp(-d * dh * dt);
  double y1 = (-b - d * (1. + g0 * e) / (1. - g0 * e)) / (2. * a);
  y1 = tmin_(y1, 0.9999);
  y1 = tmax_(y1, 0.);
  const double dh0 = uu[ND];
  const double al = coolh::aloss(y0, dh, dh0, T) / (dh * dh);
  const double tprime = 10.;
  const double ce = (2. * dh * al) / (3. * boltzm * T);
  double t1 = tprime + (T - tprime) * exp(-ce * dt);
  t1 = tmax_(t1, 0.1 * T);
  t1 = tmin_(t1, 10. * T);
  uu[ND] = y1 * uu[0];
  double e5 = p.cv * (2. * uu[0] - uu[ND]) * t1 / p.Tempsc
              + 0.5 * prim[0] * (prim[1] * prim[1] + prim[2] * prim[2] + prim[3] * prim[3]);
  if (NEQ >= 8 && p.mhd) e5 = e5 + 0.5 * (prim[5] * prim[5] + prim[6] * prim[6] + prim[7] * prim[7]);
  u[ND * p.fs + c] = from_d<typename Pol::TU>(uu[ND]);
  u[4 * p.fs + c] = from_d<typename Pol::TU>(e5);
}

// src/hydro_solver.f90:47-65 viscous_copy: u = w + eta*(sum of the six
// neighbours - 6 w); w holds the stage-2 interior, its ghosts are up's.
template <class Pol, int NEQ>
__global__ void k_visc(KParams p, typename Pol::TU* u, const typename Pol::TU* w,
                       const typename Pol::TS* up, const StepScalars* sc) {
  const int ci = blockIdx.x * blockDim.x + threadIdx.x;
  const int cj = blockIdx.y * blockDim.y + threadIdx.y;
  const int ck = blockIdx.z;
  if (ci >= p.nx || cj >= p.ny || !sc->active) return;
  const int ax = ci + NG, ay = cj + NG, az = ck + NG;
  auto val = [&](int q, int x, int y, int z) -> double {
    const bool inside = x >= NG && x < NG + p.nx && y >= NG && y < NG + p.ny && z >= NG &&
                        z < NG + p.nz;
    const long long c = cell_index(p, x, y, z);
    return inside ? to_d(w[q * p.fs + c]) : to_d(up[q * p.fs + c]);
  };
  const long long c = cell_index(p, ax, ay, az);
  if constexpr (!std::is_same<Pol, PolFP64>::value) {
    // FP32 paths: eta times the FP32 Laplacian, added to the cell's FP64 or
    // compensated w (neighbours outside the interior are up's ghosts)
    auto valf = [&](int q, int x, int y, int z) -> float {
      const bool inside = x >= NG && x < NG + p.nx && y >= NG && y < NG + p.ny && z >= NG &&
                          z < NG + p.nz;
      const long long cc = cell_index(p, x, y, z);
      if (!inside) return (float)up[q * p.fs + cc];
      if constexpr (std::is_same<Pol, PolKahan>::value) return w[q * p.fs + cc].x;
      else return (float)w[q * p.fs + cc];
    };
    const float eta = (float)p.eta;
    for (int q = 0; q < NEQ; ++q) {
      const auto wc = w[q * p.fs + c];
      const float v = valf(q, ax, ay, az);
      const float lap = valf(q, ax + 1, ay, az) + valf(q, ax - 1, ay, az) +
                        valf(q, ax, ay + 1, az) + valf(q, ax, ay - 1, az) +
                        valf(q, ax, ay, az + 1) + valf(q, ax, ay, az - 1) - 6.0f * v;
      if constexpr (std::is_same<Pol, PolKahan>::value)
        u[q * p.fs + c] = Ops<PolKahan>::addf(wc, eta * lap);
      else
        u[q * p.fs + c] = wc + (double)(eta * lap);
    }
  } else {
    for (int q = 0; q < NEQ; ++q) {
      const double v = val(q, ax, ay, az);
      u[q * p.fs + c] = from_d<typename Pol::TU>(
          v + p.eta * (val(q, ax + 1, ay, az) + val(q, ax - 1, ay, az) + val(q, ax, ay + 1, az) +
                       val(q, ax, ay - 1, az) + val(q, ax, ay, az + 1) + val(q, ax, ay, az - 1) -
                       6.0 * v));
    }
  }
}

// u2prim of one cell into primit (FP64 arithmetic on every path, as the
// reference's calcprim), stored in the stage type.
template <class Pol, int NEQ>
__device__ __forceinline__ void calcprim_cell(const KParams& p, const typename Pol::TU* u,
                                              typename Pol::TS* primit, long long c) {
  double uu[NEQ], pp[NEQ];
#pragma unroll
  for (int q = 0; q < NEQ; ++q) uu[q] = to_d(u[q * p.fs + c]);
  unsigned pfl = 0;
  Ops<PolFP64>::u2prim<NEQ>(p, uu, pp, pfl);
#pragma unroll
  for (int q = 0; q < NEQ; ++q) primit[q * p.fs + c] = (typename Pol::TS)pp[q];
}

// calcprim of the one-cell ghost shell only (src/hydro_core.f90:258-300 with
// only_ghost): one thread per shell cell of [NG-1, NG+n]^3, the two z planes,
// then the two y rows of every interior plane, then the two x cells of every
// interior row; grid-stride.
// The primitives of one cell with the policy's own recovery (the arithmetic
// of the stage kernels' conversion), stored in the stage type.
template <class Pol, int NEQ>
__device__ __forceinline__ void own_prim_cell(const KParams& p, const typename Pol::TU* u,
                                              typename Pol::TS* primit, long long c) {
  typename Ops<Pol>::TC pr[NEQ];
  unsigned pfl = 0;
  Ops<Pol>::template load_prim<NEQ>(p, u, c, pr, pfl);
#pragma unroll
  for (int q = 0; q < NEQ; ++q) primit[q * p.fs + c] = (typename Pol::TS)pr[q];
}

// OWN: the policy's own recovery (stored primitives of the first stage),
// else the reference's calcprim (table cooling)
template <class Pol, int NEQ, bool OWN = false>
__device__ __forceinline__ void calcprim_shell_body(const KParams& p, const typename Pol::TU* u,
                                                    typename Pol::TS* primit,
                                                    const StepScalars* sc, int blk, int nblk) {
  if (!sc->active) return;
  const long long mx = p.nx + 2, my = p.ny + 2;
  const long long cz = 2 * mx * my, cy = 2LL * p.nz * mx, cx = 2LL * p.nz * p.ny;
  for (long long t = blk * 256LL + threadIdx.x; t < cz + cy + cx;
       t += (long long)nblk * 256) {
    int ax, ay, az;
    if (t < cz) {
      ax = NG - 1 + (int)(t % mx);
      const long long r = t / mx;
      ay = NG - 1 + (int)(r % my);
      az = r / my == 0 ? NG - 1 : NG + p.nz;
    } else if (t < cz + cy) {
      const long long s = t - cz, r = s / mx;
      ax = NG - 1 + (int)(s % mx);
      ay = (r & 1) ? NG + p.ny : NG - 1;
      az = NG + (int)(r >> 1);
    } else {
      const long long s = t - cz - cy, r = s >> 1;
      ax = (s & 1) ? NG + p.nx : NG - 1;
      ay = NG + (int)(r % p.ny);
      az = NG + (int)(r / p.ny);
    }
    if constexpr (OWN) own_prim_cell<Pol, NEQ>(p, u, primit, cell_index(p, ax, ay, az));
    else calcprim_cell<Pol, NEQ>(p, u, primit, cell_index(p, ax, ay, az));
  }
}
template <class Pol, int NEQ>
__global__ void __launch_bounds__(256)
k_calcprim_shell(KParams p, const typename Pol::TU* u, typename Pol::TS* primit,
                 const StepScalars* sc) {
  calcprim_shell_body<Pol, NEQ>(p, u, primit, sc, blockIdx.x, gridDim.x);
}

// The shell part of get_timestep's stored primitives (after the CFL pass
// stored the interior ones); marks them fresh for the next tstep.
template <class Pol, int NEQ>
__global__ void __launch_bounds__(256)
k_prim_shell_own(KParams p, const typename Pol::TU* u, typename Pol::TS* primit,
                 StepScalars* sc) {
  calcprim_shell_body<Pol, NEQ, true>(p, u, primit, sc, blockIdx.x, gridDim.x);
  if (blockIdx.x == 0 && threadIdx.x == 0 && sc->active) sc->prim_fresh = 1;
}

// At the start of tstep: the stored primitives of the interior and the
// one-cell ghost shell, unless get_timestep stored them for this u already
// (a tstep without get_timestep, or after an upload or boundary fill).
// Grid-stride over the (nx+2)(ny+2)(nz+2) cells, a few blocks per SM: when
// the primitives are fresh every block returns at once.
template <class Pol, int NEQ>
__global__ void __launch_bounds__(256)
k_prim_refresh(KParams p, const typename Pol::TU* u, typename Pol::TS* primit,
               const StepScalars* sc) {
  if (sc->prim_fresh || !sc->active) return;
  const long long mx = p.nx + 2, my = p.ny + 2, n = mx * my * (p.nz + 2);
  for (long long t = blockIdx.x * 256LL + threadIdx.x; t < n; t += (long long)gridDim.x * 256) {
    const int ax = NG - 1 + (int)(t % mx);
    const int ay = NG - 1 + (int)((t / mx) % my);
    const int az = NG - 1 + (int)(t / (mx * my));
    own_prim_cell<Pol, NEQ>(p, u, primit, cell_index(p, ax, ay, az));
  }
}

// calcprim over the whole array (src/hydro_core.f90:245-320); writes primit in
// the stored type.  block (32, 8); grid (ceil(NX/32), ceil(NY/8), NZ).
template <class Pol, int NEQ>
__global__ void k_calcprim(KParams p, const typename Pol::TU* u, typename Pol::TS* primit,
                           const StepScalars* sc) {
  const int ax = blockIdx.x * blockDim.x + threadIdx.x;
  const int ay = blockIdx.y * blockDim.y + threadIdx.y;
  const int az = blockIdx.z;
  if (ax >= p.NX || ay >= p.NY || !sc->active) return;
  calcprim_cell<Pol, NEQ>(p, u, primit, cell_index(p, ax, ay, az));
}

// Host layout (Fortran u(neq, x, y, z), FP64, no pitch) <-> device SoA.
// A block moves kLayoutCells consecutive cells per pass: their neq doubles
// each are read (or written) on the host-layout side with consecutive
// threads on consecutive doubles, and exchanged through shared memory with
// the per-field arrays, which are written (or read) one field at a time
// with consecutive threads on consecutive cells.  The host-layout side may
// be the device staging buffer or page-locked host memory mapped into the
// device address space (then these kernels are the host-link transfer).
constexpr int kLayoutCells = 256;
constexpr int kLayoutPad = kMaxNeq + 1;  // odd row stride of the shared tile

__device__ __forceinline__ long long layout_cell(const KParams& p, long long t) {
  const int ax = (int)(t % p.NX);
  const int ay = (int)((t / p.NX) % p.NY);
  const int az = (int)(t / ((long long)p.NX * p.NY));
  return cell_index(p, ax, ay, az);
}

// block 256; any grid (grid-stride over the cells; [cb, ce) only when ce > 0)
template <class T>
__global__ void __launch_bounds__(kLayoutCells)
k_aos_to_soa(KParams p, const double* __restrict__ aos, T* __restrict__ soa, int neq,
             long long cb = 0, long long ce = 0) {
  __shared__ double buf[kLayoutCells * kLayoutPad];
  const long long n = ce > 0 ? ce : (long long)p.NX * p.NY * p.NZ;
  for (long long c0 = cb + (long long)blockIdx.x * kLayoutCells; c0 < n;
       c0 += (long long)gridDim.x * kLayoutCells) {
    const int m = (int)min((long long)kLayoutCells, n - c0);
    for (int i = threadIdx.x; i < m * neq; i += kLayoutCells) {
      const int cell = i / neq;
      buf[cell * kLayoutPad + (i - cell * neq)] = aos[c0 * neq + i];
    }
    __syncthreads();
    if (threadIdx.x < m) {
      const long long c = layout_cell(p, c0 + threadIdx.x);
      for (int q = 0; q < neq; ++q)
        soa[q * p.fs + c] = from_d<T>(buf[threadIdx.x * kLayoutPad + q]);
    }
    __syncthreads();
  }
}

// cells [cb, ce) of the host layout only when ce > 0 (a slab of planes)
template <class T>
__global__ void __launch_bounds__(kLayoutCells)
k_soa_to_aos(KParams p, const T* __restrict__ soa, double* __restrict__ aos, int neq,
             long long cb = 0, long long ce = 0) {
  __shared__ double buf[kLayoutCells * kLayoutPad];
  const long long n = ce > 0 ? ce : (long long)p.NX * p.NY * p.NZ;
  for (long long c0 = cb + (long long)blockIdx.x * kLayoutCells; c0 < n;
       c0 += (long long)gridDim.x * kLayoutCells) {
    const int m = (int)min((long long)kLayoutCells, n - c0);
    if (threadIdx.x < m) {
      const long long c = layout_cell(p, c0 + threadIdx.x);
      for (int q = 0; q < neq; ++q) buf[threadIdx.x * kLayoutPad + q] = to_d(soa[q * p.fs + c]);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < m * neq; i += kLayoutCells) {
      const int cell = i / neq;
      aos[c0 * neq + i] = buf[cell * kLayoutPad + (i - cell * neq)];
    }
    __syncthreads();
  }
}

// primit (full array, from u) straight into the host layout
template <class Pol, int NEQ>
__global__ void __launch_bounds__(kLayoutCells)
k_prim_to_aos(KParams p, const typename Pol::TU* __restrict__ u, double* __restrict__ aos) {
  __shared__ double buf[kLayoutCells * kLayoutPad];
  const long long n = (long long)p.NX * p.NY * p.NZ;
  for (long long c0 = (long long)blockIdx.x * kLayoutCells; c0 < n;
       c0 += (long long)gridDim.x * kLayoutCells) {
    const int m = (int)min((long long)kLayoutCells, n - c0);
    if (threadIdx.x < m) {
      const long long c = layout_cell(p, c0 + threadIdx.x);
      double uu[NEQ], pp[NEQ];
#pragma unroll
      for (int q = 0; q < NEQ; ++q) uu[q] = to_d(u[q * p.fs + c]);
      unsigned pfl = 0;
      Ops<PolFP64>::u2prim<NEQ>(p, uu, pp, pfl);
#pragma unroll
      for (int q = 0; q < NEQ; ++q) buf[threadIdx.x * kLayoutPad + q] = pp[q];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < m * NEQ; i += kLayoutCells) {
      const int cell = i / NEQ;
      aos[c0 * NEQ + i] = buf[cell * kLayoutPad + (i - cell * NEQ)];
    }
    __syncthreads();
  }
}

}  // namespace gch
