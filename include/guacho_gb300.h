/*
 * guacho_gb300.h -- C ABI of the GB300 (sm_103a) per-timestep update for
 * Guacho-3D.
 *
 * The entry points replace, one for one, the Fortran routines that
 * src/main.f90 calls on the hot path:
 *
 *   gch_boundaryI     <- boundaryI()               src/boundaries.f90:44
 *                                                   (called at src/main.f90:76)
 *   gch_calcprim      <- calcprim(u, primit)       src/hydro_core.f90:245
 *                                                   (called at src/main.f90:79)
 *   gch_get_timestep  <- get_timestep(...)         src/hydro_core.f90:623
 *                                                   (called at src/main.f90:97)
 *   gch_tstep         <- tstep()                   src/hydro_solver.f90:134
 *                                                   (called at src/main.f90:106)
 *
 * plus the state transfers a GPU drop-in needs around them (the reference
 * keeps u/primit as host globals, src/globals.f90:33-38):
 *
 *   gch_create / gch_destroy   <- allocate/deallocate in initmain
 *                                 (src/init.f90:145-158)
 *   gch_upload / gch_download  <- u/primit host arrays, Fortran layout
 *                                 u(neq, 1-nghost:nx+nghost, ..., ...)
 *
 * and two device-resident drivers with no host round trip per step:
 *
 *   gch_advance        <- the time loop of src/main.f90:94-125, with dt kept
 *                         on the device, steps captured as a CUDA graph
 *   gch_batch_*        <- many independent boxes of uneven size, each with
 *                         its own dt, advanced by one CUDA graph per step
 *                         whose kernels each cover all boxes
 *
 * Every call returns 0 (GCH_OK) or a bitmask of GCH_ERR_* bits.  The Fortran
 * shim prints and stops on a non-zero status, as the reference does
 * (src/hlld.f90:316-317, src/hllc.f90:135-138, src/init.f90:79-84).
 *
 * Threading: one host thread drives a domain; calls on one domain are not
 * reentrant.  All work of a domain runs on the CUDA stream given at creation
 * (0 = the legacy default stream).
 *
 * Plain C types only: no torch or CUDA types cross this boundary.
 */
#ifndef GUACHO_GB300_H
#define GUACHO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GCH_ABI_VERSION 3

/* ---- switch ids: identical values to src/constants.f90:56-98 ----------- */
#define GCH_SOLVER_HLL 1
#define GCH_SOLVER_HLLC 2
#define GCH_SOLVER_HLLE 3
#define GCH_SOLVER_HLLD 4
/* HLLE with every variable split into a background and a fluctuation
 * (src/hlle_split_all.f90); MHD on the FP64 path, background set with
 * gch_set_background */
#define GCH_SOLVER_HLLE_SPLIT_ALL 7

#define GCH_EOS_ADIABATIC 1
#define GCH_EOS_SINGLE_SPECIE 2
#define GCH_EOS_H_RATE 3

#define GCH_COOL_NONE 0
#define GCH_COOL_H 1
#define GCH_COOL_DMC 3
#define GCH_COOL_CHI 4

#define GCH_TC_OFF 0
#define GCH_TC_ISOTROPIC 1
#define GCH_TC_ANISOTROPIC 2

#define GCH_BC_OUTFLOW 1
#define GCH_BC_CLOSED 2
#define GCH_BC_PERIODIC 3
#define GCH_BC_OTHER 4

#define GCH_LIMITER_NO_AVERAGE (-1)
#define GCH_LIMITER_NO_LIMIT 0
#define GCH_LIMITER_MINMOD 1
#define GCH_LIMITER_VAN_LEER 2
#define GCH_LIMITER_VAN_ALBADA 3
#define GCH_LIMITER_UMIST 4
#define GCH_LIMITER_WOODWARD 5
#define GCH_LIMITER_SUPERBEE 6

/* ---- precision modes (no counterpart in the reference) ------------------ */
/* Plain FP64 drop-in: every value and operation in FP64, no FMA contraction,
 * bitwise equal to the reference's x86-64 FP64 build where all operations
 * are IEEE-exact (everything but the exp/log/pow of cooling and conduction). */
#define GCH_FP64 0
/* FP32 state, reconstruction and fluxes; u stored in FP64; FP64 for the
 * pressure recovery in u2prim, the u += dt*divF accumulation, dt and time.
 * Cooling, conduction, viscosity and sources compute in FP32 and add their
 * change of u in FP64. */
#define GCH_FP32_MIXED 1
/* As GCH_FP32_MIXED but u stored as a compensated (hi, lo) FP32 pair and
 * accumulated with Kahan-style error-free sums instead of FP64; the stage
 * kernels run no FP64 instruction per cell. */
#define GCH_FP32_KAHAN 2

/* ---- status bits --------------------------------------------------------- */
#define GCH_OK 0
#define GCH_ERR_PARAM 0x1            /* rejected parameter set            */
#define GCH_ERR_CUDA 0x2             /* a CUDA runtime call failed        */
#define GCH_ERR_HLLD 0x4             /* HLLD fell through (hlld.f90:316)  */
#define GCH_ERR_HLLC 0x8             /* HLLC fell through (hllc.f90:135)  */
#define GCH_ERR_DT 0x10              /* dt <= 0 or not finite             */
#define GCH_ERR_TIMEOUT 0x20         /* a bounded device wait ran out     */
#define GCH_ERR_NO_DEVICE 0x40       /* no CUDA device / not sm_103       */
#define GCH_ERR_STATE 0x80           /* call out of order                 */
#define GCH_ERR_TOO_LARGE 0x100      /* box exceeds a fixed-size work area */

#define GCH_MAX_SPHERES 8
#define GCH_MAX_GRAV 4
#define GCH_MAX_TABLE 512

/* A wind sphere re-imposed by the user boundary hook on every boundary
 * call, the pattern of impose_exo (EXO/exoplanet.f90:125-266) and
 * impose_user_bc (EXO/user_mod.f90:131-144).  Cells whose centre lies within
 * `radius` of (xc, yc, zc) (measured from the grid centre) are set to
 * rho = dens, v = vorb + vwind * r_hat, E = 1/2 rho v^2 + cv*dens*tfac
 * (+ the dipole field of strength bdip and its energy when MHD).
 * With orbit_omega != 0 the sphere moves on the planet's circular orbit in
 * the x-z plane (EXO/exoplanet.f90:143-148): at the time t of the boundary
 * call (the step's start time, as the reference's global `time` inside
 * tstep; 0 before the first step), with th = orbit_omega*t + orbit_phase,
 * the centre is (orbit_r cos th, yc, orbit_r sin th) and vorb is the orbital
 * velocity orbit_omega*orbit_r*(-sin th, 0, cos th); xc, zc and vorb are
 * then unused. */
typedef struct {
  double xc, yc, zc;
  double radius;
  double dens;
  double vwind;
  double vorb[3];
  double tfac;
  double bdip;
  double orbit_r, orbit_omega, orbit_phase;
} gch_sphere_t;

/* The parameter surface of parameters.f90 (OT/parameters.f90:48-177), as
 * runtime values.  Field names follow the Fortran names. */
typedef struct {
  int32_t abi_version;      /* = GCH_ABI_VERSION */
  int32_t precision;        /* GCH_FP64 | GCH_FP32_MIXED | GCH_FP32_KAHAN */
  /* grid: interior cells of the (single) domain, nghost = 2 fixed */
  int32_t nx, ny, nz;
  int32_t neq;              /* 8 with BFIELD, 5 without */
  /* physics switches */
  int32_t mhd, pmhd;
  int32_t riemann_solver;
  int32_t slope_limiter;
  int32_t eq_of_state;
  int32_t cooling;
  int32_t enable_flux_cd;
  int32_t eight_wave;
  int32_t user_source_terms;
  int32_t bc_left, bc_right, bc_bottom, bc_top, bc_out, bc_in;
  int32_t bc_user;
  /* spacing (dx = xmax/nxtot, src/init.f90:120-122) and EOS */
  double dx, dy, dz;
  double cv, gamma;         /* gamma = (cv+1)/cv (OT/parameters.f90:158) */
  double cfl, eta;
  double Tempsc, Psc, tsc;  /* scalings (OT/parameters.f90:163-170) */
  /* tabulated cooling (COOL_DMC / COOL_CHI): rows equally spaced in log10 T
   * (reference tables: 41 rows of 0.1 dex from 1e4 K) */
  int32_t ntab;
  int32_t tab_i0;           /* round(log10(T_first) * tab_inv_dlog) */
  double tab_inv_dlog;      /* 1 / row spacing in dex */
  double tab_tail;          /* Lambda = tab_tail*sqrt(T) above 1e8 K */
  double tab_Tmin;          /* cooling acts only above this T (1e4 K) */
  double tab_T[GCH_MAX_TABLE];
  double tab_L[GCH_MAX_TABLE];
  /* user boundary spheres (bc_user) */
  int32_t nsph;
  int32_t ngrav;
  gch_sphere_t sph[GCH_MAX_SPHERES];
  /* user source terms: point masses (EXO/user_mod.f90:158-206) */
  double grav_GM[GCH_MAX_GRAV];
  double grav_x[GCH_MAX_GRAV], grav_y[GCH_MAX_GRAV], grav_z[GCH_MAX_GRAV];
  /* thermal conduction (th_cond and tc_saturation of parameters.f90:114-119;
   * src/thermal_cond.f90) and the cgs scalings it converts with
   * (parameters.f90:159-170): rsc = xphys/xmax, rhosc = amh*mu,
   * vsc2 = gamma*Rg*T0/mu, bsc = sqrt(4*pi*Psc), mu.  Anisotropic
   * conduction needs B; conduction with table cooling is rejected. */
  int32_t th_cond;          /* GCH_TC_OFF | GCH_TC_ISOTROPIC | GCH_TC_ANISOTROPIC */
  int32_t tc_saturation;
  double rsc, rhosc, vsc2, bsc, mu;
  /* passive scalars (npas of parameters.f90:131-135, 0 or 2): the last npas
   * of the neq equations, neq = 5 or 8 dynamical + npas.  With
   * GCH_EOS_H_RATE (src/hydro_core.f90:106-111) or GCH_COOL_H
   * (src/cooling_h.f90) the first passive is the neutral hydrogen density. */
  int32_t npas;
} gch_params_t;

typedef struct gch_domain gch_domain_t;

/* Fill *p with the OT/parameters.f90 defaults (HLLD, minmod, flux-CD,
 * periodic, cv = 1.5, cfl = 0.2, eta = 0) for an nx x ny x nz box. */
void gch_params_default(gch_params_t* p, int nx, int ny, int nz);

/* Validate a parameter set without allocating; returns GCH_OK or
 * GCH_ERR_PARAM. */
int gch_params_check(const gch_params_t* p);

/* Allocate the device state of one domain (src/init.f90:145-158).  `stream`
 * is a cudaStream_t passed as an opaque pointer (NULL: default stream). */
int gch_create(const gch_params_t* p, void* stream, gch_domain_t** out);
int gch_destroy(gch_domain_t* d);

/* Host <-> device transfer of the conserved variables in the reference's
 * layout: u(neq, 1-2:nx+2, 1-2:ny+2, 1-2:nz+2), column major, FP64.
 * gch_download also writes primit (same layout) when primit != NULL. */
int gch_upload(gch_domain_t* d, const double* u);
int gch_download(gch_domain_t* d, double* u, double* primit);

/* The background state of GCH_SOLVER_HLLE_SPLIT_ALL, primit0 of
 * src/globals.f90:42, in the layout of primit (u and primit then hold the
 * fluctuation).  The reference allocates primit0 but never sets it; here it
 * is zero until this call.  Call it before gch_calcprim, as the background is
 * part of the initial state.  GCH_ERR_PARAM for the other solvers. */
int gch_set_background(gch_domain_t* d, const double* primit0);

/* src/boundaries.f90:44 boundaryI: one ghost layer of u, then the user
 * boundary spheres. */
int gch_boundaryI(gch_domain_t* d);

/* src/hydro_core.f90:245 calcprim(u, primit) over the whole array. */
int gch_calcprim(gch_domain_t* d);

/* src/hydro_core.f90:623 get_timestep: CFL dt from the interior primitives,
 * ramped over the first n_iter iterations, clipped to land on tprint (sets
 * *dump_flag = 1 then). */
int gch_get_timestep(gch_domain_t* d, int current_iter, int n_iter, double current_time,
                     double tprint, double* dt, int* dump_flag);

/* src/hydro_solver.f90:134 tstep: advance u by dt (both stages, flux-CD,
 * sources, viscosity, cooling, boundaries, primitives, and thermal
 * conduction when th_cond != 0).  With conduction the call waits for the
 * device once (the super-step count depends on the state); otherwise it is
 * asynchronous. */
int gch_tstep(gch_domain_t* d, double dt);

/* The conduction substeps of the last tstep (src/thermal_cond.f90:690-768:
 * Nsteps and dt_cond in seconds); 0 and 0.0 when conduction is off. */
int gch_tc_info(gch_domain_t* d, int* nsteps, double* dt_cond);

/* gch_get_timestep + gch_tstep with the state in HOST memory: uploads u,
 * steps once and downloads u, for callers whose hooks need the host arrays
 * current after every step.  *dt and *dump_flag as gch_get_timestep.
 * A page-locked u is read and written over the host link by the layout
 * kernels.  A pageable u goes through copy-engine copies; where
 * gch_step_host_overlaps says so, it goes up slab by slab of z while the
 * first half step's fluxes start on the slabs that have landed, and comes
 * back slab by slab while the second half step still computes the slabs
 * above (same bits as the serial order). */
int gch_step_host(gch_domain_t* d, double* u, int current_iter, int n_iter,
                  double current_time, double tprint, double* dt, int* dump_flag);

/* 1 when gch_step_host overlaps its copies of a pageable u with the step:
 * the upload with the CFL pass and the first half step's fluxes, the
 * download with the second half step.  FP32 domains without user spheres, table cooling,
 * COOL_H, resistivity, thermal conduction, source terms or passive scalars,
 * with at least three z chunks of the stage kernels (gch_get_kz); 0
 * otherwise (the serial order; always for GCH_FP64, whose step is bound by
 * its arithmetic). */
int gch_step_host_overlaps(const gch_domain_t* d);

/* The time loop of src/main.f90:94-125 on the device: up to max_steps
 * iterations while time <= tmax, dt never leaves the device.  *time, *iter
 * and *tprint are the loop state (in/out).  Returns after a host sync. */
int gch_advance(gch_domain_t* d, int max_steps, double tmax, double dtprint, int n_iter,
                double* time, int* iter, double* tprint, int* steps_done);

/* Device-side counters of the last step: number of cells whose pressure hit
 * the 1e-16 floor in u2prim (src/hydro_core.f90:78) during the step, and the
 * accumulated error bits. */
int gch_last_step_info(gch_domain_t* d, long long* pfloor_hits, int* err_bits);

/* Kernel launches of one gch_get_timestep (k_cfl, k_dtfin) plus one
 * gch_tstep of this domain (for launch accounting).  The device loop of
 * gch_advance adds one loop-tail kernel per iteration. */
int gch_launches_per_step(gch_domain_t* d);

/* ---- z-march depth of the stage kernels (no reference counterpart) -------
 * Each block of the stage kernels marches over kz planes of z.  Results are
 * identical for every depth (every plane is computed by the same code); the
 * depth trades the column warm-up per block against the number of blocks.
 * gch_create picks kz from the box size; gch_autotune times the stage-1
 * flux kernel (it writes only the stage arrays up and E) for kz in
 * {1,2,4,8,12,16,20,24,32} <= nz on the current state, keeps the fastest, and
 * reports up to `cap` candidates with their times in ms (outputs may be
 * NULL).  gch_set_kz sets the depth directly (1 <= kz <= nz). */
int gch_get_kz(gch_domain_t* d);
int gch_set_kz(gch_domain_t* d, int kz);
int gch_autotune(gch_domain_t* d, int cap, int* cand_kz, float* cand_ms, int* ncand);

/* Profiling aids (no counterpart in the reference).
 * gch_advance_timed: `steps` device-resident iterations without output
 * clipping, timed with CUDA events on the domain's stream; *ms = GPU time.
 * gch_profile_step: one get_timestep + tstep with an event after every
 * launch; writes up to `cap` per-launch durations (ms) and kernel names
 * (each a NUL-terminated string in a `name_len`-byte slot of `names`). */
int gch_advance_timed(gch_domain_t* d, int steps, int n_iter, float* ms);
int gch_profile_step(gch_domain_t* d, int cap, float* ms, char* names, int name_len, int* n);

/* get_timestep for callers that cannot allocate device memory.  No
 * counterpart in the reference.  It exists for host codes that give the
 * library a fixed, pre-sized memory budget and forbid hidden allocations (a
 * late cudaMalloc can fail or fragment memory in the middle of a run), and
 * for codes that own every device buffer through their own pool allocator.
 * It allocates nothing: the caller passes u in device memory in the
 * reference layout u(neq, 1-2:nx+2, 1-2:ny+2, 1-2:nz+2) (FP64, ghost cells
 * filled) and device slots for the outputs dt and dump_flag; the per-block
 * partial minima go to a fixed array inside the library (512 KiB on every
 * GPU that loads it, kept until exit).  Same result as gch_get_timestep in
 * FP64 arithmetic.  Limits: boxes with ceil(nx/32)*ceil(ny/8)*ceil(nz/8) >
 * 65536 (beyond 512^3 cells) return GCH_ERR_TOO_LARGE.  GCH_ERR_PARAM for
 * what the one-kernel reduction does not cover: any cooling (table cooling
 * takes dt from the stored primitives, COOL_H needs the passive n_HI),
 * passive scalars (npas != 0), and the split solver
 * GCH_SOLVER_HLLE_SPLIT_ALL (its fast speeds need the background state of a
 * domain).  All calls share the fixed array and each call clears its
 * completion counter first: calls that can overlap on the GPU race, so
 * issue them on one stream.  The first call on a device, and the first call
 * after that device's context was destroyed and created again (e.g. by
 * cudaDeviceReset), looks up the array's address; make that first call
 * before any stream capture.  Asynchronous on `stream`. */
int gch_get_timestep_noalloc(const gch_params_t* p, const double* u_dev, int current_iter,
                             int n_iter, double current_time, double tprint, double* dt_dev,
                             int* dump_dev, void* stream);

/* ---- batched boxes ------------------------------------------------------ */
typedef struct gch_batch gch_batch_t;

/* n independent domains (each its own params, size and dt) advanced
 * together.  All boxes must share precision, neq and the physics switches;
 * sizes, spacings, boundary kinds and problem data may differ.
 *
 * FP32 boxes without COOL_H, thermal conduction, resistivity or passive
 * scalars (table cooling and user spheres included) are advanced in
 * grouped mode on `stream` (0 = a
 * stream of the batch's own): one launch per kernel of the step covers up to
 * 64 boxes, the two stage kernels work (box, tile, z chunk) items either
 * one block per item or as a persistent grid whose blocks pull items from
 * a device counter, one CUDA graph holds the step, and the z-march depth of
 * an item and the launch form are chosen by timing before the first step.
 * Other batches run each box's own step graph on its own stream.  No
 * reference counterpart: the reference advances one domain per process. */
int gch_batch_create(int n, const gch_params_t* params, void* stream, gch_batch_t** out);
int gch_batch_destroy(gch_batch_t* b);
int gch_batch_upload(gch_batch_t* b, int box, const double* u);
int gch_batch_download(gch_batch_t* b, int box, double* u);
/* Advance every box by `steps` steps, each with its own CFL dt (ramp over
 * the first n_iter iterations of each box), no output clipping. */
int gch_batch_advance(gch_batch_t* b, int steps, int n_iter);
/* Per-box simulated time and iteration count. */
int gch_batch_time(gch_batch_t* b, double* times, int* iters);
/* How the batch runs: grouped (1/0), the z-march depth the autotuner chose
 * (-1 when not grouped, 0 before the first advance) and up to `cap`
 * candidate depths with their measured stage-1 times in ms (ncand of them)
 * at the chosen resident blocks per SM.  Any output pointer may be NULL. */
int gch_batch_tuning(gch_batch_t* b, int* grouped, int* kz, int cap, int* cand_kz,
                     float* cand_ms, int* ncand);
/* The autotuner's whole search: grouped (1/0), the chosen z-march depth and
 * launch form of the stage kernels (bps = resident blocks per SM of the
 * persistent grid, 0 = one block per work item; both -1 when not grouped),
 * and up to `cap` timed candidates (depth, bps, stage-1 ms).  Any output
 * pointer may be NULL. */
int gch_batch_tuning_grid(gch_batch_t* b, int* grouped, int* kz, int* bps, int cap,
                          int* cand_kz, int* cand_bps, float* cand_ms, int* ncand);

#ifdef __cplusplus
}
#endif
#endif
