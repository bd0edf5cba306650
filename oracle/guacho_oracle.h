/*
 * guacho_oracle.h -- CPU (FP64) restatement of Guacho-3D's per-timestep update.
 *
 * TEST INFRASTRUCTURE ONLY.  This oracle is the parity checker for the CUDA
 * path: only tests, the smoke check and the CPU-baseline leg of the benchmark
 * may load it.  The product library never links or calls it.
 *
 * Parity status: the reference (Fortran + MPI) has no test suite and no golden
 * vectors, and no Fortran compiler exists in the build container.  The oracle
 * is pinned by known-answer tests (Riemann consistency, conservation, div B at
 * round-off, mirror symmetry) and, where a Fortran toolchain is present, by a
 * build of the reference sources themselves (oracle/_ref).
 *
 * Layout follows the reference exactly: Fortran column-major
 * u(neq, nxmin:nxmax, nymin:nymax, nzmin:nzmax), i.e. neq fastest, then x, y,
 * z, with nghost = 2 ghost cells per side (src/globals.f90:33-38,
 * src/init.f90:145-150, OT/parameters.f90:193,222-227).
 */
#ifndef GUACHO_ORACLE_H
#define GUACHO_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Switch ids, equal to src/constants.f90:56-98. */
enum {
  GOR_SOLVER_HLL = 1, GOR_SOLVER_HLLC = 2, GOR_SOLVER_HLLE = 3, GOR_SOLVER_HLLD = 4,
  GOR_SOLVER_HLLE_SPLIT_ALL = 7,
  GOR_EOS_ADIABATIC = 1, GOR_EOS_SINGLE_SPECIE = 2, GOR_EOS_H_RATE = 3,
  GOR_COOL_NONE = 0, GOR_COOL_H = 1, GOR_COOL_DMC = 3, GOR_COOL_CHI = 4,
  GOR_BC_OUTFLOW = 1, GOR_BC_CLOSED = 2, GOR_BC_PERIODIC = 3, GOR_BC_OTHER = 4,
  GOR_LIMITER_NO_AVERAGE = -1, GOR_LIMITER_NO_LIMIT = 0, GOR_LIMITER_MINMOD = 1,
  GOR_LIMITER_VAN_LEER = 2, GOR_LIMITER_VAN_ALBADA = 3, GOR_LIMITER_UMIST = 4,
  GOR_LIMITER_WOODWARD = 5, GOR_LIMITER_SUPERBEE = 6
};

#define GOR_MAX_SPHERES 8
#define GOR_MAX_GRAV 4
#define GOR_MAX_TAB 512
#define GOR_MAX_NEQ 10  /* 8 dynamical equations + 2 passive scalars */

/* Error bits (the reference prints and stops in these cases). */
enum {
  GOR_ERR_HLLD_FALLTHROUGH = 1,   /* src/hlld.f90:316-317 */
  GOR_ERR_HLLC_FALLTHROUGH = 2,   /* src/hllc.f90:135-138 */
  GOR_ERR_BAD_PARAM = 4
};

/* One wind sphere re-imposed by the user boundary hook (EXO pattern,
 * EXO/exoplanet.f90:125-266): cells with r <= radius get rho = dens,
 * v = vorb + vwind * r_hat, E = 1/2 rho v^2 + cv*dens*tfac (+ 1/2 B^2).
 * With orbit_omega != 0 the centre and vorb follow the planet's orbit in the
 * x-z plane at the state's time (EXO/exoplanet.f90:143-148). */
typedef struct {
  double xc, yc, zc;      /* centre, measured from the grid centre */
  double radius;
  double dens;
  double vwind;
  double vorb[3];
  double tfac;            /* the "1.9999*Tsw" / "1.8*Tpw" factor, code units */
  double bdip;            /* dipole strength ("bsw"/"bpw"), MHD only */
  double orbit_r, orbit_omega, orbit_phase;  /* "Rorb", "omegap", "phi" */
} gor_sphere_t;

typedef struct {
  int nx, ny, nz;         /* interior cells (one domain, no MPI split) */
  int neq;                /* 8 with B, 5 without */
  int mhd, pmhd;
  int riemann_solver, slope_limiter, eq_of_state, cooling;
  int enable_flux_cd, eight_wave, user_source_terms;
  int bc_left, bc_right, bc_bottom, bc_top, bc_out, bc_in;
  int bc_user;
  double dx, dy, dz;
  double cv, gamma, cfl, eta;
  double Tempsc, Psc, tsc;
  /* tabulated cooling: rows T[i], L[i] (already in the units the
   * reference's table reader produces, src/cooling_dmc.f90:71-75) */
  int ntab;
  double tab_T[GOR_MAX_TAB], tab_L[GOR_MAX_TAB];
  double tab_inv_dlog;    /* 10 for the reference's 0.1 dex tables */
  int tab_i0;             /* round(log10(T_first) * tab_inv_dlog) */
  double tab_tail;        /* Lambda = tab_tail*sqrt(T) above 1e8 K */
  double tab_Tmin;        /* 1e4 in the reference */
  /* user boundary spheres */
  int nsph;
  gor_sphere_t sph[GOR_MAX_SPHERES];
  /* user source terms: point masses, EXO/user_mod.f90:158-206 */
  int ngrav;
  double grav_GM[GOR_MAX_GRAV], grav_x[GOR_MAX_GRAV], grav_y[GOR_MAX_GRAV],
         grav_z[GOR_MAX_GRAV];
  /* thermal conduction (src/thermal_cond.f90): th_cond = TC_OFF 0,
   * TC_ISOTROPIC 1, TC_ANISOTROPIC 2 (src/constants.f90:96-98); the cgs
   * scalings of parameters.f90:159-170 it converts with */
  int th_cond, tc_saturation;
  double rsc, rhosc, vsc2, bsc, mu;
  /* passive scalars (npas of parameters.f90:131-135): the last npas of the
   * neq equations, neqdyn = neq - npas; EOS_H_RATE reads the first one as
   * the neutral hydrogen density (src/hydro_core.f90:106-111) */
  int npas;
} gor_params_t;

typedef struct gor_state gor_state_t;

gor_state_t* gor_create(const gor_params_t* p);
void gor_destroy(gor_state_t* s);
int gor_nthreads(int n);  /* set OpenMP threads (<=0: keep); returns current */

/* Whole-array access, Fortran (neq, x, y, z) order with ghosts. */
void gor_set_u(gor_state_t* s, const double* u);
void gor_get_u(const gor_state_t* s, double* u);
void gor_get_primit(const gor_state_t* s, double* primit);
void gor_set_primit(gor_state_t* s, const double* primit);
/* The background state primit0 of the split solver (src/globals.f90:42),
 * same layout as primit.  The reference allocates but never sets it; here it
 * is zero until set. */
void gor_set_background(gor_state_t* s, const double* primit0);

/* Reference entry points. */
void gor_boundaryI(gor_state_t* s);                        /* src/boundaries.f90:44 */
void gor_calcprim(gor_state_t* s, int only_ghost);         /* src/hydro_core.f90:245 */
void gor_get_timestep(gor_state_t* s, int iter, int n_iter, double t,
                      double tprint, double* dt, int* dump); /* src/hydro_core.f90:623 */
void gor_tstep(gor_state_t* s, double dt);                 /* src/hydro_solver.f90:134 */
double gor_time(const gor_state_t* s);
void gor_set_time(gor_state_t* s, double t);
int gor_error(const gor_state_t* s);

/* Single-interface kernels (x-direction), for known-answer tests. */
void gor_riemann(const gor_params_t* p, const double* priml, const double* primr,
                 double* ff, int* err);
/* src/hlle_split_all.f90:51-84: fluctuations priml/primr over backgrounds
 * prim0l/prim0r (x-direction) */
void gor_riemann_split(const gor_params_t* p, const double* priml, const double* primr,
                       const double* prim0l, const double* prim0r, double* ff);
void gor_prim2f(const gor_params_t* p, const double* prim, double* ff);
void gor_u2prim(const gor_params_t* p, const double* uu, double* prim, double* T);
void gor_prim2u(const gor_params_t* p, const double* prim, double* uu);
void gor_limiter(const gor_params_t* p, const double* pll, double* pl, double* pr,
                 const double* prr);
double gor_cooltab(const gor_params_t* p, double T);

/* src/thermal_cond.f90:690-768 thermal_conduction: the conduction substeps
 * that tstep runs after the hydro step when th_cond != 0 (called by
 * gor_tstep; exposed for tests with the hydro step's dt_CFL).  *nsteps and
 * *dt_cond (may be NULL) report the substep count and the conduction
 * timescale in seconds. */
void gor_thermal_conduction(gor_state_t* s, double dt_CFL, int* nsteps, double* dt_cond);
/* Temperature of every cell from the last calcprim (src/globals.f90 Temp). */
void gor_get_temp(const gor_state_t* s, double* temp /* NX*NY*NZ, x fastest */);
/* The super-time-stepping helpers (src/thermal_cond.f90:625-681). */
double gor_superstep(int n, double snu);
double gor_substep(int j, int n, double nu);
void gor_st_steps(double fs, int* ns, double* fstep);

/* Diagnostics: centred div B over the interior (src/Out_BIN_Module.f90:214-222). */
void gor_divb(const gor_state_t* s, double* divb /* nx*ny*nz */);

/* Main-loop semantics of src/main.f90:94-125, from the current state to
 * time > tmax or max_steps steps.  *iter (starts at 1) and *tprint (starts at
 * dtprint) carry the loop state between calls.  Returns steps taken. */
int gor_run(gor_state_t* s, double tmax, double dtprint, int max_steps, int n_iter,
            int* iter, double* tprint);

#ifdef __cplusplus
}
#endif
#endif
