!=======================================================================
!> @file gpu_hydro.f90
!> @brief iso_c_binding interface to the GB300 timestep library
!> @details Binds the C ABI of include/guacho_gb300.h so that Guacho's main
!! program can call the GPU timestep in place of tstep/get_timestep/calcprim.
!! The host arrays keep the reference layout u(neq,nxmin:nxmax,...) in
!! real(8) (-fdefault-real-8 / DOUBLEP=Y); they are current on the host only
!! after gpu_download.
!=======================================================================
module gpu_hydro

  use iso_c_binding
  implicit none

  integer, parameter :: GCH_MAX_SPHERES = 8, GCH_MAX_GRAV = 4, GCH_MAX_TABLE = 512

  type, bind(C) :: gch_sphere_t
    real(c_double) :: xc, yc, zc, radius, dens, vwind
    real(c_double) :: vorb(3)
    real(c_double) :: tfac, bdip
    real(c_double) :: orbit_r, orbit_omega, orbit_phase
  end type gch_sphere_t

  type, bind(C) :: gch_params_t
    integer(c_int32_t) :: abi_version, precision
    integer(c_int32_t) :: nx, ny, nz, neq
    integer(c_int32_t) :: mhd, pmhd
    integer(c_int32_t) :: riemann_solver, slope_limiter, eq_of_state, cooling
    integer(c_int32_t) :: enable_flux_cd, eight_wave, user_source_terms
    integer(c_int32_t) :: bc_left, bc_right, bc_bottom, bc_top, bc_out, bc_in
    integer(c_int32_t) :: bc_user
    real(c_double) :: dx, dy, dz
    real(c_double) :: cv, gamma, cfl, eta
    real(c_double) :: Tempsc, Psc, tsc
    integer(c_int32_t) :: ntab, tab_i0
    real(c_double) :: tab_inv_dlog, tab_tail, tab_Tmin
    real(c_double) :: tab_T(GCH_MAX_TABLE), tab_L(GCH_MAX_TABLE)
    integer(c_int32_t) :: nsph, ngrav
    type(gch_sphere_t) :: sph(GCH_MAX_SPHERES)
    real(c_double) :: grav_GM(GCH_MAX_GRAV), grav_x(GCH_MAX_GRAV)
    real(c_double) :: grav_y(GCH_MAX_GRAV), grav_z(GCH_MAX_GRAV)
    integer(c_int32_t) :: th_cond, tc_saturation
    real(c_double) :: rsc, rhosc, vsc2, bsc, mu
    integer(c_int32_t) :: npas
  end type gch_params_t

  interface
    subroutine gch_params_default(p, nx, ny, nz) bind(C, name="gch_params_default")
      import :: gch_params_t, c_int
      type(gch_params_t), intent(out) :: p
      integer(c_int), value :: nx, ny, nz
    end subroutine
    integer(c_int) function gch_create(p, stream, dom) bind(C, name="gch_create")
      import :: gch_params_t, c_int, c_ptr
      type(gch_params_t), intent(in) :: p
      type(c_ptr), value :: stream
      type(c_ptr), intent(out) :: dom
    end function
    integer(c_int) function gch_destroy(dom) bind(C, name="gch_destroy")
      import :: c_int, c_ptr
      type(c_ptr), value :: dom
    end function
    integer(c_int) function gch_upload(dom, u) bind(C, name="gch_upload")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: dom
      real(c_double), intent(in) :: u(*)
    end function
    integer(c_int) function gch_download(dom, u, primit) bind(C, name="gch_download")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: dom
      real(c_double), intent(out) :: u(*), primit(*)
    end function
    integer(c_int) function gch_set_background(dom, primit0) bind(C, name="gch_set_background")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: dom
      real(c_double), intent(in) :: primit0(*)
    end function
    integer(c_int) function gch_boundaryI(dom) bind(C, name="gch_boundaryI")
      import :: c_int, c_ptr
      type(c_ptr), value :: dom
    end function
    integer(c_int) function gch_calcprim(dom) bind(C, name="gch_calcprim")
      import :: c_int, c_ptr
      type(c_ptr), value :: dom
    end function
    integer(c_int) function gch_get_timestep(dom, iter, n_iter, t, tprint, dt, dump) &
                                             bind(C, name="gch_get_timestep")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: dom
      integer(c_int), value :: iter, n_iter
      real(c_double), value :: t, tprint
      real(c_double), intent(out) :: dt
      integer(c_int), intent(inout) :: dump
    end function
    integer(c_int) function gch_tstep(dom, dt) bind(C, name="gch_tstep")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: dom
      real(c_double), value :: dt
    end function
    integer(c_int) function gch_tc_info(dom, nsteps, dt_cond) bind(C, name="gch_tc_info")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: dom
      integer(c_int), intent(out) :: nsteps
      real(c_double), intent(out) :: dt_cond
    end function
  end interface

  type(c_ptr), save :: gpu_dom = c_null_ptr

contains

  !> stop like the reference does on an error (src/hlld.f90:316-317)
  subroutine gpu_check(where, status)
    character(len=*), intent(in) :: where
    integer(c_int), intent(in) :: status
    if (status /= 0) then
      print '(a,a,a,z8)', 'GPU error in ', where, ': status 0x', status
      stop
    end if
  end subroutine gpu_check

end module gpu_hydro
