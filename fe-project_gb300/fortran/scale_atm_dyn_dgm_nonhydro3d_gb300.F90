!-------------------------------------------------------------------------------
!> module FElib / Fluid dyn solver / Atmosphere / Nonhydrostatic model / GB300 binding
!!
!! ISO_C_BINDING shim that points FElib's cal_tend_ex / cal_vi procedure pointers
!! (FElib/src/fluid_dyn_solver/scale_atm_dyn_dgm_driver_nonhydro3d.F90:152-250) at the
!! GB300 library libfedg.so (C ABI: include/fedg.h).  The arrays are the driver's own
!! OpenACC-resident fields; their device addresses are passed under host_data use_device.
!! Not compiled in this repository (no Fortran compiler in its build image); built with the
!! model by a maintainer, linked with -lfedg.
!-------------------------------------------------------------------------------
#include "scaleFElib.h"
module scale_atm_dyn_dgm_nonhydro3d_gb300
  use iso_c_binding
  use scale_precision
  use scale_prc, only: PRC_abort
  use scale_const, only: GRAV => CONST_GRAV, Rdry => CONST_Rdry, CPdry => CONST_CPdry, &
                         CVdry => CONST_CVdry, PRES00 => CONST_PRE00
  use scale_element_base, only: ElementBase2D, ElementBase3D
  use scale_element_operation_base, only: ElementOperationBase3D
  use scale_localmesh_2d, only: LocalMesh2D
  use scale_localmesh_3d, only: LocalMesh3D
  use scale_sparsemat, only: SparseMat
  implicit none
  private

  public :: atm_dyn_dgm_nonhydro3d_gb300_Init
  public :: atm_dyn_dgm_nonhydro3d_gb300_Final
  public :: atm_dyn_dgm_nonhydro3d_gb300_cal_tend_heve
  public :: atm_dyn_dgm_nonhydro3d_gb300_cal_tend_hevi
  public :: atm_dyn_dgm_nonhydro3d_gb300_cal_vi
  public :: atm_dyn_dgm_nonhydro3d_gb300_ctx
  public :: atm_dyn_dgm_nonhydro3d_gb300_numdiff_apply
  public :: atm_dyn_dgm_nonhydro3d_gb300_sponge_init
  public :: atm_dyn_dgm_nonhydro3d_gb300_sponge_add_tend
  public :: atm_dyn_dgm_nonhydro3d_gb300_set_base_state
  public :: atm_dyn_dgm_nonhydro3d_gb300_load_guess
  public :: atm_dyn_dgm_nonhydro3d_gb300_update
  public :: atm_dyn_dgm_nonhydro3d_gb300_restart_write
  public :: atm_dyn_dgm_nonhydro3d_gb300_restart_read

  integer(c_int), parameter :: FEDG_HEVE = 0, FEDG_HEVI = 1
  integer(c_int), parameter, public :: FEDG_PREC_FP64 = 0, FEDG_PREC_MIXED = 1, FEDG_PREC_PAIR = 2

  type, bind(C) :: fedg_update_opts
    integer(c_int) :: eqs, prec, max_iter, use_guess
    real(c_double) :: dt, tol
  end type

  type, bind(C) :: fedg_restart_info
    integer(c_long_long) :: step
    real(c_double) :: time, dt
    character(kind=c_char) :: scheme(32)
  end type

  type, bind(C) :: fedg_mesh_desc
    integer(c_int) :: porder, NeX, NeY, NeZ
    real(c_double) :: xmin, xmax, ymin, ymax, zmin, zmax
    integer(c_int) :: periodic_x, periodic_y
    real(c_double) :: grav, rdry, cpdry, cvdry, pres00
    integer(c_int) :: mf_on
    real(c_double) :: mf_etac_h, mf_alpha_h
    integer(c_int) :: mf_order_h
    real(c_double) :: mf_etac_v, mf_alpha_v
    integer(c_int) :: mf_order_v
    integer(c_int) :: device
  end type

  interface
    integer(c_int) function fedg_ctx_create(desc, ctx) bind(C, name="fedg_ctx_create")
      import :: c_int, c_ptr, fedg_mesh_desc
      type(fedg_mesh_desc), intent(in) :: desc
      type(c_ptr), intent(out) :: ctx
    end function
    subroutine fedg_ctx_destroy(ctx) bind(C, name="fedg_ctx_destroy")
      import :: c_ptr
      type(c_ptr), value :: ctx
    end subroutine
    integer(c_int) function fedg_cal_tend_ex(ctx, inp, outp, eqs) bind(C, name="fedg_cal_tend_ex")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      type(c_ptr), intent(in) :: inp(16), outp(5)
      integer(c_int), value :: eqs
    end function
    integer(c_int) function fedg_cal_vi(ctx, inp, impl_fac, dt, max_iter, tol, outp, status) &
        bind(C, name="fedg_cal_vi")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      type(c_ptr), intent(in) :: inp(12), outp(5)
      real(c_double), value :: impl_fac, dt, tol
      integer(c_int), value :: max_iter
      type(c_ptr), value :: status
    end function
    integer(c_int) function fedg_synchronize(ctx) bind(C, name="fedg_synchronize")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function fedg_numdiff_apply(ctx, q, nlap, coef_h, coef_v, dt) bind(C, name="fedg_numdiff_apply")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      type(c_ptr), intent(in) :: q(5)
      integer(c_int), value :: nlap
      real(c_double), value :: coef_h, coef_v, dt
    end function
    integer(c_int) function fedg_sponge_add_tend(ctx, tend, mom, tau, height, hveldamp) &
        bind(C, name="fedg_sponge_add_tend")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      type(c_ptr), intent(in) :: tend(3), mom(3)
      real(c_double), value :: tau, height
      integer(c_int), value :: hveldamp
    end function
    integer(c_int) function fedg_set_base_state(ctx, dens_hyd, pres_hyd, therm_hyd, rtot, cvtot, cptot, &
        dphyddx, dphyddy, coriolis) bind(C, name="fedg_set_base_state")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx, dens_hyd, pres_hyd, therm_hyd, rtot, cvtot, cptot, dphyddx, dphyddy, coriolis
    end function
    integer(c_int) function fedg_update_set_sponge(ctx, tau, height, hveldamp) bind(C, name="fedg_update_set_sponge")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), value :: tau, height
      integer(c_int), value :: hveldamp
    end function
    integer(c_int) function fedg_update(ctx, q, nsteps, opts, iters_out) bind(C, name="fedg_update")
      import :: c_int, c_ptr, c_double, fedg_update_opts
      type(c_ptr), value :: ctx
      type(c_ptr), intent(in) :: q(5)
      integer(c_int), value :: nsteps
      type(fedg_update_opts), intent(in) :: opts
      real(c_double), intent(out) :: iters_out
    end function
    integer(c_int) function fedg_guess_create(levels, hidden, g) bind(C, name="fedg_guess_create")
      import :: c_int, c_ptr
      integer(c_int), value :: levels, hidden
      type(c_ptr), intent(out) :: g
    end function
    integer(c_int) function fedg_guess_set_scales(g, in_scale, out_scale) bind(C, name="fedg_guess_set_scales")
      import :: c_int, c_ptr, c_float
      type(c_ptr), value :: g
      real(c_float), intent(in) :: in_scale(4), out_scale(3)
    end function
    integer(c_int) function fedg_guess_set_params(g, host, n) bind(C, name="fedg_guess_set_params")
      import :: c_int, c_ptr, c_float, c_long_long
      type(c_ptr), value :: g
      real(c_float), intent(in) :: host(*)
      integer(c_long_long), value :: n
    end function
    integer(c_int) function fedg_guess_load(ctx, g) bind(C, name="fedg_guess_load")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx, g
    end function
    integer(c_int) function fedg_restart_write(ctx, path, q, info) bind(C, name="fedg_restart_write")
      import :: c_int, c_ptr, c_char, fedg_restart_info
      type(c_ptr), value :: ctx
      character(kind=c_char), intent(in) :: path(*)
      type(c_ptr), intent(in) :: q(5)
      type(fedg_restart_info), intent(in) :: info
    end function
    integer(c_int) function fedg_restart_read(ctx, path, q, base, info) bind(C, name="fedg_restart_read")
      import :: c_int, c_ptr, c_char, fedg_restart_info
      type(c_ptr), value :: ctx
      character(kind=c_char), intent(in) :: path(*)
      type(c_ptr), intent(in) :: q(5)
      type(c_ptr), value :: base
      type(fedg_restart_info), intent(out) :: info
    end function
  end interface

  type(c_ptr), save :: ctx = c_null_ptr
  type(c_ptr), save :: guess = c_null_ptr    ! column-guess network (atm_dyn_dgm_nonhydro3d_gb300_load_guess)
  real(RP), save :: sl_tau = -1.0_RP, sl_height = -1.0_RP
  logical, save :: sl_hvel = .false.
  integer, save :: vi_max_iter = 1           ! 1: FElib's single linearised solve
  real(RP), save :: vi_tol = 1.0E-10_RP

contains

  !> Create the library context from the cube-domain mesh (call once, after the mesh).
  subroutine atm_dyn_dgm_nonhydro3d_gb300_Init( porder, NeX, NeY, NeZ, dom_xmin, dom_xmax, &
      dom_ymin, dom_ymax, dom_zmin, dom_zmax, modalfilter_flag, max_iter, tol )
    integer, intent(in) :: porder, NeX, NeY, NeZ
    real(RP), intent(in) :: dom_xmin, dom_xmax, dom_ymin, dom_ymax, dom_zmin, dom_zmax
    logical, intent(in) :: modalfilter_flag
    integer, intent(in), optional :: max_iter
    real(RP), intent(in), optional :: tol
    type(fedg_mesh_desc) :: d
    integer(c_int) :: ierr
    d = fedg_mesh_desc(porder, NeX, NeY, NeZ, dom_xmin, dom_xmax, dom_ymin, dom_ymax, dom_zmin, dom_zmax, &
                       1, 1, GRAV, Rdry, CPdry, CVdry, PRES00, merge(1, 0, modalfilter_flag),          &
                       2.0_RP/3.0_RP, 36.0_RP, 16, 2.0_RP/3.0_RP, 36.0_RP, 16, 0)
    ierr = fedg_ctx_create(d, ctx)
    if (ierr < 0) call PRC_abort
    if (present(max_iter)) vi_max_iter = max_iter
    if (present(tol)) vi_tol = tol
  end subroutine atm_dyn_dgm_nonhydro3d_gb300_Init

  !> the library context (shared with the tracer-advection shim)
  function atm_dyn_dgm_nonhydro3d_gb300_ctx() result(c)
    type(c_ptr) :: c
    c = ctx
  end function atm_dyn_dgm_nonhydro3d_gb300_ctx

  subroutine atm_dyn_dgm_nonhydro3d_gb300_Final()
    if (c_associated(ctx)) call fedg_ctx_destroy(ctx)
    ctx = c_null_ptr
  end subroutine atm_dyn_dgm_nonhydro3d_gb300_Final

  !> Register the base state for the whole-step update (AUX_VARS DENS_hyd, PRES_hyd, THERM_hyd and
  !! AUX_VARS2D CORIOLIS; the dry constants Rtot/CVtot/CPtot and DPhydDx/y = 0 are implied).
  subroutine atm_dyn_dgm_nonhydro3d_gb300_set_base_state( DENS_hyd, PRES_hyd, THERM_hyd, CORIOLIS )
    real(RP), intent(in), target :: DENS_hyd(:,:), PRES_hyd(:,:), THERM_hyd(:,:), CORIOLIS(:,:)
    integer(c_int) :: ierr
    !$acc host_data use_device(DENS_hyd, PRES_hyd, THERM_hyd, CORIOLIS)
    ierr = fedg_set_base_state(ctx, c_loc(DENS_hyd), c_loc(PRES_hyd), c_loc(THERM_hyd), c_null_ptr, c_null_ptr, &
                               c_null_ptr, c_null_ptr, c_null_ptr, c_loc(CORIOLIS))
    !$acc end host_data
    if (ierr < 0) call PRC_abort
  end subroutine atm_dyn_dgm_nonhydro3d_gb300_set_base_state

  !> Attach the column-guess network for update(use_guess = .true.): a (3L+1) -> hidden -> hidden -> 3L
  !! GELU MLP (L = NeZ*(porder+1)) with its parameters in the library's logical order, as written by
  !! the training (fe-project_gb300/fedg/guess.py).
  subroutine atm_dyn_dgm_nonhydro3d_gb300_load_guess( levels, hidden, in_scale, out_scale, params )
    integer, intent(in) :: levels, hidden
    real(c_float), intent(in) :: in_scale(4), out_scale(3), params(:)
    integer(c_int) :: ierr
    if (.not. c_associated(guess)) then
      ierr = fedg_guess_create(levels, hidden, guess)
      if (ierr < 0) call PRC_abort
    end if
    if (fedg_guess_set_scales(guess, in_scale, out_scale) < 0) call PRC_abort
    if (fedg_guess_set_params(guess, params, int(size(params), c_long_long)) < 0) call PRC_abort
    if (fedg_guess_load(ctx, guess) < 0) call PRC_abort
  end subroutine atm_dyn_dgm_nonhydro3d_gb300_load_guess

  !> nsteps whole time steps of AtmDynDGMDriver_nonhydro3d_update's stage loop
  !! (driver_nonhydro3d.F90:614-963) for the dry dynamics: HEVE (SSP-RK3) or HEVI (IMEX ARK232) with
  !! the modal filter, the sponge layer when sponge_init set one, in FElib's FP64 arithmetic
  !! (FEDG_PREC_FP64), or fused in float pairs (FEDG_PREC_PAIR, HEVI with tol ~1e-13) or FP32
  !! (FEDG_PREC_MIXED, HEVI).  nfail returns the number of columns whose Newton solve did not converge.
  subroutine atm_dyn_dgm_nonhydro3d_gb300_update( DDENS, MOMX, MOMY, MOMZ, DRHOT, nsteps, hevi, prec, dt, &
      use_guess, nfail, mean_solves )
    real(RP), intent(inout), target :: DDENS(:,:), MOMX(:,:), MOMY(:,:), MOMZ(:,:), DRHOT(:,:)
    integer, intent(in) :: nsteps, prec
    logical, intent(in) :: hevi, use_guess
    real(RP), intent(in) :: dt
    integer, intent(out) :: nfail
    real(RP), intent(out), optional :: mean_solves
    type(c_ptr) :: q(5)
    type(fedg_update_opts) :: o
    real(c_double) :: its
    integer(c_int) :: ierr
    o = fedg_update_opts(merge(FEDG_HEVI, FEDG_HEVE, hevi), prec, vi_max_iter, merge(1, 0, use_guess), dt, vi_tol)
    if (sl_tau > 0.0_RP) then
      ierr = fedg_update_set_sponge(ctx, sl_tau, sl_height, merge(1, 0, sl_hvel))
      if (ierr < 0) call PRC_abort
    end if
    !$acc host_data use_device(DDENS, MOMX, MOMY, MOMZ, DRHOT)
    q = [c_loc(DDENS), c_loc(MOMX), c_loc(MOMY), c_loc(MOMZ), c_loc(DRHOT)]
    ierr = fedg_update(ctx, q, int(nsteps, c_int), o, its)
    !$acc end host_data
    if (ierr < 0) call PRC_abort
    nfail = ierr
    if (present(mean_solves)) mean_solves = its
  end subroutine atm_dyn_dgm_nonhydro3d_gb300_update

  !> Write the restart state (scale_file_restart_meshfield.F90:136-186): the five prognostic fields, the
  !! registered base state and the fast paths' reference wind, in the library's flat format.
  subroutine atm_dyn_dgm_nonhydro3d_gb300_restart_write( path, DDENS, MOMX, MOMY, MOMZ, DRHOT, step, time, dt, &
      scheme )
    character(len=*), intent(in) :: path, scheme
    real(RP), intent(in), target :: DDENS(:,:), MOMX(:,:), MOMY(:,:), MOMZ(:,:), DRHOT(:,:)
    integer, intent(in) :: step
    real(RP), intent(in) :: time, dt
    type(fedg_restart_info) :: info
    type(c_ptr) :: q(5)
    integer :: i
    integer(c_int) :: ierr
    info%step = int(step, c_long_long)
    info%time = time
    info%dt = dt
    info%scheme = c_null_char
    do i = 1, min(len_trim(scheme), 31)
      info%scheme(i) = scheme(i:i)
    end do
    !$acc host_data use_device(DDENS, MOMX, MOMY, MOMZ, DRHOT)
    q = [c_loc(DDENS), c_loc(MOMX), c_loc(MOMY), c_loc(MOMZ), c_loc(DRHOT)]
    ierr = fedg_restart_write(ctx, trim(path)//c_null_char, q, info)
    !$acc end host_data
    if (ierr < 0) call PRC_abort
  end subroutine atm_dyn_dgm_nonhydro3d_gb300_restart_write

  !> Read a restart file written by restart_write into the five prognostic fields (mod_atmos_vars.F90:
  !! 580-633); the mesh must match the context's.  The base state stays the registered one.
  subroutine atm_dyn_dgm_nonhydro3d_gb300_restart_read( path, DDENS, MOMX, MOMY, MOMZ, DRHOT, step, time, dt )
    character(len=*), intent(in) :: path
    real(RP), intent(inout), target :: DDENS(:,:), MOMX(:,:), MOMY(:,:), MOMZ(:,:), DRHOT(:,:)
    integer, intent(out) :: step
    real(RP), intent(out) :: time, dt
    type(fedg_restart_info) :: info
    type(c_ptr) :: q(5)
    integer(c_int) :: ierr
    !$acc host_data use_device(DDENS, MOMX, MOMY, MOMZ, DRHOT)
    q = [c_loc(DDENS), c_loc(MOMX), c_loc(MOMY), c_loc(MOMZ), c_loc(DRHOT)]
    ierr = fedg_restart_read(ctx, trim(path)//c_null_char, q, c_null_ptr, info)
    !$acc end host_data
    if (ierr < 0) call PRC_abort
    step = int(info%step)
    time = info%time
    dt = info%dt
  end subroutine atm_dyn_dgm_nonhydro3d_gb300_restart_read

  !> atm_dyn_nonhydro3d_cal_tend_ex for EQS_TYPE = "NONHYDRO3D_HEVE_GB300"
  subroutine atm_dyn_dgm_nonhydro3d_gb300_cal_tend_heve( &
    DENS_dt, MOMX_dt, MOMY_dt, MOMZ_dt, RHOT_dt, DDENS_, MOMX_, MOMY_, MOMZ_, THERM_, DPRES_, &
    DENS_hyd, PRES_hyd, PRES_hyd_ref, THERM_hyd, CORIOLIS, Rtot, CVtot, CPtot, DPhydDx, DPhydDy, &
    element3D_operation, Dx, Dy, Dz, Sx, Sy, Sz, Lift, lmesh, elem, lmesh2D, elem2D )
    class(LocalMesh3D), intent(in) :: lmesh
    class(ElementBase3D), intent(in) :: elem
    class(LocalMesh2D), intent(in) :: lmesh2D
    class(ElementBase2D), intent(in) :: elem2D
    class(ElementOperationBase3D), intent(in) :: element3D_operation
    type(SparseMat), intent(in) :: Dx, Dy, Dz, Sx, Sy, Sz, Lift
    real(RP), intent(out), target :: DENS_dt(elem%Np,lmesh%NeA), MOMX_dt(elem%Np,lmesh%NeA), &
      MOMY_dt(elem%Np,lmesh%NeA), MOMZ_dt(elem%Np,lmesh%NeA), RHOT_dt(elem%Np,lmesh%NeA)
    real(RP), intent(in), target :: DDENS_(elem%Np,lmesh%NeA), MOMX_(elem%Np,lmesh%NeA), &
      MOMY_(elem%Np,lmesh%NeA), MOMZ_(elem%Np,lmesh%NeA), THERM_(elem%Np,lmesh%NeA),      &
      DPRES_(elem%Np,lmesh%NeA), DENS_hyd(elem%Np,lmesh%NeA), PRES_hyd(elem%Np,lmesh%NeA), &
      PRES_hyd_ref(elem%Np,lmesh%NeA), THERM_hyd(elem%Np,lmesh%NeA),                       &
      CORIOLIS(elem2D%Np,lmesh2D%NeA), Rtot(elem%Np,lmesh%NeA), CVtot(elem%Np,lmesh%NeA),   &
      CPtot(elem%Np,lmesh%NeA), DPhydDx(elem%Np,lmesh%NeA), DPhydDy(elem%Np,lmesh%NeA)
    call cal_tend( FEDG_HEVE )
  contains
    subroutine cal_tend( eqs )
      integer(c_int), intent(in) :: eqs
      type(c_ptr) :: inp(16), outp(5)
      integer(c_int) :: ierr
      !$acc host_data use_device(DENS_dt, MOMX_dt, MOMY_dt, MOMZ_dt, RHOT_dt, DDENS_, MOMX_, MOMY_, &
      !$acc   MOMZ_, THERM_, DPRES_, DENS_hyd, PRES_hyd, PRES_hyd_ref, THERM_hyd, CORIOLIS, Rtot,      &
      !$acc   CVtot, CPtot, DPhydDx, DPhydDy)
      inp = [ c_loc(DDENS_), c_loc(MOMX_), c_loc(MOMY_), c_loc(MOMZ_), c_loc(THERM_), c_loc(DPRES_), &
              c_loc(DENS_hyd), c_loc(PRES_hyd), c_loc(PRES_hyd_ref), c_loc(THERM_hyd), c_loc(CORIOLIS), &
              c_loc(Rtot), c_loc(CVtot), c_loc(CPtot), c_loc(DPhydDx), c_loc(DPhydDy) ]
      outp = [ c_loc(DENS_dt), c_loc(MOMX_dt), c_loc(MOMY_dt), c_loc(MOMZ_dt), c_loc(RHOT_dt) ]
      !$acc end host_data
      ierr = fedg_cal_tend_ex( ctx, inp, outp, eqs )
      if (ierr < 0) call PRC_abort
      ierr = fedg_synchronize( ctx )   ! FElib's next statement may touch the tendencies on another queue
    end subroutine cal_tend
  end subroutine atm_dyn_dgm_nonhydro3d_gb300_cal_tend_heve

  !> atm_dyn_nonhydro3d_cal_tend_ex for EQS_TYPE = "NONHYDRO3D_HEVI_GB300"
  subroutine atm_dyn_dgm_nonhydro3d_gb300_cal_tend_hevi( &
    DENS_dt, MOMX_dt, MOMY_dt, MOMZ_dt, RHOT_dt, DDENS_, MOMX_, MOMY_, MOMZ_, THERM_, DPRES_, &
    DENS_hyd, PRES_hyd, PRES_hyd_ref, THERM_hyd, CORIOLIS, Rtot, CVtot, CPtot, DPhydDx, DPhydDy, &
    element3D_operation, Dx, Dy, Dz, Sx, Sy, Sz, Lift, lmesh, elem, lmesh2D, elem2D )
    class(LocalMesh3D), intent(in) :: lmesh
    class(ElementBase3D), intent(in) :: elem
    class(LocalMesh2D), intent(in) :: lmesh2D
    class(ElementBase2D), intent(in) :: elem2D
    class(ElementOperationBase3D), intent(in) :: element3D_operation
    type(SparseMat), intent(in) :: Dx, Dy, Dz, Sx, Sy, Sz, Lift
    real(RP), intent(out), target :: DENS_dt(elem%Np,lmesh%NeA), MOMX_dt(elem%Np,lmesh%NeA), &
      MOMY_dt(elem%Np,lmesh%NeA), MOMZ_dt(elem%Np,lmesh%NeA), RHOT_dt(elem%Np,lmesh%NeA)
    real(RP), intent(in), target :: DDENS_(elem%Np,lmesh%NeA), MOMX_(elem%Np,lmesh%NeA), &
      MOMY_(elem%Np,lmesh%NeA), MOMZ_(elem%Np,lmesh%NeA), THERM_(elem%Np,lmesh%NeA),      &
      DPRES_(elem%Np,lmesh%NeA), DENS_hyd(elem%Np,lmesh%NeA), PRES_hyd(elem%Np,lmesh%NeA), &
      PRES_hyd_ref(elem%Np,lmesh%NeA), THERM_hyd(elem%Np,lmesh%NeA),                       &
      CORIOLIS(elem2D%Np,lmesh2D%NeA), Rtot(elem%Np,lmesh%NeA), CVtot(elem%Np,lmesh%NeA),   &
      CPtot(elem%Np,lmesh%NeA), DPhydDx(elem%Np,lmesh%NeA), DPhydDy(elem%Np,lmesh%NeA)
    type(c_ptr) :: inp(16), outp(5)
    integer(c_int) :: ierr
    !$acc host_data use_device(DENS_dt, MOMX_dt, MOMY_dt, MOMZ_dt, RHOT_dt, DDENS_, MOMX_, MOMY_, &
    !$acc   MOMZ_, THERM_, DPRES_, DENS_hyd, PRES_hyd, PRES_hyd_ref, THERM_hyd, CORIOLIS, Rtot,      &
    !$acc   CVtot, CPtot, DPhydDx, DPhydDy)
    inp = [ c_loc(DDENS_), c_loc(MOMX_), c_loc(MOMY_), c_loc(MOMZ_), c_loc(THERM_), c_loc(DPRES_), &
            c_loc(DENS_hyd), c_loc(PRES_hyd), c_loc(PRES_hyd_ref), c_loc(THERM_hyd), c_loc(CORIOLIS), &
            c_loc(Rtot), c_loc(CVtot), c_loc(CPtot), c_loc(DPhydDx), c_loc(DPhydDy) ]
    outp = [ c_loc(DENS_dt), c_loc(MOMX_dt), c_loc(MOMY_dt), c_loc(MOMZ_dt), c_loc(RHOT_dt) ]
    !$acc end host_data
    ierr = fedg_cal_tend_ex( ctx, inp, outp, FEDG_HEVI )
    if (ierr < 0) call PRC_abort
    ierr = fedg_synchronize( ctx )
  end subroutine atm_dyn_dgm_nonhydro3d_gb300_cal_tend_hevi

  !> atm_dyn_nonhydro3d_cal_vi for EQS_TYPE = "NONHYDRO3D_HEVI_GB300"
  subroutine atm_dyn_dgm_nonhydro3d_gb300_cal_vi( &
    DENS_dt, MOMX_dt, MOMY_dt, MOMZ_dt, RHOT_dt, DDENS_, MOMX_, MOMY_, MOMZ_, THERM_, DENS_hyd, PRES_hyd, &
    DDENS0_, MOMX0_, MOMY0_, MOMZ0_, THERM0_, Rtot, CVtot, CPtot, element3D_operation, Dz, Lift,          &
    impl_fac, dt, lmesh, elem, lmesh2D, elem2D )
    class(LocalMesh3D), intent(in) :: lmesh
    class(ElementBase3D), intent(in) :: elem
    class(LocalMesh2D), intent(in) :: lmesh2D
    class(ElementBase2D), intent(in) :: elem2D
    class(ElementOperationBase3D), intent(in) :: element3D_operation
    class(SparseMat), intent(in) :: Dz, Lift
    real(RP), intent(out), target :: DENS_dt(elem%Np,lmesh%NeA), MOMX_dt(elem%Np,lmesh%NeA), &
      MOMY_dt(elem%Np,lmesh%NeA), MOMZ_dt(elem%Np,lmesh%NeA), RHOT_dt(elem%Np,lmesh%NeA)
    real(RP), intent(in), target :: DDENS_(elem%Np,lmesh%NeA), MOMX_(elem%Np,lmesh%NeA),        &
      MOMY_(elem%Np,lmesh%NeA), MOMZ_(elem%Np,lmesh%NeA), THERM_(elem%Np,lmesh%NeA),             &
      DENS_hyd(elem%Np,lmesh%NeA), PRES_hyd(elem%Np,lmesh%NeA), DDENS0_(elem%Np,lmesh%NeA),      &
      MOMX0_(elem%Np,lmesh%NeA), MOMY0_(elem%Np,lmesh%NeA), MOMZ0_(elem%Np,lmesh%NeA),          &
      THERM0_(elem%Np,lmesh%NeA), Rtot(elem%Np,lmesh%NeA), CVtot(elem%Np,lmesh%NeA),            &
      CPtot(elem%Np,lmesh%NeA)
    real(RP), intent(in) :: impl_fac, dt
    type(c_ptr) :: inp(12), outp(5)
    integer(c_int) :: ierr
    !$acc host_data use_device(DENS_dt, MOMX_dt, MOMY_dt, MOMZ_dt, RHOT_dt, DDENS_, MOMX_, MOMY_, MOMZ_, &
    !$acc   THERM_, DENS_hyd, PRES_hyd, DDENS0_, MOMX0_, MOMY0_, MOMZ0_, THERM0_)
    inp = [ c_loc(DDENS_), c_loc(MOMX_), c_loc(MOMY_), c_loc(MOMZ_), c_loc(THERM_), c_loc(DENS_hyd), &
            c_loc(PRES_hyd), c_loc(DDENS0_), c_loc(MOMX0_), c_loc(MOMY0_), c_loc(MOMZ0_), c_loc(THERM0_) ]
    outp = [ c_loc(DENS_dt), c_loc(MOMX_dt), c_loc(MOMY_dt), c_loc(MOMZ_dt), c_loc(RHOT_dt) ]
    !$acc end host_data
    ierr = fedg_cal_vi( ctx, inp, impl_fac, dt, vi_max_iter, vi_tol, outp, c_null_ptr )
    if (ierr < 0) call PRC_abort
    if (ierr > 0) then
      LOG_INFO("atm_dyn_dgm_nonhydro3d_gb300_cal_vi",*) 'Newton not converged in columns:', ierr
    end if
  end subroutine atm_dyn_dgm_nonhydro3d_gb300_cal_vi

  !> AtmDyn_Nonhydro3D_Numdiff%Apply (…_nonhydro3d_numdiff.F90:214-242) on the prognostic fields
  subroutine atm_dyn_dgm_nonhydro3d_gb300_numdiff_apply( DDENS, MOMX, MOMY, MOMZ, THERM, &
    ND_LAPLACIAN_NUM, ND_COEF_H, ND_COEF_V, dtsec, lmesh, elem )
    class(LocalMesh3D), intent(in) :: lmesh
    class(ElementBase3D), intent(in) :: elem
    real(RP), intent(inout), target :: DDENS(elem%Np,lmesh%NeA), MOMX(elem%Np,lmesh%NeA), &
      MOMY(elem%Np,lmesh%NeA), MOMZ(elem%Np,lmesh%NeA), THERM(elem%Np,lmesh%NeA)
    integer, intent(in) :: ND_LAPLACIAN_NUM
    real(RP), intent(in) :: ND_COEF_H, ND_COEF_V, dtsec
    type(c_ptr) :: q(5)
    integer(c_int) :: ierr
    !$acc host_data use_device(DDENS, MOMX, MOMY, MOMZ, THERM)
    q = [ c_loc(DDENS), c_loc(MOMX), c_loc(MOMY), c_loc(MOMZ), c_loc(THERM) ]
    !$acc end host_data
    ierr = fedg_numdiff_apply( ctx, q, ND_LAPLACIAN_NUM, ND_COEF_H, ND_COEF_V, dtsec )
    if (ierr < 0) call PRC_abort
    ierr = fedg_synchronize( ctx )
  end subroutine atm_dyn_dgm_nonhydro3d_gb300_numdiff_apply

  !> the &PARAM_ATMOS_DYN_SPONGELAYER settings (…_dgm_spongelayer.F90:57-123: tau defaults to 10 dt)
  subroutine atm_dyn_dgm_nonhydro3d_gb300_sponge_init( wdamp_tau, wdamp_height, hveldamp_flag )
    real(RP), intent(in) :: wdamp_tau, wdamp_height
    logical, intent(in) :: hveldamp_flag
    sl_tau = wdamp_tau
    sl_height = wdamp_height
    sl_hvel = hveldamp_flag
  end subroutine atm_dyn_dgm_nonhydro3d_gb300_sponge_init

  !> AtmDynSpongeLayer%AddTend (…_dgm_spongelayer.F90:134-185)
  subroutine atm_dyn_dgm_nonhydro3d_gb300_sponge_add_tend( MOMX_dt, MOMY_dt, MOMZ_dt, MOMX_, MOMY_, MOMZ_, &
    lmesh, elem )
    class(LocalMesh3D), intent(in) :: lmesh
    class(ElementBase3D), intent(in) :: elem
    real(RP), intent(inout), target :: MOMX_dt(elem%Np,lmesh%NeA), MOMY_dt(elem%Np,lmesh%NeA), &
      MOMZ_dt(elem%Np,lmesh%NeA)
    real(RP), intent(in), target :: MOMX_(elem%Np,lmesh%NeA), MOMY_(elem%Np,lmesh%NeA), MOMZ_(elem%Np,lmesh%NeA)
    type(c_ptr) :: tend(3), mom(3)
    integer(c_int) :: ierr
    !$acc host_data use_device(MOMX_dt, MOMY_dt, MOMZ_dt, MOMX_, MOMY_, MOMZ_)
    tend = [ c_loc(MOMX_dt), c_loc(MOMY_dt), c_loc(MOMZ_dt) ]
    mom = [ c_loc(MOMX_), c_loc(MOMY_), c_loc(MOMZ_) ]
    !$acc end host_data
    ierr = fedg_sponge_add_tend( ctx, tend, mom, sl_tau, sl_height, merge(1, 0, sl_hvel) )
    if (ierr < 0) call PRC_abort
  end subroutine atm_dyn_dgm_nonhydro3d_gb300_sponge_add_tend

end module scale_atm_dyn_dgm_nonhydro3d_gb300
