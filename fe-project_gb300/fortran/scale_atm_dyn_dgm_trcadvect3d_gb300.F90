!-------------------------------------------------------------------------------
!> module FElib / Fluid dyn solver / Atmosphere / Tracer advection / GB300 binding
!!
!! ISO_C_BINDING shim with the argument lists of FElib's tracer-advection routines
!! (FElib/src/fluid_dyn_solver/scale_atm_dyn_dgm_trcadvect3d_heve.F90: calc_fct_coef :234-306,
!! cal_tend :149-231, TMAR :311-340, save_massflux :343-401) and of the negative fixer the tracer
!! driver runs after its step (FElib/src/microphysics/scale_atm_phy_mp_dgm_common.F90:429-556, called
!! from fix_negative_val, ..._driver_trcadv3d.F90:596-651), calling the GB300 library libfedg.so
!! (C ABI: include/fedg.h) on the driver's OpenACC-resident fields.  It shares the library context
!! of scale_atm_dyn_dgm_nonhydro3d_gb300 (create that one first).  Not compiled in this repository
!! (no Fortran compiler in its build image); built with the model by a maintainer, linked with -lfedg.
!-------------------------------------------------------------------------------
#include "scaleFElib.h"
module scale_atm_dyn_dgm_trcadvect3d_gb300
  use iso_c_binding
  use scale_precision
  use scale_prc, only: PRC_abort
  use scale_element_base, only: ElementBase2D, ElementBase3D
  use scale_element_operation_base, only: ElementOperationBase3D
  use scale_localmesh_2d, only: LocalMesh2D
  use scale_localmesh_3d, only: LocalMesh3D
  use scale_sparsemat, only: SparseMat
  use scale_atm_dyn_dgm_nonhydro3d_gb300, only: atm_dyn_dgm_nonhydro3d_gb300_ctx
  implicit none
  private

  public :: atm_dyn_dgm_trcadvect3d_gb300_calc_fct_coef
  public :: atm_dyn_dgm_trcadvect3d_gb300_cal_tend
  public :: atm_dyn_dgm_trcadvect3d_gb300_TMAR
  public :: atm_dyn_dgm_trcadvect3d_gb300_save_massflux
  public :: atm_phy_mp_dgm_common_gb300_negative_fixer
  public :: atm_dyn_dgm_trcadvect3d_gb300_update_pressure_specific_heat

  interface
    integer(c_int) function fedg_trc_fct_coef(ctx, qtrc, mflx, rhoq_tp, alph_m, alph_p, ddens, ddens0, &
        c_ssm1, dt, fct) bind(C, name="fedg_trc_fct_coef")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx, qtrc, rhoq_tp, alph_m, alph_p, ddens, ddens0, fct
      type(c_ptr), intent(in) :: mflx(3)
      real(c_double), value :: c_ssm1, dt
    end function
    integer(c_int) function fedg_trc_cal_tend(ctx, qtrc, mflx, alph_m, alph_p, fct, rhoq_tp, qtrc_dt) &
        bind(C, name="fedg_trc_cal_tend")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx, qtrc, alph_m, alph_p, fct, rhoq_tp, qtrc_dt
      type(c_ptr), intent(in) :: mflx(3)
    end function
    integer(c_int) function fedg_trc_tmar(ctx, qtrc, ddens) bind(C, name="fedg_trc_tmar")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx, qtrc, ddens
    end function
    integer(c_int) function fedg_trc_save_massflux(ctx, rkstage, q, dpres, w_h, w_v, is_hevi, mflx, &
        alph_m, alph_p) bind(C, name="fedg_trc_save_massflux")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx, dpres, alph_m, alph_p
      integer(c_int), value :: rkstage, is_hevi
      type(c_ptr), intent(in) :: q(5), mflx(3)
      real(c_double), value :: w_h, w_v
    end function
    integer(c_int) function fedg_trc_negative_fixer(ctx, qtrc, qa, qla, qia, mass, r, cv, cp, ddens, pres, &
        cvtot, cptot, rtot, dens_hyd, pres_hyd, drhot, dt) bind(C, name="fedg_trc_negative_fixer")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx, ddens, pres, cvtot, cptot, rtot, dens_hyd, pres_hyd, drhot
      type(c_ptr), intent(in) :: qtrc(*)
      integer(c_int), value :: qa, qla, qia
      real(c_double), intent(in) :: mass(*), r(*), cv(*), cp(*)
      real(c_double), value :: dt
    end function
    integer(c_int) function fedg_trc_specific_heat_pressure(ctx, qtrc, qa, mass, r, cv, cp, drhot, pres_hyd, &
        therm_hyd, rtot, cvtot, cptot, pres, dpres) bind(C, name="fedg_trc_specific_heat_pressure")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx, drhot, pres_hyd, therm_hyd, rtot, cvtot, cptot, pres, dpres
      type(c_ptr), intent(in) :: qtrc(*)
      integer(c_int), value :: qa
      real(c_double), intent(in) :: mass(*), r(*), cv(*), cp(*)
    end function
    integer(c_int) function fedg_synchronize(ctx) bind(C, name="fedg_synchronize")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
  end interface

contains

  !> atm_dyn_dgm_trcadvect3d_heve_calc_fct_coef (FaceIntMat: the library forms the LGL face weights)
  subroutine atm_dyn_dgm_trcadvect3d_gb300_calc_fct_coef( &
    fct_coef, QTRC_, MOMX_, MOMY_, MOMZ_, RHOQ_tp_, AlphDens_M, AlphDens_P, &
    DENS_hyd, DDENS_, DDENS0_, rk_c_ssm1, dt, FaceIntMat, lmesh, elem, lmesh2D, elem2D, disable_limiter )
    class(LocalMesh3D), intent(in) :: lmesh
    class(ElementBase3D), intent(in) :: elem
    class(LocalMesh2D), intent(in) :: lmesh2D
    class(ElementBase2D), intent(in) :: elem2D
    real(RP), intent(out), target :: fct_coef(elem%Np,lmesh%NeA)
    real(RP), intent(in), target :: QTRC_(elem%Np,lmesh%NeA), MOMX_(elem%Np,lmesh%NeA), &
      MOMY_(elem%Np,lmesh%NeA), MOMZ_(elem%Np,lmesh%NeA), RHOQ_tp_(elem%Np,lmesh%NeA),  &
      AlphDens_M(elem%NfpTot,lmesh%Ne), AlphDens_P(elem%NfpTot,lmesh%Ne),               &
      DENS_hyd(elem%Np,lmesh%NeA), DDENS_(elem%Np,lmesh%NeA), DDENS0_(elem%Np,lmesh%NeA)
    real(RP), intent(in) :: rk_c_ssm1, dt
    type(SparseMat), intent(in) :: FaceIntMat
    logical, intent(in), optional :: disable_limiter
    type(c_ptr) :: mflx(3)
    integer(c_int) :: ierr
    if ( present(disable_limiter) ) then
      if ( disable_limiter ) then
        !$acc kernels present(fct_coef)
        fct_coef(:,:) = 1.0_RP
        !$acc end kernels
        return
      end if
    end if
    !$acc host_data use_device(fct_coef, QTRC_, MOMX_, MOMY_, MOMZ_, RHOQ_tp_, AlphDens_M, AlphDens_P, &
    !$acc   DDENS_, DDENS0_)
    mflx = [ c_loc(MOMX_), c_loc(MOMY_), c_loc(MOMZ_) ]
    ierr = fedg_trc_fct_coef( atm_dyn_dgm_nonhydro3d_gb300_ctx(), c_loc(QTRC_), mflx, c_loc(RHOQ_tp_), &
      c_loc(AlphDens_M), c_loc(AlphDens_P), c_loc(DDENS_), c_loc(DDENS0_), rk_c_ssm1, dt, c_loc(fct_coef) )
    !$acc end host_data
    if (ierr < 0) call PRC_abort
    ierr = fedg_synchronize( atm_dyn_dgm_nonhydro3d_gb300_ctx() )
  end subroutine atm_dyn_dgm_trcadvect3d_gb300_calc_fct_coef

  !> atm_dyn_dgm_trcadvect3d_heve_cal_tend
  subroutine atm_dyn_dgm_trcadvect3d_gb300_cal_tend( &
    QTRC_dt, QTRC_, MOMX_, MOMY_, MOMZ_, alphDENS_M, alphDENS_P, fct_coef, RHOQ_tp, &
    element3D_operation, FaceIntMat, lmesh, elem, lmesh2D, elem2D )
    class(LocalMesh3D), intent(in) :: lmesh
    class(ElementBase3D), intent(in) :: elem
    class(LocalMesh2D), intent(in) :: lmesh2D
    class(ElementBase2D), intent(in) :: elem2D
    real(RP), intent(out), target :: QTRC_dt(elem%Np,lmesh%NeA)
    real(RP), intent(in), target :: QTRC_(elem%Np,lmesh%NeA), MOMX_(elem%Np,lmesh%NeA), &
      MOMY_(elem%Np,lmesh%NeA), MOMZ_(elem%Np,lmesh%NeA),                               &
      alphDENS_M(elem%NfpTot,lmesh%Ne), alphDENS_P(elem%NfpTot,lmesh%Ne),               &
      fct_coef(elem%Np,lmesh%NeA), RHOQ_tp(elem%Np,lmesh%NeA)
    class(ElementOperationBase3D), intent(in) :: element3D_operation
    type(SparseMat), intent(in) :: FaceIntMat
    type(c_ptr) :: mflx(3)
    integer(c_int) :: ierr
    !$acc host_data use_device(QTRC_dt, QTRC_, MOMX_, MOMY_, MOMZ_, alphDENS_M, alphDENS_P, fct_coef, RHOQ_tp)
    mflx = [ c_loc(MOMX_), c_loc(MOMY_), c_loc(MOMZ_) ]
    ierr = fedg_trc_cal_tend( atm_dyn_dgm_nonhydro3d_gb300_ctx(), c_loc(QTRC_), mflx, c_loc(alphDENS_M), &
      c_loc(alphDENS_P), c_loc(fct_coef), c_loc(RHOQ_tp), c_loc(QTRC_dt) )
    !$acc end host_data
    if (ierr < 0) call PRC_abort
    ierr = fedg_synchronize( atm_dyn_dgm_nonhydro3d_gb300_ctx() )
  end subroutine atm_dyn_dgm_trcadvect3d_gb300_cal_tend

  !> atm_dyn_dgm_trcadvect3d_TMAR (DENS_hyd is the registered base state)
  subroutine atm_dyn_dgm_trcadvect3d_gb300_TMAR( QTRC_, DENS_hyd, DDENS_, lmesh, elem, lmesh2D, elem2D )
    class(LocalMesh3D), intent(in) :: lmesh
    class(ElementBase3D), intent(in) :: elem
    class(LocalMesh2D), intent(in) :: lmesh2D
    class(ElementBase2D), intent(in) :: elem2D
    real(RP), intent(inout), target :: QTRC_(elem%Np,lmesh%NeA)
    real(RP), intent(in), target :: DENS_hyd(elem%Np,lmesh%NeA), DDENS_(elem%Np,lmesh%NeA)
    integer(c_int) :: ierr
    !$acc host_data use_device(QTRC_, DDENS_)
    ierr = fedg_trc_tmar( atm_dyn_dgm_nonhydro3d_gb300_ctx(), c_loc(QTRC_), c_loc(DDENS_) )
    !$acc end host_data
    if (ierr < 0) call PRC_abort
    ierr = fedg_synchronize( atm_dyn_dgm_nonhydro3d_gb300_ctx() )
  end subroutine atm_dyn_dgm_trcadvect3d_gb300_TMAR

  !> atm_dyn_dgm_trcadvect3d_save_massflux (Rtot/CVtot/CPtot: the registered dry constants)
  subroutine atm_dyn_dgm_trcadvect3d_gb300_save_massflux( &
    MFLX_x_tavg, MFLX_y_tavg, MFLX_z_tavg, alph_dens_M, alph_dens_P, &
    DDENS, MOMX, MOMY, MOMZ, DPRES, DENS_hyd, PRES_hyd, Rtot, CVtot, CPtot, &
    lmesh, elem, rkstage, tavg_weight_h, tavg_weight_v, is_hevi )
    class(LocalMesh3D), intent(in) :: lmesh
    class(ElementBase3D), intent(in) :: elem
    real(RP), intent(inout), target :: MFLX_x_tavg(elem%Np,lmesh%NeA), MFLX_y_tavg(elem%Np,lmesh%NeA), &
      MFLX_z_tavg(elem%Np,lmesh%NeA), alph_dens_M(elem%NfpTot,lmesh%Ne), alph_dens_P(elem%NfpTot,lmesh%Ne)
    real(RP), intent(in), target :: DDENS(elem%Np,lmesh%NeA), MOMX(elem%Np,lmesh%NeA),   &
      MOMY(elem%Np,lmesh%NeA), MOMZ(elem%Np,lmesh%NeA), DPRES(elem%Np,lmesh%NeA),        &
      DENS_hyd(elem%Np,lmesh%NeA), PRES_hyd(elem%Np,lmesh%NeA), Rtot(elem%Np,lmesh%NeA),  &
      CVtot(elem%Np,lmesh%NeA), CPtot(elem%Np,lmesh%NeA)
    integer, intent(in) :: rkstage
    real(RP), intent(in) :: tavg_weight_h, tavg_weight_v
    logical, intent(in) :: is_hevi
    type(c_ptr) :: q(5), mflx(3)
    integer(c_int) :: ierr
    !$acc host_data use_device(MFLX_x_tavg, MFLX_y_tavg, MFLX_z_tavg, alph_dens_M, alph_dens_P, &
    !$acc   DDENS, MOMX, MOMY, MOMZ, DPRES)
    ! the fifth state field (DRHOT) is only read when DPRES is not given
    q = [ c_loc(DDENS), c_loc(MOMX), c_loc(MOMY), c_loc(MOMZ), c_loc(DPRES) ]
    mflx = [ c_loc(MFLX_x_tavg), c_loc(MFLX_y_tavg), c_loc(MFLX_z_tavg) ]
    ierr = fedg_trc_save_massflux( atm_dyn_dgm_nonhydro3d_gb300_ctx(), rkstage, q, c_loc(DPRES), &
      tavg_weight_h, tavg_weight_v, merge(1, 0, is_hevi), mflx, c_loc(alph_dens_M), c_loc(alph_dens_P) )
    !$acc end host_data
    if (ierr < 0) call PRC_abort
    ierr = fedg_synchronize( atm_dyn_dgm_nonhydro3d_gb300_ctx() )
  end subroutine atm_dyn_dgm_trcadvect3d_gb300_save_massflux

  !> atm_phy_mp_dgm_common_negative_fixer with FElib's argument list (the tracer properties are
  !! scale_tracer's; QA must equal 1 + QLA + QIA, the case in which FElib's routine defines every
  !! tracer's result)
  subroutine atm_phy_mp_dgm_common_gb300_negative_fixer( &
    QTRC, DDENS, PRES, CVtot, CPtot, Rtot, DENS_hyd, PRES_hyd, &
    dt, lmesh, elem, QA, QLA, QIA, DRHOT )
    use openacc, only: acc_deviceptr
    use scale_tracer, only: TRACER_MASS, TRACER_R, TRACER_CV, TRACER_CP
    use scale_localmeshfield_base, only: LocalMeshFieldBaseList
    class(LocalMesh3D), intent(in) :: lmesh
    class(ElementBase3D), intent(in) :: elem
    integer, intent(in) :: QA
    type(LocalMeshFieldBaseList), intent(inout) :: QTRC(QA)
    real(RP), intent(inout), target :: DDENS(elem%Np,lmesh%NeA)
    real(RP), intent(inout), target :: PRES(elem%Np,lmesh%NeA)
    real(RP), intent(inout), target :: CVtot(elem%Np,lmesh%NeA)
    real(RP), intent(inout), target :: CPtot(elem%Np,lmesh%NeA)
    real(RP), intent(inout), target :: Rtot(elem%Np,lmesh%NeA)
    real(RP), intent(in), target :: DENS_hyd(elem%Np,lmesh%NeA)
    real(RP), intent(in), target :: PRES_hyd(elem%Np,lmesh%NeA)
    real(RP), intent(in) :: dt
    integer, intent(in) :: QLA, QIA
    real(RP), intent(inout), optional, target :: DRHOT(elem%Np,lmesh%NeA)

    type(c_ptr) :: qp(QA), drp
    integer :: iq
    integer(c_int) :: ierr
    do iq = 1, QA
      qp(iq) = acc_deviceptr( QTRC(iq)%ptr%val )
    end do
    drp = c_null_ptr
    if ( present(DRHOT) ) drp = acc_deviceptr( DRHOT )
    ierr = fedg_trc_negative_fixer( atm_dyn_dgm_nonhydro3d_gb300_ctx(), qp, QA, QLA, QIA, &
      TRACER_MASS, TRACER_R, TRACER_CV, TRACER_CP, &
      acc_deviceptr(DDENS), acc_deviceptr(PRES), acc_deviceptr(CVtot), acc_deviceptr(CPtot), &
      acc_deviceptr(Rtot), acc_deviceptr(DENS_hyd), acc_deviceptr(PRES_hyd), drp, dt )
    if (ierr < 0) call PRC_abort
    ierr = fedg_synchronize( atm_dyn_dgm_nonhydro3d_gb300_ctx() )
  end subroutine atm_phy_mp_dgm_common_gb300_negative_fixer

  !> the tracer driver's update_pressure_specific_heat (driver_trcadv3d.F90:653-716) on one local
  !! mesh's arrays: Rtot, CVtot, CPtot from the QA tracers and PRES (DPRES) from DRHOT through the
  !! mixture's exponent
  subroutine atm_dyn_dgm_trcadvect3d_gb300_update_pressure_specific_heat( &
    PRES, DPRES, Rtot, CVtot, CPtot, QTRC, DRHOT, PRES_hyd, THERM_hyd, lmesh, elem, QA )
    use openacc, only: acc_deviceptr
    use scale_tracer, only: TRACER_MASS, TRACER_R, TRACER_CV, TRACER_CP
    use scale_localmeshfield_base, only: LocalMeshFieldBaseList
    class(LocalMesh3D), intent(in) :: lmesh
    class(ElementBase3D), intent(in) :: elem
    integer, intent(in) :: QA
    real(RP), intent(inout), target :: PRES(elem%Np,lmesh%NeA)
    real(RP), intent(inout), target :: DPRES(elem%Np,lmesh%NeA)
    real(RP), intent(inout), target :: Rtot(elem%Np,lmesh%NeA)
    real(RP), intent(inout), target :: CVtot(elem%Np,lmesh%NeA)
    real(RP), intent(inout), target :: CPtot(elem%Np,lmesh%NeA)
    type(LocalMeshFieldBaseList), intent(in) :: QTRC(QA)
    real(RP), intent(in), target :: DRHOT(elem%Np,lmesh%NeA)
    real(RP), intent(in), target :: PRES_hyd(elem%Np,lmesh%NeA)
    real(RP), intent(in), target :: THERM_hyd(elem%Np,lmesh%NeA)

    type(c_ptr) :: qp(max(QA, 1))
    integer :: iq
    integer(c_int) :: ierr
    qp(1) = c_null_ptr
    do iq = 1, QA
      qp(iq) = acc_deviceptr( QTRC(iq)%ptr%val )
    end do
    ierr = fedg_trc_specific_heat_pressure( atm_dyn_dgm_nonhydro3d_gb300_ctx(), qp, QA, &
      TRACER_MASS, TRACER_R, TRACER_CV, TRACER_CP, &
      acc_deviceptr(DRHOT), acc_deviceptr(PRES_hyd), acc_deviceptr(THERM_hyd), &
      acc_deviceptr(Rtot), acc_deviceptr(CVtot), acc_deviceptr(CPtot), acc_deviceptr(PRES), acc_deviceptr(DPRES) )
    if (ierr < 0) call PRC_abort
    ierr = fedg_synchronize( atm_dyn_dgm_nonhydro3d_gb300_ctx() )
  end subroutine atm_dyn_dgm_trcadvect3d_gb300_update_pressure_specific_heat

end module scale_atm_dyn_dgm_trcadvect3d_gb300
