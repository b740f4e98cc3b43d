!-----------------------------------------------------------------------------
! ISO_C_BINDING shim: drop-in GPU bodies for the reference's pressure solve.
!
! Replaces, with the same argument lists,
!   SUBROUTINE MG_initial()                                    IBM/CORE_MG.F90:31
!   SUBROUTINE MG_Solver(var, rr, MG_itSolver, MG_itResidual, compTime)
!                                                              IBM/CORE_MG.F90:281
!   SUBROUTINE solve_poisson()                                 IBM/CORE_POISSON.F90:493
! and adds
!   SUBROUTINE fsi_mg_update_geometry()   -- call after every set_boundary
!   SUBROUTINE fsi_mg_finalize()          -- call from deallocate_memory
!
! Link this file instead of the reference's MG_initial / MG_Solver /
! solve_poisson (compile CORE_MG.F90 and CORE_POISSON.F90 with
! -DFSI_MG_GPU_SHIM and guard those three bodies with #ifndef FSI_MG_GPU_SHIM),
! and link libfsi_mg.so.  All arrays are the reference's module arrays,
! passed by address as contiguous Fortran arrays with lower bound 0.
!-----------------------------------------------------------------------------
MODULE fsi_mg_gpu

  USE, INTRINSIC :: iso_c_binding
  IMPLICIT NONE

  TYPE, BIND(C) :: fsi_mg_params
    INTEGER(C_INT) :: ndim, nx, ny, nz, pp_solver_type, iRedBlack
    INTEGER(C_INT) :: mgcycle(3), iterFinest, iterCoarsest, mgLevels(3)
    INTEGER(C_INT) :: iterMax_Poisson, iterMax_ad, bc(6), pbc(6)
    INTEGER(C_INT) :: internal_boundary_present, boundary_formulation
    INTEGER(C_INT) :: coarse_flag_mode, precision_mode, outer_krylov
    REAL(C_DOUBLE) :: omega, restol_Poisson, restol_ad, ppp(6), outflow_area, alfa
  END TYPE fsi_mg_params

  ! device pointers of the momentum right-hand side (fsi_mg_rhs_ad_fields)
  TYPE, BIND(C) :: fsi_mg_rhs_ad_fields
    TYPE(C_PTR) :: u, v, w, face_u, face_v, face_w
    TYPE(C_PTR) :: bc(9)                 ! bcxu, bcyu, bczu, bcxv, bcyv, bczv, bcxw, bcyw, bczw
    TYPE(C_PTR) :: viscTot, bcvisc(3), exp_weight
    TYPE(C_PTR) :: nluOld, nlvOld, nlwOld, p, nlu, nlv, nlw
    REAL(C_DOUBLE) :: reinv              ! 1/Re (solve_ad with zero-gradient sides and a GCM body)
  END TYPE fsi_mg_rhs_ad_fields

  ! fsi_mg_bc_values: vel(component u/v/w, side x1..z2) = ux1, vx1, wx1, ux2, ...;
  ! freq likewise (pulsatile inflow)
  TYPE, BIND(C) :: fsi_mg_bc_values
    REAL(C_DOUBLE) :: vel(3,6), freq(3,6)
    REAL(C_DOUBLE) :: time, tstart_gust, xout, yout
  END TYPE fsi_mg_bc_values

  TYPE(C_PTR), SAVE :: fsi_mg_handle = C_NULL_PTR
  INTEGER, SAVE :: fsi_mg_precision = 0      ! 0 FP64, 1 mixed (set before MG_initial)

  INTERFACE
    INTEGER(C_INT) FUNCTION fsi_mg_create(p, x, y, z, h) BIND(C, NAME='fsi_mg_create')
      IMPORT :: C_INT, C_DOUBLE, C_PTR, fsi_mg_params
      TYPE(fsi_mg_params), INTENT(IN) :: p
      REAL(C_DOUBLE), INTENT(IN) :: x(*), y(*), z(*)
      TYPE(C_PTR), INTENT(OUT) :: h
    END FUNCTION
    INTEGER(C_INT) FUNCTION fsi_mg_set_geometry(h, iblank, ghost, ium, iup, jum, jup, kum, kup, &
        nGhost, iG, jG, kG, iCI, jCI, kCI, coeff, probe, pgrad) BIND(C, NAME='fsi_mg_set_geometry')
      IMPORT :: C_INT, C_INT8_T, C_DOUBLE, C_PTR
      TYPE(C_PTR), VALUE :: h
      INTEGER(C_INT8_T), INTENT(IN) :: iblank(*), ghost(*), ium(*), iup(*), jum(*), jup(*), kum(*), kup(*)
      INTEGER(C_INT), VALUE :: nGhost
      INTEGER(C_INT), INTENT(IN) :: iG(*), jG(*), kG(*), iCI(*), jCI(*), kCI(*)
      REAL(C_DOUBLE), INTENT(IN) :: coeff(*), probe(*), pgrad(*)
    END FUNCTION
    INTEGER(C_INT) FUNCTION fsi_mg_set_fresh_cells(h, fresh) BIND(C, NAME='fsi_mg_set_fresh_cells')
      IMPORT :: C_INT, C_INT8_T, C_PTR
      TYPE(C_PTR), VALUE :: h
      INTEGER(C_INT8_T), INTENT(IN) :: fresh(*)
    END FUNCTION
    INTEGER(C_INT) FUNCTION fsi_mg_solve(h, pPrime, nlu0, nlw0, iters, maxres, loc, compTime) &
        BIND(C, NAME='fsi_mg_solve')
      IMPORT :: C_INT, C_DOUBLE, C_PTR
      TYPE(C_PTR), VALUE :: h
      REAL(C_DOUBLE), INTENT(INOUT) :: pPrime(*)
      REAL(C_DOUBLE), INTENT(IN) :: nlu0(*)
      REAL(C_DOUBLE), INTENT(OUT) :: nlw0(*)
      INTEGER(C_INT), INTENT(OUT) :: iters, loc(3)
      REAL(C_DOUBLE), INTENT(OUT) :: maxres, compTime
    END FUNCTION
    INTEGER(C_INT) FUNCTION fsi_mg_mg_solver(h, var, rr, compTime) BIND(C, NAME='fsi_mg_mg_solver')
      IMPORT :: C_INT, C_DOUBLE, C_PTR
      TYPE(C_PTR), VALUE :: h
      REAL(C_DOUBLE), INTENT(INOUT) :: var(*)
      REAL(C_DOUBLE), INTENT(IN) :: rr(*)
      REAL(C_DOUBLE), INTENT(OUT) :: compTime
    END FUNCTION
    ! Steps either side of the solve on DEVICE arrays (a CUDA Fortran or
    ! OpenACC caller passes device addresses, e.g. via host_data use_device;
    ! C_NULL_PTR for an absent bc array).  face_vel + rhs_poisson
    ! (IBM/CORE_FRAC_STEP_ROUTINES.F90:6, IBM/CORE_POISSON.F90:123),
    ! correct_vel (:244) without its ghost-cell velocity steps, update_pressure (:949).
    INTEGER(C_INT) FUNCTION fsi_mg_face_vel_rhs(h, frac_step_type, dt, u, v, w, p, bcxu, bcyv, bczw, &
        face_u, face_v, face_w, nlu0, total) BIND(C, NAME='fsi_mg_face_vel_rhs')
      IMPORT :: C_INT, C_DOUBLE, C_PTR
      TYPE(C_PTR), VALUE :: h, u, v, w, p, bcxu, bcyv, bczw, face_u, face_v, face_w, nlu0
      INTEGER(C_INT), VALUE :: frac_step_type
      REAL(C_DOUBLE), VALUE :: dt
      REAL(C_DOUBLE), INTENT(OUT) :: total
    END FUNCTION
    INTEGER(C_INT) FUNCTION fsi_mg_correct_vel(h, dt, pPrime, u, v, w, bcxu, bcyv, bczw, &
        face_u, face_v, face_w) BIND(C, NAME='fsi_mg_correct_vel')
      IMPORT :: C_INT, C_DOUBLE, C_PTR
      TYPE(C_PTR), VALUE :: h, pPrime, u, v, w, bcxu, bcyv, bczw, face_u, face_v, face_w
      REAL(C_DOUBLE), VALUE :: dt
    END FUNCTION
    ! momentum predictor on device arrays: rhs_advec_diff (IBM/CORE_RHS_AD.F90:13),
    ! rhs_adjust_bc (:588), solve_ad (IBM/CORE_SOLVE_AD.F90:12)
    INTEGER(C_INT) FUNCTION fsi_mg_rhs_advec_diff(h, advec_scheme, frac_step_type, dt, fields) &
        BIND(C, NAME='fsi_mg_rhs_advec_diff')
      IMPORT :: C_INT, C_DOUBLE, C_PTR, fsi_mg_rhs_ad_fields
      TYPE(C_PTR), VALUE :: h
      INTEGER(C_INT), VALUE :: advec_scheme, frac_step_type
      REAL(C_DOUBLE), VALUE :: dt
      TYPE(fsi_mg_rhs_ad_fields), INTENT(IN) :: fields
    END FUNCTION
    INTEGER(C_INT) FUNCTION fsi_mg_rhs_adjust_bc(h, advec_scheme, dt, fields) BIND(C, NAME='fsi_mg_rhs_adjust_bc')
      IMPORT :: C_INT, C_DOUBLE, C_PTR, fsi_mg_rhs_ad_fields
      TYPE(C_PTR), VALUE :: h
      INTEGER(C_INT), VALUE :: advec_scheme
      REAL(C_DOUBLE), VALUE :: dt
      TYPE(fsi_mg_rhs_ad_fields), INTENT(IN) :: fields
    END FUNCTION
    INTEGER(C_INT) FUNCTION fsi_mg_solve_ad(h, advec_scheme, dt, fields, u, v, w, iters, maxres) &
        BIND(C, NAME='fsi_mg_solve_ad')
      IMPORT :: C_INT, C_DOUBLE, C_PTR, fsi_mg_rhs_ad_fields
      TYPE(C_PTR), VALUE :: h, u, v, w
      INTEGER(C_INT), VALUE :: advec_scheme
      REAL(C_DOUBLE), VALUE :: dt
      TYPE(fsi_mg_rhs_ad_fields), INTENT(IN) :: fields
      INTEGER(C_INT), INTENT(OUT) :: iters
      REAL(C_DOUBLE), INTENT(OUT) :: maxres
    END FUNCTION
    ! coeffGCMD(8,nGhost), u/v/wBodyIntercept(nGhost) (host; C_NULL_PTR for a body at rest)
    INTEGER(C_INT) FUNCTION fsi_mg_set_velocity_ghosts(h, coeffGCMD, uBI, vBI, wBI, bodyInterceptWeight, &
        imagePointWeight) BIND(C, NAME='fsi_mg_set_velocity_ghosts')
      IMPORT :: C_INT, C_DOUBLE, C_PTR
      TYPE(C_PTR), VALUE :: h, coeffGCMD, uBI, vBI, wBI
      REAL(C_DOUBLE), VALUE :: bodyInterceptWeight, imagePointWeight
    END FUNCTION
    INTEGER(C_INT) FUNCTION fsi_mg_set_bc(h, values, u, v, w, bc, correction_vel) &
        BIND(C, NAME='fsi_mg_set_bc')
      IMPORT :: C_INT, C_DOUBLE, C_PTR, fsi_mg_bc_values
      TYPE(C_PTR), VALUE :: h, u, v, w
      TYPE(fsi_mg_bc_values), INTENT(IN) :: values
      TYPE(C_PTR), INTENT(IN) :: bc(9)     ! bcxu, bcyu, bczu, bcxv, bcyv, bczv, bcxw, bcyw, bczw
      REAL(C_DOUBLE), INTENT(OUT) :: correction_vel
    END FUNCTION
    INTEGER(C_INT) FUNCTION fsi_mg_update_pressure(h, frac_step_type, pPrime, p) &
        BIND(C, NAME='fsi_mg_update_pressure')
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: h, pPrime, p
      INTEGER(C_INT), VALUE :: frac_step_type
    END FUNCTION
    TYPE(C_PTR) FUNCTION fsi_mg_last_error() BIND(C, NAME='fsi_mg_last_error')
      IMPORT :: C_PTR
    END FUNCTION
    SUBROUTINE fsi_mg_destroy(h) BIND(C, NAME='fsi_mg_destroy')
      IMPORT :: C_PTR
      TYPE(C_PTR), VALUE :: h
    END SUBROUTINE
  END INTERFACE

CONTAINS

  SUBROUTINE fsi_mg_abort(where, rc)
    CHARACTER(LEN=*), INTENT(IN) :: where
    INTEGER(C_INT), INTENT(IN) :: rc
    CHARACTER(KIND=C_CHAR), POINTER :: msg(:)
    INTEGER :: n
    CALL C_F_POINTER(fsi_mg_last_error(), msg, [1024])
    n = 0
    DO WHILE (n < 1024)
      IF (msg(n+1) == C_NULL_CHAR) EXIT
      n = n + 1
    END DO
    WRITE(*,*) where, ': fsi_mg error ', rc, ' ', msg(1:n)
    STOP
  END SUBROUTINE fsi_mg_abort

END MODULE fsi_mg_gpu

!-----------------------------------------------------------------------------
SUBROUTINE MG_initial()
  USE global_parameters
  USE flow_parameters
  USE grid_arrays
  USE mg_parameters
  USE fsi_mg_gpu
  IMPLICIT NONE
  TYPE(fsi_mg_params) :: p
  INTEGER(C_INT) :: rc
  p%ndim = ndim; p%nx = nx; p%ny = ny; p%nz = nz
  p%pp_solver_type = pp_solver_type; p%iRedBlack = iRedBlack
  p%mgcycle = [mgcyclex, mgcycley, mgcyclez]
  p%iterFinest = iterFinest; p%iterCoarsest = iterCoarsest
  p%mgLevels = [mgLevels_X, mgLevels_Y, mgLevels_Z]
  p%iterMax_Poisson = iterMax_Poisson; p%iterMax_ad = iterMax_ad
  p%bc = [bcx1, bcx2, bcy1, bcy2, bcz1, bcz2]
  p%pbc = [pbcx1, pbcx2, pbcy1, pbcy2, pbcz1, pbcz2]
  p%internal_boundary_present = internal_boundary_present
  p%boundary_formulation = boundary_formulation
  p%coarse_flag_mode = 1
  p%precision_mode = fsi_mg_precision
  p%outer_krylov = 0                         ! the reference's stationary outer iteration
  p%omega = omega; p%restol_Poisson = restol_Poisson; p%restol_ad = restol_ad
  p%ppp = [pppx1, pppx2, pppy1, pppy2, pppz1, pppz2]
  p%outflow_area = outflow_area
  p%alfa = alfa                              ! hybrid advection weight (flow_parameters)
  rc = fsi_mg_create(p, x, y, z, fsi_mg_handle)
  IF (rc /= 0) CALL fsi_mg_abort('MG_initial', rc)
END SUBROUTINE MG_initial

!-----------------------------------------------------------------------------
SUBROUTINE fsi_mg_update_geometry()
  USE global_parameters
  USE flow_parameters
  USE boundary_arrays
  USE GCM_arrays
  USE fsi_mg_gpu
  IMPLICIT NONE
  REAL(C_DOUBLE), ALLOCATABLE :: pg(:)
  INTEGER(C_INT) :: rc
  INTEGER :: nyz, nxz, nxy, n
  INTEGER(C_INT) :: idum(1)
  REAL(C_DOUBLE) :: ddum(1)
  nyz = (ny+2)*(nz+2); nxz = (nx+2)*(nz+2); nxy = (nx+2)*(ny+2)
  ALLOCATE(pg(2*nyz + 2*nxz + 2*nxy))
  pg(1:nyz)                         = RESHAPE(pgradx1, [nyz])
  pg(nyz+1:2*nyz)                   = RESHAPE(pgradx2, [nyz])
  pg(2*nyz+1:2*nyz+nxz)             = RESHAPE(pgrady1, [nxz])
  pg(2*nyz+nxz+1:2*nyz+2*nxz)       = RESHAPE(pgrady2, [nxz])
  n = 2*nyz + 2*nxz
  pg(n+1:n+nxy)                     = RESHAPE(pgradz1, [nxy])
  pg(n+nxy+1:n+2*nxy)               = RESHAPE(pgradz2, [nxy])
  idum = 0; ddum = 0.0_C_DOUBLE
  IF (boundary_formulation == GCM_METHOD .AND. nGhost > 0) THEN
    rc = fsi_mg_set_geometry(fsi_mg_handle, iblank, ghostCellMark, ium, iup, jum, jup, kum, kup, &
                             nGhost, iGhost, jGhost, kGhost, iCellIndex, jCellIndex, kCellIndex, &
                             coeffGCMN, probeLength, pg)
  ELSE
    rc = fsi_mg_set_geometry(fsi_mg_handle, iblank, ghostCellMark, ium, iup, jum, jup, kum, kup, &
                             0, idum, idum, idum, idum, idum, idum, ddum, ddum, pg)
  ENDIF
  DEALLOCATE(pg)
  IF (rc /= 0) CALL fsi_mg_abort('fsi_mg_update_geometry', rc)
  ! fresh cells of a moving body (allocated with the GCM arrays, GCM_MEMORY_ALLOCATE.F90:27)
  IF (ALLOCATED(fresh_cell)) THEN
    rc = fsi_mg_set_fresh_cells(fsi_mg_handle, fresh_cell)
    IF (rc /= 0) CALL fsi_mg_abort('fsi_mg_set_fresh_cells', rc)
  ENDIF
END SUBROUTINE fsi_mg_update_geometry

!-----------------------------------------------------------------------------
SUBROUTINE MG_Solver(var, rr, MG_itSolver, MG_itResidual, compTime)
  USE global_parameters
  USE flow_parameters
  USE fsi_mg_gpu
  IMPLICIT NONE
  EXTERNAL MG_itSolver, MG_itResidual        ! fixed on the GPU: line SOR and MG_Residual
  REAL(KIND=CGREAL), DIMENSION(0:nx+1,0:ny+1,0:nz+1), INTENT(IN)    :: rr
  REAL(KIND=CGREAL), DIMENSION(0:nx+1,0:ny+1,0:nz+1), INTENT(INOUT) :: var
  REAL(KIND=CGREAL), INTENT(OUT) :: compTime
  INTEGER(C_INT) :: rc
  rc = fsi_mg_mg_solver(fsi_mg_handle, var, rr, compTime)
  IF (rc /= 0) CALL fsi_mg_abort('MG_Solver', rc)
END SUBROUTINE MG_Solver

!-----------------------------------------------------------------------------
SUBROUTINE solve_poisson()
  USE global_parameters
  USE flow_parameters
  USE pressure_arrays
  USE multiuse_arrays
  USE fsi_mg_gpu
  IMPLICIT NONE
  INTEGER(C_INT) :: rc, iters, loc(3)
  REAL(C_DOUBLE) :: maxres, compTime
  rc = fsi_mg_solve(fsi_mg_handle, pPrime, nlu0, nlw0, iters, maxres, loc, compTime)
  IF (rc < 0) CALL fsi_mg_abort('solve_poisson', rc)
  IF (rc == 1) THEN                      ! IBM/CORE_POISSON.F90:665-669, continue as the reference does
    PRINT*,'MG-LSOR: Pressure Convergence at NTIME = ',ntime
    PRINT*,'MG-LSOR: Pressure did not converge in ',iterMax_Poisson,' iterations'
    PRINT*,'Final residual = ',maxres,' at',loc(1),loc(2),loc(3)
  ELSE IF (rc == 2) THEN                 ! IBM/GCM_GHOSTCELL_VEL_UPDATE_UNSTRUC.F90:374-378
    PRINT*,'GhostCell Pressure did not converge in ',iterMax_ad,' iterations'
  ELSE IF (MOD(ntime,nmonitor) == 0) THEN
    WRITE(STDOUT,'(A,I4,2X,1PE15.7,3(2X,I4),2X,F7.3)') &
      'MG-LSOR: Pressure Convergence : ',iters,maxres,loc(1),loc(2),loc(3),compTime
  ENDIF
END SUBROUTINE solve_poisson

!-----------------------------------------------------------------------------
SUBROUTINE fsi_mg_finalize()
  USE fsi_mg_gpu
  IMPLICIT NONE
  IF (C_ASSOCIATED(fsi_mg_handle)) CALL fsi_mg_destroy(fsi_mg_handle)
  fsi_mg_handle = C_NULL_PTR
END SUBROUTINE fsi_mg_finalize
