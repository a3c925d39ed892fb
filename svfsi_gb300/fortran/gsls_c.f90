! ISO_C_BINDING interface to libgsls.so for the svFSI Fortran driver.
!
! The svFSILS-shaped entry points keep the reference's argument order and
! 1-based indices (Code/Source/svFSILS/FSILS_API.h:51-135), so the driver's
! call sites change only their callee.  Every function returns an INTEGER
! status (0 = GSLS_OK); gsls_last_error gives the message.  Declarations
! follow include/gsls.h.  The driver's FSILS_lsType (L/FSILS_STRUCT.h:
! 103-140, C mirror L/FSILS_struct_c.h:114-140) has the field layout of
! gsls_ls, so lEq%FSILS is passed as is (assumed type, TYPE(*)).
!
! Built only where gfortran exists (the library itself needs none):
!   gfortran -c gsls_c.f90
MODULE GSLS_C
  USE, INTRINSIC :: ISO_C_BINDING
  IMPLICIT NONE

  INTEGER(C_INT), PARAMETER :: GSLS_OK = 0
  INTEGER(C_INT), PARAMETER :: GSLS_LS_TYPE_CG = 798, GSLS_LS_TYPE_GMRES = 797, &
       GSLS_LS_TYPE_NS = 796, GSLS_LS_TYPE_BICGS = 795
  INTEGER(C_INT), PARAMETER :: GSLS_PRECOND_FSILS = 701, GSLS_PRECOND_RCS = 709
  INTEGER(C_INT), PARAMETER :: GSLS_BC_TYPE_DIR = 0, GSLS_BC_TYPE_NEU = 1
  INTEGER(C_INT), PARAMETER :: GSLS_PREC_FP64 = 0, GSLS_PREC_MIXED = 1
  INTEGER(C_INT), PARAMETER :: GSLS_PHYS_HEATS = 1, GSLS_PHYS_STRUCT = 2, &
       GSLS_PHYS_CEP = 3, GSLS_PHYS_FLUID = 4, GSLS_PHYS_LELAS = 5, GSLS_PHYS_HEATF = 6, &
       GSLS_PHYS_USTRUCT = 7
  INTEGER(C_INT), PARAMETER :: GSLS_VISC_CONST = 0, GSLS_VISC_CY = 1, GSLS_VISC_CASSON = 2

  ! FSILS_subLsType / FSILS_lsType (LOGICAL as C int)
  TYPE, BIND(C) :: gsls_sub_ls
     INTEGER(C_INT) :: suc, mItr, sD, itr, cM, cN, cD, reserve
     REAL(C_DOUBLE) :: absTol, relTol, iNorm, fNorm, dB, callD
  END TYPE gsls_sub_ls
  TYPE, BIND(C) :: gsls_ls
     INTEGER(C_INT) :: foC, LS_type, Resm, Resc
     TYPE(gsls_sub_ls) :: GM, CG, RI
  END TYPE gsls_ls

  ! gsls_eq_params (include/gsls.h)
  TYPE, BIND(C) :: gsls_eq_params
     INTEGER(C_INT) :: phys, dof, tDof, s
     REAL(C_DOUBLE) :: am, af, beta, gam, dt
     REAL(C_DOUBLE) :: rho, cond, src, C10, Kpen, visc, dmp
     REAL(C_DOUBLE) :: fb(3)
     REAL(C_DOUBLE) :: Diso, mu_f, ctM, ctC
     TYPE(C_PTR) :: eparam = C_NULL_PTR
     REAL(C_DOUBLE) :: elM, nu
     INTEGER(C_INT) :: viscType
     REAL(C_DOUBLE) :: mu_o, vlam, va, vn
     REAL(C_DOUBLE) :: bstab
     INTEGER(C_INT) :: volType
     INTEGER(C_INT) :: nFn = 0
     REAL(C_DOUBLE) :: Dani(3) = 0.0_C_DOUBLE
     TYPE(C_PTR) :: fN = C_NULL_PTR
  END TYPE gsls_eq_params

  INTERFACE
     INTEGER(C_INT) FUNCTION gsls_init(device) BIND(C, NAME="gsls_init")
       IMPORT :: C_INT
       INTEGER(C_INT), VALUE :: device
     END FUNCTION gsls_init

     TYPE(C_PTR) FUNCTION gsls_last_error() BIND(C, NAME="gsls_last_error")
       IMPORT :: C_PTR
     END FUNCTION gsls_last_error

     ! FSILS_LHS_CREATE (L/LHS.f:51); commu dropped: one process, one GPU
     INTEGER(C_INT) FUNCTION gsls_lhs_create(lhs, gnNo, nNo, nnz, gNodes, rowPtr, colPtr, &
          nFaces) BIND(C, NAME="gsls_lhs_create")
       IMPORT :: C_INT, C_PTR
       TYPE(C_PTR) :: lhs
       INTEGER(C_INT), VALUE :: gnNo, nNo, nnz, nFaces
       INTEGER(C_INT) :: gNodes(*), rowPtr(*), colPtr(*)
     END FUNCTION gsls_lhs_create

     INTEGER(C_INT) FUNCTION gsls_lhs_free(lhs) BIND(C, NAME="gsls_lhs_free")
       IMPORT :: C_INT, C_PTR
       TYPE(C_PTR), VALUE :: lhs
     END FUNCTION gsls_lhs_free

     ! FSILS_BC_CREATE (L/BC.f:50); Val(dof,nNo) optional in the reference
     INTEGER(C_INT) FUNCTION gsls_bc_create(lhs, faIn, nNo, dof, BC_type, gNodes, Val) &
          BIND(C, NAME="gsls_bc_create")
       IMPORT :: C_INT, C_PTR, C_DOUBLE
       TYPE(C_PTR), VALUE :: lhs
       INTEGER(C_INT), VALUE :: faIn, nNo, dof, BC_type
       INTEGER(C_INT) :: gNodes(*)
       REAL(C_DOUBLE) :: Val(*)
     END FUNCTION gsls_bc_create

     ! FSILS_LS_CREATE (L/LS.f:50): pass C_NULL_PTR for an absent OPTIONAL
     INTEGER(C_INT) FUNCTION gsls_ls_create(ls, LS_type, relTol, absTol, maxItr, dimKry, &
          relTolIn, absTolIn, maxItrIn) BIND(C, NAME="gsls_ls_create")
       IMPORT :: C_INT, C_PTR
       TYPE(*) :: ls
       INTEGER(C_INT), VALUE :: LS_type
       TYPE(C_PTR), VALUE :: relTol, absTol, maxItr, dimKry, relTolIn, absTolIn, maxItrIn
     END FUNCTION gsls_ls_create

     ! FSILS_SOLVE (L/SOLVE.f:51): Ri overwritten with the solution, Val
     ! left preconditioned, as in the reference
     INTEGER(C_INT) FUNCTION gsls_solve(lhs, ls, dof, Ri, Val, prec, incL, res) &
          BIND(C, NAME="gsls_solve")
       IMPORT :: C_INT, C_PTR, C_DOUBLE
       TYPE(C_PTR), VALUE :: lhs
       TYPE(*) :: ls
       INTEGER(C_INT), VALUE :: dof, prec
       REAL(C_DOUBLE) :: Ri(*), Val(*)
       INTEGER(C_INT) :: incL(*)
       REAL(C_DOUBLE) :: res(*)
     END FUNCTION gsls_solve

     ! tet4 mesh bound to the lhs's CSR (IEN 1-based, eNoN 4, nsd 3)
     INTEGER(C_INT) FUNCTION gsls_mesh_create(mesh, lhs, nEl, eNoN, IEN, nsd, x) &
          BIND(C, NAME="gsls_mesh_create")
       IMPORT :: C_INT, C_PTR, C_DOUBLE
       TYPE(C_PTR) :: mesh
       TYPE(C_PTR), VALUE :: lhs
       INTEGER(C_INT), VALUE :: nEl, eNoN, nsd
       INTEGER(C_INT) :: IEN(*)
       REAL(C_DOUBLE) :: x(*)
     END FUNCTION gsls_mesh_create

     INTEGER(C_INT) FUNCTION gsls_mesh_free(mesh) BIND(C, NAME="gsls_mesh_free")
       IMPORT :: C_INT, C_PTR
       TYPE(C_PTR), VALUE :: mesh
     END FUNCTION gsls_mesh_free

     ! GLOBALEQASSEM -> CONSTRUCT_* -> DOASSEM (F/EQASSEM.f:38-87) on host
     ! arrays: R(dof,nNo) and Val(dof*dof,nnz) overwritten
     INTEGER(C_INT) FUNCTION gsls_assemble(mesh, p, Ag, Yg, Dg, R, Val) &
          BIND(C, NAME="gsls_assemble")
       IMPORT :: C_INT, C_PTR, C_DOUBLE, gsls_eq_params
       TYPE(C_PTR), VALUE :: mesh
       TYPE(gsls_eq_params) :: p
       REAL(C_DOUBLE) :: Ag(*), Yg(*), Dg(*), R(*), Val(*)
     END FUNCTION gsls_assemble
  END INTERFACE

CONTAINS

  ! The library's last error message as a Fortran string.
  FUNCTION gsls_error_text() RESULT(msg)
    CHARACTER(LEN=256) :: msg
    CHARACTER(KIND=C_CHAR), POINTER :: c(:)
    TYPE(C_PTR) :: p
    INTEGER :: i
    msg = ""
    p = gsls_last_error()
    IF (.NOT. C_ASSOCIATED(p)) RETURN
    CALL C_F_POINTER(p, c, [256])
    DO i = 1, 256
       IF (c(i) == C_NULL_CHAR) EXIT
       msg(i:i) = c(i)
    END DO
  END FUNCTION gsls_error_text

END MODULE GSLS_C
