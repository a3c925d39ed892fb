! svFSI-side glue: the gsls handles and the four call sites the driver
! switches when it is built with -DWITH_GSLS (svfsi_driver.patch):
!
!   F/INITIALIZE.f:207  FSILS_LHS_CREATE  -> GSLS_LHS_INIT
!   F/BAFINI.f:510      FSILS_BC_CREATE   -> GSLS_BC_DIR
!   F/MAIN.f:141        GLOBALEQASSEM     -> GSLS_GLOBALEQASSEM
!   F/LS.f:98           FSILS_SOLVE       -> GSLS_LSSOLVE
!
! Scope: one mesh and one domain per equation (the tet4 meshes and the
! HEATS, STRUCT (neo-Hookean + ST91), FLUID, CEP (isotropic), LELAS and
! HEATF physics of the library); other configurations keep the reference
! path.  Compiled inside the svFSI build (it uses COMMOD) with
! gsls_c.f90, and linked with -lgsls.  Not compiled here: it needs
! gfortran and the svFSI sources.
MODULE GSLS_SVFSI
  USE, INTRINSIC :: ISO_C_BINDING
  USE GSLS_C
  USE COMMOD
  IMPLICIT NONE

  TYPE(C_PTR), SAVE :: gslsLhs = C_NULL_PTR
  TYPE(C_PTR), SAVE, ALLOCATABLE :: gslsMesh(:)

CONTAINS

  ! After FSILS_LHS_CREATE: the same CSR pattern on the GPU.
  SUBROUTINE GSLS_LHS_INIT(gnNo, nNo, nz, gNodes, rp, cp, nFaces)
    INTEGER(KIND=IKIND), INTENT(IN) :: gnNo, nNo, nz, nFaces
    INTEGER(KIND=IKIND), INTENT(IN) :: gNodes(nNo), rp(nNo+1), cp(nz)
    INTEGER(C_INT) :: istat
    INTEGER(C_INT), ALLOCATABLE :: g(:), r(:), c(:)
    IF (C_ASSOCIATED(gslsLhs)) istat = gsls_lhs_free(gslsLhs)
    istat = gsls_init(0_C_INT)
    IF (istat .NE. GSLS_OK) err = "gsls_init: "//TRIM(gsls_error_text())
    g = INT(gNodes, C_INT)
    r = INT(rp, C_INT)
    c = INT(cp, C_INT)
    istat = gsls_lhs_create(gslsLhs, INT(gnNo, C_INT), INT(nNo, C_INT), INT(nz, C_INT), &
         g, r, c, INT(nFaces, C_INT))
    IF (istat .NE. GSLS_OK) err = "gsls_lhs_create: "//TRIM(gsls_error_text())
    IF (ALLOCATED(gslsMesh)) DEALLOCATE(gslsMesh)
    ALLOCATE(gslsMesh(nMsh))
    gslsMesh = C_NULL_PTR
  END SUBROUTINE GSLS_LHS_INIT

  ! After FSILS_BC_CREATE of a Dirichlet face (FSILSINI, F/BAFINI.f:510).
  SUBROUTINE GSLS_BC_DIR(faIn, nNo, dof, gNodes, sVl)
    INTEGER(KIND=IKIND), INTENT(IN) :: faIn, nNo, dof
    INTEGER(KIND=IKIND), INTENT(IN) :: gNodes(nNo)
    REAL(KIND=RKIND), INTENT(IN) :: sVl(dof, nNo)
    INTEGER(C_INT) :: istat
    INTEGER(C_INT), ALLOCATABLE :: g(:)
    REAL(C_DOUBLE), ALLOCATABLE :: v(:,:)
    g = INT(gNodes, C_INT)
    v = REAL(sVl, C_DOUBLE)
    istat = gsls_bc_create(gslsLhs, INT(faIn, C_INT), INT(nNo, C_INT), INT(dof, C_INT), &
         GSLS_BC_TYPE_DIR, g, v)
    IF (istat .NE. GSLS_OK) err = "gsls_bc_create: "//TRIM(gsls_error_text())
  END SUBROUTINE GSLS_BC_DIR

  ! GLOBALEQASSEM (F/EQASSEM.f:38-87) for mesh iM of equation cEq: R and
  ! Val (zeroed by LSALLOC) receive the assembled residual and tangent.
  SUBROUTINE GSLS_GLOBALEQASSEM(iM, lM, Ag, Yg, Dg)
    INTEGER(KIND=IKIND), INTENT(IN) :: iM
    TYPE(mshType), INTENT(IN) :: lM
    REAL(KIND=RKIND), INTENT(IN) :: Ag(tDof,tnNo), Yg(tDof,tnNo), Dg(tDof,tnNo)
    TYPE(gsls_eq_params) :: p
    INTEGER(C_INT) :: istat
    INTEGER(C_INT), ALLOCATABLE :: ien(:,:)
    REAL(C_DOUBLE), ALLOCATABLE :: xx(:,:)
    REAL(C_DOUBLE), ALLOCATABLE, TARGET, SAVE :: fib(:,:)
    INTEGER :: i

    IF (.NOT. C_ASSOCIATED(gslsMesh(iM))) THEN
       ien = INT(lM%IEN, C_INT)
       xx = REAL(x, C_DOUBLE)
       istat = gsls_mesh_create(gslsMesh(iM), gslsLhs, INT(lM%nEl, C_INT), &
            INT(lM%eNoN, C_INT), ien, INT(nsd, C_INT), xx)
       IF (istat .NE. GSLS_OK) err = "gsls_mesh_create: "//TRIM(gsls_error_text())
    END IF
    CALL GSLS_PARAMS(p)
    IF (p%phys .EQ. GSLS_PHYS_CEP .AND. ALLOCATED(lM%fN)) THEN
       ! CEP3D's fibres (F/CEP.f:89-93) and one Dani per family, the last
       ! configured value repeated (F/CEP.f:158-165)
       fib = REAL(lM%fN, C_DOUBLE)
       p%nFn = INT(MIN(lM%nFn, 3), C_INT)
       DO i = 1, p%nFn
          IF (i .LE. eq(cEq)%dmn(1)%cep%nFn) THEN
             p%Dani(i) = eq(cEq)%dmn(1)%cep%Dani(i)
          ELSE IF (i .GT. 1) THEN
             p%Dani(i) = p%Dani(i-1)
          END IF
       END DO
       p%fN = C_LOC(fib)
    END IF
    istat = gsls_assemble(gslsMesh(iM), p, Ag, Yg, Dg, R, Val)
    IF (istat .NE. GSLS_OK) err = "gsls_assemble: "//TRIM(gsls_error_text())
  END SUBROUTINE GSLS_GLOBALEQASSEM

  ! Parameters of equation cEq, domain 1, as the CONSTRUCT_* routines read
  ! them (F/READFILES.f READDOMAIN, READVISCMODEL; F/MATMODELS.f).
  SUBROUTINE GSLS_PARAMS(p)
    TYPE(gsls_eq_params), INTENT(OUT) :: p
    ASSOCIATE (lEq => eq(cEq), d => eq(cEq)%dmn(1))
      SELECT CASE (lEq%phys)
      CASE (phys_heatS)
         p%phys = GSLS_PHYS_HEATS
      CASE (phys_struct)
         p%phys = GSLS_PHYS_STRUCT
      CASE (phys_CEP)
         p%phys = GSLS_PHYS_CEP
      CASE (phys_fluid)
         p%phys = GSLS_PHYS_FLUID
      CASE (phys_lElas)
         p%phys = GSLS_PHYS_LELAS
      CASE (phys_heatF)
         p%phys = GSLS_PHYS_HEATF
      CASE (phys_ustruct)
         p%phys = GSLS_PHYS_USTRUCT
      CASE DEFAULT
         err = "GSLS_PARAMS: physics not on the GPU path"
      END SELECT
      p%dof = INT(lEq%dof, C_INT)
      p%tDof = INT(tDof, C_INT)
      p%s = INT(lEq%s - 1, C_INT)
      p%am = lEq%am
      p%af = lEq%af
      p%beta = lEq%beta
      p%gam = lEq%gam
      p%dt = dt
      p%rho = d%prop(solid_density)
      IF (lEq%phys .EQ. phys_fluid) p%rho = d%prop(fluid_density)
      p%cond = d%prop(conductivity)
      p%src = d%prop(source_term)
      p%C10 = d%stM%C10
      p%Kpen = d%stM%Kpen
      p%visc = d%prop(solid_viscosity)
      p%dmp = d%prop(damping)
      p%fb = [d%prop(f_x), d%prop(f_y), d%prop(f_z)]
      p%Diso = d%cep%Diso
      p%mu_f = d%visc%mu_i
      p%ctM = d%prop(ctau_M)
      p%ctC = d%prop(ctau_C)
      p%eparam = C_NULL_PTR
      p%elM = d%prop(elasticity_modulus)
      p%nu = d%prop(poisson_ratio)
      SELECT CASE (d%visc%viscType)
      CASE (viscType_CY)
         p%viscType = GSLS_VISC_CY
      CASE (viscType_Cass)
         p%viscType = GSLS_VISC_CASSON
      CASE DEFAULT
         p%viscType = GSLS_VISC_CONST
      END SELECT
      p%mu_o = d%visc%mu_o
      p%vlam = d%visc%lam
      p%va = d%visc%a
      p%vn = d%visc%n
      p%bstab = d%prop(backflow_stab)
      SELECT CASE (d%stM%volType)
      CASE (stVol_Quad)
         p%volType = 0
      CASE (stVol_M94)
         p%volType = 2
      CASE DEFAULT
         p%volType = 1
      END SELECT
    END ASSOCIATE
  END SUBROUTINE GSLS_PARAMS

  ! LSSOLVE's FSILS_SOLVE (F/LS.f:98): lEq%FSILS carries the settings in
  ! and RI%suc/itr/iNorm/fNorm/dB/callD out, field for field.
  SUBROUTINE GSLS_LSSOLVE(lEq, dof, Ri, Vl, incL, res)
    TYPE(eqType), INTENT(INOUT), TARGET :: lEq
    INTEGER(KIND=IKIND), INTENT(IN) :: dof
    REAL(KIND=RKIND), INTENT(INOUT) :: Ri(:,:), Vl(:,:)
    INTEGER(KIND=IKIND), INTENT(IN) :: incL(:)
    REAL(KIND=RKIND), INTENT(IN) :: res(:)
    INTEGER(C_INT) :: istat
    INTEGER(C_INT), ALLOCATABLE :: il(:)
    REAL(C_DOUBLE), ALLOCATABLE :: rs(:)
    il = INT(incL, C_INT)
    rs = REAL(res, C_DOUBLE)
    IF (SIZE(il) .EQ. 0) THEN
       il = [0_C_INT]
       rs = [0._C_DOUBLE]
    END IF
    istat = gsls_solve(gslsLhs, lEq%FSILS, INT(dof, C_INT), Ri, Vl, &
         INT(lEq%ls%PREC_Type, C_INT), il, rs)
    IF (istat .NE. GSLS_OK) err = "gsls_solve: "//TRIM(gsls_error_text())
  END SUBROUTINE GSLS_LSSOLVE

END MODULE GSLS_SVFSI
