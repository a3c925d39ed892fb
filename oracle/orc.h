/*
 * Oracle: a plain-C, FP64, single-threaded restatement of the svFSI
 * implicit-step hot path (element assembly + svFSILS Krylov solve).
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, calls or
 * executes this code.  It is the checker used by tests/, by
 * __graft_entry__.smoke() and by bench.py's cpu_baseline / reference arm.
 *
 * Every routine cites the reference Fortran it restates (paths are relative
 * to the svFSI project root; F/ = Code/Source/svFSI, L/ = Code/Source/svFSILS).
 *
 * Conventions (identical to the reference's column-major arrays):
 *   Val[j*dof*dof + r*dof + c]  block j of the CSR, row r, column c
 *                               (Fortran Val(dof*dof,nnz), row-major in block)
 *   U[a*dof + i]                node a, component i (Fortran U(dof,nNo))
 *   IEN[e*eNoN + a]             0-based node of local vertex a of element e
 *   rowPtr[nNo+1], colPtr[nnz]  0-based CSR, columns sorted ascending
 */
#ifndef ORC_H
#define ORC_H

#ifdef __cplusplus
extern "C" {
#endif

/* constants identical to L/FSILS_STRUCT.h:53-62 */
#define ORC_LS_TYPE_CG 798
#define ORC_LS_TYPE_GMRES 797
#define ORC_LS_TYPE_NS 796
#define ORC_LS_TYPE_BICGS 795
#define ORC_PRECOND_FSILS 701
#define ORC_PRECOND_RCS 709
#define ORC_BC_TYPE_Dir 0
#define ORC_BC_TYPE_Neu 1

/* FSILS_subLsType, L/FSILS_STRUCT.h:162-191 (LOGICAL stored as int) */
typedef struct {
  int suc, mItr, sD, itr, cM, cN, cD, reserve;
  double absTol, relTol, iNorm, fNorm, dB, callD;
} orc_subls;

/* FSILS_lsType, L/FSILS_STRUCT.h:193-204 */
typedef struct {
  int foC, LS_type, Resm, Resc;
  orc_subls GM, CG, RI;
} orc_ls;

/* FSILS_faceType, L/FSILS_STRUCT.h:87-114 */
typedef struct {
  int foC, coupledFlag, sharedFlag, incFlag, nNo, dof, bGrp;
  int *glob;      /* 0-based local node ids */
  double nS, res;
  double *val;    /* val(dof,nNo) */
  double *valM;
} orc_face;

/* FSILS_lhsType (serial branch), L/FSILS_STRUCT.h:126-158 */
typedef struct {
  int nNo, nnz, nFaces, mynNo;
  int *rowS, *rowE; /* rowPtr(1,:), rowPtr(2,:) as 0-based inclusive ranges */
  int *colPtr, *diagPtr;
  orc_face *face;
} orc_lhs;

/* ---- library-level knobs ---- */
void orc_set_threads(int n);
int orc_get_threads(void);

/* ---- svFSILS restatement (orc_fsils.c) ---- */
orc_lhs *orc_lhs_create(int nNo, int nnz, const int *rowPtr, const int *colPtr,
                        int nFaces);
void orc_lhs_free(orc_lhs *lhs);
int orc_bc_create(orc_lhs *lhs, int faIn, int nNo, int dof, int BC_type,
                  const int *gNodes, const double *val);
void orc_ls_create(orc_ls *ls, int LS_type);
void orc_spar_vv(const orc_lhs *lhs, int dof, const double *K, const double *U,
                 double *KU);
void orc_spar_ss(const orc_lhs *lhs, const double *K, const double *U, double *KU);
void orc_spar_vs(const orc_lhs *lhs, int dof, const double *K, const double *U,
                 double *KU);
void orc_spar_sv(const orc_lhs *lhs, int dof, const double *K, const double *U,
                 double *KU);
double orc_dotv(int dof, int nNo, const double *U, const double *V);
double orc_normv(int dof, int nNo, const double *U);
void orc_precond_diag(orc_lhs *lhs, int dof, double *Val, double *R, double *W);
void orc_precond_rcs(orc_lhs *lhs, int dof, double *Val, double *R, double *W1,
                     double *W2);
void orc_cgrad_v(orc_lhs *lhs, orc_subls *ls, int dof, const double *K, double *R);
void orc_bicgs_v(orc_lhs *lhs, orc_subls *ls, int dof, const double *K, double *R);
void orc_gmres_v(orc_lhs *lhs, orc_subls *ls, int dof, const double *Val,
                 double *R);
void orc_gmres_ns(orc_lhs *lhs, orc_subls *ls, int dof, const double *Val,
                  const double *R, double *X);
/* ADDBCMUL, L/ADDBCMUL.f:53-114 (serial faces): op 0 = BCOP_TYPE_ADD
   (coef = res), 1 = BCOP_TYPE_PRE (coef = -res/(1 + res nS)); Y += coef
   valM (valM . X) for every coupled face */
void orc_addbcmul(orc_lhs *lhs, int op, int dof, const double *X, double *Y);
/* BCPRE, L/NSSOLVER.f:307-343: nS = |valM(1:nsd,:)|^2 of each coupled face */
void orc_bcpre(orc_lhs *lhs, int nsd);
int orc_any_coupled(const orc_lhs *lhs);
void orc_cgrad_schur(orc_lhs *lhs, orc_subls *ls, int dof, const double *D,
                     const double *G, const double *L, double *R);
int orc_ge(int nV, int N, const double *A, double *B);
void orc_nssolver(orc_lhs *lhs, orc_ls *ls, int dof, const double *Val, double *Ri);
int orc_solve(orc_lhs *lhs, orc_ls *ls, int dof, double *Ri, double *Val,
              int prec, const int *incL, const double *res);

/* ---- driver-side restatement (orc_asm.c) ---- */
int orc_lhsa(int nNo, int nEl, int eNoN, const int *IEN, int *rowPtr,
             int *colPtr, int nnzCap);
int orc_lhsa_count(int nNo, int nEl, int eNoN, const int *IEN);
void orc_doassem(int dof, int eNoN, const int *ptr, const double *lK,
                 const double *lR, const int *rowPtr, const int *colPtr,
                 double *R, double *Val);

/* Equation parameters for one assembly call (one domain, constant props). */
typedef struct {
  int phys;      /* 1 HEATS, 2 STRUCT, 3 CEP, 4 FLUID, 5 LELAS, 6 HEATF, 7 USTRUCT */
  int dof, tDof, s; /* eq dof, total dof, 0-based start of this eq in tDof */
  double am, af, beta, gam, dt;
  double rho, cond, src;       /* HEATS: solid_density, conductivity, source */
  double C10, Kpen, visc, dmp; /* STRUCT nHK + ST91, solid_viscosity, damping */
  double fb[3];                /* body force */
  double Diso;                 /* CEP isotropic diffusivity */
  double mu_f;                 /* FLUID viscosity (density: rho) */
  double ctM, ctC;             /* FLUID stabilisation constants */
  const double *eparam;        /* optional per-element parameter (mu or Diso) */
  double elM, nu;              /* LELAS elasticity modulus, Poisson ratio (f in fb) */
  int viscType;                /* FLUID viscosity: 0 constant (mu_f), 1 Carreau-Yasuda,
                                  2 Casson (F/FLUID.f:1690-1739) */
  double mu_o, vlam, va, vn;   /* mu_o, lam, a, n of the model (mu_i = mu_f) */
  double bstab;                /* FLUID backflow_stab (F/READFILES.f:1089-1091) */
  int volType;                 /* USTRUCT volumetric penalty: 0 Quad, 1 ST91, 2 M94 */
  int nFn;                     /* CEP fibre families per element (lM%nFn), 0..3 */
  double Dani[3];              /* CEP anisotropic diffusivity per family (cep%Dani) */
  const double *fN;            /* CEP fibre directions, 3*nFn per element (lM%fN) */
} orc_eqp;

int orc_assemble(const orc_eqp *p, int nNo, int nEl, const int *IEN,
                 const double *x, const double *Ag, const double *Yg,
                 const double *Dg, const int *rowPtr, const int *colPtr,
                 double *R, double *Val);
int orc_assemble_colored(const orc_eqp *p, int nNo, int nEl, const int *IEN,
                         const double *x, const double *Ag, const double *Yg,
                         const double *Dg, const int *rowPtr, const int *colPtr,
                         double *R, double *Val, int ncolor, const int *color_off,
                         const int *order);
void orc_elem_fluid(const orc_eqp *p, const double xl[12], const double *al,
                    const double *yl, double lR[16], double lK[256]);
void orc_elem_heats(const orc_eqp *p, const double xl[12], const double *al,
                    const double *yl, double lR[4], double lK[16]);
/* LELAS3D, F/LELAS.f:130-238 (no prestress, no nodal body force Bf), one
   tet4 element: lR(3,4), lK(9,4,4) */
void orc_elem_lelas(const orc_eqp *p, const double xl[12], const double *al,
                    const double *dl, double lR[12], double lK[144]);
/* HEATF3D, F/HEATF.f:116-205 (no mesh motion): velocity in state
   components 0..2, temperature in component s; lR(1,4), lK(1,4,4) */
void orc_elem_heatf(const orc_eqp *p, const double xl[12], const double *al,
                    const double *yl, double lR[4], double lK[16]);
void orc_elem_struct(const orc_eqp *p, double mu_e, const double xl[12],
                     const double *al, const double *yl, const double *dl,
                     double lR[12], double lK[144]);
void orc_pk2cc_nhk(double C10, double Kpen, const double F[9], double S[9],
                   double Dm[36]);
void orc_traction(int dof, int nFel, const int *fIEN, const double *x,
                  const double h[3], double *R);
/* BASSEMNEUBC with BHEATF (F/EQASSEM.f:90-192, F/HEATF.f:289-319) on tri3
   faces: h = -g (F/SETBC.f:300), outward normal from the parent element
   (GNNB, F/NN.f:1856-1990), into R(1,nNo) and the scalar CSR Val */
void orc_bheatf(const orc_eqp *p, int nFel, const int *fIEN, double g, int nEl,
                const int *IEN, const double *x, const double *Yg, const int *rowPtr,
                const int *colPtr, double *R, double *Val);

/* BASSEMNEUBC with BFLUID (F/EQASSEM.f:90-192, F/FLUID.f:1280-1334) on
   tri3 faces of a fluid equation (dof 4, velocity at s..s+2): h = -g,
   backflow coefficient p->bstab, into R(4,nNo) and Val(16,nnz) */
void orc_bfluid(const orc_eqp *p, int nFel, const int *fIEN, double g, int nEl,
                const int *IEN, const double *x, const double *Yg, const int *rowPtr,
                const int *colPtr, double *R, double *Val);
/* node of each face's parent element that is off the face (-1: none) */
void orc_face_inner(int nFel, const int *fIEN, int nEl, const int *IEN, int *inner);

/* CEP3D, F/CEP.f:136-266 without electromechanical coupling: D = Diso I +
   sum_i Dani_i f_i f_i^T with the element's fibres fN_e (3*p->nFn, or
   NULL: isotropic) */
void orc_elem_cep(const orc_eqp *p, double Diso, const double *fN_e, const double xl[12],
                  const double *al, const double *yl, double lR[4], double lK[16]);

/* Aliev-Panfilov cell model (F/CEPMOD_AP.f, F/PARAMS_AP.f:53-86) and the
   per-node integration of CEPINTEGL (F/CEPION.f:319-400). */
typedef struct {
  int ode;          /* 0 forward Euler (AP_INTEGFE), 1 RK4 (AP_INTEGRK) */
  double dt_ode;    /* cep%dt (substep), nt = NINT(dt/dt_ode) */
  double A, Ts, Td, CL; /* stimulus amplitude, start, duration, cycle */
  double Ksac;
} orc_cep;
void orc_ap_getf(const double X[2], double f[2], double fext);
void orc_ap_step(double X[2], double t, double dt, double Istim, double Ksac,
                 int rk4);
/* integrate one node over [t1, t1+dt] (CEPINTEGL for cepModel_AP) */
void orc_cep_integ_node(const orc_cep *c, double t1, double dt, int stim,
                        double X[2]);

/* gen-alpha coefficients, F/INITIALIZE.f:76-139 */
void orc_genalpha(double roInf, int second_order, double *am, double *af,
                  double *beta, double *gam);

/* Time stepping (F/MAIN.f:89-215, F/PIC.f) for one equation.
   Dirichlet BC: node list with value g*gx per constrained component. */
typedef struct {
  int nNo;
  const int *nodes;   /* 0-based */
  const double *gx;   /* spatial profile, length nNo (NULL = 1) */
  const double *nV;   /* unit normals 3 x nNo for a vector BC (NULL = none) */
  double g;           /* value (dirY); dirA = 0 */
  int mask;           /* bit i set = component i constrained; 0 = all */
} orc_dirbc;

typedef struct {
  int nFel;
  const int *fIEN;    /* 3 x nFel, 0-based */
  double h[3];
} orc_tracbc;

/* Neumann face set of a HEATF equation: value g (BASSEMNEUBC + BHEATF) */
typedef struct {
  int nFel;
  const int *fIEN;    /* 3 x nFel, 0-based */
  double g;
} orc_neubc;

typedef struct {
  orc_eqp p;
  int nNo, nEl;
  const int *IEN;
  const double *x;
  const int *rowPtr, *colPtr; int nnz;
  int nDir; const orc_dirbc *dir;
  int nTrac; const orc_tracbc *trac;
  int LS_type, prec;
  double ls_relTol, ls_absTol; int ls_mItr, ls_sD;
  double ls_relTolIn[2]; double ls_absTolIn[2]; int ls_mItrIn[2];
  int minItr, maxItr; double tol, eqAbsTol;
  /* state (tDof x nNo) */
  double *Ao, *Yo, *Do, *An, *Yn, *Dn;
  /* eq%iNorm (first Newton residual of the run) and eq%pNorm (first of the
     current step), F/MOD.f:700-706; start at 0 */
  double eq_iNorm, eq_pNorm;
  /* CEP: cell model, stimulated-node flags (nNo, may be NULL), Xion(2,nNo),
     simulation time and the first-pass flag of CEPINTEG */
  orc_cep cep;
  const int *stim;
  double *Xion;
  double time;
  int cep_ipass_done;
  int nNeu; const orc_neubc *neu;  /* HEATF Neumann faces */
  /* optional element colouring for the multi-core CPU baseline: ncolor > 0
     runs each colour's elements with OpenMP (orc_assemble_colored); 0 keeps
     the serial element loop of GLOBALEQASSEM */
  int ncolor; const int *color_off; const int *color_order;
  /* USTRUCT (phys 7): Ad(3,nNo), the acceleration of the displacement
     kept across steps (F/INITIALIZE.f:227-231); NULL otherwise */
  double *Ad;
} orc_eq;

/* USTRUCT element (tet4, equal order, VMS): USTRUCT3D_M + USTRUCT3D_C,
   F/USTRUCT.f:205-612, 880-1102 */
void orc_elem_ustruct(const orc_eqp *p, const double xl[12], const double *al,
                      const double *yl, const double *dl, double lR[16], double lK[256],
                      double lKd[192]);
/* CONSTRUCT_uSOLID + USTRUCT_DOASSEM (F/USTRUCT.f:39-203, 1419-1555):
   R(4,nNo), Val(16,nnz), Kd(12,nnz) accumulated */
int orc_assemble_ustruct(const orc_eqp *p, int nNo, int nEl, const int *IEN,
                         const double *x, const double *Ag, const double *Yg,
                         const double *Dg, const int *rowPtr, const int *colPtr,
                         double *R, double *Val, double *Kd);
int orc_assemble_ustruct_colored(const orc_eqp *p, int nEl, const int *IEN, const double *x,
                                 const double *Ag, const double *Yg, const double *Dg,
                                 const int *rowPtr, const int *colPtr, double *R, double *Val,
                                 double *Kd, int ncolor, const int *color_off,
                                 const int *order);

/* Greedy element colouring: elements of one colour share no node.  Writes
   color_off[ncolor+1] (at most 65 entries) and order[nEl] (element ids
   colour by colour, ascending within a colour); returns ncolor (<= 64) or
   -1 when 64 colours do not suffice. */
int orc_color_elements(int nNo, int nEl, const int *IEN, int *color_off, int *order);

typedef struct {
  int newton_itr;
  int ls_itr_total;
  double last_iNorm;
  double r1_last;
  int last_suc;
} orc_stepinfo;

int orc_eq_step(orc_eq *eq, orc_stepinfo *info);

#ifdef __cplusplus
}
#endif
#endif
