/*
 * gsls -- GB300-native implicit-step engine for svFSI-style finite-element
 * solves: element residual/tangent assembly + svFSILS-compatible Krylov
 * solve, hand-written CUDA for sm_103a, one process on one GPU.
 *
 * Plain C ABI: plain pointers and sizes, no C++ or torch types.  Every
 * function returns an int status (GSLS_OK = 0).  The svFSILS-shaped calls
 * keep the argument order of the reference's Fortran interface
 * (Code/Source/svFSILS/FSILS_API.h:51-135, C mirror FSILS_api_c.h:52-64) so
 * a Fortran BIND(C) interface maps 1:1; indices are 1-based there as in the
 * reference.  Reference paths below are relative to the svFSI project root.
 *
 * Array layouts are the reference's column-major ones:
 *   Val[j*dof*dof + r*dof + c]  block j (CSR order), row r, column c
 *   R[a*dof + i]                node a, component i
 *   state[a*tDof + i]           node a, unknown i (An/Yn/Dn, Ag/Yg/Dg)
 *   IEN[e*eNoN + a]             node (1-based) of local vertex a of element e
 *   x[a*nsd + i]                coordinate i of node a
 */
#ifndef GSLS_H
#define GSLS_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GSLS_VERSION 1

/* ---- status codes ---- */
#define GSLS_OK 0
#define GSLS_ERR_ARG (-1)      /* bad argument (the reference STOPs instead) */
#define GSLS_ERR_CUDA (-2)     /* CUDA runtime error */
#define GSLS_ERR_STATE (-3)    /* object not created / already created */
#define GSLS_ERR_NAN (-4)      /* NaN/Inf met in the residual or Krylov scalars */
#define GSLS_ERR_JAC (-5)      /* non-positive element Jacobian */
#define GSLS_ERR_UNSUPPORTED (-6)
#define GSLS_ERR_NOMEM (-7)

/* ---- constants identical to Code/Source/svFSILS/FSILS_STRUCT.h:53-62 ---- */
#define GSLS_LS_TYPE_CG 798
#define GSLS_LS_TYPE_GMRES 797
#define GSLS_LS_TYPE_NS 796
#define GSLS_LS_TYPE_BICGS 795
#define GSLS_PRECOND_FSILS 701
#define GSLS_PRECOND_RCS 709
#define GSLS_BC_TYPE_DIR 0
#define GSLS_BC_TYPE_NEU 1

/* ---- arithmetic modes ---- */
#define GSLS_PREC_FP64 0  /* plain FP64 everywhere (the drop-in) */
#define GSLS_PREC_MIXED 1 /* FP32 tangent + FP32 inner Krylov; FP64 residual,
                             det F, Newton update, reductions, Gram-Schmidt */

/* ---- physics ids for assembly ---- */
#define GSLS_PHYS_HEATS 1
#define GSLS_PHYS_STRUCT 2
#define GSLS_PHYS_CEP 3
#define GSLS_PHYS_FLUID 4
#define GSLS_PHYS_LELAS 5  /* linear elasticity, Code/Source/svFSI/LELAS.f */
#define GSLS_PHYS_HEATF 6  /* heat in a fluid (advection-diffusion), HEATF.f;
                              velocity in state components 0..2 */
#define GSLS_PHYS_USTRUCT 7 /* velocity-pressure nonlinear solid, USTRUCT.f
                              (tet4, equal order, VMS; dof 4: v, p) */

/* Mirrors FSILS_subLsType, Code/Source/svFSILS/FSILS_STRUCT.h:162-191
   (Fortran LOGICAL stored as int32). */
typedef struct {
  int suc, mItr, sD, itr, cM, cN, cD, reserve;
  double absTol, relTol, iNorm, fNorm, dB, callD;
} gsls_sub_ls;

/* Mirrors FSILS_lsType, Code/Source/svFSILS/FSILS_STRUCT.h:193-204. */
typedef struct {
  int foC, LS_type, Resm, Resc;
  gsls_sub_ls GM, CG, RI;
} gsls_ls;

typedef struct gsls_lhs gsls_lhs;   /* replaces FSILS_lhsType */
typedef struct gsls_mesh gsls_mesh; /* element data for assembly */
typedef struct gsls_eq gsls_eq;     /* one equation's time integrator */

/* ------------------------------------------------------------------------ */
/* Library */

/* Select the CUDA device for this process (and place gsls_dot_noalloc's
   fixed scratch array on it). */
int gsls_init(int device);
/* No counterpart in the reference.  Poll limit of the grid barrier that
   the persistent Schur-complement CG of the NS solver waits on between its
   phases (0 = the default, 2^24 polls: seconds).  When a wait reaches the
   limit the kernel sets an error word, every block leaves, and the solve
   returns GSLS_ERR_CUDA with the CUDA context intact.  A test hook for the
   timeout path; a small limit makes waits expire on healthy launches. */
int gsls_set_wait_limit(unsigned polls);
/* Library version (GSLS_VERSION). */
int gsls_version(void);
/* Human-readable text for the last error of this thread. */
const char *gsls_last_error(void);

/* ------------------------------------------------------------------------ */
/* svFSILS-shaped linear-solver API */

/* Replaces FSILS_LHS_CREATE, Code/Source/svFSILS/LHS.f:51-111 (serial
   branch): rowPtr[nNo+1] and colPtr[nnz] are 1-based, columns sorted per
   row; gNodes is accepted for interface parity (map = identity on 1 GPU). */
int gsls_lhs_create(gsls_lhs **lhs, int gnNo, int nNo, int nnz,
                    const int *gNodes, const int *rowPtr, const int *colPtr,
                    int nFaces);
/* Replaces FSILS_LHS_FREE, Code/Source/svFSILS/LHS.f:295-325.  Meshes,
   equations and tapes built on the lhs may still be freed afterwards, in
   any order (their free calls then touch no lhs); no other call on them is
   valid once their lhs is freed. */
int gsls_lhs_free(gsls_lhs *lhs);

/* Replaces FSILS_BC_CREATE, Code/Source/svFSILS/BC.f:50-121: faIn 1-based,
   gNodes 1-based, val(dof,nNo) nullable (NULL = zeros). */
int gsls_bc_create(gsls_lhs *lhs, int faIn, int nNo, int dof, int BC_type,
                   const int *gNodes, const double *val);

/* Replaces FSILS_LS_CREATE, Code/Source/svFSILS/LS.f:50-119: defaults per
   LS_type, then every non-NULL optional argument overrides. */
int gsls_ls_create(gsls_ls *ls, int LS_type, const double *relTol,
                   const double *absTol, const int *maxItr, const int *dimKry,
                   const double *relTolIn, const double *absTolIn,
                   const int *maxItrIn);

/* Replaces FSILS_SOLVE, Code/Source/svFSILS/SOLVE.f:51-143, host arrays:
   Ri(dof,nNo) is overwritten with the solution and Val(dof*dof,nnz) is left
   scaled by the preconditioner, exactly as the reference does.  incL and res
   (length nFaces) are nullable.  Non-convergence is reported through
   ls->RI.suc = 0 with GSLS_OK, as in the reference. */
int gsls_solve(gsls_lhs *lhs, gsls_ls *ls, int dof, double *Ri, double *Val,
               int prec, const int *incL, const double *res);

/* Same as gsls_solve on device arrays.  val_prec selects the element type of
   dVal (GSLS_PREC_FP64: double, GSLS_PREC_MIXED: float, inner Krylov in
   FP32).  dRi is always double. */
int gsls_solve_dev(gsls_lhs *lhs, gsls_ls *ls, int dof, double *dRi,
                   void *dVal, int val_prec, int prec, const int *incL,
                   const double *res);

/* y = K x for block-CSR K (FSILS_SPARMULVV, Code/Source/svFSILS/SPARMUL.f:
   51-133) on device arrays; val_prec as above, x and y double. */
int gsls_spmv_dev(gsls_lhs *lhs, int dof, const void *dVal, int val_prec,
                  const double *dx, double *dy);

/* Dot product and 2-norm on device arrays (FSILS_DOTV / FSILS_NORMV,
   Code/Source/svFSILS/DOT.f:56-110, NORM.f:55-110); result on the host. */
int gsls_dot_dev(gsls_lhs *lhs, int dof, const double *du, const double *dv,
                 double *result);

/* No counterpart in the reference.  Dot product of two device vectors of
   length n (result on the host), for callers that cannot call cudaMalloc:
   it allocates no device memory.  Its reduction scratch is a fixed
   137,476-byte array in the library's device image; n <= 67,108,864,
   larger n is rejected with GSLS_ERR_ARG.  CUDA loads modules lazily, so
   the array is placed on a device when its address is first resolved
   (cudaGetSymbolAddress, with that device current): gsls_init does this
   for the device it selects, and the array then stays until the process
   exits.  Without gsls_init the first gsls_dot_noalloc call on a device
   does it; make that call before any stream capture and before a pool
   takes the whole heap (or set CUDA_MODULE_LOADING=EAGER).  The address is
   kept for the process: after cudaDeviceReset call gsls_init again.  All
   calls share the array: calls that overlap on the GPU (other streams,
   other host threads) race.  stream is a cudaStream_t (NULL = the default
   stream). */
int gsls_dot_noalloc(long long n, const double *du, const double *dv,
                     double *result, void *stream);
int gsls_norm_dev(gsls_lhs *lhs, int dof, const double *du, double *result);

/* CUDA stream used by every call on this lhs (cudaStream_t as void*;
   NULL = the library's own stream). */
int gsls_set_stream(gsls_lhs *lhs, void *stream);
void *gsls_get_stream(gsls_lhs *lhs);

/* ------------------------------------------------------------------------ */
/* Assembly (replaces GLOBALEQASSEM -> CONSTRUCT_* -> DOASSEM,
   Code/Source/svFSI/EQASSEM.f:38-87 and LHSA.f:266-298) */

/* Upload a tet4 mesh (IEN 1-based, eNoN = 4, nsd = 3) bound to lhs's CSR.
   Builds the element -> CSR position map and a conflict-free element
   colouring (deterministic scatter). */
int gsls_mesh_create(gsls_mesh **mesh, gsls_lhs *lhs, int nEl, int eNoN,
                     const int *IEN, int nsd, const double *x);
int gsls_mesh_free(gsls_mesh *mesh);
/* Number of colours of the element colouring. */
int gsls_mesh_ncolors(const gsls_mesh *mesh);

/* Parameters of one equation/domain (constant properties, optional
   per-element parameter). */
typedef struct {
  int phys;         /* GSLS_PHYS_* */
  int dof;          /* unknowns of this equation */
  int tDof;         /* total unknowns per node in the state arrays */
  int s;            /* 0-based first unknown of this equation */
  double am, af, beta, gam, dt;   /* generalized-alpha */
  double rho;       /* density (solid_density / fluid_density) */
  double cond;      /* HEATS conductivity */
  double src;       /* HEATS source term */
  double C10;       /* STRUCT neo-Hookean C10 = mu/2 */
  double Kpen;      /* STRUCT ST91 penalty (bulk modulus) */
  double visc;      /* STRUCT solid viscosity */
  double dmp;       /* STRUCT damping */
  double fb[3];     /* body force */
  double Diso;      /* CEP isotropic diffusivity */
  double mu_f;      /* FLUID viscosity */
  double ctM, ctC;  /* FLUID stabilisation constants */
  const double *eparam; /* host, per element (original order) or NULL:
                           STRUCT C10, CEP Diso, HEATS conductivity */
  double elM, nu;   /* LELAS elasticity modulus and Poisson ratio (body
                       force f_x, f_y, f_z in fb) */
  /* FLUID viscosity model (GETVISCOSITY, Code/Source/svFSI/FLUID.f:1690-1739;
     READVISCMODEL, READFILES.f:2875-2925): GSLS_VISC_CONST uses mu_f;
     GSLS_VISC_CY (Carreau-Yasuda): mu_f = high shear-rate limit, mu_o = low
     shear-rate limit, vlam = lambda, va = a, vn = power-law index n;
     GSLS_VISC_CASSON: mu_f = asymptotic viscosity parameter, mu_o = yield
     stress parameter, vlam = low shear-rate threshold (0.5 by default in
     the reference's input). */
  int viscType;
  double mu_o, vlam, va, vn;
  double bstab;     /* FLUID backflow stabilisation coefficient of the
                       Neumann faces (BFLUID, backflow_stab; the reference's
                       input default is 0.2, READFILES.f:1089-1091) */
  int volType;      /* USTRUCT volumetric penalty of GVOLPEN
                       (MATMODELS.f:1020-1070): 0 quadratic, 1 ST91, 2 M94;
                       USTRUCT also reads rho, C10 (neo-Hookean), Kpen
                       (0: incompressible), visc, fb, elM, nu, ctM, ctC */
  /* CEP fibres (CEP3D without electromechanical coupling,
     Code/Source/svFSI/CEP.f:136-266): the diffusion tensor of element e is
     D_e = Diso I + sum_i Dani[i] f_i f_i^T with the fibre directions
     f_i = fN[e*3*nFn + 3*i + (0..2)] used as given (lM%fN).  The reference
     repeats its last configured Dani for further mesh fibres (CEP.f:
     158-165); here Dani holds one value per fibre.  nFn = 0: isotropic
     (fN NULL).  Other physics take no fibres (GSLS_ERR_ARG). */
  int nFn;          /* fibre families per element, 0..3 */
  double Dani[3];   /* anisotropic diffusivity of each family */
  const double *fN; /* host, 3*nFn per element (original order), or NULL */
} gsls_eq_params;

#define GSLS_VISC_CONST 0
#define GSLS_VISC_CY 1
#define GSLS_VISC_CASSON 2

/* Assemble R(dof,nNo) (double) and Val(dof*dof,nnz) (double or float per
   val_prec) on device arrays from device state arrays Ag/Yg/Dg(tDof,nNo).
   R and Val are overwritten (LSALLOC zeroing included). */
int gsls_assemble_dev(gsls_mesh *mesh, const gsls_eq_params *p,
                      const double *dAg, const double *dYg, const double *dDg,
                      double *dR, void *dVal, int val_prec);
/* Same on host arrays (copies in and out). */
int gsls_assemble(gsls_mesh *mesh, const gsls_eq_params *p, const double *Ag,
                  const double *Yg, const double *Dg, double *R, double *Val);
/* USTRUCT (GSLS_PHYS_USTRUCT): CONSTRUCT_uSOLID with USTRUCT_DOASSEM
   (Code/Source/svFSI/USTRUCT.f:39-203, 1419-1555) on device arrays: R(4,nNo)
   and Val(16,nnz) as gsls_assemble_dev, and the displacement tangent
   Kd(12,nnz) (double: rows v1..v3, p times columns d1..d3, row-major per
   block) that USTRUCTR applies on the first Newton iteration.  All three
   are overwritten. */
int gsls_assemble_ustruct_dev(gsls_mesh *mesh, const gsls_eq_params *p,
                              const double *dAg, const double *dYg, const double *dDg,
                              double *dR, void *dVal, double *dKd, int val_prec);

/* ------------------------------------------------------------------------ */
/* Time integration of one equation (replaces the per-step work of
   Code/Source/svFSI/MAIN.f:89-281 for one equation: PICP, SETBCDIR, Newton
   loop of PICI / LSALLOC / assembly / SETBCNEU / LSSOLVE / PICC). */

typedef struct {
  int LS_type, prec;            /* GSLS_LS_TYPE_*, GSLS_PRECOND_* */
  double ls_relTol, ls_absTol;  /* <= 0: library default */
  int ls_mItr, ls_sD;           /* <= 0: library default */
  double ls_relTolIn[2];        /* NS GM/CG relTol, <= 0: default */
  int ls_mItrIn[2];             /* NS GM/CG mItr, <= 0: default */
  int minItr, maxItr;           /* Newton limits (defaults 1, 5) */
  double tol;                   /* Newton relative tolerance */
  double absTol;                /* Newton absolute tolerance (eq%absTol) */
  int precision;                /* GSLS_PREC_FP64 or GSLS_PREC_MIXED */
} gsls_eq_solver;

int gsls_eq_create(gsls_eq **eq, gsls_mesh *mesh, const gsls_eq_params *p,
                   const gsls_eq_solver *sv);
/* Frees the equation and releases the LS faces its Dirichlet sets claimed
   on the lhs (faces 1 .. number of sets), so that the next equation on the
   same lhs and mesh can claim them. */
int gsls_eq_free(gsls_eq *eq);

/* Strong Dirichlet BC on a node list (1-based): component c of the
   equation is set to g*gx[a] (Yn) with An = 0 when bit c of mask is set
   (mask = 0: all components); the face also enters the linear solver as a
   BC_TYPE_DIR face.  gx nullable (= 1).  For a dof = 4 (fluid) equation
   only the three velocity components are constrained.  Replaces the
   SETBCDIR/FSILSINI pair (Code/Source/svFSI/SETBC.f:39-228,
   BAFINI.f:488-512). */
int gsls_eq_add_dirichlet(gsls_eq *eq, int nNo, const int *gNodes,
                          const double *gx, double g, int mask);
/* Same with unit normals nV (3 x nNo): component c is set to
   g*gx[a]*nV[a][c], the vector form SETBCDIRL uses when the BC carries nsd
   values (Code/Source/svFSI/SETBC.f:212-217), e.g. an inflow profile along
   the inward normal.  nV nullable (= plain form). */
int gsls_eq_add_dirichlet_nv(gsls_eq *eq, int nNo, const int *gNodes,
                             const double *gx, const double *nV, double g,
                             int mask);
/* Neumann BC of value g on tri3 faces (fIEN 1-based, 3 x nFel), applied
   by BASSEMNEUBC (Code/Source/svFSI/EQASSEM.f:90-192) at every Newton
   iteration with h = -g (SETBCNEUL, SETBC.f:300).  HEATF: BHEATF
   (HEATF.f:289-319), the flux and the backflow term min(u.n, 0) T with its
   tangent.  FLUID: BFLUID (FLUID.f:1280-1334), the traction h n and the
   backflow stabilisation 1/2 bstab rho (u.n - |u.n|) u with its tangent on
   the velocity diagonal.  The outward normal is oriented away from the
   parent element's fourth node (GNNB, NN.f:1856-1990).  Other physics:
   GSLS_ERR_UNSUPPORTED. */
int gsls_eq_add_neumann(gsls_eq *eq, int nFel, const int *fIEN, double g);
/* Constant traction h on tri3 faces (fIEN 1-based, 3 x nFel), integrated
   as SETBCTRACL does (Code/Source/svFSI/SETBC.f:319-416). */
int gsls_eq_add_traction(gsls_eq *eq, int nFel, const int *fIEN,
                         const double h[3]);

/* Old-step state (tDof x nNo, host) in and current state out. */
int gsls_eq_set_state(gsls_eq *eq, const double *Ao, const double *Yo,
                      const double *Do);
int gsls_eq_get_state(gsls_eq *eq, double *Ao, double *Yo, double *Do);
/* Device pointers of the resident old-step state (valid until the next
   step); for callers that keep the state on the GPU. */
int gsls_eq_state_dev(gsls_eq *eq, double **dAo, double **dYo, double **dDo);

typedef struct {
  int newton_itr;       /* Newton iterations taken */
  int ls_itr_total;     /* Krylov iterations summed over Newton iterations */
  double last_iNorm;    /* RI%iNorm of the last linear solve */
  double r1_last;       /* RI%iNorm / eq%iNorm at exit */
  int last_suc;         /* RI%suc of the last linear solve */
  double t_assembly_ms; /* device time in assembly (CUDA events) */
  double t_solve_ms;    /* device time in the linear solve */
} gsls_step_info;

/* Aliev-Panfilov cell model for a GSLS_PHYS_CEP equation: the reaction
   step of CEPINTEG/CEPINTEGL (Code/Source/svFSI/CEPION.f:166-400,
   CEPMOD_AP.f:125-184), run per node at the start of every step before
   the diffusion solve.  The stimulus of amplitude A is applied on
   [Ts + k CL, Ts + k CL + Td] to the listed nodes (1-based). */
typedef struct {
  int ode;          /* 0 forward Euler, 1 RK4 */
  double dt_ode;    /* ODE substep (cep%dt); nt = round(dt/dt_ode) */
  double A, Ts, Td, CL;
  double V0, X20;   /* initial voltage and recovery variable */
} gsls_cep_params;
int gsls_eq_set_cep(gsls_eq *eq, const gsls_cep_params *c, int nStim,
                    const int *stimNodes);
/* Cell state Xion(2,nNo) (voltage, recovery) to the host. */
int gsls_eq_get_cep_state(gsls_eq *eq, double *Xion);

/* Advance one time step. */
int gsls_eq_step(gsls_eq *eq, gsls_step_info *info);

/* Restart file of one equation in the reference's layout
   (Code/Source/svFSI/OUTPUT.f:132-232 WRITERESTART, read back as
   INITIALIZE.f:508-621 INITFROMBIN; record length INITIALIZE.f:152-163),
   serial form: one direct-access record of
     stamp(7) = (1, 1, 1, nNo, 0, tDof, dFlag), cTS      int32
     time, cpu_time, eq%iNorm                           float64
     Y(tDof,nNo), A(tDof,nNo) [, D(tDof,nNo) if dFlag]  float64
     [Xion(2,nNo) for CEP]                              float64
   in native byte order, no record markers.  The state written is the one
   after the last step (the reference's Yn, An, Dn at WRITERESTART).
   Reading checks the stamp as INITFROMBIN does (an error names the first
   field that differs) and restores the state, the simulation time, the
   Newton normalisation eq%iNorm and the cell state. */
int gsls_eq_write_restart(gsls_eq *eq, const char *path, int cTS, double cpu_time);
int gsls_eq_read_restart(gsls_eq *eq, const char *path, int *cTS, double *cpu_time);
/* Per-element parameter update (host, original element order). */
int gsls_eq_set_eparam(gsls_eq *eq, const double *eparam);

/* Count of this library's kernel launches so far (for launch accounting). */
long long gsls_launch_count(void);

/* Kernel timing (no counterpart in the reference, which only keeps wall
   clock per call in ls%callD).  When enabled, the library brackets its
   dominant launches with CUDA events on its own stream and accumulates,
   per name, the number of launches that did work and their device time:
   "cg_spmv" (SpMV + fused dot of one CG iteration), "cg_update" (X, R and
   |R|^2), "cg_pupdate" (direction update), "gm_spmv"/"gm_spmv_d3" (GMRES
   Arnoldi SpMV), "assembly" (all colour launches of one assembly).  Off by
   default; profiled solves run without graphs or programmatic launch. */
int gsls_profile_enable(int on);
int gsls_profile_reset(void);
int gsls_profile_read(const char *name, long long *count, double *total_ms);
/* FP64 FMA throughput of the current device (FMAs per second), measured
   with a short probe kernel (8 independent FMA chains per thread, 4 blocks
   of 256 per SM, CUDA events): the compute roof of the FP64 drop-in path,
   whose SpMV issues one FP64 FMA per matrix entry.  No counterpart in the
   reference. */
int gsls_fp64_fma_rate(double *fma_per_s);
/* No counterpart in the reference.  L2 read bandwidth of the device
   (bytes/s): a 48 MiB buffer, resident in L2, swept 20 times by every
   resident thread with 16-byte loads; the roof of kernels whose operator
   stays in L2 between launches (the persistent Schur-complement CG). */
int gsls_l2_read_rate(double *bytes_per_s);

/* ---- discrete adjoint (forward/backward pair) --------------------------
   Gradient of an objective of the final state with respect to the
   per-element parameter of the equation (gsls_eq_set_eparam: STRUCT C10 =
   mu/2, HEATS conductivity), through every implicit step: transpose solve
   on the assembled tangent, element kernel for dR/dp, checkpoint every
   `every` steps and recompute of each segment on the way back.  New
   capability (the reference has no adjoint).  An FP64 equation runs FP64
   throughout; a GSLS_PREC_MIXED equation takes its forward and recomputed
   steps on the mixed path and refines each transpose solve (FP32 solves of
   the normalised FP64 residual) to the FP64 tolerance. */
typedef struct gsls_tape gsls_tape;
/* Take nsteps steps of eq (as gsls_eq_step), storing checkpoints. */
int gsls_adjoint_forward(gsls_eq *eq, int nsteps, int every, gsls_tape **tape);
/* Given dJ/dA_N, dJ/dY_N, dJ/dD_N (host, tDof x nNo, each nullable = 0),
   write dJ/dp (host, nEl, original element order).  eq is left at step N. */
int gsls_adjoint_backward(gsls_tape *tape, const double *Abar, const double *Ybar,
                          const double *Dbar, double *grad);
int gsls_tape_free(gsls_tape *tape);

/* Activation-time adjoint of a CEP equation (monodomain, forward-Euler or
   RK4 cell step, isotropic or with fibres; per-element isotropic
   diffusivity by gsls_eq_set_eparam).  The
   smoothed activation time of node a over the nsteps steps is
     T_a = sum_n dt (1 - s(V_n(a))),  s(V) = 1 / (1 + exp(-(V - vth) / vw))
   (vw > 0; T_a tends to the first crossing of vth as vw -> 0 for a node
   that depolarises once and stays up over the window).  The forward call
   steps eq as gsls_eq_step does, checkpointing the state and the cell
   state every `every` steps, and returns T (host, nNo).  The backward call
   takes dJ/dT (host, nNo) and writes dJ/dDiso_e (host, nEl, original
   element order): each reverse step adds dJ/dV_n, reverses the diffusion
   solve (transpose solve + dR/dDiso) and the cell step's substeps.  eq is
   left at step N.  New capability (the reference has no adjoint); the
   precision follows the equation's, as for gsls_adjoint_forward. */
int gsls_cep_adjoint_forward(gsls_eq *eq, int nsteps, int every, double vth, double vw,
                             double *T, gsls_tape **tape);
int gsls_cep_adjoint_backward(gsls_tape *tape, const double *Tbar, double *grad);

/* Linearisation point of one step: old and new state (device, tDof x nNo). */
typedef struct {
  const double *Ao, *Yo, *Do, *An, *Yn, *Dn;
} gsls_adj_point;
/* lambda = K^-T rhs with K = dR/dA_n assembled at pt (Dirichlet rows
   masked as in the forward solve); rhs, lambda: device, dof x nNo. */
int gsls_adjoint_solve(gsls_eq *eq, const gsls_adj_point *pt, const double *rhs,
                       double *lambda);
/* out[e] = (d R / d p_e)^T lambda at pt (device, nEl, original element order). */
int gsls_dRdp(gsls_eq *eq, const gsls_adj_point *pt, const double *lambda, double *out);

#ifdef __cplusplus
}
#endif
#endif
