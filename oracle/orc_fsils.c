/*
 * Oracle (test infrastructure only): restatement of the svFSILS linear
 * solver library, serial branch (nTasks == 1), FP64.
 * L/ = Code/Source/svFSILS in the svFSI project.
 */
#include "orc.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int g_threads = 1;
void orc_set_threads(int n) { g_threads = n > 0 ? n : 1; }
int orc_get_threads(void) { return g_threads; }

static void *xcalloc(size_t n, size_t s) {
  void *p = calloc(n ? n : 1, s);
  if (!p) {
    fprintf(stderr, "oracle: out of memory\n");
    abort();
  }
  return p;
}

/* FSILS_LHS_CREATE serial branch, L/LHS.f:88-111: copy CSR, find diagPtr,
   rowPtr(2,nNo) = [start,end], map = identity. */
orc_lhs *orc_lhs_create(int nNo, int nnz, const int *rowPtr, const int *colPtr,
                        int nFaces) {
  orc_lhs *lhs = (orc_lhs *)xcalloc(1, sizeof(orc_lhs));
  lhs->nNo = nNo;
  lhs->nnz = nnz;
  lhs->nFaces = nFaces;
  lhs->mynNo = nNo;
  lhs->rowS = (int *)xcalloc(nNo, sizeof(int));
  lhs->rowE = (int *)xcalloc(nNo, sizeof(int));
  lhs->colPtr = (int *)xcalloc(nnz, sizeof(int));
  lhs->diagPtr = (int *)xcalloc(nNo, sizeof(int));
  lhs->face = (orc_face *)xcalloc(nFaces, sizeof(orc_face));
  memcpy(lhs->colPtr, colPtr, sizeof(int) * (size_t)nnz);
  for (int Ac = 0; Ac < nNo; Ac++) {
    int s = rowPtr[Ac], e = rowPtr[Ac + 1] - 1;
    lhs->diagPtr[Ac] = -1;
    for (int i = s; i <= e; i++)
      if (colPtr[i] == Ac) {
        lhs->diagPtr[Ac] = i;
        break;
      }
    lhs->rowS[Ac] = s;
    lhs->rowE[Ac] = e;
  }
  return lhs;
}

void orc_lhs_free(orc_lhs *lhs) {
  if (!lhs) return;
  for (int f = 0; f < lhs->nFaces; f++) {
    free(lhs->face[f].glob);
    free(lhs->face[f].val);
    free(lhs->face[f].valM);
  }
  free(lhs->face);
  free(lhs->rowS);
  free(lhs->rowE);
  free(lhs->colPtr);
  free(lhs->diagPtr);
  free(lhs);
}

/* FSILS_BC_CREATE, L/BC.f:50-121 (faIn is 1-based as in the reference). */
int orc_bc_create(orc_lhs *lhs, int faIn, int nNo, int dof, int BC_type,
                  const int *gNodes, const double *val) {
  if (faIn > lhs->nFaces || faIn <= 0) return -1;
  orc_face *f = &lhs->face[faIn - 1];
  if (f->foC) return -2;
  f->foC = 1;
  f->nNo = nNo;
  f->dof = dof;
  f->bGrp = BC_type;
  f->glob = (int *)xcalloc(nNo, sizeof(int));
  f->val = (double *)xcalloc((size_t)dof * nNo, sizeof(double));
  f->valM = (double *)xcalloc((size_t)dof * nNo, sizeof(double));
  for (int a = 0; a < nNo; a++) f->glob[a] = gNodes[a];
  if (val)
    memcpy(f->val, val, sizeof(double) * (size_t)dof * nNo);
  return 0;
}

/* FSILS_LS_CREATE defaults, L/LS.f:50-119 */
void orc_ls_create(orc_ls *ls, int LS_type) {
  memset(ls, 0, sizeof(*ls));
  ls->foC = 1;
  ls->LS_type = LS_type;
  switch (LS_type) {
  case ORC_LS_TYPE_NS:
    ls->RI.relTol = 0.4;
    ls->GM.relTol = 1e-2;
    ls->CG.relTol = 0.2;
    ls->RI.mItr = 10;
    ls->GM.mItr = 2;
    ls->CG.mItr = 500;
    ls->GM.sD = 100;
    ls->RI.sD = 100;
    break;
  case ORC_LS_TYPE_GMRES:
    ls->RI.relTol = 0.1;
    ls->RI.mItr = 4;
    ls->RI.sD = 250;
    break;
  case ORC_LS_TYPE_CG:
    ls->RI.relTol = 1e-2;
    ls->RI.mItr = 1000;
    break;
  case ORC_LS_TYPE_BICGS:
    ls->RI.relTol = 1e-2;
    ls->RI.mItr = 500;
    break;
  default:
    break;
  }
  ls->RI.absTol = 1e-10;
  ls->GM.absTol = 1e-10;
  ls->CG.absTol = 1e-10;
}

/* FSILS_SPARMULVV, L/SPARMUL.f:51-133: KU(:,i) = sum_j K(:,:,j) U(:,col(j)) */
void orc_spar_vv(const orc_lhs *lhs, int dof, const double *K, const double *U,
                 double *KU) {
  const int nNo = lhs->nNo, dd = dof * dof;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (int i = 0; i < nNo; i++) {
    double acc[16];
    for (int l = 0; l < dof; l++) acc[l] = 0.0;
    for (int j = lhs->rowS[i]; j <= lhs->rowE[i]; j++) {
      const int col = lhs->colPtr[j];
      const double *Kj = K + (size_t)j * dd;
      const double *Uc = U + (size_t)col * dof;
      for (int l = 0; l < dof; l++) {
        double s = 0.0;
        for (int m = 0; m < dof; m++) s += Kj[l * dof + m] * Uc[m];
        acc[l] += s;
      }
    }
    for (int l = 0; l < dof; l++) KU[(size_t)i * dof + l] = acc[l];
  }
}

/* FSILS_SPARMULSS, L/SPARMUL.f:273-297 */
void orc_spar_ss(const orc_lhs *lhs, const double *K, const double *U,
                 double *KU) {
  orc_spar_vv(lhs, 1, K, U, KU);
}

/* FSILS_SPARMULVS, L/SPARMUL.f:135-200: K(dof,nnz) row-vector blocks times
   vector U(dof,nNo) -> scalar KU(nNo) */
void orc_spar_vs(const orc_lhs *lhs, int dof, const double *K, const double *U,
                 double *KU) {
  const int nNo = lhs->nNo;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (int i = 0; i < nNo; i++) {
    double acc = 0.0;
    for (int j = lhs->rowS[i]; j <= lhs->rowE[i]; j++) {
      const int col = lhs->colPtr[j];
      for (int m = 0; m < dof; m++)  /* ((KU + K1 U1) + K2 U2) + ... */
        acc += K[(size_t)j * dof + m] * U[(size_t)col * dof + m];
    }
    KU[i] = acc;
  }
}

/* FSILS_SPARMULSV, L/SPARMUL.f:202-271: K(dof,nnz) column blocks times
   scalar U(nNo) -> vector KU(dof,nNo) */
void orc_spar_sv(const orc_lhs *lhs, int dof, const double *K, const double *U,
                 double *KU) {
  const int nNo = lhs->nNo;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (int i = 0; i < nNo; i++) {
    double acc[16];
    for (int l = 0; l < dof; l++) acc[l] = 0.0;
    for (int j = lhs->rowS[i]; j <= lhs->rowE[i]; j++) {
      const int col = lhs->colPtr[j];
      for (int l = 0; l < dof; l++) acc[l] += K[(size_t)j * dof + l] * U[col];
    }
    for (int l = 0; l < dof; l++) KU[(size_t)i * dof + l] = acc[l];
  }
}

/* FSILS_DOTV, L/DOT.f:56-110 (serial: no ALLREDUCE) */
double orc_dotv(int dof, int nNo, const double *U, const double *V) {
  double s = 0.0;
  const size_t n = (size_t)dof * nNo;
  if (g_threads > 1) {
    /* fixed chunks, partial sums added in chunk order: the same bits on
       every run for a given thread count (an OpenMP reduction clause
       combines the partials in arrival order) */
    enum { kMaxChunks = 256 };
    double part[kMaxChunks];
    const int nt = g_threads < kMaxChunks ? g_threads : kMaxChunks;
    const size_t chunk = (n + (size_t)nt - 1) / (size_t)nt;
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int t = 0; t < nt; t++) {
      const size_t i0 = (size_t)t * chunk, i1 = i0 + chunk < n ? i0 + chunk : n;
      double a = 0.0;
      for (size_t i = i0; i < i1; i++) a += U[i] * V[i];
      part[t] = a;
    }
    for (int t = 0; t < nt; t++) s += part[t];
    return s;
  }
  for (int i = 0; i < nNo; i++) {
    double t = 0.0;
    for (int k = 0; k < dof; k++) t += U[(size_t)i * dof + k] * V[(size_t)i * dof + k];
    s += t;
  }
  return s;
}

/* FSILS_NORMV, L/NORM.f:55-110 */
double orc_normv(int dof, int nNo, const double *U) {
  return sqrt(orc_dotv(dof, nNo, U, U));
}

/* PREMUL / POSMUL, L/PRECOND.f:372-489 */
static void premul(const orc_lhs *lhs, int dof, double *Val, const double *W) {
  const int dd = dof * dof;
  for (int Ac = 0; Ac < lhs->nNo; Ac++)
    for (int j = lhs->rowS[Ac]; j <= lhs->rowE[Ac]; j++)
      for (int r = 0; r < dof; r++)
        for (int c = 0; c < dof; c++) Val[(size_t)j * dd + r * dof + c] *= W[(size_t)Ac * dof + r];
}
static void posmul(const orc_lhs *lhs, int dof, double *Val, const double *W) {
  const int dd = dof * dof;
  for (int Ac = 0; Ac < lhs->nNo; Ac++)
    for (int j = lhs->rowS[Ac]; j <= lhs->rowE[Ac]; j++) {
      const int a = lhs->colPtr[j];
      for (int r = 0; r < dof; r++)
        for (int c = 0; c < dof; c++) Val[(size_t)j * dd + r * dof + c] *= W[(size_t)a * dof + c];
    }
}

/* PRECONDDIAG, L/PRECOND.f:50-145 */
void orc_precond_diag(orc_lhs *lhs, int dof, double *Val, double *R, double *W) {
  const int nNo = lhs->nNo, dd = dof * dof;
  for (int Ac = 0; Ac < nNo; Ac++) {
    const int d = lhs->diagPtr[Ac];
    for (int i = 0; i < dof; i++) W[(size_t)Ac * dof + i] = Val[(size_t)d * dd + i * dof + i];
  }
  for (size_t k = 0; k < (size_t)nNo * dof; k++) {
    if (W[k] == 0.0) W[k] = 1.0;
    W[k] = 1.0 / sqrt(fabs(W[k]));
  }
  for (int f = 0; f < lhs->nFaces; f++) {
    orc_face *fa = &lhs->face[f];
    if (!fa->incFlag) continue;
    const int i = fa->dof < dof ? fa->dof : dof;
    if (fa->bGrp == ORC_BC_TYPE_Dir)
      for (int a = 0; a < fa->nNo; a++) {
        const int Ac = fa->glob[a];
        for (int k = 0; k < i; k++) W[(size_t)Ac * dof + k] *= fa->val[(size_t)a * fa->dof + k];
      }
  }
  premul(lhs, dof, Val, W);
  for (size_t k = 0; k < (size_t)nNo * dof; k++) R[k] *= W[k];
  posmul(lhs, dof, Val, W);
  for (int f = 0; f < lhs->nFaces; f++) {
    orc_face *fa = &lhs->face[f];
    if (!fa->coupledFlag) continue;
    const int m = fa->dof < dof ? fa->dof : dof;
    for (int a = 0; a < fa->nNo; a++) {
      const int Ac = fa->glob[a];
      for (int i = 0; i < m; i++)
        fa->valM[(size_t)a * fa->dof + i] = fa->val[(size_t)a * fa->dof + i] * W[(size_t)Ac * dof + i];
    }
  }
}

/* PRECONDRCS, L/PRECOND.f:150-368 */
void orc_precond_rcs(orc_lhs *lhs, int dof, double *Val, double *R, double *W1,
                     double *W2) {
  const int nNo = lhs->nNo, dd = dof * dof;
  const size_t n = (size_t)nNo * dof;
  const int maxiter = 10;
  const double tol = 2.0;
  int iter = 0, flag = 1;
  double *Wr = (double *)xcalloc(n, sizeof(double));
  double *Wc = (double *)xcalloc(n, sizeof(double));
  for (size_t k = 0; k < n; k++) {
    W1[k] = 1.0;
    W2[k] = 1.0;
    Wr[k] = 1.0;
  }
  for (int f = 0; f < lhs->nFaces; f++) {
    orc_face *fa = &lhs->face[f];
    if (!fa->incFlag) continue;
    const int i = fa->dof < dof ? fa->dof : dof;
    if (fa->bGrp == ORC_BC_TYPE_Dir)
      for (int a = 0; a < fa->nNo; a++) {
        const int Ac = fa->glob[a];
        for (int k = 0; k < i; k++) Wr[(size_t)Ac * dof + k] *= fa->val[(size_t)a * fa->dof + k];
      }
  }
  /* renormalisation Wr = (sign(Wr-0.5)+|.|)/2 -> 1 if Wr > 0.5 else 0 */
  for (size_t k = 0; k < n; k++) {
    double t = Wr[k] - 0.5;
    t = t / fabs(t);
    Wr[k] = (t + fabs(t)) * 0.5;
  }
  premul(lhs, dof, Val, Wr);
  for (size_t k = 0; k < n; k++) R[k] *= Wr[k];
  posmul(lhs, dof, Val, Wr);
  for (int Ac = 0; Ac < nNo; Ac++) {
    const int d = lhs->diagPtr[Ac];
    for (int i = 0; i < dof; i++) {
      double *v = &Val[(size_t)d * dd + i * dof + i];
      *v = Wr[(size_t)Ac * dof + i] * (*v - 1.0) + 1.0;
    }
  }
  while (flag) {
    for (size_t k = 0; k < n; k++) {
      Wr[k] = 0.0;
      Wc[k] = 0.0;
    }
    iter++;
    if (iter >= maxiter) flag = 0;
    for (int Ac = 0; Ac < nNo; Ac++) {
      for (int j = lhs->rowS[Ac]; j <= lhs->rowE[Ac]; j++) {
        const int a = lhs->colPtr[j];
        for (int r = 0; r < dof; r++)
          for (int c = 0; c < dof; c++) {
            const double v = fabs(Val[(size_t)j * dd + r * dof + c]);
            if (v > Wr[(size_t)Ac * dof + r]) Wr[(size_t)Ac * dof + r] = v;
            if (v > Wc[(size_t)a * dof + c]) Wc[(size_t)a * dof + c] = v;
          }
      }
    }
    double mr = 0.0, mc = 0.0;
    for (size_t k = 0; k < n; k++) {
      if (fabs(1.0 - Wr[k]) > mr) mr = fabs(1.0 - Wr[k]);
      if (fabs(1.0 - Wc[k]) > mc) mc = fabs(1.0 - Wc[k]);
    }
    if (mr < tol && mc < tol) flag = 0;
    for (size_t k = 0; k < n; k++) {
      Wr[k] = 1.0 / sqrt(Wr[k]);
      Wc[k] = 1.0 / sqrt(Wc[k]);
    }
    premul(lhs, dof, Val, Wr);
    posmul(lhs, dof, Val, Wc);
    for (size_t k = 0; k < n; k++) {
      W1[k] *= Wr[k];
      W2[k] *= Wc[k];
    }
  }
  for (size_t k = 0; k < n; k++) R[k] *= W1[k];
  free(Wr);
  free(Wc);
}

/* ADDBCMUL, L/ADDBCMUL.f:53-114 (non-shared faces) */
void orc_addbcmul(orc_lhs *lhs, int op, int dof, const double *X, double *Y) {
  for (int f = 0; f < lhs->nFaces; f++) {
    orc_face *fa = &lhs->face[f];
    if (!fa->coupledFlag) continue;
    const double coef = (op == 0) ? fa->res : -fa->res / (1.0 + fa->res * fa->nS);
    const int nsd = fa->dof < dof ? fa->dof : dof;
    double S = 0.0;
    for (int a = 0; a < fa->nNo; a++) {
      const int Ac = fa->glob[a];
      for (int i = 0; i < nsd; i++) S = S + fa->valM[(size_t)a * fa->dof + i] * X[(size_t)Ac * dof + i];
    }
    S = coef * S;
    for (int a = 0; a < fa->nNo; a++) {
      const int Ac = fa->glob[a];
      for (int i = 0; i < nsd; i++)
        Y[(size_t)Ac * dof + i] = Y[(size_t)Ac * dof + i] + fa->valM[(size_t)a * fa->dof + i] * S;
    }
  }
}

/* BCPRE, L/NSSOLVER.f:307-343 and L/GMRES.f:395-431 (non-shared faces) */
void orc_bcpre(orc_lhs *lhs, int nsd) {
  for (int f = 0; f < lhs->nFaces; f++) {
    orc_face *fa = &lhs->face[f];
    if (!fa->coupledFlag) continue;
    fa->nS = 0.0;
    for (int a = 0; a < fa->nNo; a++)
      for (int i = 0; i < nsd; i++)
        fa->nS = fa->nS + pow(fa->valM[(size_t)a * fa->dof + i], 2.0);
  }
}

int orc_any_coupled(const orc_lhs *lhs) {
  for (int f = 0; f < lhs->nFaces; f++)
    if (lhs->face[f].coupledFlag) return 1;
  return 0;
}

/* BICGSS / BICGSV, L/BICGS.f:51-230 */
void orc_bicgs_v(orc_lhs *lhs, orc_subls *ls, int dof, const double *K, double *R) {
  const int nNo = lhs->nNo, mynNo = lhs->mynNo;
  const size_t n = (size_t)nNo * dof;
  double *P = (double *)xcalloc(n, sizeof(double));
  double *Rh = (double *)xcalloc(n, sizeof(double));
  double *X = (double *)xcalloc(n, sizeof(double));
  double *V = (double *)xcalloc(n, sizeof(double));
  double *S = (double *)xcalloc(n, sizeof(double));
  double *T = (double *)xcalloc(n, sizeof(double));
  ls->suc = 0;
  double err = orc_normv(dof, mynNo, R);
  ls->iNorm = err;
  double errO = err;
  const double eps = fmax(ls->absTol, ls->relTol * err);
  double rho = err * err, rhoO, beta = rho, alpha, omega;
  (void)beta;
  memcpy(P, R, n * sizeof(double));
  memcpy(Rh, R, n * sizeof(double));
  int i;
  for (i = 1; i <= ls->mItr; i++) {
    if (err < eps) {
      ls->suc = 1;
      break;
    }
    orc_spar_vv(lhs, dof, K, P, V);
    alpha = rho / orc_dotv(dof, mynNo, Rh, V);
    for (size_t k = 0; k < n; k++) S[k] = R[k] - alpha * V[k];
    orc_spar_vv(lhs, dof, K, S, T);
    omega = orc_normv(dof, mynNo, T);
    omega = orc_dotv(dof, mynNo, T, S) / (omega * omega);
    for (size_t k = 0; k < n; k++) X[k] = X[k] + alpha * P[k] + omega * S[k];
    for (size_t k = 0; k < n; k++) R[k] = S[k] - omega * T[k];
    errO = err;
    err = orc_normv(dof, mynNo, R);
    rhoO = rho;
    rho = orc_dotv(dof, mynNo, R, Rh);
    beta = rho * alpha / (rhoO * omega);
    for (size_t k = 0; k < n; k++) P[k] = R[k] + beta * (P[k] - omega * V[k]);
  }
  memcpy(R, X, n * sizeof(double));
  ls->itr = i - 1;
  ls->fNorm = err;
  ls->dB = (errO < 2.220446049250313e-16) ? 0.0 : 10.0 * log(err / errO);
  free(P);
  free(Rh);
  free(X);
  free(V);
  free(S);
  free(T);
}

/* CGRADS / CGRADV, L/CGRAD.f:125-242 */
void orc_cgrad_v(orc_lhs *lhs, orc_subls *ls, int dof, const double *K, double *R) {
  const int nNo = lhs->nNo, mynNo = lhs->mynNo;
  const size_t n = (size_t)nNo * dof;
  double *P = (double *)xcalloc(n, sizeof(double));
  double *KP = (double *)xcalloc(n, sizeof(double));
  double *X = (double *)xcalloc(n, sizeof(double));
  ls->suc = 0;
  ls->iNorm = orc_normv(dof, mynNo, R);
  double eps = fmax(ls->absTol, ls->relTol * ls->iNorm);
  eps = eps * eps;
  double errO = ls->iNorm * ls->iNorm, err = errO, alpha;
  memcpy(P, R, n * sizeof(double));
  int i;
  for (i = 1; i <= ls->mItr; i++) {
    if (err < eps) {
      ls->suc = 1;
      break;
    }
    errO = err;
    orc_spar_vv(lhs, dof, K, P, KP);
    alpha = errO / orc_dotv(dof, mynNo, P, KP);
    for (size_t k = 0; k < n; k++) X[k] += alpha * P[k];
    for (size_t k = 0; k < n; k++) R[k] += -alpha * KP[k];
    err = orc_normv(dof, mynNo, R);
    err = err * err;
    for (size_t k = 0; k < n; k++) P[k] += (errO / err) * R[k];
    for (size_t k = 0; k < n; k++) P[k] *= err / errO;
  }
  memcpy(R, X, n * sizeof(double));
  ls->itr = i - 1;
  ls->fNorm = sqrt(err);
  ls->dB = (errO < 2.220446049250313e-16) ? 0.0 : 5.0 * log(err / errO);
  free(P);
  free(KP);
  free(X);
}

/* Arnoldi with classical Gram-Schmidt + Givens, shared by GMRESS/GMRESV,
   L/GMRES.f:171-431 (no coupled-Neumann faces). */
void orc_gmres_v(orc_lhs *lhs, orc_subls *ls, int dof, const double *Val, double *R) {
  const int nNo = lhs->nNo, mynNo = lhs->mynNo, sD = ls->sD;
  const size_t n = (size_t)nNo * dof;
  double *u = (double *)xcalloc(n * (size_t)(sD + 1), sizeof(double));
  double *h = (double *)xcalloc((size_t)(sD + 1) * sD, sizeof(double));
#define H(j, i) h[(size_t)(i) * (sD + 1) + (j)]
  double *X = (double *)xcalloc(n, sizeof(double));
  double *y = (double *)xcalloc(sD + 1, sizeof(double));
  double *c = (double *)xcalloc(sD + 1, sizeof(double));
  double *s = (double *)xcalloc(sD + 1, sizeof(double));
  double *err = (double *)xcalloc(sD + 2, sizeof(double));
  ls->suc = 0;
  double eps = orc_normv(dof, mynNo, R);
  ls->iNorm = eps;
  ls->fNorm = eps;
  eps = fmax(ls->absTol, ls->relTol * eps);
  ls->itr = 0;
  if (ls->iNorm <= ls->absTol) {
    /* the reference returns here with R untouched (L/GMRES.f:310-314) */
    ls->callD = 2.220446049250313e-16;
    ls->dB = 0.0;
    goto done;
  }
  for (int l = 1; l <= ls->mItr; l++) {
    ls->dB = ls->fNorm;
    ls->itr++;
    orc_spar_vv(lhs, dof, Val, X, u);
    orc_addbcmul(lhs, 0, dof, X, u);
    for (size_t k = 0; k < n; k++) u[k] = R[k] - u[k];
    err[0] = orc_normv(dof, mynNo, u);
    for (size_t k = 0; k < n; k++) u[k] /= err[0];
    int i;
    for (i = 1; i <= sD; i++) {
      ls->itr++;
      double *ui = u + n * (size_t)(i - 1), *ui1 = u + n * (size_t)i;
      orc_spar_vv(lhs, dof, Val, ui, ui1);
      orc_addbcmul(lhs, 0, dof, ui, ui1);
      for (int j = 1; j <= i + 1; j++) H(j - 1, i - 1) = orc_dotv(dof, mynNo, u + n * (size_t)(j - 1), ui1);
      for (int j = 1; j <= i; j++) {
        const double hj = H(j - 1, i - 1);
        const double *uj = u + n * (size_t)(j - 1);
        for (size_t k = 0; k < n; k++) ui1[k] += -hj * uj[k];
        H(i, i - 1) = H(i, i - 1) - hj * hj;
      }
      H(i, i - 1) = sqrt(fabs(H(i, i - 1)));
      const double inv = 1.0 / H(i, i - 1);
      for (size_t k = 0; k < n; k++) ui1[k] *= inv;
      for (int j = 1; j <= i - 1; j++) {
        const double tmp = c[j - 1] * H(j - 1, i - 1) + s[j - 1] * H(j, i - 1);
        H(j, i - 1) = -s[j - 1] * H(j - 1, i - 1) + c[j - 1] * H(j, i - 1);
        H(j - 1, i - 1) = tmp;
      }
      const double tmp = sqrt(H(i - 1, i - 1) * H(i - 1, i - 1) + H(i, i - 1) * H(i, i - 1));
      c[i - 1] = H(i - 1, i - 1) / tmp;
      s[i - 1] = H(i, i - 1) / tmp;
      H(i - 1, i - 1) = tmp;
      H(i, i - 1) = 0.0;
      err[i] = -s[i - 1] * err[i - 1];
      err[i - 1] = c[i - 1] * err[i - 1];
      if (fabs(err[i]) < eps) {
        ls->suc = 1;
        break;
      }
    }
    if (i > sD) i = sD;
    for (int j = 0; j < i; j++) y[j] = err[j];
    for (int j = i; j >= 1; j--) {
      for (int k = j + 1; k <= i; k++) y[j - 1] -= H(j - 1, k - 1) * y[k - 1];
      y[j - 1] /= H(j - 1, j - 1);
    }
    for (int j = 1; j <= i; j++) {
      const double *uj = u + n * (size_t)(j - 1);
      for (size_t k = 0; k < n; k++) X[k] += y[j - 1] * uj[k];
    }
    ls->fNorm = fabs(err[i]);
    if (ls->suc) break;
  }
  memcpy(R, X, n * sizeof(double));
  ls->dB = 10.0 * log(ls->fNorm / ls->dB);
done:
#undef H
  free(u);
  free(h);
  free(X);
  free(y);
  free(c);
  free(s);
  free(err);
}

/* FSILS_SOLVE, L/SOLVE.f:51-143 (serial: map = identity) */
int orc_solve(orc_lhs *lhs, orc_ls *ls, int dof, double *Ri, double *Val,
              int prec, const int *incL, const double *res) {
  const int nNo = lhs->nNo;
  const size_t n = (size_t)nNo * dof;
  if (lhs->nFaces) {
    for (int f = 0; f < lhs->nFaces; f++) {
      lhs->face[f].incFlag = 1;
      if (incL && incL[f] == 0) lhs->face[f].incFlag = 0;
    }
    for (int f = 0; f < lhs->nFaces; f++) {
      orc_face *fa = &lhs->face[f];
      fa->coupledFlag = 0;
      if (!fa->incFlag) continue;
      if (fa->bGrp == ORC_BC_TYPE_Neu && res && res[f] != 0.0) {
        fa->res = res[f];
        fa->coupledFlag = 1;
      }
    }
  }
  double *Wr = (double *)xcalloc(n, sizeof(double));
  double *Wc = (double *)xcalloc(n, sizeof(double));
  double *R = Ri; /* map is the identity in the serial branch */
  if (prec == ORC_PRECOND_FSILS)
    orc_precond_diag(lhs, dof, Val, R, Wc);
  else if (prec == ORC_PRECOND_RCS)
    orc_precond_rcs(lhs, dof, Val, R, Wr, Wc);
  else {
    free(Wr);
    free(Wc);
    return -3;
  }
  int rc = 0;
  switch (ls->LS_type) {
  case ORC_LS_TYPE_NS:
    orc_nssolver(lhs, ls, dof, Val, R);
    break;
  case ORC_LS_TYPE_GMRES:
    orc_gmres_v(lhs, &ls->RI, dof, Val, R);
    break;
  case ORC_LS_TYPE_CG:
    orc_cgrad_v(lhs, &ls->RI, dof, Val, R);
    break;
  case ORC_LS_TYPE_BICGS:
    orc_bicgs_v(lhs, &ls->RI, dof, Val, R);
    break;
  default:
    rc = -4;
  }
  for (size_t k = 0; k < n; k++) R[k] = Wc[k] * R[k];
  free(Wr);
  free(Wc);
  return rc;
}
