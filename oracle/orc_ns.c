/*
 * Oracle (test infrastructure only): restatement of the svFSILS NS block
 * solver (L/NSSOLVER.f:52-382, L/GE.f:51-151, L/CGRAD.f:51-123,
 * L/GMRES.f:51-169), with the coupled-Neumann terms of ADDBCMUL where the
 * reference applies them.  Serial branch: no MPI reductions.
 */
#include "orc.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static void *xcalloc(size_t n, size_t s) {
  void *p = calloc(n ? n : 1, s);
  if (!p) {
    fprintf(stderr, "oracle: out of memory\n");
    abort();
  }
  return p;
}

static const double kEps = 2.220446049250313e-16; /* EPSILON(1._LSRP) */
static const double kTiny = 2.2250738585072014e-308; /* TINY(1._LSRP) */

/* FSILS_NCDOTS, L/DOT.f:193-210 */
static double ncdots(int nNo, const double *U, const double *V) {
  double s = 0.0;
  for (int i = 0; i < nNo; i++) s += U[i] * V[i];
  return s;
}

/* FSILS_NCDOTV for dof 3, L/DOT.f:141-191: s + U1 V1 + U2 V2 + U3 V3 */
static double ncdotv(int dof, int nNo, const double *U, const double *V) {
  double s = 0.0;
  for (int i = 0; i < nNo; i++)
    for (int m = 0; m < dof; m++) s += U[(size_t)i * dof + m] * V[(size_t)i * dof + m];
  return s;
}

/* GMRES, L/GMRES.f:51-169: the variant called by NSSOLVER.  X starts at 0,
   R is not modified, itr and callD accumulate over calls (the caller resets
   them), and an initial residual at or below absTol returns X = 0. */
void orc_gmres_ns(orc_lhs *lhs, orc_subls *ls, int dof, const double *Val, const double *R,
                  double *X) {
  const int nNo = lhs->nNo, mynNo = lhs->mynNo, sD = ls->sD;
  const size_t n = (size_t)nNo * dof;
  double *u = (double *)xcalloc(n * (size_t)(sD + 1), sizeof(double));
  double *h = (double *)xcalloc((size_t)(sD + 1) * sD, sizeof(double));
#define H(j, i) h[(size_t)(i) * (sD + 1) + (j)]
  double *y = (double *)xcalloc(sD + 1, sizeof(double));
  double *c = (double *)xcalloc(sD + 1, sizeof(double));
  double *s = (double *)xcalloc(sD + 1, sizeof(double));
  double *err = (double *)xcalloc(sD + 2, sizeof(double));
  double *unc = (double *)xcalloc(n, sizeof(double));
  ls->suc = 0;
  double eps = 0.0;
  memset(X, 0, n * sizeof(double));
  for (int l = 1; l <= ls->mItr; l++) {
    if (l == 1) {
      memcpy(u, R, n * sizeof(double));
    } else {
      ls->itr++;
      orc_spar_vv(lhs, dof, Val, X, u);
      orc_addbcmul(lhs, 0, dof, X, u);
      for (size_t k = 0; k < n; k++) u[k] = R[k] - u[k];
    }
    if (orc_any_coupled(lhs)) {
      memcpy(unc, u, n * sizeof(double));
      orc_addbcmul(lhs, 1, dof, unc, u);
    }
    err[0] = orc_normv(dof, mynNo, u);
    if (l == 1) {
      eps = err[0];
      if (eps <= ls->absTol) {
        ls->callD = kEps;
        ls->dB = 0.0;
        goto done;
      }
      ls->iNorm = eps;
      ls->fNorm = eps;
      eps = fmax(ls->absTol, ls->relTol * eps);
    }
    ls->dB = ls->fNorm;
    for (size_t k = 0; k < n; k++) u[k] /= err[0];
    int i;
    for (i = 1; i <= sD; i++) {
      ls->itr++;
      double *ui = u + n * (size_t)(i - 1), *ui1 = u + n * (size_t)i;
      orc_spar_vv(lhs, dof, Val, ui, ui1);
      orc_addbcmul(lhs, 0, dof, ui, ui1);
      if (orc_any_coupled(lhs)) {
        memcpy(unc, ui1, n * sizeof(double));
        orc_addbcmul(lhs, 1, dof, unc, ui1);
      }
      for (int j = 1; j <= i + 1; j++)
        H(j - 1, i - 1) = ncdotv(dof, mynNo, u + n * (size_t)(j - 1), ui1);
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
  ls->dB = 10.0 * log(ls->fNorm / ls->dB);
done:
#undef H
  free(u);
  free(h);
  free(y);
  free(c);
  free(s);
  free(err);
  free(unc);
}

/* CGRAD_SCHUR, L/CGRAD.f:51-123: CG on S = L - D G for the pressure block;
   R in, X out (in R).  itr accumulates over calls. */
void orc_cgrad_schur(orc_lhs *lhs, orc_subls *ls, int dof, const double *D, const double *G,
                     const double *L, double *R) {
  const int nNo = lhs->nNo, mynNo = lhs->mynNo;
  double *X = (double *)xcalloc(nNo, sizeof(double));
  double *P = (double *)xcalloc(nNo, sizeof(double));
  double *SP = (double *)xcalloc(nNo, sizeof(double));
  double *DGP = (double *)xcalloc(nNo, sizeof(double));
  double *GP = (double *)xcalloc((size_t)dof * nNo, sizeof(double));
  double *unc = (double *)xcalloc((size_t)dof * nNo, sizeof(double));
  ls->suc = 0;
  ls->iNorm = sqrt(ncdots(mynNo, R, R));
  double eps = fmax(ls->absTol, ls->relTol * ls->iNorm);
  eps = eps * eps;
  double errO = ls->iNorm * ls->iNorm, err = errO;
  memcpy(P, R, sizeof(double) * nNo);
  int i;
  for (i = 1; i <= ls->mItr; i++) {
    if (err < eps) {
      ls->suc = 1;
      break;
    }
    errO = err;
    orc_spar_sv(lhs, dof, G, P, GP);
    if (orc_any_coupled(lhs)) {
      memcpy(unc, GP, sizeof(double) * (size_t)dof * nNo);
      orc_addbcmul(lhs, 1, dof, unc, GP);
    }
    orc_spar_vs(lhs, dof, D, GP, DGP);
    orc_spar_ss(lhs, L, P, SP);
    for (int k = 0; k < nNo; k++) SP[k] = SP[k] + (-1.0) * DGP[k];
    const double alpha = errO / ncdots(mynNo, P, SP);
    for (int k = 0; k < nNo; k++) X[k] = X[k] + alpha * P[k];
    for (int k = 0; k < nNo; k++) R[k] = R[k] + (-alpha) * SP[k];
    err = sqrt(ncdots(mynNo, R, R));
    err = err * err;
    for (int k = 0; k < nNo; k++) P[k] = P[k] + (errO / err) * R[k];
    for (int k = 0; k < nNo; k++) P[k] = (err / errO) * P[k];
  }
  memcpy(R, X, sizeof(double) * nNo);
  ls->fNorm = sqrt(err);
  ls->itr = ls->itr + i - 1;
  ls->dB = (errO < kEps) ? 0.0 : 5.0 * log(err / errO);
  free(X);
  free(P);
  free(SP);
  free(DGP);
  free(GP);
  free(unc);
}

/* GE, L/GE.f:51-151: symmetric diagonal scaling, then Gaussian elimination
   with partial pivoting on the leading N x N block of A (leading dimension
   nV).  Returns 1 on success, 0 when singular (B set to 0). */
int orc_ge(int nV, int N, const double *A, double *B) {
#define AA(i, j) A[(size_t)(j) * nV + (i)]
  double *W = (double *)xcalloc(N, sizeof(double));
  for (int i = 0; i < N; i++) {
    if (fabs(AA(i, i)) < kTiny) {
      for (int k = 0; k < N; k++) B[k] = 0.0;
      free(W);
      return 0;
    }
    W[i] = 1.0 / sqrt(fabs(AA(i, i)));
  }
  const int ld = N;
  double *C = (double *)xcalloc((size_t)N * (N + 1), sizeof(double));
#define CC(i, j) C[(size_t)(j) * ld + (i)]
  for (int i = 0; i < N; i++) {
    for (int j = 0; j < N; j++) CC(i, j) = W[i] * W[j] * AA(i, j);
    CC(i, N) = W[i] * B[i];
  }
  int ok = 1;
  if (N <= 0) {
    ok = 0;
  } else if (N == 1) {
    B[0] = CC(0, 1) / CC(0, 0);
    B[0] = B[0] * W[0];
  } else if (N == 2) {
    const double pivot = CC(0, 0) * CC(1, 1) - CC(1, 0) * CC(0, 1);
    if (fabs(pivot) < kEps) {
      B[0] = B[1] = 0.0;
      ok = 0;
    } else {
      B[0] = (CC(0, 2) * CC(1, 1) - CC(1, 2) * CC(0, 1)) / pivot;
      B[1] = (CC(1, 2) * CC(0, 0) - CC(0, 2) * CC(1, 0)) / pivot;
      B[0] = W[0] * B[0];
      B[1] = W[1] * B[1];
    }
  } else {
    for (int m = 0; m < N - 1 && ok; m++) {
      int ipv = m;
      double pivot = fabs(CC(m, m));
      for (int i = m + 1; i < N; i++)
        if (fabs(CC(i, m)) > pivot) {
          ipv = i;
          pivot = fabs(CC(i, m));
        }
      if (fabs(pivot) < kEps) {
        for (int k = 0; k < N; k++) B[k] = 0.0;
        ok = 0;
        break;
      }
      if (ipv != m)
        for (int j = m; j <= N; j++) {
          const double t = CC(m, j);
          CC(m, j) = CC(ipv, j);
          CC(ipv, j) = t;
        }
      for (int i = m + 1; i < N; i++) {
        const double f = CC(i, m) / CC(m, m);
        CC(i, m) = 0.0;
        for (int j = m + 1; j <= N; j++) CC(i, j) = CC(i, j) - f * CC(m, j);
      }
    }
    if (ok) {
      for (int j = N - 1; j >= 0; j--) {
        for (int i = j + 1; i < N; i++) CC(j, N) = CC(j, N) - CC(j, i) * CC(i, N);
        CC(j, N) = CC(j, N) / CC(j, j);
      }
      for (int i = 0; i < N; i++) B[i] = W[i] * CC(i, N);
    }
  }
#undef CC
#undef AA
  free(C);
  free(W);
  return ok;
}

/* DEPART, L/NSSOLVER.f:237-305 for nsd = 3: split the 4x4 blocks into
   mK(9), mG(3), mD(3), mL(1); Gt at the transposed block = -mG. */
static void depart3(const orc_lhs *lhs, const double *Val, double *mK, double *mG, double *mD,
                    double *mL, double *Gt) {
  const int nNo = lhs->nNo, nnz = lhs->nnz;
  for (int j = 0; j < nnz; j++) {
    const double *t = Val + (size_t)j * 16;
    double *k = mK + (size_t)j * 9;
    k[0] = t[0]; k[1] = t[1]; k[2] = t[2];
    k[3] = t[4]; k[4] = t[5]; k[5] = t[6];
    k[6] = t[8]; k[7] = t[9]; k[8] = t[10];
    mG[(size_t)j * 3 + 0] = t[3];
    mG[(size_t)j * 3 + 1] = t[7];
    mG[(size_t)j * 3 + 2] = t[11];
    mD[(size_t)j * 3 + 0] = t[12];
    mD[(size_t)j * 3 + 1] = t[13];
    mD[(size_t)j * 3 + 2] = t[14];
    mL[j] = t[15];
  }
  for (int i = 0; i < nNo; i++)
    for (int j = lhs->rowS[i]; j <= lhs->rowE[i]; j++) {
      const int k = lhs->colPtr[j];
      for (int l = lhs->rowS[k]; l <= lhs->rowE[k]; l++)
        if (lhs->colPtr[l] == i) {
          for (int m = 0; m < 3; m++) Gt[(size_t)l * 3 + m] = -mG[(size_t)j * 3 + m];
          break;
        }
    }
}

/* NSSOLVER, L/NSSOLVER.f:52-235 (nsd = 3, dof = 4) */
void orc_nssolver(orc_lhs *lhs, orc_ls *ls, int dof, const double *Val, double *Ri) {
  const int nNo = lhs->nNo, nnz = lhs->nnz, mynNo = lhs->mynNo;
  const int nsd = dof - 1;
  if (nsd != 3) {
    fprintf(stderr, "oracle: NS solver restated for nsd = 3 only\n");
    abort();
  }
  const int mI = ls->RI.mItr;
  const int nB = 2 * mI;
  const size_t nv = (size_t)nsd * nNo;
  double *Rm = (double *)xcalloc(nv, sizeof(double));
  double *Rc = (double *)xcalloc(nNo, sizeof(double));
  double *Rmi = (double *)xcalloc(nv, sizeof(double));
  double *Rci = (double *)xcalloc(nNo, sizeof(double));
  double *U = (double *)xcalloc(nv * mI, sizeof(double));
  double *P = (double *)xcalloc((size_t)nNo * mI, sizeof(double));
  double *MU = (double *)xcalloc(nv * nB, sizeof(double));
  double *MP = (double *)xcalloc((size_t)nNo * nB, sizeof(double));
  double *A = (double *)xcalloc((size_t)nB * nB, sizeof(double));
  double *B = (double *)xcalloc(nB, sizeof(double));
  double *xB = (double *)xcalloc(nB, sizeof(double));
  double *oldxB = (double *)xcalloc(nB, sizeof(double));
  double *tmp = (double *)xcalloc((size_t)nB * nB + nB, sizeof(double));
  double *mK = (double *)xcalloc((size_t)9 * nnz, sizeof(double));
  double *mG = (double *)xcalloc((size_t)3 * nnz, sizeof(double));
  double *mD = (double *)xcalloc((size_t)3 * nnz, sizeof(double));
  double *mL = (double *)xcalloc(nnz, sizeof(double));
  double *Gt = (double *)xcalloc((size_t)3 * nnz, sizeof(double));
#define UI(i) (U + nv * (size_t)((i) - 1))
#define PI(i) (P + (size_t)nNo * ((i) - 1))
#define MUI(i) (MU + nv * (size_t)((i) - 1))
#define MPI_(i) (MP + (size_t)nNo * ((i) - 1))
#define AM(j, k) A[(size_t)((k) - 1) * nB + ((j) - 1)]

  for (int a = 0; a < nNo; a++) {
    for (int m = 0; m < nsd; m++) Rmi[(size_t)a * nsd + m] = Ri[(size_t)a * dof + m];
    Rci[a] = Ri[(size_t)a * dof + nsd];
  }
  memcpy(Rm, Rmi, nv * sizeof(double));
  memcpy(Rc, Rci, nNo * sizeof(double));
  const double nm = orc_normv(nsd, mynNo, Rm), nc = sqrt(ncdots(mynNo, Rc, Rc));
  double eps = sqrt(nm * nm + nc * nc);
  ls->RI.iNorm = eps;
  ls->RI.fNorm = eps * eps;
  ls->CG.callD = 0.0;
  ls->GM.callD = 0.0;
  ls->CG.itr = 0;
  ls->GM.itr = 0;
  ls->RI.callD = 0.0;
  ls->RI.suc = 0;
  eps = fmax(ls->RI.absTol, ls->RI.relTol * eps);

  depart3(lhs, Val, mK, mG, mD, mL, Gt);
  orc_bcpre(lhs, nsd);

  int i, iB = 0, iBB = 0;
  for (i = 1; i <= ls->RI.mItr; i++) {
    iB = 2 * i - 1;
    iBB = 2 * i;
    ls->RI.dB = ls->RI.fNorm;

    orc_gmres_ns(lhs, &ls->GM, nsd, mK, Rm, UI(i));
    orc_spar_vs(lhs, nsd, mD, UI(i), PI(i));
    for (int a = 0; a < nNo; a++) PI(i)[a] = Rc[a] - PI(i)[a];
    orc_cgrad_schur(lhs, &ls->CG, nsd, Gt, mG, mL, PI(i));
    orc_spar_sv(lhs, nsd, mG, PI(i), MUI(iB));
    for (size_t k = 0; k < nv; k++) MUI(iBB)[k] = Rm[k] - MUI(iB)[k];
    orc_gmres_ns(lhs, &ls->GM, nsd, mK, MUI(iBB), UI(i));
    orc_spar_vv(lhs, nsd, mK, UI(i), MUI(iBB));
    orc_addbcmul(lhs, 0, nsd, UI(i), MUI(iBB));
    orc_spar_ss(lhs, mL, PI(i), MPI_(iB));
    orc_spar_vs(lhs, nsd, mD, UI(i), MPI_(iBB));

    int c = 0;
    for (int k = iB; k <= iBB; k++) {
      for (int j = 1; j <= k; j++)
        tmp[c++] = ncdotv(nsd, mynNo, MUI(j), MUI(k)) + ncdots(mynNo, MPI_(j), MPI_(k));
      tmp[c++] = ncdotv(nsd, mynNo, MUI(k), Rmi) + ncdots(mynNo, MPI_(k), Rci);
    }
    c = 0;
    for (int k = iB; k <= iBB; k++) {
      for (int j = 1; j <= k; j++) {
        AM(j, k) = tmp[c];
        AM(k, j) = tmp[c];
        c++;
      }
      B[k - 1] = tmp[c++];
    }
    memcpy(xB, B, sizeof(double) * nB);
    if (orc_ge(nB, iBB, A, xB)) {
      memcpy(oldxB, xB, sizeof(double) * nB);
    } else {
      memcpy(xB, oldxB, sizeof(double) * nB);
      if (i > 1) {
        iB -= 2;
        iBB -= 2;
      }
      break;
    }
    double sxb = 0.0;
    for (int k = 0; k < iBB; k++) sxb += xB[k] * B[k];
    ls->RI.fNorm = ls->RI.iNorm * ls->RI.iNorm - sxb;
    if (ls->RI.fNorm < eps * eps) {
      ls->RI.suc = 1;
      break;
    }
    for (size_t k = 0; k < nv; k++) Rm[k] = Rmi[k] - xB[0] * MUI(1)[k];
    for (int a = 0; a < nNo; a++) Rc[a] = Rci[a] - xB[0] * MPI_(1)[a];
    for (int j = 2; j <= iBB; j++) {
      for (size_t k = 0; k < nv; k++) Rm[k] = Rm[k] - xB[j - 1] * MUI(j)[k];
      for (int a = 0; a < nNo; a++) Rc[a] = Rc[a] - xB[j - 1] * MPI_(j)[a];
    }
  }
  if (i > ls->RI.mItr) {
    ls->RI.itr = ls->RI.mItr;
  } else {
    ls->RI.itr = i;
    for (int a = 0; a < nNo; a++) Rc[a] = Rci[a] - xB[0] * MPI_(1)[a];
    for (int j = 2; j <= iBB; j++)
      for (int a = 0; a < nNo; a++) Rc[a] = Rc[a] - xB[j - 1] * MPI_(j)[a];
  }
  {
    const double rc = sqrt(ncdots(mynNo, Rc, Rc));
    const double q = 100.0 * rc * rc / ls->RI.fNorm;
    ls->Resc = isfinite(q) && fabs(q) < 2e9 ? (int)lround(q) : -1;
    ls->Resm = 100 - ls->Resc;
  }
  for (size_t k = 0; k < nv; k++) Rmi[k] = xB[1] * UI(1)[k];
  for (int a = 0; a < nNo; a++) Rci[a] = xB[0] * PI(1)[a];
  for (int ii = 2; ii <= ls->RI.itr; ii++) {
    const int jB = 2 * ii - 1, jBB = 2 * ii;
    for (size_t k = 0; k < nv; k++) Rmi[k] = Rmi[k] + xB[jBB - 1] * UI(ii)[k];
    for (int a = 0; a < nNo; a++) Rci[a] = Rci[a] + xB[jB - 1] * PI(ii)[a];
  }
  ls->RI.dB = 5.0 * log(ls->RI.fNorm / ls->RI.dB);
  if (ls->Resc < 0 || ls->Resm < 0) {
    ls->Resc = 0;
    ls->Resm = 0;
    ls->RI.dB = 0.0;
    ls->RI.fNorm = 0.0;
  }
  ls->RI.fNorm = sqrt(ls->RI.fNorm);
  for (int a = 0; a < nNo; a++) {
    for (int m = 0; m < nsd; m++) Ri[(size_t)a * dof + m] = Rmi[(size_t)a * nsd + m];
    Ri[(size_t)a * dof + nsd] = Rci[a];
  }
#undef UI
#undef PI
#undef MUI
#undef MPI_
#undef AM
  free(Rm); free(Rc); free(Rmi); free(Rci); free(U); free(P); free(MU); free(MP);
  free(A); free(B); free(xB); free(oldxB); free(tmp);
  free(mK); free(mG); free(mD); free(mL); free(Gt);
}
