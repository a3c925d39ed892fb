/*
 * Oracle (test infrastructure only): restatement of the svFSI driver-side
 * hot path -- sparsity (LHSA), element assembly (HEATS3D, STRUCT3D with the
 * neo-Hookean + ST91 material), scatter (DOASSEM), traction loads, and the
 * generalized-alpha predictor / initiator / corrector with the Newton loop.
 * F/ = Code/Source/svFSI in the svFSI project.  All arithmetic is FP64.
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

/* ---------------------------------------------------------------------- */
/* LHSA + ADDCOL, F/LHSA.f:38-241: per row a sorted list of unique columns */
typedef struct {
  int n, cap;
  int *c;
} rowlist;

static void addcol(rowlist *r, int col) {
  int i = 0;
  while (i < r->n && r->c[i] < col) i++;
  if (i < r->n && r->c[i] == col) return;
  if (r->n == r->cap) {
    r->cap = r->cap ? r->cap + (r->cap / 5 > 5 ? r->cap / 5 : 5) : 40;
    r->c = (int *)realloc(r->c, sizeof(int) * (size_t)r->cap);
  }
  memmove(r->c + i + 1, r->c + i, sizeof(int) * (size_t)(r->n - i));
  r->c[i] = col;
  r->n++;
}

static rowlist *lhsa_rows(int nNo, int nEl, int eNoN, const int *IEN) {
  rowlist *rows = (rowlist *)xcalloc(nNo, sizeof(rowlist));
  for (int e = 0; e < nEl; e++)
    for (int a = 0; a < eNoN; a++) {
      const int rowN = IEN[(size_t)e * eNoN + a];
      for (int b = 0; b < eNoN; b++) addcol(&rows[rowN], IEN[(size_t)e * eNoN + b]);
    }
  return rows;
}

int orc_lhsa_count(int nNo, int nEl, int eNoN, const int *IEN) {
  rowlist *rows = lhsa_rows(nNo, nEl, eNoN, IEN);
  long long nnz = 0;
  for (int i = 0; i < nNo; i++) {
    nnz += rows[i].n;
    free(rows[i].c);
  }
  free(rows);
  return (int)nnz;
}

int orc_lhsa(int nNo, int nEl, int eNoN, const int *IEN, int *rowPtr,
             int *colPtr, int nnzCap) {
  rowlist *rows = lhsa_rows(nNo, nEl, eNoN, IEN);
  int j = 0, rc = 0;
  rowPtr[0] = 0;
  for (int i = 0; i < nNo; i++) {
    if (rows[i].n == 0) rc = -1; /* "Node is isolated" */
    for (int k = 0; k < rows[i].n; k++) {
      if (j < nnzCap) colPtr[j] = rows[i].c[k];
      j++;
    }
    rowPtr[i + 1] = j;
    free(rows[i].c);
  }
  free(rows);
  if (j > nnzCap) return -2;
  return rc ? rc : j;
}

/* DOASSEM, F/LHSA.f:266-298: bisection for the column inside the row. */
void orc_doassem(int dof, int eNoN, const int *ptr, const double *lK,
                 const double *lR, const int *rowPtr, const int *colPtr,
                 double *R, double *Val) {
  const int dd = dof * dof;
  for (int a = 0; a < eNoN; a++) {
    const int rowN = ptr[a];
    for (int k = 0; k < dof; k++) R[(size_t)rowN * dof + k] += lR[a * dof + k];
    for (int b = 0; b < eNoN; b++) {
      const int colN = ptr[b];
      /* the Fortran bisection runs on 1-based [left,right]; same search in
         0-based form: left = rowPtr(rowN), right = rowPtr(rowN+1) */
      int left = rowPtr[rowN] + 1, right = rowPtr[rowN + 1] + 1;
      int p = (right + left) / 2;
      while (colN != colPtr[p - 1]) {
        if (colN > colPtr[p - 1])
          left = p;
        else
          right = p;
        p = (right + left) / 2;
      }
      for (int k = 0; k < dd; k++)
        Val[(size_t)(p - 1) * dd + k] += lK[(size_t)(a * eNoN + b) * dd + k];
    }
  }
}

/* ---------------------------------------------------------------------- */
/* tet4 quadrature and shape functions, F/NN.f:268-275 and F/NN.f:654-671 */
static void tet4_gauss(double w[4], double N[4][4]) {
  const double s = (5.0 + 3.0 * sqrt(5.0)) / 20.0;
  const double t = (5.0 - sqrt(5.0)) / 20.0;
  const double xi[4][3] = {{s, t, t}, {t, s, t}, {t, t, s}, {t, t, t}};
  for (int g = 0; g < 4; g++) {
    w[g] = 1.0 / 24.0;
    N[g][0] = xi[g][0];
    N[g][1] = xi[g][1];
    N[g][2] = xi[g][2];
    N[g][3] = 1.0 - xi[g][0] - xi[g][1] - xi[g][2];
  }
}
static const double TET4_NXI[3][4] = {{1, 0, 0, -1}, {0, 1, 0, -1}, {0, 0, 1, -1}};

/* GNN (insd = 3), F/NN.f:1469-1565 */
static void gnn3(const double xl[12], double Nx[3][4], double *Jac) {
  double xXi[3][3] = {{0}}, xiX[3][3];
  for (int a = 0; a < 4; a++)
    for (int i = 0; i < 3; i++)
      for (int k = 0; k < 3; k++) xXi[i][k] += xl[a * 3 + i] * TET4_NXI[k][a];
  const double J = xXi[0][0] * xXi[1][1] * xXi[2][2] + xXi[0][1] * xXi[1][2] * xXi[2][0] +
                   xXi[0][2] * xXi[1][0] * xXi[2][1] - xXi[0][0] * xXi[1][2] * xXi[2][1] -
                   xXi[0][1] * xXi[1][0] * xXi[2][2] - xXi[0][2] * xXi[1][1] * xXi[2][0];
  xiX[0][0] = (xXi[1][1] * xXi[2][2] - xXi[1][2] * xXi[2][1]) / J;
  xiX[0][1] = (xXi[2][1] * xXi[0][2] - xXi[2][2] * xXi[0][1]) / J;
  xiX[0][2] = (xXi[0][1] * xXi[1][2] - xXi[0][2] * xXi[1][1]) / J;
  xiX[1][0] = (xXi[1][2] * xXi[2][0] - xXi[1][0] * xXi[2][2]) / J;
  xiX[1][1] = (xXi[2][2] * xXi[0][0] - xXi[2][0] * xXi[0][2]) / J;
  xiX[1][2] = (xXi[0][2] * xXi[1][0] - xXi[0][0] * xXi[1][2]) / J;
  xiX[2][0] = (xXi[1][0] * xXi[2][1] - xXi[1][1] * xXi[2][0]) / J;
  xiX[2][1] = (xXi[2][0] * xXi[0][1] - xXi[2][1] * xXi[0][0]) / J;
  xiX[2][2] = (xXi[0][0] * xXi[1][1] - xXi[0][1] * xXi[1][0]) / J;
  for (int a = 0; a < 4; a++)
    for (int i = 0; i < 3; i++)
      Nx[i][a] = 0.0 + TET4_NXI[0][a] * xiX[0][i] + TET4_NXI[1][a] * xiX[1][i] +
                 TET4_NXI[2][a] * xiX[2][i];
  *Jac = J;
}

/* GNN (insd = 3) with the metric ks = xiX^T xiX, F/NN.f:1527-1545 */
static void gnn3k(const double xl[12], double Nx[3][4], double *Jac, double ks[3][3]) {
  double xXi[3][3] = {{0}}, xiX[3][3];
  for (int a = 0; a < 4; a++)
    for (int i = 0; i < 3; i++)
      for (int k = 0; k < 3; k++) xXi[i][k] += xl[a * 3 + i] * TET4_NXI[k][a];
  const double J = xXi[0][0] * xXi[1][1] * xXi[2][2] + xXi[0][1] * xXi[1][2] * xXi[2][0] +
                   xXi[0][2] * xXi[1][0] * xXi[2][1] - xXi[0][0] * xXi[1][2] * xXi[2][1] -
                   xXi[0][1] * xXi[1][0] * xXi[2][2] - xXi[0][2] * xXi[1][1] * xXi[2][0];
  xiX[0][0] = (xXi[1][1] * xXi[2][2] - xXi[1][2] * xXi[2][1]) / J;
  xiX[0][1] = (xXi[2][1] * xXi[0][2] - xXi[2][2] * xXi[0][1]) / J;
  xiX[0][2] = (xXi[0][1] * xXi[1][2] - xXi[0][2] * xXi[1][1]) / J;
  xiX[1][0] = (xXi[1][2] * xXi[2][0] - xXi[1][0] * xXi[2][2]) / J;
  xiX[1][1] = (xXi[2][2] * xXi[0][0] - xXi[2][0] * xXi[0][2]) / J;
  xiX[1][2] = (xXi[0][2] * xXi[1][0] - xXi[0][0] * xXi[1][2]) / J;
  xiX[2][0] = (xXi[1][0] * xXi[2][1] - xXi[1][1] * xXi[2][0]) / J;
  xiX[2][1] = (xXi[2][0] * xXi[0][1] - xXi[2][1] * xXi[0][0]) / J;
  xiX[2][2] = (xXi[0][0] * xXi[1][1] - xXi[0][1] * xXi[1][0]) / J;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      ks[i][j] = xiX[0][i] * xiX[0][j] + xiX[1][i] * xiX[1][j] + xiX[2][i] * xiX[2][j];
  for (int a = 0; a < 4; a++)
    for (int i = 0; i < 3; i++)
      Nx[i][a] = 0.0 + TET4_NXI[0][a] * xiX[0][i] + TET4_NXI[1][a] * xiX[1][i] +
                 TET4_NXI[2][a] * xiX[2][i];
  *Jac = J;
}

/* ISZERO, F/MATFUN.f:763-780: |a| / max(|a|, eps) < eps */
static int iszero(double v) {
  const double e = 2.220446049250313e-16;
  const double a = fabs(v);
  return a / fmax(a, e) < e;
}

/* CONSTRUCT_FLUID with FLUID3D_M and FLUID3D_C, F/FLUID.f:40-190,
   :192-560, :813-1084, for one P1-P1 tet4 element with VMS stabilisation
   (GETTHOODFS gives both passes the element's own basis and 4-point rule,
   F/FS.f:270-286) and constant viscosity (GETVISCOSITY, F/FLUID.f:1705-1708:
   mu_g = 0).  For tet4 the second derivatives Nwxx vanish (affine map), so
   uxx, d2u2, es_x, mu_x and rS are identically zero and are left out; no
   mesh motion.  al, yl: tDof x 4 (u, v, w, p first); lR[a*4+i]; lK[(a*4+b)*16
   + r*4 + c] with the reference's lK(k,a,b), k = r*4 + c + 1. */
/* GETVISCOSITY, F/FLUID.f:1690-1739: mu, mu_s and mu_x = d mu / d gamma
   at shear rate gam; the Casson model raises gam to its threshold lam. */
static void orc_getviscosity(const orc_eqp *p, double *gam, double *mu, double *mu_s,
                             double *mu_x) {
  if (p->viscType == 1) {
    const double mu_i = p->mu_f, mu_o = p->mu_o, lam = p->vlam, a = p->va, n = p->vn;
    double T1 = 1.0 + pow(lam * (*gam), a);
    double T2 = pow(T1, (n - 1.0) / a);
    *mu = mu_i + (mu_o - mu_i) * T2;
    *mu_s = mu_i;
    T1 = T2 / T1;
    T2 = pow(lam, a) * pow(*gam, a - 1.0) * T1;
    *mu_x = (mu_o - mu_i) * (n - 1.0) * T2;
  } else if (p->viscType == 2) {
    const double mu_i = p->mu_f, lam = p->vlam;
    double mu_o = p->mu_o;
    if (*gam < lam) {
      mu_o = mu_o / sqrt(lam);
      *gam = lam;
    } else {
      mu_o = mu_o / sqrt(*gam);
    }
    *mu = (mu_i + mu_o) * (mu_i + mu_o);
    *mu_s = mu_i * mu_i;
    *mu_x = 2.0 * mu_o * (mu_o + mu_i) / (*gam);
  } else {
    *mu = p->mu_f;
    *mu_s = *mu;
    *mu_x = 0.0;
  }
}

void orc_elem_fluid(const orc_eqp *p, const double xl[12], const double *al,
                    const double *yl, double lR[16], double lK[256]) {
  double w4[4], N4[4][4], Nx[3][4], Jac, Kxi[3][3];
  tet4_gauss(w4, N4);
  gnn3k(xl, Nx, &Jac, Kxi);
  for (int k = 0; k < 16; k++) lR[k] = 0.0;
  for (int k = 0; k < 256; k++) lK[k] = 0.0;
  const int tD = p->tDof;
  const double ctM = p->ctM, ctC = p->ctC;
  const double rho = p->rho;
  const double f[3] = {p->fb[0], p->fb[1], p->fb[2]};
  const double T1c = p->af * p->gam * p->dt;
  const double amd = p->am / T1c;
  const double eps = 2.220446049250313e-16;
#define LK(k, a, b) lK[((a) * 4 + (b)) * 16 + (k) - 1]
  /* pass 1: momentum (FLUID3D_M); pass 2: continuity (FLUID3D_C) -- both over
     the same four Gauss points; they write disjoint lR/lK entries. */
  for (int pass = 0; pass < 2; pass++)
    for (int g = 0; g < 4; g++) {
      const double w = w4[g] * Jac;
      const double *N = N4[g];
      const double wl = w * T1c, wr = w * rho;
      double ud[3] = {-f[0], -f[1], -f[2]}, u[3] = {0, 0, 0}, ux[3][3] = {{0}};
      for (int a = 0; a < 4; a++) {
        for (int i = 0; i < 3; i++) {
          ud[i] = ud[i] + N[a] * (al[a * tD + i] - 0.0);
          u[i] = u[i] + N[a] * yl[a * tD + i];
        }
        for (int j = 0; j < 3; j++)
          for (int i = 0; i < 3; i++) ux[i][j] = ux[i][j] + Nx[i][a] * yl[a * tD + j];
      }
      const double divU = ux[0][0] + ux[1][1] + ux[2][2];
      double pr = 0.0, px[3] = {0, 0, 0};
      for (int a = 0; a < 4; a++) {
        pr = pr + N[a] * yl[a * tD + 3];
        for (int i = 0; i < 3; i++) px[i] = px[i] + Nx[i][a] * yl[a * tD + 3];
      }
      double es[3][3];
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) es[i][j] = ux[i][j] + ux[j][i];
      double esNx[3][4];
      for (int a = 0; a < 4; a++)
        for (int i = 0; i < 3; i++)
          esNx[i][a] = es[0][i] * Nx[0][a] + es[1][i] * Nx[1][a] + es[2][i] * Nx[2][a];
      /* shear rate (2 e_ij e_ij)^(1/2) and the viscosity model, F/FLUID.f:358-373;
         mu_x(:) = mu_g es_x . es vanishes for tet4 (no second derivatives) */
      double gam = 0.0;
      for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) gam = gam + es[i][j] * es[i][j];
      gam = sqrt(0.5 * gam);
      double mu, mu_s, mu_g;
      orc_getviscosity(p, &gam, &mu, &mu_s, &mu_g);
      (void)mu_s;
      if (iszero(gam))
        mu_g = 0.0;
      else
        mu_g = mu_g / gam;
      const double kT = 4.0 * pow(ctM / p->dt, 2.0);
      double kU = 0.0, kS = 0.0;
      for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) {
          kU = kU + u[i] * u[j] * Kxi[i][j];
          kS = kS + Kxi[i][j] * Kxi[i][j];
        }
      kS = ctC * kS * pow(mu / rho, 2.0);
      const double tauM = 1.0 / (rho * sqrt(kT + kU + kS));
      double rV[3], up[3];
      for (int j = 0; j < 3; j++) rV[j] = ud[j] + u[0] * ux[0][j] + u[1] * ux[1][j] + u[2] * ux[2][j];
      for (int j = 0; j < 3; j++) up[j] = -tauM * (rho * rV[j] + px[j] - 0.0);
      if (pass == 0) {
        const double tauC = 1.0 / (tauM * (Kxi[0][0] + Kxi[1][1] + Kxi[2][2]));
        double tauB = 0.0;
        for (int j = 0; j < 3; j++)
          for (int i = 0; i < 3; i++) tauB = tauB + up[i] * up[j] * Kxi[i][j];
        if (iszero(tauB)) tauB = eps;
        tauB = rho / sqrt(tauB);
        double ua[3];
        for (int i = 0; i < 3; i++) ua[i] = u[i] + up[i];
        const double pa = pr - tauC * divU;
        double rM[3][3];
        for (int j = 0; j < 3; j++)
          rV[j] = tauB * (up[0] * ux[0][j] + up[1] * ux[1][j] + up[2] * ux[2][j]);
        for (int j = 0; j < 3; j++)
          for (int i = 0; i < 3; i++)
            rM[i][j] = mu * es[i][j] - rho * up[j] * ua[i] + rV[j] * up[i] - (i == j ? pa : 0.0);
        for (int j = 0; j < 3; j++)
          rV[j] = ud[j] + ua[0] * ux[0][j] + ua[1] * ux[1][j] + ua[2] * ux[2][j];
        double uNx[4], upNx[4], uaNx[4];
        for (int a = 0; a < 4; a++) {
          for (int j = 0; j < 3; j++)
            lR[a * 4 + j] = lR[a * 4 + j] + wr * N[a] * rV[j] +
                            w * (Nx[0][a] * rM[0][j] + Nx[1][a] * rM[1][j] + Nx[2][a] * rM[2][j]);
          uNx[a] = u[0] * Nx[0][a] + u[1] * Nx[1][a] + u[2] * Nx[2][a];
          upNx[a] = up[0] * Nx[0][a] + up[1] * Nx[1][a] + up[2] * Nx[2][a];
          uaNx[a] = uNx[a] + upNx[a];
        }
        /* updu(i,j,b) = delta_ij (-rho uNx(b)) when Nwxx = mu_x = 0 */
        for (int b = 0; b < 4; b++)
          for (int a = 0; a < 4; a++) {
            double NN[3][3];
            for (int i = 0; i < 3; i++)
              for (int j = 0; j < 3; j++) NN[i][j] = Nx[i][a] * Nx[j][b];
            const double NxNx = Nx[0][a] * Nx[0][b] + Nx[1][a] * Nx[1][b] + Nx[2][a] * Nx[2][b];
            const double T1 = mu * NxNx + rho * amd * N[b] * (N[a] + rho * tauM * uaNx[a]) +
                              rho * N[a] * (uNx[b] + upNx[b]) + tauB * upNx[a] * upNx[b];
            const double upd = -rho * uNx[b];
            /* row i (momentum component), column j (velocity component) */
            for (int i = 0; i < 3; i++)
              for (int j = 0; j < 3; j++) {
                double T2 = (i == j ? (mu + tauC) * NN[i][i] : mu * NN[j][i] + tauC * NN[i][j]) +
                            esNx[i][a] * mu_g * esNx[j][b] -
                            rho * tauM * uaNx[a] * (i == j ? upd : 0.0);
                LK(i * 4 + j + 1, a, b) += wl * (i == j ? T2 + T1 : T2);
              }
          }
        for (int b = 0; b < 4; b++)
          for (int a = 0; a < 4; a++) {
            const double T1 = rho * tauM * uaNx[a];
            for (int i = 0; i < 3; i++)
              LK(i * 4 + 4, a, b) -= wl * (Nx[i][a] * N[b] - Nx[i][b] * T1);
          }
      } else {
        for (int a = 0; a < 4; a++) {
          const double upNx = up[0] * Nx[0][a] + up[1] * Nx[1][a] + up[2] * Nx[2][a];
          lR[a * 4 + 3] = lR[a * 4 + 3] + w * (N[a] * divU - upNx);
        }
        for (int b = 0; b < 4; b++) {
          const double T1 = rho * amd * N[b];
          const double uNxb = u[0] * Nx[0][b] + u[1] * Nx[1][b] + u[2] * Nx[2][b];
          const double upd = -rho * uNxb; /* updu(j,j,b) */
          for (int a = 0; a < 4; a++)
            for (int j = 0; j < 3; j++) {
              /* T2 = sum_i Nqx(i,a) updu(j,i,b) - Nqx(j,a) T1 */
              const double T2 = Nx[j][a] * (upd - T1);
              LK(13 + j, a, b) += wl * (N[a] * Nx[j][b] - tauM * T2);
            }
        }
        for (int b = 0; b < 4; b++)
          for (int a = 0; a < 4; a++) {
            const double NxNx = Nx[0][a] * Nx[0][b] + Nx[1][a] * Nx[1][b] + Nx[2][a] * Nx[2][b];
            LK(16, a, b) += wl * tauM * NxNx;
          }
      }
    }
#undef LK
}

/* ---------------------------------------------------------------------- */
/* CONSTRUCT_HEATS / HEATS3D, F/HEATS.f:39-159 for one tet4 element.
   al, yl: tDof x 4 local copies; uses component p->s. */
void orc_elem_heats(const orc_eqp *p, const double xl[12], const double *al,
                    const double *yl, double lR[4], double lK[16]) {
  double w4[4], N4[4][4], Nx[3][4], Jac;
  tet4_gauss(w4, N4);
  gnn3(xl, Nx, &Jac);
  for (int a = 0; a < 4; a++) lR[a] = 0.0;
  for (int k = 0; k < 16; k++) lK[k] = 0.0;
  const double nu = p->cond, s = p->src, rho = p->rho;
  const double T1 = p->af * p->gam * p->dt;
  const double amd = p->am * rho / T1;
  const int i = p->s, tD = p->tDof;
  for (int g = 0; g < 4; g++) {
    const double w = w4[g] * Jac;
    const double *N = N4[g];
    const double wl = w * T1;
    double Td = -s, Tx[3] = {0, 0, 0};
    for (int a = 0; a < 4; a++) {
      Td = Td + N[a] * al[a * tD + i];
      Tx[0] = Tx[0] + Nx[0][a] * yl[a * tD + i];
      Tx[1] = Tx[1] + Nx[1][a] * yl[a * tD + i];
      Tx[2] = Tx[2] + Nx[2][a] * yl[a * tD + i];
    }
    Td = Td * rho;
    for (int a = 0; a < 4; a++) {
      lR[a] = lR[a] + w * (N[a] * Td + (Nx[0][a] * Tx[0] + Nx[1][a] * Tx[1] + Nx[2][a] * Tx[2]) * nu);
      for (int b = 0; b < 4; b++)
        lK[a * 4 + b] = lK[a * 4 + b] +
                        wl * (N[a] * N[b] * amd +
                              nu * (Nx[0][a] * Nx[0][b] + Nx[1][a] * Nx[1][b] + Nx[2][a] * Nx[2][b]));
    }
  }
}

/* LELAS3D, F/LELAS.f:130-238, one tet4 element, per Gauss point as the
   reference: lambda = E nu/(1+nu)/(1-2nu), mu = E/2/(1+nu), lDm = lambda/mu,
   T1 = af beta dt^2, amd = am/T1 rho, wl = w T1 mu; ud = -f + sum N al,
   ed = symmetric gradient of dl (Voigt, engineering shear), S = lambda tr I
   + 2 mu eps (pS0 = 0, Bf = 0); lR(:,a) += w (rho N_a ud + Nx_a . S);
   lK(rc,a,b) += wl (d_rc (amd N_a N_b / mu + Nx_a.Nx_b) + lDm Nx(r,a) Nx(c,b)
   + Nx(c,a) Nx(r,b)). */
void orc_elem_lelas(const orc_eqp *p, const double xl[12], const double *al,
                    const double *dl, double lR[12], double lK[144]) {
  double w4[4], N4[4][4], Nx[3][4], Jac;
  tet4_gauss(w4, N4);
  gnn3(xl, Nx, &Jac);
  for (int k = 0; k < 12; k++) lR[k] = 0.0;
  for (int k = 0; k < 144; k++) lK[k] = 0.0;
  const int dof = 3, tD = p->tDof;
  const int i = p->s, j = i + 1, k = j + 1;
  const double rho = p->rho, elM = p->elM, nu = p->nu;
  const double lambda = elM * nu / (1.0 + nu) / (1.0 - 2.0 * nu);
  const double mu = elM * 0.5 / (1.0 + nu);
  const double lDm = lambda / mu;
  const double T1 = p->af * p->beta * p->dt * p->dt;
  const double amd = p->am / T1 * rho;
  for (int g = 0; g < 4; g++) {
    const double w = w4[g] * Jac;
    const double *N = N4[g];
    const double wl = w * T1 * mu;
    double ed[6] = {0, 0, 0, 0, 0, 0};
    double ud[3] = {-p->fb[0], -p->fb[1], -p->fb[2]};
    for (int a = 0; a < 4; a++) {
      ud[0] = ud[0] + N[a] * al[a * tD + i];
      ud[1] = ud[1] + N[a] * al[a * tD + j];
      ud[2] = ud[2] + N[a] * al[a * tD + k];
      ed[0] = ed[0] + Nx[0][a] * dl[a * tD + i];
      ed[1] = ed[1] + Nx[1][a] * dl[a * tD + j];
      ed[2] = ed[2] + Nx[2][a] * dl[a * tD + k];
      ed[3] = ed[3] + Nx[1][a] * dl[a * tD + i] + Nx[0][a] * dl[a * tD + j];
      ed[4] = ed[4] + Nx[2][a] * dl[a * tD + j] + Nx[1][a] * dl[a * tD + k];
      ed[5] = ed[5] + Nx[0][a] * dl[a * tD + k] + Nx[2][a] * dl[a * tD + i];
    }
    const double divD = lambda * (ed[0] + ed[1] + ed[2]);
    double S[6];
    S[0] = divD + 2.0 * mu * ed[0];
    S[1] = divD + 2.0 * mu * ed[1];
    S[2] = divD + 2.0 * mu * ed[2];
    S[3] = mu * ed[3];
    S[4] = mu * ed[4];
    S[5] = mu * ed[5];
    for (int a = 0; a < 4; a++) {
      lR[a * dof + 0] += w * (rho * N[a] * ud[0] + Nx[0][a] * S[0] + Nx[1][a] * S[3] + Nx[2][a] * S[5]);
      lR[a * dof + 1] += w * (rho * N[a] * ud[1] + Nx[0][a] * S[3] + Nx[1][a] * S[1] + Nx[2][a] * S[4]);
      lR[a * dof + 2] += w * (rho * N[a] * ud[2] + Nx[0][a] * S[5] + Nx[1][a] * S[4] + Nx[2][a] * S[2]);
      for (int b = 0; b < 4; b++) {
        const double NxdNx = Nx[0][a] * Nx[0][b] + Nx[1][a] * Nx[1][b] + Nx[2][a] * Nx[2][b];
        const double T = amd * N[a] * N[b] / mu + NxdNx;
        double *K = lK + (size_t)(a * 4 + b) * 9;
        for (int r = 0; r < 3; r++)
          for (int c = 0; c < 3; c++) {
            double v = lDm * Nx[r][a] * Nx[c][b] + Nx[c][a] * Nx[r][b];
            if (r == c) v = T + (1.0 + lDm) * Nx[r][a] * Nx[r][b];
            K[r * 3 + c] += wl * v;
          }
      }
    }
  }
}

/* HEATF3D, F/HEATF.f:116-205 (no mesh motion), one tet4 element per
   Gauss point as the reference: advection-diffusion of component s with the
   velocity in components 0..2 of the state, SUPG-type stabilisation tauM =
   ct4/sqrt(ct1/dt^2 + ct2 u.ks.u + ct3 nu^2 ks:ks), ct = (4, 1, 3, 1), and
   the discontinuity-capturing diffusivity nu + |Td + u.Tx| / (2 sqrt(Tx.ks.Tx))
   (ISZERO(Tx.ks.Tx) -> eps).  lR(1,4), lK(1,4,4). */
void orc_elem_heatf(const orc_eqp *p, const double xl[12], const double *al,
                    const double *yl, double lR[4], double lK[16]) {
  static const double ct[4] = {4.0, 1.0, 3.0, 1.0};
  const double eps = 2.220446049250313e-16;
  double w4[4], N4[4][4], Nx[3][4], Jac, ks[3][3];
  tet4_gauss(w4, N4);
  gnn3k(xl, Nx, &Jac, ks);
  for (int a = 0; a < 4; a++) lR[a] = 0.0;
  for (int k = 0; k < 16; k++) lK[k] = 0.0;
  const int i = p->s, tD = p->tDof;
  const double dt = p->dt;
  const double T1 = p->af * p->gam * dt;
  const double amd = p->am / T1;
  const double s = p->src;
  for (int g = 0; g < 4; g++) {
    const double w = w4[g] * Jac;
    const double *N = N4[g];
    const double wl = w * T1;
    double nu = p->cond;
    double u[3] = {0, 0, 0}, Tx[3] = {0, 0, 0}, Td = -s;
    for (int a = 0; a < 4; a++) {
      u[0] = u[0] + N[a] * yl[a * tD + 0];
      u[1] = u[1] + N[a] * yl[a * tD + 1];
      u[2] = u[2] + N[a] * yl[a * tD + 2];
      Td = Td + N[a] * al[a * tD + i];
      Tx[0] = Tx[0] + Nx[0][a] * yl[a * tD + i];
      Tx[1] = Tx[1] + Nx[1][a] * yl[a * tD + i];
      Tx[2] = Tx[2] + Nx[2][a] * yl[a * tD + i];
    }
    const double kU = u[0] * u[0] * ks[0][0] + u[1] * u[0] * ks[1][0] + u[2] * u[0] * ks[2][0] +
                      u[0] * u[1] * ks[0][1] + u[1] * u[1] * ks[1][1] + u[2] * u[1] * ks[2][1] +
                      u[0] * u[2] * ks[0][2] + u[1] * u[2] * ks[1][2] + u[2] * u[2] * ks[2][2];
    const double kS = ks[0][0] * ks[0][0] + ks[1][0] * ks[1][0] + ks[2][0] * ks[2][0] +
                      ks[0][1] * ks[0][1] + ks[1][1] * ks[1][1] + ks[2][1] * ks[2][1] +
                      ks[0][2] * ks[0][2] + ks[1][2] * ks[1][2] + ks[2][2] * ks[2][2];
    double nTx = ks[0][0] * Tx[0] * Tx[0] + ks[1][1] * Tx[1] * Tx[1] + ks[2][2] * Tx[2] * Tx[2] +
                 (ks[0][1] + ks[1][0]) * Tx[0] * Tx[1] + (ks[0][2] + ks[2][0]) * Tx[0] * Tx[2] +
                 (ks[1][2] + ks[2][1]) * Tx[1] * Tx[2];
    if (iszero(nTx)) nTx = eps;
    const double udTx = u[0] * Tx[0] + u[1] * Tx[1] + u[2] * Tx[2];
    double Tp = fabs(Td + udTx);
    nu = nu + 0.5 * Tp / sqrt(nTx);
    const double tauM = ct[3] / sqrt((ct[0] / (dt * dt)) + ct[1] * kU + ct[2] * nu * nu * kS);
    Tp = -tauM * (Td + udTx);
    double udNx[4];
    for (int a = 0; a < 4; a++) udNx[a] = u[0] * Nx[0][a] + u[1] * Nx[1][a] + u[2] * Nx[2][a];
    for (int a = 0; a < 4; a++) {
      lR[a] = lR[a] + w * (N[a] * (Td + udTx) +
                           (Nx[0][a] * Tx[0] + Nx[1][a] * Tx[1] + Nx[2][a] * Tx[2]) * nu -
                           udNx[a] * Tp);
      for (int b = 0; b < 4; b++)
        lK[a * 4 + b] = lK[a * 4 + b] +
                        wl * (nu * (Nx[0][a] * Nx[0][b] + Nx[1][a] * Nx[1][b] + Nx[2][a] * Nx[2][b]) +
                              (N[a] + tauM * udNx[a]) * (N[b] * amd + udNx[b]));
    }
  }
}

/* CEP3D, F/CEP.f:136-266 without electromechanical coupling (ecCpld
   false: fl = fN, F/CEP.f:213-218), one tet4 element.  The diffusion
   tensor D = Diso I plus Dani(i) fl(:,i) fl(:,i)^T per fibre
   (F/CEP.f:221-233); fN_e NULL or p->nFn = 0: isotropic. */
void orc_elem_cep(const orc_eqp *p, double Diso, const double *fN_e, const double xl[12],
                  const double *al, const double *yl, double lR[4], double lK[16]) {
  double w4[4], N4[4][4], Nx[3][4], Jac;
  tet4_gauss(w4, N4);
  gnn3(xl, Nx, &Jac);
  for (int a = 0; a < 4; a++) lR[a] = 0.0;
  for (int k = 0; k < 16; k++) lK[k] = 0.0;
  const double T1 = p->af * p->gam * p->dt;
  const double amd = p->am / T1;
  const int i = p->s, tD = p->tDof;
  double D[3][3] = {{Diso, 0, 0}, {0, Diso, 0}, {0, 0, Diso}};
  if (fN_e)
    for (int f = 0; f < p->nFn; f++) {
      const double *fl = fN_e + 3 * f;
      for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) D[r][c] = D[r][c] + p->Dani[f] * fl[r] * fl[c];
    }
  for (int g = 0; g < 4; g++) {
    const double w = w4[g] * Jac, wl = w * T1;
    const double *N = N4[g];
    double Vd = 0.0, Vx[3] = {0, 0, 0}, DNx[3][4];
    for (int a = 0; a < 4; a++) {
      Vd = Vd + N[a] * al[a * tD + i];
      for (int k = 0; k < 3; k++) Vx[k] = Vx[k] + Nx[k][a] * yl[a * tD + i];
      for (int k = 0; k < 3; k++) DNx[k][a] = D[k][0] * Nx[0][a] + D[k][1] * Nx[1][a] + D[k][2] * Nx[2][a];
    }
    double DVx[3];
    for (int k = 0; k < 3; k++) DVx[k] = D[k][0] * Vx[0] + D[k][1] * Vx[1] + D[k][2] * Vx[2];
    for (int a = 0; a < 4; a++) {
      lR[a] = lR[a] + w * (N[a] * Vd + Nx[0][a] * DVx[0] + Nx[1][a] * DVx[1] + Nx[2][a] * DVx[2]);
      for (int b = 0; b < 4; b++)
        lK[a * 4 + b] = lK[a * 4 + b] +
                        wl * (N[a] * N[b] * amd + Nx[0][a] * DNx[0][b] + Nx[1][a] * DNx[1][b] +
                              Nx[2][a] * DNx[2][b]);
    }
  }
}

/* ---------------------------------------------------------------------- */
/* Aliev-Panfilov: parameters F/PARAMS_AP.f:53-86, AP_GETF
   F/CEPMOD_AP.f:255-267, AP_INTEGFE/AP_INTEGRK F/CEPMOD_AP.f:125-184 */
static const double AP_Vscale = 100.0, AP_Tscale = 12.9, AP_Voffset = -80.0;
static const double AP_alpha = 1e-2, AP_a = 2e-3, AP_b = 0.15, AP_c = 8.0;
static const double AP_mu1 = 0.2, AP_mu2 = 0.3, AP_Vrest = -80.0;

void orc_ap_getf(const double X[2], double f[2], double fext) {
  f[0] = X[0] * (AP_c * (X[0] - AP_alpha) * (1.0 - X[0]) - X[1]) + fext;
  f[1] = (AP_a + AP_mu1 * X[1] / (AP_mu2 + X[0])) * (-X[1] - AP_c * X[0] * (X[0] - AP_b - 1.0));
}

void orc_ap_step(double X[2], double Ts, double Ti, double Istim, double Ksac, int rk4) {
  const double dt = Ti / AP_Tscale;
  const double Isac = Ksac * (AP_Vrest - X[0]);
  const double fext = (Istim + Isac) * AP_Tscale / AP_Vscale;
  (void)Ts;
  X[0] = (X[0] - AP_Voffset) / AP_Vscale;
  if (!rk4) {
    double f[2];
    orc_ap_getf(X, f, fext);
    X[0] = X[0] + dt * f[0];
    X[1] = X[1] + dt * f[1];
  } else {
    const double dt6 = dt / 6.0;
    double Xr[2], f1[2], f2[2], f3[2], f4[2];
    Xr[0] = X[0];
    Xr[1] = X[1];
    orc_ap_getf(Xr, f1, fext);
    for (int k = 0; k < 2; k++) Xr[k] = X[k] + 0.5 * dt * f1[k];
    orc_ap_getf(Xr, f2, fext);
    for (int k = 0; k < 2; k++) Xr[k] = X[k] + 0.5 * dt * f2[k];
    orc_ap_getf(Xr, f3, fext);
    for (int k = 0; k < 2; k++) Xr[k] = X[k] + dt * f3[k];
    orc_ap_getf(Xr, f4, fext);
    for (int k = 0; k < 2; k++) X[k] = X[k] + dt6 * (f1[k] + 2.0 * (f2[k] + f3[k]) + f4[k]);
  }
  X[0] = X[0] * AP_Vscale + AP_Voffset;
}

/* CEPINTEGL for cepModel_AP, F/CEPION.f:319-370 (no stretch: I4f <= 1). */
void orc_cep_integ_node(const orc_cep *c, double t1, double dt, int stim, double X[2]) {
  const double eps = 2.220446049250313e-16;
  const double Ksac = 0.0;
  (void)c->Ksac;
  const int nt = (int)lround(dt / c->dt_ode);
  int icl = (int)floor(t1 / c->CL);
  if (icl < 0) icl = 0;
  const double Ts = c->Ts + (double)icl * c->CL;
  const double Te = Ts + c->Td;
  for (int i = 1; i <= nt; i++) {
    const double t = t1 + (double)(i - 1) * c->dt_ode;
    const double Istim = (stim && t >= Ts - eps && t <= Te + eps) ? c->A : 0.0;
    orc_ap_step(X, t, c->dt_ode, Istim, Ksac, c->ode == 1);
  }
}

/* ---------------------------------------------------------------------- */
/* 3x3 helpers, F/MATFUN.f (MAT_DET:177, MAT_INV:238, TEN_*:419-478) */
#define M3(A, i, j) A[(i)*3 + (j)]
static double det3(const double *A) {
  return M3(A, 0, 0) * (M3(A, 1, 1) * M3(A, 2, 2) - M3(A, 1, 2) * M3(A, 2, 1)) -
         M3(A, 0, 1) * (M3(A, 1, 0) * M3(A, 2, 2) - M3(A, 1, 2) * M3(A, 2, 0)) +
         M3(A, 0, 2) * (M3(A, 1, 0) * M3(A, 2, 1) - M3(A, 1, 1) * M3(A, 2, 0));
}
static void inv3(const double *A, double *B) {
  const double d = det3(A);
  M3(B, 0, 0) = (M3(A, 1, 1) * M3(A, 2, 2) - M3(A, 1, 2) * M3(A, 2, 1)) / d;
  M3(B, 0, 1) = (M3(A, 0, 2) * M3(A, 2, 1) - M3(A, 0, 1) * M3(A, 2, 2)) / d;
  M3(B, 0, 2) = (M3(A, 0, 1) * M3(A, 1, 2) - M3(A, 0, 2) * M3(A, 1, 1)) / d;
  M3(B, 1, 0) = (M3(A, 1, 2) * M3(A, 2, 0) - M3(A, 1, 0) * M3(A, 2, 2)) / d;
  M3(B, 1, 1) = (M3(A, 0, 0) * M3(A, 2, 2) - M3(A, 0, 2) * M3(A, 2, 0)) / d;
  M3(B, 1, 2) = (M3(A, 0, 2) * M3(A, 1, 0) - M3(A, 0, 0) * M3(A, 1, 2)) / d;
  M3(B, 2, 0) = (M3(A, 1, 0) * M3(A, 2, 1) - M3(A, 1, 1) * M3(A, 2, 0)) / d;
  M3(B, 2, 1) = (M3(A, 0, 1) * M3(A, 2, 0) - M3(A, 0, 0) * M3(A, 2, 1)) / d;
  M3(B, 2, 2) = (M3(A, 0, 0) * M3(A, 1, 1) - M3(A, 0, 1) * M3(A, 1, 0)) / d;
}
static void matmul3(const double *A, const double *B, double *C) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double s = 0.0;
      for (int k = 0; k < 3; k++) s += M3(A, i, k) * M3(B, k, j);
      M3(C, i, j) = s;
    }
}

/* GETPK2CC, neo-Hookean branch + ST91 volumetric penalty (GETSVOLP) and
   CCTOVOIGT: F/MATMODELS.f:41-150, 539-564, 1588-1647.  No fibres, no
   active stress/strain.  Dm is 6x6 row-major, Voigt order 11,22,33,12,23,31. */
void orc_pk2cc_nhk(double C10, double Kpen, const double F[9], double S[9],
                   double Dm[36]) {
  const double nd = 3.0;
  const double J = det3(F);
  const double J2d = pow(J, -2.0 / nd);
  double C[9], Ci[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double s = 0.0;
      for (int k = 0; k < 3; k++) s += M3(F, k, i) * M3(F, k, j);
      M3(C, i, j) = s;
    }
  inv3(C, Ci);
  double p = 0.0, pl = 0.0;
  if (Kpen != 0.0) {
    p = 0.5 * Kpen * (J - 1.0 / J);
    pl = Kpen * J;
  }
  const double g1 = 2.0 * C10;
  double Sb[9] = {g1, 0, 0, 0, g1, 0, 0, 0, g1};
  double CSb = 0.0;
  for (int k = 0; k < 9; k++) CSb += C[k] * Sb[k];
  const double r1 = J2d * CSb / nd;
  for (int k = 0; k < 9; k++) S[k] = J2d * Sb[k] - r1 * Ci[k];
  double CC[81];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      for (int k = 0; k < 3; k++)
        for (int l = 0; l < 3; l++)
          CC[((i * 3 + j) * 3 + k) * 3 + l] =
              (-2.0 / nd) * (M3(Ci, i, j) * M3(S, k, l) + M3(S, i, j) * M3(Ci, k, l));
  for (int k = 0; k < 9; k++) S[k] = S[k] + p * J * Ci[k];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      for (int k = 0; k < 3; k++)
        for (int l = 0; l < 3; l++) {
          const double sym = 0.5 * (M3(Ci, i, k) * M3(Ci, j, l) + M3(Ci, i, l) * M3(Ci, j, k));
          const double dy = M3(Ci, i, j) * M3(Ci, k, l);
          CC[((i * 3 + j) * 3 + k) * 3 + l] += 2.0 * (r1 - p * J) * sym + (pl * J - 2.0 * r1 / nd) * dy;
        }
  static const int vi[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {1, 2}, {2, 0}};
  for (int I = 0; I < 6; I++)
    for (int Jv = I; Jv < 6; Jv++) {
      const double v = CC[((vi[I][0] * 3 + vi[I][1]) * 3 + vi[Jv][0]) * 3 + vi[Jv][1]];
      Dm[I * 6 + Jv] = v;
      Dm[Jv * 6 + I] = v;
    }
}

/* CONSTRUCT_dSOLID / STRUCT3D for one tet4 element, F/STRUCT.f:39-496.
   mu_e: per-element C10 override if > 0 (else p->C10). */
void orc_elem_struct(const orc_eqp *p, double C10_e, const double xl[12],
                     const double *al, const double *yl, const double *dl,
                     double lR[12], double lK[144]) {
  double w4[4], N4[4][4], Nx[3][4], Jac;
  tet4_gauss(w4, N4);
  gnn3(xl, Nx, &Jac);
  for (int k = 0; k < 12; k++) lR[k] = 0.0;
  for (int k = 0; k < 144; k++) lK[k] = 0.0;
  const int dof = 3, tD = p->tDof;
  const double rho = p->rho, mu = p->visc, dmp = p->dmp;
  const double afu = p->af * p->beta * p->dt * p->dt;
  const double afv = p->af * p->gam * p->dt;
  const double amd = p->am * rho + afv * dmp;
  const int i0 = p->s, j0 = i0 + 1, k0 = j0 + 1;
  const double C10 = C10_e > 0.0 ? C10_e : p->C10;
  for (int g = 0; g < 4; g++) {
    const double w = w4[g] * Jac;
    const double *N = N4[g];
    double ud[3], vx[9] = {0}, F[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    for (int c = 0; c < 3; c++) ud[c] = -rho * p->fb[c];
    for (int a = 0; a < 4; a++) {
      const int ids[3] = {i0, j0, k0};
      for (int c = 0; c < 3; c++) {
        ud[c] = ud[c] + N[a] * (rho * (al[a * tD + ids[c]] - 0.0) + dmp * yl[a * tD + ids[c]]);
        for (int m = 0; m < 3; m++) {
          M3(vx, c, m) = M3(vx, c, m) + Nx[m][a] * yl[a * tD + ids[c]];
          M3(F, c, m) = M3(F, c, m) + Nx[m][a] * dl[a * tD + ids[c]];
        }
      }
    }
    const double J = det3(F);
    double Fi[9];
    inv3(F, Fi);
    /* viscous contribution */
    double VxFi[9], ddev[9], Svis[9], tmp[9], FiT[9];
    matmul3(vx, Fi, VxFi);
    for (int a = 0; a < 3; a++)
      for (int b = 0; b < 3; b++) M3(ddev, a, b) = 0.5 * (M3(VxFi, a, b) + M3(VxFi, b, a));
    const double trd = (M3(ddev, 0, 0) + M3(ddev, 1, 1) + M3(ddev, 2, 2)) / 3.0;
    for (int a = 0; a < 3; a++) M3(ddev, a, a) -= trd;
    for (int a = 0; a < 3; a++)
      for (int b = 0; b < 3; b++) M3(FiT, a, b) = M3(Fi, b, a);
    matmul3(ddev, FiT, tmp);
    matmul3(Fi, tmp, Svis);
    for (int k = 0; k < 9; k++) Svis[k] *= 2.0 * mu * J;
    double S[9], Dm[36], P[9];
    orc_pk2cc_nhk(C10, p->Kpen, F, S, Dm);
    for (int k = 0; k < 9; k++) S[k] += Svis[k];
    matmul3(F, S, P);
    for (int a = 0; a < 4; a++)
      for (int c = 0; c < 3; c++)
        lR[a * dof + c] += w * (N[a] * ud[c] + Nx[0][a] * M3(P, c, 0) + Nx[1][a] * M3(P, c, 1) +
                                Nx[2][a] * M3(P, c, 2));
    double Bm[4][6][3], NxFi[4][3], DdNx[4][3], VxNx[4][3];
    for (int a = 0; a < 4; a++) {
      for (int c = 0; c < 3; c++) {
        Bm[a][0][c] = Nx[0][a] * M3(F, c, 0);
        Bm[a][1][c] = Nx[1][a] * M3(F, c, 1);
        Bm[a][2][c] = Nx[2][a] * M3(F, c, 2);
        Bm[a][3][c] = Nx[0][a] * M3(F, c, 1) + M3(F, c, 0) * Nx[1][a];
        Bm[a][4][c] = Nx[1][a] * M3(F, c, 2) + M3(F, c, 1) * Nx[2][a];
        Bm[a][5][c] = Nx[2][a] * M3(F, c, 0) + M3(F, c, 2) * Nx[0][a];
      }
      for (int c = 0; c < 3; c++)
        NxFi[a][c] = Nx[0][a] * M3(Fi, 0, c) + Nx[1][a] * M3(Fi, 1, c) + Nx[2][a] * M3(Fi, 2, c);
      for (int c = 0; c < 3; c++) {
        DdNx[a][c] = M3(ddev, c, 0) * NxFi[a][0] + M3(ddev, c, 1) * NxFi[a][1] + M3(ddev, c, 2) * NxFi[a][2];
        VxNx[a][c] = M3(VxFi, 0, c) * NxFi[a][0] + M3(VxFi, 1, c) * NxFi[a][1] + M3(VxFi, 2, c) * NxFi[a][2];
      }
    }
    const double r13 = 1.0 / 3.0, r23 = 2.0 / 3.0;
    const double rmu = afu * mu * J, rmv = afv * mu * J;
    for (int b = 0; b < 4; b++)
      for (int a = 0; a < 4; a++) {
        double NxSNx = 0.0;
        for (int m = 0; m < 3; m++)
          for (int q = 0; q < 3; q++) NxSNx += Nx[m][a] * M3(S, m, q) * Nx[q][b];
        const double T1 = amd * N[a] * N[b] + afu * NxSNx;
        double DBm[6][3];
        for (int I = 0; I < 6; I++)
          for (int c = 0; c < 3; c++) {
            double s = 0.0;
            for (int K = 0; K < 6; K++) s += Dm[I * 6 + K] * Bm[b][K][c];
            DBm[I][c] = s;
          }
        const double NxNx = NxFi[a][0] * NxFi[b][0] + NxFi[a][1] * NxFi[b][1] + NxFi[a][2] * NxFi[b][2];
        for (int r = 0; r < 3; r++)
          for (int c = 0; c < 3; c++) {
            double BmDBm = 0.0;
            for (int I = 0; I < 6; I++) BmDBm += Bm[a][I][r] * DBm[I][c];
            double Tv = (2.0 * (DdNx[a][r] * NxFi[b][c] - DdNx[b][r] * NxFi[a][c]) -
                         (NxNx * M3(VxFi, r, c) + NxFi[b][r] * VxNx[a][c] - r23 * NxFi[a][r] * VxNx[b][c])) *
                        rmu;
            if (r == c)
              Tv += (r13 * NxFi[a][r] * NxFi[b][r] + NxNx) * rmv;
            else
              Tv += (NxFi[a][c] * NxFi[b][r] - r23 * NxFi[a][r] * NxFi[b][c]) * rmv;
            const double diag = (r == c) ? T1 : 0.0;
            lK[(size_t)(a * 4 + b) * 9 + r * 3 + c] += w * (diag + afu * BmDBm + Tv);
          }
      }
  }
}

/* ---------------------------------------------------------------------- */
/* GLOBALEQASSEM -> CONSTRUCT_* -> DOASSEM over all elements (one domain),
   F/EQASSEM.f:38-87. */
int orc_assemble(const orc_eqp *p, int nNo, int nEl, const int *IEN,
                 const double *x, const double *Ag, const double *Yg,
                 const double *Dg, const int *rowPtr, const int *colPtr,
                 double *R, double *Val) {
  (void)nNo;
  const int tD = p->tDof;
  double xl[12], al[4 * 16], yl[4 * 16], dl[4 * 16];
  int ptr[4];
  if (tD > 16) return -1;
  for (int e = 0; e < nEl; e++) {
    for (int a = 0; a < 4; a++) {
      const int Ac = IEN[(size_t)e * 4 + a];
      ptr[a] = Ac;
      for (int i = 0; i < 3; i++) xl[a * 3 + i] = x[(size_t)Ac * 3 + i];
      for (int i = 0; i < tD; i++) {
        al[a * tD + i] = Ag[(size_t)Ac * tD + i];
        yl[a * tD + i] = Yg[(size_t)Ac * tD + i];
        dl[a * tD + i] = Dg ? Dg[(size_t)Ac * tD + i] : 0.0;
      }
    }
    if (p->phys == 1) {
      double lR[4], lK[16];
      orc_elem_heats(p, xl, al, yl, lR, lK);
      orc_doassem(1, 4, ptr, lK, lR, rowPtr, colPtr, R, Val);
    } else if (p->phys == 2) {
      double lR[12], lK[144];
      const double C10e = p->eparam ? p->eparam[e] : 0.0;
      orc_elem_struct(p, C10e, xl, al, yl, dl, lR, lK);
      orc_doassem(3, 4, ptr, lK, lR, rowPtr, colPtr, R, Val);
    } else if (p->phys == 3) {
      double lR[4], lK[16];
      orc_elem_cep(p, p->eparam ? p->eparam[e] : p->Diso,
                   (p->fN && p->nFn > 0) ? p->fN + (size_t)e * 3 * p->nFn : NULL, xl, al, yl,
                   lR, lK);
      orc_doassem(1, 4, ptr, lK, lR, rowPtr, colPtr, R, Val);
    } else if (p->phys == 4) {
      double lR[16], lK[256];
      orc_elem_fluid(p, xl, al, yl, lR, lK);
      orc_doassem(4, 4, ptr, lK, lR, rowPtr, colPtr, R, Val);
    } else if (p->phys == 5) {
      double lR[12], lK[144];
      orc_elem_lelas(p, xl, al, dl, lR, lK);
      orc_doassem(3, 4, ptr, lK, lR, rowPtr, colPtr, R, Val);
    } else if (p->phys == 6) {
      double lR[4], lK[16];
      orc_elem_heatf(p, xl, al, yl, lR, lK);
      orc_doassem(1, 4, ptr, lK, lR, rowPtr, colPtr, R, Val);
    } else {
      return -2;
    }
  }
  return 0;
}

/* Same as orc_assemble with the element loop split by a conflict-free
   colouring (elements of one colour share no node) and run with OpenMP
   inside each colour -- the multi-core CPU baseline.  order[] lists element
   ids colour by colour, color_off[ncolor+1] delimits the colours. */
int orc_assemble_colored(const orc_eqp *p, int nNo, int nEl, const int *IEN,
                         const double *x, const double *Ag, const double *Yg,
                         const double *Dg, const int *rowPtr, const int *colPtr,
                         double *R, double *Val, int ncolor, const int *color_off,
                         const int *order) {
  (void)nNo;
  (void)nEl;
  const int tD = p->tDof;
  if (tD > 16) return -1;
  for (int c = 0; c < ncolor; c++) {
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
    for (int k = color_off[c]; k < color_off[c + 1]; k++) {
      const int e = order[k];
      double xl[12], al[4 * 16], yl[4 * 16], dl[4 * 16];
      int ptr[4];
      for (int a = 0; a < 4; a++) {
        const int Ac = IEN[(size_t)e * 4 + a];
        ptr[a] = Ac;
        for (int i = 0; i < 3; i++) xl[a * 3 + i] = x[(size_t)Ac * 3 + i];
        for (int i = 0; i < tD; i++) {
          al[a * tD + i] = Ag[(size_t)Ac * tD + i];
          yl[a * tD + i] = Yg[(size_t)Ac * tD + i];
          dl[a * tD + i] = Dg ? Dg[(size_t)Ac * tD + i] : 0.0;
        }
      }
      if (p->phys == 1) {
        double lR[4], lK[16];
        orc_elem_heats(p, xl, al, yl, lR, lK);
        orc_doassem(1, 4, ptr, lK, lR, rowPtr, colPtr, R, Val);
      } else if (p->phys == 2) {
        double lR[12], lK[144];
        orc_elem_struct(p, p->eparam ? p->eparam[e] : 0.0, xl, al, yl, dl, lR, lK);
        orc_doassem(3, 4, ptr, lK, lR, rowPtr, colPtr, R, Val);
      } else if (p->phys == 3) {
        double lR[4], lK[16];
        orc_elem_cep(p, p->eparam ? p->eparam[e] : p->Diso,
                     (p->fN && p->nFn > 0) ? p->fN + (size_t)e * 3 * p->nFn : NULL, xl, al,
                     yl, lR, lK);
        orc_doassem(1, 4, ptr, lK, lR, rowPtr, colPtr, R, Val);
      } else if (p->phys == 4) {
        double lR[16], lK[256];
        orc_elem_fluid(p, xl, al, yl, lR, lK);
        orc_doassem(4, 4, ptr, lK, lR, rowPtr, colPtr, R, Val);
      } else if (p->phys == 5) {
        double lR[12], lK[144];
        orc_elem_lelas(p, xl, al, dl, lR, lK);
        orc_doassem(3, 4, ptr, lK, lR, rowPtr, colPtr, R, Val);
      } else if (p->phys == 6) {
        double lR[4], lK[16];
        orc_elem_heatf(p, xl, al, yl, lR, lK);
        orc_doassem(1, 4, ptr, lK, lR, rowPtr, colPtr, R, Val);
      }
    }
  }
  return 0;
}

int orc_color_elements(int nNo, int nEl, const int *IEN, int *color_off, int *order) {
  /* one 64-bit mask of used colours per node; an element takes the lowest
     colour free at all four of its nodes */
  unsigned long long *used = (unsigned long long *)xcalloc((size_t)nNo, sizeof(*used));
  unsigned char *col = (unsigned char *)xcalloc((size_t)(nEl > 0 ? nEl : 1), 1);
  int ncolor = 0;
  for (int e = 0; e < nEl; e++) {
    unsigned long long m = 0;
    for (int a = 0; a < 4; a++) m |= used[IEN[(size_t)e * 4 + a]];
    if (m == ~0ULL) {
      free(used);
      free(col);
      return -1;
    }
    int c = 0;
    while ((m >> c) & 1ULL) c++;
    col[e] = (unsigned char)c;
    for (int a = 0; a < 4; a++) used[IEN[(size_t)e * 4 + a]] |= 1ULL << c;
    if (c + 1 > ncolor) ncolor = c + 1;
  }
  for (int c = 0; c <= ncolor; c++) color_off[c] = 0;
  for (int e = 0; e < nEl; e++) color_off[col[e] + 1]++;
  for (int c = 0; c < ncolor; c++) color_off[c + 1] += color_off[c];
  int fill[64];
  for (int c = 0; c < ncolor; c++) fill[c] = color_off[c];
  for (int e = 0; e < nEl; e++) order[fill[col[e]]++] = e;
  free(used);
  free(col);
  return ncolor;
}

/* SETBCTRACL for tri3 faces with a constant traction vector h,
   F/SETBC.f:319-416; 3-point rule F/NN.f:416-422, w = 1/6. */
void orc_bheatf(const orc_eqp *p, int nFel, const int *fIEN, double g, int nEl,
                const int *IEN, const double *x, const double *Yg, const int *rowPtr,
                const int *colPtr, double *R, double *Val) {
  const int tD = p->tDof;
  const double h = -g;
  const double s = 2.0 / 3.0, t = 1.0 / 6.0;
  const double xi[3][2] = {{t, t}, {s, t}, {t, s}};
  int *innerv = (int *)xcalloc((size_t)(nFel > 0 ? nFel : 1), sizeof(int));
  orc_face_inner(nFel, fIEN, nEl, IEN, innerv);
  for (int f = 0; f < nFel; f++) {
    const int *q = fIEN + 3 * f;
    /* the element holding the face, and its node off the face */
    const int inner = innerv[f];
    if (inner < 0) continue;
    /* GNNB for tri3: n = (x1 - x3) x (x2 - x3), pointing away from the
       element's other node */
    double e1[3], e2[3], n[3], v[3];
    for (int i = 0; i < 3; i++) {
      e1[i] = x[3 * q[0] + i] - x[3 * q[2] + i];
      e2[i] = x[3 * q[1] + i] - x[3 * q[2] + i];
      v[i] = x[3 * q[0] + i] - x[3 * inner + i];
    }
    n[0] = e1[1] * e2[2] - e1[2] * e2[1];
    n[1] = e1[2] * e2[0] - e1[0] * e2[2];
    n[2] = e1[0] * e2[1] - e1[1] * e2[0];
    if (n[0] * v[0] + n[1] * v[1] + n[2] * v[2] < 0.0)
      for (int i = 0; i < 3; i++) n[i] = -n[i];
    const double Jac = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    double nV[3];
    for (int i = 0; i < 3; i++) nV[i] = n[i] / Jac;
    double lR[3] = {0, 0, 0}, lK[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int gp = 0; gp < 3; gp++) {
      const double N[3] = {xi[gp][0], xi[gp][1], 1.0 - xi[gp][0] - xi[gp][1]};
      const double w = (1.0 / 6.0) * Jac;
      const double wl = w * p->af * p->gam * p->dt;
      double y[4] = {0, 0, 0, 0};
      for (int a = 0; a < 3; a++) {
        for (int i = 0; i < 3; i++) y[i] = y[i] + N[a] * Yg[(size_t)q[a] * tD + i];
        y[3] = y[3] + N[a] * Yg[(size_t)q[a] * tD + p->s];
      }
      double udn = 0.0;
      for (int i = 0; i < 3; i++) udn = udn + y[i] * nV[i];
      udn = 0.5 * (udn - fabs(udn));
      const double T1 = h - udn * y[3];
      for (int a = 0; a < 3; a++) {
        lR[a] = lR[a] + w * N[a] * T1;
        for (int b = 0; b < 3; b++) lK[3 * a + b] = lK[3 * a + b] - wl * N[a] * N[b] * udn;
      }
    }
    /* DOASSEM for the face element */
    for (int a = 0; a < 3; a++) {
      R[q[a]] += lR[a];
      for (int b = 0; b < 3; b++)
        for (int j = rowPtr[q[a]]; j < rowPtr[q[a] + 1]; j++)
          if (colPtr[j] == q[b]) {
            Val[j] += lK[3 * a + b];
            break;
          }
    }
  }
  free(innerv);
}

void orc_face_inner(int nFel, const int *fIEN, int nEl, const int *IEN, int *inner) {
  /* elements of each node that lies on a face (counting sort) */
  int nNo = 0;
  for (int k = 0; k < 4 * nEl; k++)
    if (IEN[k] + 1 > nNo) nNo = IEN[k] + 1;
  int *cnt = (int *)xcalloc((size_t)nNo + 1, sizeof(int));
  char *onF = (char *)xcalloc((size_t)(nNo > 0 ? nNo : 1), 1);
  for (int k = 0; k < 3 * nFel; k++) onF[fIEN[k]] = 1;
  for (int k = 0; k < 4 * nEl; k++)
    if (onF[IEN[k]]) cnt[IEN[k] + 1]++;
  for (int v = 0; v < nNo; v++) cnt[v + 1] += cnt[v];
  int *els = (int *)xcalloc((size_t)(cnt[nNo] > 0 ? cnt[nNo] : 1), sizeof(int));
  int *fill = (int *)xcalloc((size_t)nNo + 1, sizeof(int));
  memcpy(fill, cnt, sizeof(int) * ((size_t)nNo + 1));
  for (int e = 0; e < nEl; e++)
    for (int a = 0; a < 4; a++)
      if (onF[IEN[4 * e + a]]) els[fill[IEN[4 * e + a]]++] = e;
  for (int f = 0; f < nFel; f++) {
    const int *q = fIEN + 3 * f;
    inner[f] = -1;
    for (int k = cnt[q[0]]; k < cnt[q[0] + 1] && inner[f] < 0; k++) {
      const int e = els[k];
      int hit = 0, other = -1;
      for (int a = 0; a < 4; a++) {
        const int v = IEN[4 * e + a];
        if (v == q[0] || v == q[1] || v == q[2])
          hit++;
        else if (other < 0)
          other = v;
      }
      if (hit == 3) inner[f] = other;
    }
  }
  free(cnt);
  free(onF);
  free(els);
  free(fill);
}

/* BFLUID (F/FLUID.f:1280-1334) through BASSEMNEUBC (F/EQASSEM.f:90-192):
   at each point of the tri3 rule, udn = 1/2 bstab rho (u.n - |u.n|),
   hc = h n + udn u, lR(i,a) -= w N_a hc_i and the velocity diagonal of
   lK (entries 1, 6, 11 of the 4x4 block) -= w af gam dt N_a N_b udn. */
void orc_bfluid(const orc_eqp *p, int nFel, const int *fIEN, double g, int nEl,
                const int *IEN, const double *x, const double *Yg, const int *rowPtr,
                const int *colPtr, double *R, double *Val) {
  const int tD = p->tDof, s0 = p->s;
  const double h = -g;
  const double s = 2.0 / 3.0, t = 1.0 / 6.0;
  const double xi[3][2] = {{t, t}, {s, t}, {t, s}};
  int *innerv = (int *)xcalloc((size_t)(nFel > 0 ? nFel : 1), sizeof(int));
  orc_face_inner(nFel, fIEN, nEl, IEN, innerv);
  for (int f = 0; f < nFel; f++) {
    const int *q = fIEN + 3 * f;
    const int inner = innerv[f];
    if (inner < 0) continue;
    double e1[3], e2[3], n[3], v[3];
    for (int i = 0; i < 3; i++) {
      e1[i] = x[3 * q[0] + i] - x[3 * q[2] + i];
      e2[i] = x[3 * q[1] + i] - x[3 * q[2] + i];
      v[i] = x[3 * q[0] + i] - x[3 * inner + i];
    }
    n[0] = e1[1] * e2[2] - e1[2] * e2[1];
    n[1] = e1[2] * e2[0] - e1[0] * e2[2];
    n[2] = e1[0] * e2[1] - e1[1] * e2[0];
    if (n[0] * v[0] + n[1] * v[1] + n[2] * v[2] < 0.0)
      for (int i = 0; i < 3; i++) n[i] = -n[i];
    const double Jac = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    double nV[3];
    for (int i = 0; i < 3; i++) nV[i] = n[i] / Jac;
    double lR[3][3] = {{0}}, lK[3][3] = {{0}};
    for (int gp = 0; gp < 3; gp++) {
      const double N[3] = {xi[gp][0], xi[gp][1], 1.0 - xi[gp][0] - xi[gp][1]};
      const double w = (1.0 / 6.0) * Jac;
      const double wl = w * p->af * p->gam * p->dt;
      double u[3] = {0, 0, 0};
      for (int a = 0; a < 3; a++)
        for (int i = 0; i < 3; i++) u[i] = u[i] + N[a] * Yg[(size_t)q[a] * tD + s0 + i];
      double udn = 0.0;
      for (int i = 0; i < 3; i++) udn = udn + u[i] * nV[i];
      udn = 0.5 * p->bstab * p->rho * (udn - fabs(udn));
      double hc[3];
      for (int i = 0; i < 3; i++) hc[i] = h * nV[i] + udn * u[i];
      for (int a = 0; a < 3; a++) {
        for (int i = 0; i < 3; i++) lR[a][i] = lR[a][i] - w * N[a] * hc[i];
        for (int b = 0; b < 3; b++) lK[a][b] = lK[a][b] - wl * N[a] * N[b] * udn;
      }
    }
    for (int a = 0; a < 3; a++) {
      for (int i = 0; i < 3; i++) R[(size_t)q[a] * 4 + i] += lR[a][i];
      for (int b = 0; b < 3; b++)
        for (int j = rowPtr[q[a]]; j < rowPtr[q[a] + 1]; j++)
          if (colPtr[j] == q[b]) {
            Val[(size_t)j * 16 + 0] += lK[a][b];
            Val[(size_t)j * 16 + 5] += lK[a][b];
            Val[(size_t)j * 16 + 10] += lK[a][b];
            break;
          }
    }
  }
  free(innerv);
}

void orc_traction(int dof, int nFel, const int *fIEN, const double *x,
                  const double h[3], double *R) {
  const double s = 2.0 / 3.0, t = 1.0 / 6.0;
  const double xi[3][2] = {{t, t}, {s, t}, {t, s}};
  for (int e = 0; e < nFel; e++) {
    const int *n = fIEN + (size_t)e * 3;
    double v1[3], v2[3], nV[3];
    for (int i = 0; i < 3; i++) {
      v1[i] = x[(size_t)n[0] * 3 + i] - x[(size_t)n[2] * 3 + i];
      v2[i] = x[(size_t)n[1] * 3 + i] - x[(size_t)n[2] * 3 + i];
    }
    nV[0] = v1[1] * v2[2] - v1[2] * v2[1];
    nV[1] = v1[2] * v2[0] - v1[0] * v2[2];
    nV[2] = v1[0] * v2[1] - v1[1] * v2[0];
    const double Jac = sqrt(nV[0] * nV[0] + nV[1] * nV[1] + nV[2] * nV[2]);
    double lR[3][3] = {{0}};
    for (int g = 0; g < 3; g++) {
      const double w = Jac / 6.0;
      const double N[3] = {xi[g][0], xi[g][1], 1.0 - xi[g][0] - xi[g][1]};
      double hh[3] = {0, 0, 0};
      for (int a = 0; a < 3; a++)
        for (int i = 0; i < 3; i++) hh[i] += N[a] * h[i];
      for (int a = 0; a < 3; a++)
        for (int i = 0; i < 3; i++) lR[a][i] -= w * N[a] * hh[i];
    }
    for (int a = 0; a < 3; a++)
      for (int i = 0; i < 3 && i < dof; i++) R[(size_t)n[a] * dof + i] += lR[a][i];
  }
}

/* gen-alpha coefficients, F/INITIALIZE.f:76-139 */
void orc_genalpha(double roInf, int second_order, double *am, double *af,
                  double *beta, double *gam) {
  *am = second_order ? (2.0 - roInf) / (1.0 + roInf)
                     : 0.5 * (3.0 - roInf) / (1.0 + roInf);
  *af = 1.0 / (1.0 + roInf);
  *beta = 0.25 * pow(1.0 + *am - *af, 2.0);
  *gam = 0.5 + *am - *af;
}

/* ---------------------------------------------------------------------- */
/* One time step of one equation: PICP (F/PIC.f:40-130), SETBCDIR
   (F/SETBC.f:39-228), then the Newton loop of F/MAIN.f:116-215 with
   PICI (F/PIC.f:133-166), LSALLOC, assembly, SETBCNEU, LSSOLVE and PICC
   (F/PIC.f:169-297).  At the end An/Yn/Dn are copied to Ao/Yo/Do
   (F/MAIN.f:277-279).  eq->p.s must be 0 (single equation). */
static void apply_dir(orc_eq *eq, double *lA, double *lY) {
  const int tD = eq->p.tDof, s = eq->p.s, dof = eq->p.dof;
  for (int ib = 0; ib < eq->nDir; ib++) {
    const orc_dirbc *bc = &eq->dir[ib];
    /* the pressure of a dof = nsd+1 equation is never constrained
       (F/SETBC.f:77); with lDof = nsd the value is g*gx*nV (SETBCDIRL,
       F/SETBC.f:212-217), else g*gx */
    const int ncomp = (dof == 4) ? 3 : dof;
    for (int a = 0; a < bc->nNo; a++) {
      const int Ac = bc->nodes[a];
      const double gx = bc->gx ? bc->gx[a] : 1.0;
      for (int c = 0; c < ncomp; c++) {
        if (bc->mask && !((bc->mask >> c) & 1)) continue;
        const double nv = (bc->nV && ncomp == 3) ? bc->nV[(size_t)a * 3 + c] : 1.0;
        lA[(size_t)Ac * tD + s + c] = 0.0 * gx * nv;
        lY[(size_t)Ac * tD + s + c] = bc->g * gx * nv;
      }
    }
  }
}

/* SETBCDIRL for ustruct (F/SETBC.f:133-175, plain Dirichlet): for each
   constrained velocity component, Dn = gam dt Yn - (gam - 1) dt Ad + Do
   and Ad = Yn */
static void ust_dir(orc_eq *eq, const double *lY, double *lD) {
  const int tD = eq->p.tDof, s = eq->p.s;
  const double c1 = eq->p.gam * eq->p.dt, c2 = (eq->p.gam - 1.0) * eq->p.dt;
  for (int ib = 0; ib < eq->nDir; ib++) {
    const orc_dirbc *bc = &eq->dir[ib];
    for (int a = 0; a < bc->nNo; a++) {
      const int Ac = bc->nodes[a];
      for (int i = 0; i < 3; i++) {
        if (bc->mask && !((bc->mask >> i) & 1)) continue;
        const size_t j = (size_t)Ac * tD + s + i;
        lD[j] = c1 * lY[j] - c2 * eq->Ad[(size_t)Ac * 3 + i] + eq->Do[j];
        eq->Ad[(size_t)Ac * 3 + i] = lY[j];
      }
    }
  }
}

int orc_eq_step(orc_eq *eq, orc_stepinfo *info) {
  const int nNo = eq->nNo, tD = eq->p.tDof, dof = eq->p.dof;
  const size_t nS = (size_t)nNo * tD;
  const double dt = eq->p.dt, gam = eq->p.gam, beta = eq->p.beta;
  const int dFlag = (eq->p.phys == 2 || eq->p.phys == 5);
  const int ust = (eq->p.phys == 7);
  if (ust && (!eq->Ad || dof != 4 || eq->p.s != 0)) return -4;
  memset(info, 0, sizeof(*info));
  eq->time += dt;
  /* CEP: reaction step (CEPINTEG, F/CEPION.f:166-314, called from PICP):
     Xion(1) = Yo(v) (not on the first pass), integrate the cell model from
     time-dt over dt, Yo(v) = Xion(1) */
  if (eq->p.phys == 3) {
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
    for (int a = 0; a < nNo; a++) {
      double X[2];
      X[0] = eq->cep_ipass_done ? eq->Yo[(size_t)a * tD + eq->p.s] : eq->Xion[(size_t)a * 2];
      X[1] = eq->Xion[(size_t)a * 2 + 1];
      orc_cep_integ_node(&eq->cep, eq->time - dt, dt, eq->stim ? eq->stim[a] : 0, X);
      eq->Xion[(size_t)a * 2] = X[0];
      eq->Xion[(size_t)a * 2 + 1] = X[1];
      eq->Yo[(size_t)a * tD + eq->p.s] = X[0];
    }
    eq->cep_ipass_done = 1;
  }
  /* PICP */
  const double coef = (gam - 1.0) / gam;
  for (size_t k = 0; k < nS; k++) eq->An[k] = eq->Ao[k] * coef;
  for (size_t k = 0; k < nS; k++) eq->Yn[k] = eq->Yo[k];
  if (dFlag) {
    const double c2 = dt * dt * (0.5 * gam - beta) / (gam - 1.0);
    for (size_t k = 0; k < nS; k++) eq->Dn[k] = eq->Do[k] + eq->Yn[k] * dt + eq->An[k] * c2;
  } else {
    for (size_t k = 0; k < nS; k++) eq->Dn[k] = eq->Do[k];
  }
  if (ust) /* ustruct: Ad = Ad (gam - 1)/gam, Dn = Do (F/PIC.f:111-116) */
    for (size_t k = 0; k < (size_t)nNo * 3; k++) eq->Ad[k] = eq->Ad[k] * coef;
  /* SETBCDIR */
  apply_dir(eq, eq->An, eq->Yn);
  if (ust) ust_dir(eq, eq->Yn, eq->Dn);

  /* LS structures: one face per Dirichlet BC (FSILSINI, F/BAFINI.f:468-513) */
  orc_lhs *lhs = orc_lhs_create(nNo, eq->nnz, eq->rowPtr, eq->colPtr, eq->nDir);
  for (int ib = 0; ib < eq->nDir; ib++) {
    const orc_dirbc *bc = &eq->dir[ib];
    double *sv = (double *)xcalloc((size_t)3 * bc->nNo, sizeof(double));
    if (bc->mask)
      for (int a = 0; a < bc->nNo; a++)
        for (int c = 0; c < 3; c++) sv[a * 3 + c] = ((bc->mask >> c) & 1) ? 0.0 : 1.0;
    orc_bc_create(lhs, ib + 1, bc->nNo, 3, ORC_BC_TYPE_Dir, bc->nodes, sv);
    free(sv);
  }
  orc_ls ls;
  orc_ls_create(&ls, eq->LS_type);
  if (eq->ls_relTol > 0) ls.RI.relTol = eq->ls_relTol;
  if (eq->ls_absTol > 0) ls.RI.absTol = eq->ls_absTol;
  if (eq->ls_mItr > 0) ls.RI.mItr = eq->ls_mItr;
  if (eq->ls_sD > 0) {
    ls.RI.sD = eq->ls_sD;
    ls.GM.sD = eq->ls_sD;
  }
  if (eq->ls_relTolIn[0] > 0) {
    ls.GM.relTol = eq->ls_relTolIn[0];
    ls.CG.relTol = eq->ls_relTolIn[1];
  }
  if (eq->ls_mItrIn[0] > 0) {
    ls.GM.mItr = eq->ls_mItrIn[0];
    ls.CG.mItr = eq->ls_mItrIn[1];
  }

  double *Ag = (double *)xcalloc(nS, sizeof(double));
  double *Yg = (double *)xcalloc(nS, sizeof(double));
  double *Dg = (double *)xcalloc(nS, sizeof(double));
  double *R = (double *)xcalloc((size_t)nNo * dof, sizeof(double));
  double *Val = (double *)xcalloc((size_t)eq->nnz * dof * dof, sizeof(double));
  double *Kd = ust ? (double *)xcalloc((size_t)eq->nnz * 12, sizeof(double)) : NULL;
  double *Rd = ust ? (double *)xcalloc((size_t)nNo * 3, sizeof(double)) : NULL;
  int *incL = (int *)xcalloc(eq->nDir > 0 ? eq->nDir : 1, sizeof(int));
  double *res = (double *)xcalloc(eq->nDir > 0 ? eq->nDir : 1, sizeof(double));
  for (int f = 0; f < eq->nDir; f++) incL[f] = 1;

  int itr = 0, ok = 0, rc = 0;
  const double am = eq->p.am, af = eq->p.af;
  while (!ok) {
    /* PICI */
    itr++;
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
    for (size_t k = 0; k < nS; k++) {
      Ag[k] = eq->Ao[k] * (1.0 - am) + eq->An[k] * am;
      Yg[k] = eq->Yo[k] * (1.0 - af) + eq->Yn[k] * af;
      Dg[k] = eq->Do[k] * (1.0 - af) + eq->Dn[k] * af;
    }
    /* LSALLOC */
    memset(R, 0, sizeof(double) * (size_t)nNo * dof);
    memset(Val, 0, sizeof(double) * (size_t)eq->nnz * dof * dof);
    if (ust) {
      memset(Kd, 0, sizeof(double) * (size_t)eq->nnz * 12);
      if (eq->ncolor > 0)
        rc = orc_assemble_ustruct_colored(&eq->p, eq->nEl, eq->IEN, eq->x, Ag, Yg, Dg,
                                          eq->rowPtr, eq->colPtr, R, Val, Kd, eq->ncolor,
                                          eq->color_off, eq->color_order);
      else
        rc = orc_assemble_ustruct(&eq->p, nNo, eq->nEl, eq->IEN, eq->x, Ag, Yg, Dg, eq->rowPtr,
                                  eq->colPtr, R, Val, Kd);
    } else if (eq->ncolor > 0)
      rc = orc_assemble_colored(&eq->p, nNo, eq->nEl, eq->IEN, eq->x, Ag, Yg, Dg, eq->rowPtr,
                                eq->colPtr, R, Val, eq->ncolor, eq->color_off, eq->color_order);
    else
      rc = orc_assemble(&eq->p, nNo, eq->nEl, eq->IEN, eq->x, Ag, Yg, Dg, eq->rowPtr,
                        eq->colPtr, R, Val);
    if (rc) break;
    /* SETBCNEU (traction) */
    for (int t = 0; t < eq->nTrac; t++)
      orc_traction(dof, eq->trac[t].nFel, eq->trac[t].fIEN, eq->x, eq->trac[t].h, R);
    /* BASSEMNEUBC (Neumann faces: BFLUID for a fluid, BHEATF for HEATF) */
    for (int k = 0; k < eq->nNeu; k++) {
      if (eq->p.phys == 4)
        orc_bfluid(&eq->p, eq->neu[k].nFel, eq->neu[k].fIEN, eq->neu[k].g, eq->nEl, eq->IEN,
                   eq->x, Yg, eq->rowPtr, eq->colPtr, R, Val);
      else
        orc_bheatf(&eq->p, eq->neu[k].nFel, eq->neu[k].fIEN, eq->neu[k].g, eq->nEl, eq->IEN,
                   eq->x, Yg, eq->rowPtr, eq->colPtr, R, Val);
    }
    /* USTRUCTR (F/USTRUCT.f:1557-1637): on the first Newton iteration
       Rd = amg Ad - Yg(velocity) and R -= Kd Rd / am; afterwards Rd = 0 */
    if (ust) {
      if (itr > 1) {
        memset(Rd, 0, sizeof(double) * (size_t)nNo * 3);
      } else {
        const double amg = (gam - am) / (gam - 1.0), ami = 1.0 / am;
        for (int a = 0; a < nNo; a++)
          for (int i = 0; i < 3; i++)
            Rd[(size_t)a * 3 + i] = amg * eq->Ad[(size_t)a * 3 + i] - Yg[(size_t)a * tD + i];
        for (int a = 0; a < nNo; a++) {
          double KU[4] = {0, 0, 0, 0};
          for (int j = eq->rowPtr[a]; j < eq->rowPtr[a + 1]; j++) {
            const int c = eq->colPtr[j];
            const double *kd = Kd + (size_t)j * 12;
            for (int r = 0; r < 4; r++)
              KU[r] = KU[r] + kd[3 * r] * Rd[(size_t)c * 3] + kd[3 * r + 1] * Rd[(size_t)c * 3 + 1] +
                      kd[3 * r + 2] * Rd[(size_t)c * 3 + 2];
          }
          for (int r = 0; r < 4; r++) R[(size_t)a * 4 + r] = R[(size_t)a * 4 + r] - ami * KU[r];
        }
      }
    }
    /* LSSOLVE */
    rc = orc_solve(lhs, &ls, dof, R, Val, eq->prec, incL, res);
    if (rc) break;
    info->ls_itr_total += ls.RI.itr;
    info->last_suc = ls.RI.suc;
    /* PICC */
    const double c1 = gam * dt, c2 = beta * dt * dt;
    if (ust) { /* F/PIC.f:185-196 */
      const double c3 = 1.0 / am, c4 = af * c1 * c3;
      for (int a = 0; a < nNo; a++)
        for (int i = 0; i < 3; i++) {
          const double dU = Rd[(size_t)a * 3 + i] * c3 + R[(size_t)a * 4 + i] * c4;
          eq->Ad[(size_t)a * 3 + i] = eq->Ad[(size_t)a * 3 + i] - dU;
          eq->Dn[(size_t)a * tD + i] = eq->Dn[(size_t)a * tD + i] - dU * c1;
        }
    }
    for (int a = 0; a < nNo; a++)
      for (int c = 0; c < dof; c++) {
        const double r = R[(size_t)a * dof + c];
        const size_t k = (size_t)a * tD + eq->p.s + c;
        eq->An[k] = eq->An[k] - r;
        eq->Yn[k] = eq->Yn[k] - r * c1;
        if (!ust) eq->Dn[k] = eq->Dn[k] - r * c2;
      }
    if (ls.RI.iNorm == 0.0) ls.RI.iNorm = 2.220446049250313e-16;
    if (eq->eq_iNorm == 0.0) eq->eq_iNorm = ls.RI.iNorm;
    if (itr == 1) eq->eq_pNorm = ls.RI.iNorm / eq->eq_iNorm;
    const double r1 = ls.RI.iNorm / eq->eq_iNorm;
    const int l1 = eq->eq_iNorm <= eq->eqAbsTol;
    const int l2 = itr >= eq->maxItr;
    const int l3 = r1 <= eq->tol;
    const int l4 = r1 <= eq->tol * eq->eq_pNorm;
    const int l5 = itr >= eq->minItr;
    if (l1 || l2 || ((l3 || l4) && l5)) ok = 1;
    info->last_iNorm = ls.RI.iNorm;
    info->r1_last = r1;
  }
  info->newton_itr = itr;
  /* PICC for CEP: Xion(1) = Yn(s) (F/PIC.f:232-238) */
  if (eq->p.phys == 3)
    for (int a = 0; a < nNo; a++) eq->Xion[(size_t)a * 2] = eq->Yn[(size_t)a * tD + eq->p.s];
  memcpy(eq->Ao, eq->An, nS * sizeof(double));
  memcpy(eq->Yo, eq->Yn, nS * sizeof(double));
  if (dFlag || ust) memcpy(eq->Do, eq->Dn, nS * sizeof(double));
  orc_lhs_free(lhs);
  free(Ag);
  free(Yg);
  free(Dg);
  free(R);
  free(Val);
  free(Kd);
  free(Rd);
  free(incL);
  free(res);
  return rc;
}

/* ---------------------------------------------------------------------- */
/* USTRUCT: velocity-pressure (mixed) nonlinear solid, F/USTRUCT.f.  The
   tet4 mesh uses one function space for velocity and pressure (nFs = 1,
   VMS stabilisation on), the neo-Hookean isochoric model (GETPK2CCdev,
   F/MATMODELS.f:568-1016, without fibres or active coupling: Ja = 1) and
   the volumetric penalty of GVOLPEN (F/MATMODELS.f:1020-1070); tauM/tauC
   of GETTAU (F/MATMODELS.f:1073-1104).  lR(4,4), lK(16,4,4), lKd(12,4,4):
   index [a*4+i], [(a*4+b)*16+k], [(a*4+b)*12+k]. */
static void ust_gvolpen(const orc_eqp *p, double pr, double Ja, double *ro, double *bt,
                        double *dro, double *dbt) {
  *ro = p->rho / Ja;
  *bt = 0.0;
  *dbt = 0.0;
  *dro = 0.0;
  const double Kp = p->Kpen;
  if (iszero(Kp)) return;
  if (p->volType == 0) {        /* stVol_Quad */
    const double r1 = 1.0 / (Kp - pr);
    *ro = *ro * Kp * r1;
    *bt = r1;
    *dro = *ro * r1;
    *dbt = r1 * r1;
  } else if (p->volType == 1) { /* stVol_ST91 */
    const double r1 = *ro / Kp, r2 = sqrt(pr * pr + Kp * Kp);
    *ro = r1 * (pr + r2);
    *bt = 1.0 / r2;
    *dro = *ro * *bt;
    *dbt = -*bt * pr / (pr * pr + Kp * Kp);
  } else {                      /* stVol_M94 */
    const double r1 = *ro / Kp, r2 = Kp + pr;
    *ro = r1 * r2;
    *bt = 1.0 / r2;
    *dro = r1;
    *dbt = -*bt * *bt;
  }
}

static void ust_gettau(const orc_eqp *p, double detF, double Je, double *tauM, double *tauC) {
  const double he = 0.5 * pow(Je, 1.0 / 3.0);
  const double rho0 = p->rho, Em = p->elM, nu = p->nu;
  const double mu = 0.5 * Em / (1.0 + nu);
  double c;
  if (iszero(nu - 0.5)) {
    c = sqrt(mu / rho0);
  } else {
    const double lam = 2.0 * mu * nu / (1.0 - 2.0 * nu);
    c = sqrt((lam + 2.0 * mu) / rho0);
  }
  *tauM = p->ctM * (he / c) * (detF / rho0);
  *tauC = p->ctC * (he * c) * (rho0 / detF);
}

void orc_elem_ustruct(const orc_eqp *p, const double xl[12], const double *al,
                      const double *yl, const double *dl, double lR[16], double lK[256],
                      double lKd[192]) {
  const int tD = p->tDof, s = p->s;
  double w4[4], N4[4][4], Nx[3][4], Je, ksix[3][3];
  tet4_gauss(w4, N4);
  gnn3k(xl, Nx, &Je, ksix);
  for (int k = 0; k < 16; k++) lR[k] = 0.0;
  for (int k = 0; k < 256; k++) lK[k] = 0.0;
  for (int k = 0; k < 192; k++) lKd[k] = 0.0;
  const double mu = p->visc;
  const double am = p->am, af = p->af * p->gam * p->dt, afm = af / am;
  const double r13 = 1.0 / 3.0, r23 = 2.0 / 3.0;
#define AL(c, a) al[(a) * tD + s + (c)]
#define YL(c, a) yl[(a) * tD + s + (c)]
#define DL(c, a) dl[(a) * tD + s + (c)]
#define LK(k, a, b) lK[((a) * 4 + (b)) * 16 + (k) - 1]
#define LKD(k, a, b) lKd[((a) * 4 + (b)) * 12 + (k) - 1]
  /* kinematics are constant on a tet4 */
  double vx[3][3] = {{0}}, F[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  for (int a = 0; a < 4; a++)
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        vx[i][j] += Nx[j][a] * YL(i, a);
        M3(F, i, j) += Nx[j][a] * DL(i, a);
      }
  const double Jac = det3(F);
  double Fi[9];
  inv3(F, Fi);
  /* ---- Gauss integration 1: momentum, USTRUCT3D_M (F/USTRUCT.f:205-612) */
  for (int g = 0; g < 4; g++) {
    const double w = w4[g] * Je;
    const double *Nw = N4[g];
    double vd[3] = {-p->fb[0], -p->fb[1], -p->fb[2]};
    for (int a = 0; a < 4; a++)
      for (int i = 0; i < 3; i++) vd[i] = vd[i] + Nw[a] * AL(i, a);
    double pr = 0.0, pd = 0.0;
    for (int a = 0; a < 4; a++) {
      pr = pr + Nw[a] * YL(3, a);
      pd = pd + Nw[a] * AL(3, a);
    }
    /* GETPK2CCdev = GETPK2CC's neo-Hookean isochoric part (Kpen = 0) */
    double Siso[9], Dm[36];
    orc_pk2cc_nhk(p->C10, 0.0, F, Siso, Dm);
    const double Ja = 1.0;
    /* viscous contribution */
    double VxFi[3][3], ddev[3][3], Svis[9];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        double t = 0.0;
        for (int k = 0; k < 3; k++) t += vx[i][k] * M3(Fi, k, j);
        VxFi[i][j] = t;
      }
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) ddev[i][j] = 0.5 * (VxFi[i][j] + VxFi[j][i]);
    {
      const double tr = (ddev[0][0] + ddev[1][1] + ddev[2][2]) / 3.0;
      for (int i = 0; i < 3; i++) ddev[i][i] -= tr;
    }
    {
      double tmp[3][3];
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
          double t = 0.0;
          for (int k = 0; k < 3; k++) t += ddev[i][k] * M3(Fi, j, k);
          tmp[i][j] = t;
        }
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
          double t = 0.0;
          for (int k = 0; k < 3; k++) t += M3(Fi, i, k) * tmp[k][j];
          M3(Svis, i, j) = 2.0 * mu * Jac * t;
        }
    }
    double rho, beta, drho, dbeta;
    ust_gvolpen(p, pr, Ja, &rho, &beta, &drho, &dbeta);
    double tauM, tauC;
    ust_gettau(p, Jac, Je, &tauM, &tauC);
    for (int k = 0; k < 9; k++) Siso[k] += Svis[k];
    double Pdev[9];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        double t = 0.0;
        for (int k = 0; k < 3; k++) t += M3(F, i, k) * M3(Siso, k, j);
        M3(Pdev, i, j) = t;
      }
    double NxFi[3][4];
    for (int a = 0; a < 4; a++)
      for (int i = 0; i < 3; i++)
        NxFi[i][a] = Nx[0][a] * M3(Fi, 0, i) + Nx[1][a] * M3(Fi, 1, i) + Nx[2][a] * M3(Fi, 2, i);
    const double rC = beta * pd + VxFi[0][0] + VxFi[1][1] + VxFi[2][2];
    const double rCl = -pr + tauC * rC;
    for (int a = 0; a < 4; a++)
      for (int i = 0; i < 3; i++) {
        const double T1 = Jac * rho * vd[i] * Nw[a];
        const double T2 = M3(Pdev, i, 0) * Nx[0][a] + M3(Pdev, i, 1) * Nx[1][a] +
                          M3(Pdev, i, 2) * Nx[2][a];
        const double T3 = Jac * rCl * NxFi[i][a];
        lR[a * 4 + i] = lR[a * 4 + i] + w * (T1 + T2 + T3);
      }
    /* Bm(6,3,a): rows (11, 22, 33, 12, 23, 31) of the strain variation */
    double Bm[6][3][4];
    for (int a = 0; a < 4; a++)
      for (int c = 0; c < 3; c++) {
        Bm[0][c][a] = Nx[0][a] * M3(F, c, 0);
        Bm[1][c][a] = Nx[1][a] * M3(F, c, 1);
        Bm[2][c][a] = Nx[2][a] * M3(F, c, 2);
        Bm[3][c][a] = Nx[0][a] * M3(F, c, 1) + M3(F, c, 0) * Nx[1][a];
        Bm[4][c][a] = Nx[1][a] * M3(F, c, 2) + M3(F, c, 1) * Nx[2][a];
        Bm[5][c][a] = Nx[2][a] * M3(F, c, 0) + M3(F, c, 2) * Nx[0][a];
      }
    double DdNx[3][4], VxNx[3][4];
    for (int a = 0; a < 4; a++)
      for (int i = 0; i < 3; i++) {
        DdNx[i][a] = ddev[i][0] * NxFi[0][a] + ddev[i][1] * NxFi[1][a] + ddev[i][2] * NxFi[2][a];
        VxNx[i][a] = VxFi[0][i] * NxFi[0][a] + VxFi[1][i] * NxFi[1][a] + VxFi[2][i] * NxFi[2][a];
      }
    for (int b = 0; b < 4; b++)
      for (int a = 0; a < 4; a++) {
        double NxSNx = 0.0;
        for (int i = 0; i < 3; i++)
          for (int j = 0; j < 3; j++) NxSNx += Nx[i][a] * M3(Siso, i, j) * Nx[j][b];
        double DBm[6][3];
        for (int I = 0; I < 6; I++)
          for (int c = 0; c < 3; c++) {
            double t = 0.0;
            for (int K = 0; K < 6; K++) t += Dm[I * 6 + K] * Bm[K][c][b];
            DBm[I][c] = t;
          }
        const double NxNx = NxFi[0][a] * NxFi[0][b] + NxFi[1][a] * NxFi[1][b] +
                            NxFi[2][a] * NxFi[2][b];
        /* dM_r/dV_c + af/am dM_r/dU_c, r, c = 0..2 (lKd k = 3r+c+1,
           lK k = 4r+c+1) */
        for (int r = 0; r < 3; r++)
          for (int c = 0; c < 3; c++) {
            double BtDB = 0.0;
            for (int I = 0; I < 6; I++) BtDB += Bm[I][r][a] * DBm[I][c];
            const double T1 = Jac * rho * vd[r] * Nw[a] * NxFi[c][b];
            const double T2 = -tauC * Jac * NxFi[r][a] * VxNx[c][b];
            const double T3 = (r == c) ? 0.0
                                       : Jac * rCl * (NxFi[r][a] * NxFi[c][b] - NxFi[c][a] * NxFi[r][b]);
            const double Tv = (2.0 * (DdNx[r][a] * NxFi[c][b] - DdNx[r][b] * NxFi[c][a]) -
                               (NxNx * VxFi[r][c] + NxFi[r][b] * VxNx[c][a] -
                                r23 * NxFi[r][a] * VxNx[c][b])) * mu * Jac;
            const double Ku = w * af * (T1 + T2 + T3 + Tv + BtDB + ((r == c) ? NxSNx : 0.0));
            LKD(3 * r + c + 1, a, b) += Ku;
            double T2k, Tvk;
            if (r == c) {
              const double T1m = am * Jac * rho * Nw[a] * Nw[b];
              T2k = T1m + af * Jac * tauC * rho * NxFi[r][a] * NxFi[r][b];
              Tvk = af * mu * Jac * (r13 * NxFi[r][a] * NxFi[r][b] + NxNx);
            } else {
              T2k = af * Jac * tauC * rho * NxFi[r][a] * NxFi[c][b];
              Tvk = af * mu * Jac * (NxFi[c][a] * NxFi[r][b] - r23 * NxFi[r][a] * NxFi[c][b]);
            }
            LK(4 * r + c + 1, a, b) += w * (T2k + Tvk) + afm * Ku;
          }
      }
    for (int b = 0; b < 4; b++)
      for (int a = 0; a < 4; a++) {
        const double T1 = am * tauC * beta + af * (tauC * dbeta * pd - 1.0);
        for (int r = 0; r < 3; r++) {
          const double T2 = T1 * NxFi[r][a] * Nw[b] + af * drho * vd[r] * Nw[a] * Nw[b];
          LK(4 * r + 4, a, b) += w * Jac * T2;
        }
      }
  }
  /* ---- Gauss integration 2: continuity, USTRUCT3D_C (F/USTRUCT.f:880-1102) */
  const double ctV = 36.0;
  for (int g = 0; g < 4; g++) {
    const double w = w4[g] * Je;
    const double *Nw = N4[g], *Nq = N4[g];
    double vd[3] = {-p->fb[0], -p->fb[1], -p->fb[2]};
    for (int a = 0; a < 4; a++)
      for (int i = 0; i < 3; i++) vd[i] = vd[i] + Nw[a] * AL(i, a);
    double pr = 0.0, pd = 0.0, px[3] = {0, 0, 0};
    for (int a = 0; a < 4; a++) {
      pr = pr + Nq[a] * YL(3, a);
      pd = pd + Nq[a] * AL(3, a);
      for (int i = 0; i < 3; i++) px[i] = px[i] + Nx[i][a] * YL(3, a);
    }
    double rho, beta, drho, dbeta;
    ust_gvolpen(p, pr, 1.0, &rho, &beta, &drho, &dbeta);
    double tauM, tauC;
    ust_gettau(p, Jac, Je, &tauM, &tauC);
    {
      double Kx[3][3], tmp[3][3];
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
          double t = 0.0;
          for (int k = 0; k < 3; k++) t += ksix[i][k] * M3(Fi, k, j);
          tmp[i][j] = t;
        }
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
          double t = 0.0;
          for (int k = 0; k < 3; k++) t += M3(Fi, k, i) * tmp[k][j];
          Kx[i][j] = t;
        }
      double tauV = 0.0;
      for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) tauV += Kx[i][j] * Kx[i][j];
      tauV = ctV * mu * mu * tauV;
      tauM = 1.0 / sqrt(tauV + pow(1.0 / tauM, 2.0));
    }
    double NwxFi[3][4], VxFi[3][3], PxFi[3];
    for (int a = 0; a < 4; a++)
      for (int i = 0; i < 3; i++)
        NwxFi[i][a] = Nx[0][a] * M3(Fi, 0, i) + Nx[1][a] * M3(Fi, 1, i) + Nx[2][a] * M3(Fi, 2, i);
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++)
        VxFi[i][j] = vx[i][0] * M3(Fi, 0, j) + vx[i][1] * M3(Fi, 1, j) + vx[i][2] * M3(Fi, 2, j);
    for (int i = 0; i < 3; i++) PxFi[i] = px[0] * M3(Fi, 0, i) + px[1] * M3(Fi, 1, i) + px[2] * M3(Fi, 2, i);
    const double rC = beta * pd + VxFi[0][0] + VxFi[1][1] + VxFi[2][2];
    double rM[3];
    for (int i = 0; i < 3; i++) rM[i] = rho * vd[i] + PxFi[i];
    double rMNqx[4], rMNwx[4], VxNwx[3][4];
    for (int a = 0; a < 4; a++) {
      rMNqx[a] = rM[0] * NwxFi[0][a] + rM[1] * NwxFi[1][a] + rM[2] * NwxFi[2][a];
      lR[a * 4 + 3] = lR[a * 4 + 3] + w * Jac * (Nq[a] * rC + tauM * rMNqx[a]);
    }
    for (int a = 0; a < 4; a++) {
      rMNwx[a] = rM[0] * NwxFi[0][a] + rM[1] * NwxFi[1][a] + rM[2] * NwxFi[2][a];
      for (int i = 0; i < 3; i++)
        VxNwx[i][a] = VxFi[0][i] * NwxFi[0][a] + VxFi[1][i] * NwxFi[1][a] + VxFi[2][i] * NwxFi[2][a];
    }
    for (int b = 0; b < 4; b++)
      for (int a = 0; a < 4; a++) {
        const double NxNx = NwxFi[0][a] * NwxFi[0][b] + NwxFi[1][a] * NwxFi[1][b] +
                            NwxFi[2][a] * NwxFi[2][b];
        for (int c = 0; c < 3; c++) {
          const double T1 = Nq[a] * (rC * NwxFi[c][b] - VxNwx[c][b]);
          const double T2 = tauM * (rMNqx[a] * NwxFi[c][b] - rMNwx[b] * NwxFi[c][a]);
          const double T3 = -tauM * NxNx * PxFi[c];
          const double Ku = w * af * Jac * (T1 + T2 + T3);
          LKD(10 + c, a, b) += Ku;
          const double T2k = (am * tauM * rho) * NwxFi[c][a] * Nw[b] + af * Nq[a] * NwxFi[c][b];
          LK(13 + c, a, b) += w * Jac * T2k + afm * Ku;
        }
      }
    for (int b = 0; b < 4; b++)
      for (int a = 0; a < 4; a++) {
        const double NxNx = NwxFi[0][a] * NwxFi[0][b] + NwxFi[1][a] * NwxFi[1][b] +
                            NwxFi[2][a] * NwxFi[2][b];
        const double T1 = (am * beta + af * dbeta * pd) * Nq[a] * Nq[b];
        const double T2 = NwxFi[0][a] * vd[0] + NwxFi[1][a] * vd[1] + NwxFi[2][a] * vd[2];
        const double T3 = T1 + af * tauM * (NxNx + drho * T2 * Nq[b]);
        LK(16, a, b) += w * Jac * T3;
      }
  }
#undef AL
#undef YL
#undef DL
#undef LK
#undef LKD
}

static int ust_elem_assemble(const orc_eqp *p, int e, const int *IEN, const double *x,
                             const double *Ag, const double *Yg, const double *Dg,
                             const int *rowPtr, const int *colPtr, double *R, double *Val,
                             double *Kd);

int orc_assemble_ustruct(const orc_eqp *p, int nNo, int nEl, const int *IEN,
                         const double *x, const double *Ag, const double *Yg,
                         const double *Dg, const int *rowPtr, const int *colPtr,
                         double *R, double *Val, double *Kd) {
  (void)nNo;
  if (p->tDof > 16 || p->dof != 4) return -1;
  for (int e = 0; e < nEl; e++) {
    const int rc = ust_elem_assemble(p, e, IEN, x, Ag, Yg, Dg, rowPtr, colPtr, R, Val, Kd);
    if (rc) return rc;
  }
  return 0;
}

/* The same colour by colour with OpenMP (the multi-core CPU baseline). */
int orc_assemble_ustruct_colored(const orc_eqp *p, int nEl, const int *IEN, const double *x,
                                 const double *Ag, const double *Yg, const double *Dg,
                                 const int *rowPtr, const int *colPtr, double *R, double *Val,
                                 double *Kd, int ncolor, const int *color_off,
                                 const int *order) {
  (void)nEl;
  if (p->tDof > 16 || p->dof != 4) return -1;
  int bad = 0;
  for (int c = 0; c < ncolor; c++) {
#pragma omp parallel for schedule(static) num_threads(orc_get_threads()) reduction(| : bad)
    for (int k = color_off[c]; k < color_off[c + 1]; k++)
      bad |= ust_elem_assemble(p, order[k], IEN, x, Ag, Yg, Dg, rowPtr, colPtr, R, Val, Kd) != 0;
  }
  return bad ? -3 : 0;
}

static int ust_elem_assemble(const orc_eqp *p, int e, const int *IEN, const double *x,
                             const double *Ag, const double *Yg, const double *Dg,
                             const int *rowPtr, const int *colPtr, double *R, double *Val,
                             double *Kd) {
  const int tD = p->tDof;
  double xl[12], al[4 * 16], yl[4 * 16], dl[4 * 16], lR[16], lK[256], lKd[192];
  {
    int ptr[4];
    for (int a = 0; a < 4; a++) {
      const int Ac = IEN[(size_t)e * 4 + a];
      ptr[a] = Ac;
      for (int i = 0; i < 3; i++) xl[a * 3 + i] = x[(size_t)Ac * 3 + i];
      for (int i = 0; i < tD; i++) {
        al[a * tD + i] = Ag[(size_t)Ac * tD + i];
        yl[a * tD + i] = Yg[(size_t)Ac * tD + i];
        dl[a * tD + i] = Dg[(size_t)Ac * tD + i];
      }
    }
    orc_elem_ustruct(p, xl, al, yl, dl, lR, lK, lKd);
    /* USTRUCT_DOASSEM with the identity node map of one mesh: every entry
       of lK goes to Val, every entry of lKd to Kd, at the (a,b) block */
    for (int a = 0; a < 4; a++) {
      const int rowN = ptr[a];
      for (int i = 0; i < 4; i++) R[(size_t)rowN * 4 + i] += lR[a * 4 + i];
      for (int b = 0; b < 4; b++) {
        const int colN = ptr[b];
        int left = rowPtr[rowN], right = rowPtr[rowN + 1] - 1, q = -1;
        while (left <= right) {
          const int mid = (left + right) / 2;
          if (colPtr[mid] == colN) {
            q = mid;
            break;
          }
          if (colPtr[mid] < colN) left = mid + 1;
          else right = mid - 1;
        }
        if (q < 0) return -3;
        for (int k = 0; k < 16; k++) Val[(size_t)q * 16 + k] += lK[(a * 4 + b) * 16 + k];
        for (int k = 0; k < 12; k++) Kd[(size_t)q * 12 + k] += lKd[(a * 4 + b) * 12 + k];
      }
    }
  }
  return 0;
}
