// Element assembly for tet4 meshes: HEATS (Code/Source/svFSI/HEATS.f:39-159)
// and STRUCT with the neo-Hookean + ST91 material
// (Code/Source/svFSI/STRUCT.f:39-496, MATMODELS.f:41-150,539-564,1588-1647),
// scattered into block CSR as DOASSEM does (Code/Source/svFSI/LHSA.f:266-298).
//
// GB300 design: the binary search of DOASSEM is replaced by a precomputed
// element -> CSR position map (16 int32 per tet); the RMW scatter is made
// race-free and deterministic by a greedy node-conflict colouring (one
// launch per colour, elements stored in colour order).  One thread owns one
// element; the residual is always FP64, the tangent is FP64 (drop-in) or
// FP32 (mixed precision, with det F, S and P kept in FP64).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "gsls_internal.cuh"

struct gsls_mesh {
  gsls_lhs *lhs = nullptr;
  int nEl = 0, nNo = 0, ncolors = 0;
  std::vector<int> color_off;     // ncolors + 1, offsets into colour-ordered elements
  std::vector<int> perm;          // colour order -> original element index
  std::vector<int> h_ien;         // 0-based, colour order, 4 per element
  gsls::DevBuf d_ien;             // int4 per element (colour order)
  gsls::DevBuf d_map;             // int4[4] per element: CSR position of (a,b)
  gsls::DevBuf d_x;               // double nNo*3
  gsls::DevBuf d_eparam;          // double per element (colour order)
  gsls::DevBuf d_err;             // int error word
  const double *eparam_src = nullptr;
  bool has_eparam = false;
};

namespace gsls {

constexpr int kAsmThreads = 128;

// tet4 Gauss rule and shape functions (Code/Source/svFSI/NN.f:268-275,
// 654-671): 4 points, w = 1/24.
struct Tet4Rule {
  double N[4][4];  // N[g][a]
  double w;
};
__constant__ Tet4Rule c_rule;

static Tet4Rule make_rule() {
  Tet4Rule r;
  const double s = (5.0 + 3.0 * sqrt(5.0)) / 20.0;
  const double t = (5.0 - sqrt(5.0)) / 20.0;
  const double xi[4][3] = {{s, t, t}, {t, s, t}, {t, t, s}, {t, t, t}};
  for (int g = 0; g < 4; g++) {
    r.N[g][0] = xi[g][0];
    r.N[g][1] = xi[g][1];
    r.N[g][2] = xi[g][2];
    r.N[g][3] = 1.0 - xi[g][0] - xi[g][1] - xi[g][2];
  }
  r.w = 1.0 / 24.0;
  return r;
}

// GNN for tet4 (Code/Source/svFSI/NN.f:1469-1565, insd = 3):
// Nxi = [[1,0,0,-1],[0,1,0,-1],[0,0,1,-1]], so xXi(:,k) = x_k - x_4.
__device__ __forceinline__ void gnn_tet4(const double xl[4][3], double Nx[3][4], double &Jac) {
  double xXi[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int k = 0; k < 3; k++) xXi[i][k] = xl[k][i] - xl[3][i];
  const double J = xXi[0][0] * xXi[1][1] * xXi[2][2] + xXi[0][1] * xXi[1][2] * xXi[2][0] +
                   xXi[0][2] * xXi[1][0] * xXi[2][1] - xXi[0][0] * xXi[1][2] * xXi[2][1] -
                   xXi[0][1] * xXi[1][0] * xXi[2][2] - xXi[0][2] * xXi[1][1] * xXi[2][0];
  double xiX[3][3];
  xiX[0][0] = (xXi[1][1] * xXi[2][2] - xXi[1][2] * xXi[2][1]) / J;
  xiX[0][1] = (xXi[2][1] * xXi[0][2] - xXi[2][2] * xXi[0][1]) / J;
  xiX[0][2] = (xXi[0][1] * xXi[1][2] - xXi[0][2] * xXi[1][1]) / J;
  xiX[1][0] = (xXi[1][2] * xXi[2][0] - xXi[1][0] * xXi[2][2]) / J;
  xiX[1][1] = (xXi[2][2] * xXi[0][0] - xXi[2][0] * xXi[0][2]) / J;
  xiX[1][2] = (xXi[0][2] * xXi[1][0] - xXi[0][0] * xXi[1][2]) / J;
  xiX[2][0] = (xXi[1][0] * xXi[2][1] - xXi[1][1] * xXi[2][0]) / J;
  xiX[2][1] = (xXi[2][0] * xXi[0][1] - xXi[2][1] * xXi[0][0]) / J;
  xiX[2][2] = (xXi[0][0] * xXi[1][1] - xXi[0][1] * xXi[1][0]) / J;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    Nx[i][0] = xiX[0][i];
    Nx[i][1] = xiX[1][i];
    Nx[i][2] = xiX[2][i];
    Nx[i][3] = -xiX[0][i] - xiX[1][i] - xiX[2][i];
  }
  Jac = J;
}

struct AsmArgs {
  int nColorEl, el0;
  int tDof, s;
  double am, af, beta, gam, dt;
  double rho, cond, src;
  double C10, Kpen, visc, dmp;
  double fb[3];
  const int4 *ien;
  const int4 *map;  // 4 int4 per element: map[e*4 + a] = (b0..b3)
  const double *x;
  const double *Ag, *Yg, *Dg;
  const double *eparam;
  double *R;
  void *Val;
  int *err;
};

// ---------------------------------------------------------------------------
// HEATS3D (one tet per thread)
template <class VT>
__global__ void __launch_bounds__(kAsmThreads) k_asm_heats(AsmArgs A) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= A.nColorEl) return;
  const int e = A.el0 + t;
  const int4 nd = A.ien[e];
  const int n4[4] = {nd.x, nd.y, nd.z, nd.w};
  double xl[4][3], al[4], yl[4];
#pragma unroll
  for (int a = 0; a < 4; a++) {
#pragma unroll
    for (int i = 0; i < 3; i++) xl[a][i] = A.x[(size_t)n4[a] * 3 + i];
    al[a] = A.Ag[(size_t)n4[a] * A.tDof + A.s];
    yl[a] = A.Yg[(size_t)n4[a] * A.tDof + A.s];
  }
  double Nx[3][4], Jac;
  gnn_tet4(xl, Nx, Jac);
  if (!(Jac != 0.0) || !isfinite(Jac)) atomicOr(A.err, 1);
  const double nu = A.eparam ? A.eparam[e] : A.cond;
  const double T1 = A.af * A.gam * A.dt;
  const double amd = A.am * A.rho / T1;
  using AT = VT;
  double lR[4] = {0, 0, 0, 0};
  AT lK[16];
#pragma unroll
  for (int k = 0; k < 16; k++) lK[k] = AT(0);
  const AT NxNx_scale = AT(nu);
#pragma unroll
  for (int g = 0; g < 4; g++) {
    const double w = c_rule.w * Jac;
    const double wl = w * T1;
    double Td = -A.src, Tx0 = 0, Tx1 = 0, Tx2 = 0;
#pragma unroll
    for (int a = 0; a < 4; a++) {
      const double N = c_rule.N[g][a];
      Td = Td + N * al[a];
      Tx0 = Tx0 + Nx[0][a] * yl[a];
      Tx1 = Tx1 + Nx[1][a] * yl[a];
      Tx2 = Tx2 + Nx[2][a] * yl[a];
    }
    Td = Td * A.rho;
#pragma unroll
    for (int a = 0; a < 4; a++) {
      const double Na = c_rule.N[g][a];
      lR[a] = lR[a] + w * (Na * Td + (Nx[0][a] * Tx0 + Nx[1][a] * Tx1 + Nx[2][a] * Tx2) * nu);
#pragma unroll
      for (int b = 0; b < 4; b++) {
        const AT Nb = AT(c_rule.N[g][b]);
        const AT dd = AT(Nx[0][a]) * AT(Nx[0][b]) + AT(Nx[1][a]) * AT(Nx[1][b]) +
                      AT(Nx[2][a]) * AT(Nx[2][b]);
        lK[a * 4 + b] = lK[a * 4 + b] + AT(wl) * (AT(Na) * Nb * AT(amd) + NxNx_scale * dd);
      }
    }
  }
  VT *Val = reinterpret_cast<VT *>(A.Val);
#pragma unroll
  for (int a = 0; a < 4; a++) {
    A.R[n4[a]] += lR[a];
    const int4 m = A.map[(size_t)e * 4 + a];
    Val[m.x] += VT(lK[a * 4 + 0]);
    Val[m.y] += VT(lK[a * 4 + 1]);
    Val[m.z] += VT(lK[a * 4 + 2]);
    Val[m.w] += VT(lK[a * 4 + 3]);
  }
}

// ---------------------------------------------------------------------------
// STRUCT3D with neo-Hookean (GETPK2CC stIso_nHook) + ST91 (GETSVOLP).
template <class T>
__device__ __forceinline__ T det3(const T F[3][3]) {
  return F[0][0] * (F[1][1] * F[2][2] - F[1][2] * F[2][1]) -
         F[0][1] * (F[1][0] * F[2][2] - F[1][2] * F[2][0]) +
         F[0][2] * (F[1][0] * F[2][1] - F[1][1] * F[2][0]);
}
template <class T>
__device__ __forceinline__ void inv3(const T A[3][3], T B[3][3]) {
  const T d = det3(A);
  B[0][0] = (A[1][1] * A[2][2] - A[1][2] * A[2][1]) / d;
  B[0][1] = (A[0][2] * A[2][1] - A[0][1] * A[2][2]) / d;
  B[0][2] = (A[0][1] * A[1][2] - A[0][2] * A[1][1]) / d;
  B[1][0] = (A[1][2] * A[2][0] - A[1][0] * A[2][2]) / d;
  B[1][1] = (A[0][0] * A[2][2] - A[0][2] * A[2][0]) / d;
  B[1][2] = (A[0][2] * A[1][0] - A[0][0] * A[1][2]) / d;
  B[2][0] = (A[1][0] * A[2][1] - A[1][1] * A[2][0]) / d;
  B[2][1] = (A[0][1] * A[2][0] - A[0][0] * A[2][1]) / d;
  B[2][2] = (A[0][0] * A[1][1] - A[0][1] * A[1][0]) / d;
}

__device__ __forceinline__ int vo(int I, int k) {
  // Voigt pairs 11,22,33,12,23,31 (CCTOVOIGT)
  const int p0[6] = {0, 1, 2, 0, 1, 2};
  const int p1[6] = {0, 1, 2, 1, 2, 0};
  return k == 0 ? p0[I] : p1[I];
}

template <class VT>
__global__ void __launch_bounds__(kAsmThreads) k_asm_struct(AsmArgs A) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= A.nColorEl) return;
  using AT = VT;  // tangent precision
  const int e = A.el0 + t;
  const int4 nd = A.ien[e];
  const int n4[4] = {nd.x, nd.y, nd.z, nd.w};
  const int tD = A.tDof, s0 = A.s;
  double xl[4][3];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int i = 0; i < 3; i++) xl[a][i] = A.x[(size_t)n4[a] * 3 + i];
  double Nx[3][4], Jac;
  gnn_tet4(xl, Nx, Jac);
  if (!(Jac != 0.0) || !isfinite(Jac)) atomicOr(A.err, 1);

  // F, velocity gradient, inertia (per Gauss point sums handled below)
  double F[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  double vx[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  double ala[4][3], yla[4][3];
#pragma unroll
  for (int a = 0; a < 4; a++) {
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const size_t k = (size_t)n4[a] * tD + s0 + c;
      const double d = A.Dg[k];
      ala[a][c] = A.Ag[k];
      yla[a][c] = A.Yg[k];
#pragma unroll
      for (int m = 0; m < 3; m++) {
        F[c][m] += Nx[m][a] * d;
        vx[c][m] += Nx[m][a] * yla[a][c];
      }
    }
  }
  const double rho = A.rho, mu = A.visc, dmp = A.dmp;
  const double afu = A.af * A.beta * A.dt * A.dt;
  const double afv = A.af * A.gam * A.dt;
  const double amd = A.am * rho + afv * dmp;
  const double C10 = A.eparam ? A.eparam[e] : A.C10;

  // ---- material (FP64): J, C, Ci, S_iso, p, pl (GETPK2CC nHK + GETSVOLP)
  const double J = det3(F);
  double Fi[3][3];
  inv3(F, Fi);
  double C[3][3], Ci[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) C[i][j] = F[0][i] * F[0][j] + F[1][i] * F[1][j] + F[2][i] * F[2][j];
  inv3(C, Ci);
  const double J2d = pow(J, -2.0 / 3.0);
  double p = 0.0, pl = 0.0;
  if (A.Kpen != 0.0) {
    p = 0.5 * A.Kpen * (J - 1.0 / J);
    pl = A.Kpen * J;
  }
  const double g1 = 2.0 * C10;
  const double r1 = J2d * (g1 * (C[0][0] + C[1][1] + C[2][2])) / 3.0;
  double Siso[3][3], S[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      Siso[i][j] = J2d * (i == j ? g1 : 0.0) - r1 * Ci[i][j];
      S[i][j] = Siso[i][j] + p * J * Ci[i][j];
    }
  // ---- viscous stress (Code/Source/svFSI/STRUCT.f:258-269)
  double VxFi[3][3], ddev[3][3];
  const bool visc = (mu != 0.0);
  if (visc) {
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) VxFi[i][j] = vx[i][0] * Fi[0][j] + vx[i][1] * Fi[1][j] + vx[i][2] * Fi[2][j];
    double tr = 0.0;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) ddev[i][j] = 0.5 * (VxFi[i][j] + VxFi[j][i]);
    tr = (ddev[0][0] + ddev[1][1] + ddev[2][2]) / 3.0;
#pragma unroll
    for (int i = 0; i < 3; i++) ddev[i][i] -= tr;
    double tmp[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) tmp[i][j] = ddev[i][0] * Fi[j][0] + ddev[i][1] * Fi[j][1] + ddev[i][2] * Fi[j][2];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++)
        S[i][j] += 2.0 * mu * J * (Fi[i][0] * tmp[0][j] + Fi[i][1] * tmp[1][j] + Fi[i][2] * tmp[2][j]);
  }
  // ---- residual (FP64)
  double P[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) P[i][j] = F[i][0] * S[0][j] + F[i][1] * S[1][j] + F[i][2] * S[2][j];
  const double w = c_rule.w * Jac;
  double lR[4][3];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int c = 0; c < 3; c++) lR[a][c] = 0.0;
#pragma unroll
  for (int g = 0; g < 4; g++) {
    double ud[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      ud[c] = -rho * A.fb[c];
#pragma unroll
      for (int a = 0; a < 4; a++) ud[c] += c_rule.N[g][a] * (rho * ala[a][c] + dmp * yla[a][c]);
    }
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
      for (int c = 0; c < 3; c++)
        lR[a][c] += w * (c_rule.N[g][a] * ud[c] + Nx[0][a] * P[c][0] + Nx[1][a] * P[c][1] +
                         Nx[2][a] * P[c][2]);
  }
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int c = 0; c < 3; c++) A.R[(size_t)n4[a] * 3 + c] += lR[a][c];

  // ---- tangent (AT): Dm from CC in closed form
  AT Cia[3][3], Sia[3][3], Sa[3][3], Fa[3][3], Nxa[3][4];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      Cia[i][j] = AT(Ci[i][j]);
      Sia[i][j] = AT(Siso[i][j]);
      Sa[i][j] = AT(S[i][j]);
      Fa[i][j] = AT(F[i][j]);
    }
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int a = 0; a < 4; a++) Nxa[i][a] = AT(Nx[i][a]);
  const AT cA = AT(2.0 * (r1 - p * J));
  const AT cB = AT(pl * J - 2.0 * r1 / 3.0);
  const AT c23 = AT(-2.0 / 3.0);
  AT Dm[6][6];
#pragma unroll
  for (int I = 0; I < 6; I++)
#pragma unroll
    for (int K = I; K < 6; K++) {
      const int i = vo(I, 0), j = vo(I, 1), k = vo(K, 0), l = vo(K, 1);
      const AT v = c23 * (Cia[i][j] * Sia[k][l] + Sia[i][j] * Cia[k][l]) +
                   cA * (AT(0.5) * (Cia[i][k] * Cia[j][l] + Cia[i][l] * Cia[j][k])) +
                   cB * (Cia[i][j] * Cia[k][l]);
      Dm[I][K] = v;
      Dm[K][I] = v;
    }
  const AT Wsum = AT(4.0 * w);            // sum_g w_g
  const AT afuW = AT(afu) * Wsum;
  // viscous tangent quantities
  AT NxFi[4][3], DdNx[4][3], VxNx[4][3], VxFa[3][3];
  const AT rmu = AT(afu * mu * J), rmv = AT(afv * mu * J);
  if (visc) {
#pragma unroll
    for (int a = 0; a < 4; a++) {
#pragma unroll
      for (int c = 0; c < 3; c++)
        NxFi[a][c] = AT(Nx[0][a] * Fi[0][c] + Nx[1][a] * Fi[1][c] + Nx[2][a] * Fi[2][c]);
#pragma unroll
      for (int c = 0; c < 3; c++) {
        DdNx[a][c] = AT(ddev[c][0]) * NxFi[a][0] + AT(ddev[c][1]) * NxFi[a][1] + AT(ddev[c][2]) * NxFi[a][2];
        VxNx[a][c] = AT(VxFi[0][c]) * NxFi[a][0] + AT(VxFi[1][c]) * NxFi[a][1] + AT(VxFi[2][c]) * NxFi[a][2];
      }
    }
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) VxFa[i][j] = AT(VxFi[i][j]);
  }
  VT *Val = reinterpret_cast<VT *>(A.Val);
#pragma unroll 1
  for (int b = 0; b < 4; b++) {
    // Bm(:,:,b) (Code/Source/svFSI/STRUCT.f:300-318) and DBm = Dm Bm_b
    AT Bb[6][3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      Bb[0][c] = Nxa[0][b] * Fa[c][0];
      Bb[1][c] = Nxa[1][b] * Fa[c][1];
      Bb[2][c] = Nxa[2][b] * Fa[c][2];
      Bb[3][c] = Nxa[0][b] * Fa[c][1] + Fa[c][0] * Nxa[1][b];
      Bb[4][c] = Nxa[1][b] * Fa[c][2] + Fa[c][1] * Nxa[2][b];
      Bb[5][c] = Nxa[2][b] * Fa[c][0] + Fa[c][2] * Nxa[0][b];
    }
    AT DB[6][3];
#pragma unroll
    for (int I = 0; I < 6; I++)
#pragma unroll
      for (int c = 0; c < 3; c++) {
        AT acc = AT(0);
#pragma unroll
        for (int K = 0; K < 6; K++) acc += Dm[I][K] * Bb[K][c];
        DB[I][c] = acc;
      }
    AT SNxb[3];
#pragma unroll
    for (int m = 0; m < 3; m++) SNxb[m] = Sa[m][0] * Nxa[0][b] + Sa[m][1] * Nxa[1][b] + Sa[m][2] * Nxa[2][b];
#pragma unroll
    for (int a = 0; a < 4; a++) {
      AT Ba[6][3];
#pragma unroll
      for (int c = 0; c < 3; c++) {
        Ba[0][c] = Nxa[0][a] * Fa[c][0];
        Ba[1][c] = Nxa[1][a] * Fa[c][1];
        Ba[2][c] = Nxa[2][a] * Fa[c][2];
        Ba[3][c] = Nxa[0][a] * Fa[c][1] + Fa[c][0] * Nxa[1][a];
        Ba[4][c] = Nxa[1][a] * Fa[c][2] + Fa[c][1] * Nxa[2][a];
        Ba[5][c] = Nxa[2][a] * Fa[c][0] + Fa[c][2] * Nxa[0][a];
      }
      const AT NxSNx = Nxa[0][a] * SNxb[0] + Nxa[1][a] * SNxb[1] + Nxa[2][a] * SNxb[2];
      double Mab = 0.0;
#pragma unroll
      for (int g = 0; g < 4; g++) Mab += w * c_rule.N[g][a] * c_rule.N[g][b];
      const AT T1 = AT(amd * Mab) + afuW * NxSNx;
      AT blk[9];
#pragma unroll
      for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
          AT BmDBm = AT(0);
#pragma unroll
          for (int I = 0; I < 6; I++) BmDBm += Ba[I][r] * DB[I][c];
          AT v = afuW * BmDBm + ((r == c) ? T1 : AT(0));
          if (visc) {
            const AT NxNx = NxFi[a][0] * NxFi[b][0] + NxFi[a][1] * NxFi[b][1] + NxFi[a][2] * NxFi[b][2];
            AT Tv = (AT(2) * (DdNx[a][r] * NxFi[b][c] - DdNx[b][r] * NxFi[a][c]) -
                     (NxNx * VxFa[r][c] + NxFi[b][r] * VxNx[a][c] - AT(2.0 / 3.0) * NxFi[a][r] * VxNx[b][c])) *
                    rmu;
            if (r == c)
              Tv += (AT(1.0 / 3.0) * NxFi[a][r] * NxFi[b][r] + NxNx) * rmv;
            else
              Tv += (NxFi[a][c] * NxFi[b][r] - AT(2.0 / 3.0) * NxFi[a][r] * NxFi[b][c]) * rmv;
            v += Wsum * Tv;
          }
          blk[r * 3 + c] = v;
        }
      const int4 m4 = A.map[(size_t)e * 4 + a];
      const int pos = (b == 0) ? m4.x : (b == 1) ? m4.y : (b == 2) ? m4.z : m4.w;
      VT *dst = Val + (size_t)pos * 9;
#pragma unroll
      for (int k = 0; k < 9; k++) dst[k] += VT(blk[k]);
    }
  }
}

// ---------------------------------------------------------------------------
static int launch_assembly(gsls_mesh *m, const gsls_eq_params *p, const double *Ag,
                           const double *Yg, const double *Dg, double *R, void *Val,
                           int val_prec) {
  gsls_lhs *lhs = m->lhs;
  cudaStream_t st = lhs->stream;
  const int dof = p->dof;
  const size_t vbytes = (size_t)lhs->nnz * dof * dof * (val_prec == GSLS_PREC_MIXED ? 4 : 8);
  GSLS_CUDA(cudaMemsetAsync(R, 0, sizeof(double) * (size_t)lhs->nNo * dof, st));
  GSLS_CUDA(cudaMemsetAsync(Val, 0, vbytes, st));
  AsmArgs A;
  memset(&A, 0, sizeof(A));
  A.tDof = p->tDof;
  A.s = p->s;
  A.am = p->am;
  A.af = p->af;
  A.beta = p->beta;
  A.gam = p->gam;
  A.dt = p->dt;
  A.rho = p->rho;
  A.cond = p->cond;
  A.src = p->src;
  A.C10 = p->C10;
  A.Kpen = p->Kpen;
  A.visc = p->visc;
  A.dmp = p->dmp;
  for (int i = 0; i < 3; i++) A.fb[i] = p->fb[i];
  A.ien = m->d_ien.as<int4>();
  A.map = m->d_map.as<int4>();
  A.x = m->d_x.as<double>();
  A.Ag = Ag;
  A.Yg = Yg;
  A.Dg = Dg;
  A.eparam = m->has_eparam ? m->d_eparam.as<double>() : nullptr;
  A.R = R;
  A.Val = Val;
  A.err = m->d_err.as<int>();
  const bool mixed = (val_prec == GSLS_PREC_MIXED);
  for (int c = 0; c < m->ncolors; c++) {
    A.el0 = m->color_off[c];
    A.nColorEl = m->color_off[c + 1] - m->color_off[c];
    if (A.nColorEl <= 0) continue;
    const int nb = (A.nColorEl + kAsmThreads - 1) / kAsmThreads;
    if (p->phys == GSLS_PHYS_HEATS) {
      if (dof != 1) return GSLS_ERR_ARG;
      if (mixed)
        k_asm_heats<float><<<nb, kAsmThreads, 0, st>>>(A);
      else
        k_asm_heats<double><<<nb, kAsmThreads, 0, st>>>(A);
    } else if (p->phys == GSLS_PHYS_STRUCT) {
      if (dof != 3 || p->s + 3 > p->tDof || !Dg) return GSLS_ERR_ARG;
      if (mixed)
        k_asm_struct<float><<<nb, kAsmThreads, 0, st>>>(A);
      else
        k_asm_struct<double><<<nb, kAsmThreads, 0, st>>>(A);
    } else {
      set_error("assembly: physics not built in this version of the library");
      return GSLS_ERR_UNSUPPORTED;
    }
    GSLS_CHECK_LAUNCH();
  }
  return GSLS_OK;
}

int mesh_set_eparam(gsls_mesh *m, const double *eparam) {
  if (!eparam) {
    m->has_eparam = false;
    return GSLS_OK;
  }
  std::vector<double> v(m->nEl);
  for (int i = 0; i < m->nEl; i++) v[i] = eparam[m->perm[i]];
  GSLS_TRY(m->d_eparam.alloc(sizeof(double) * m->nEl));
  GSLS_CUDA(cudaMemcpyAsync(m->d_eparam.p, v.data(), sizeof(double) * m->nEl,
                            cudaMemcpyHostToDevice, m->lhs->stream));
  GSLS_CUDA(cudaStreamSynchronize(m->lhs->stream));
  m->has_eparam = true;
  return GSLS_OK;
}

int assemble_dev(gsls_mesh *m, const gsls_eq_params *p, const double *Ag, const double *Yg,
                 const double *Dg, double *R, void *Val, int val_prec) {
  return launch_assembly(m, p, Ag, Yg, Dg, R, Val, val_prec);
}

gsls_lhs *mesh_lhs(gsls_mesh *m) { return m->lhs; }

int mesh_coords_host(gsls_mesh *m, double *x) {
  GSLS_CUDA(cudaMemcpy(x, m->d_x.p, sizeof(double) * 3 * (size_t)m->nNo, cudaMemcpyDeviceToHost));
  return GSLS_OK;
}

int mesh_check_error(gsls_mesh *m) {
  int h = 0;
  GSLS_CUDA(cudaMemcpyAsync(&h, m->d_err.p, sizeof(int), cudaMemcpyDeviceToHost, m->lhs->stream));
  GSLS_CUDA(cudaStreamSynchronize(m->lhs->stream));
  if (h) {
    GSLS_CUDA(cudaMemsetAsync(m->d_err.p, 0, sizeof(int), m->lhs->stream));
    set_error("assembly: zero or non-finite element Jacobian");
    return GSLS_ERR_JAC;
  }
  return GSLS_OK;
}

}  // namespace gsls

using namespace gsls;

extern "C" {

int gsls_mesh_create(gsls_mesh **out, gsls_lhs *lhs, int nEl, int eNoN, const int *IEN, int nsd,
                     const double *x) {
  if (!out || !lhs || nEl <= 0 || !IEN || !x) return GSLS_ERR_ARG;
  if (eNoN != 4 || nsd != 3) {
    set_error("gsls_mesh_create: only tet4 meshes (eNoN = 4, nsd = 3) are supported");
    return GSLS_ERR_UNSUPPORTED;
  }
  static bool rule_set = false;
  if (!rule_set) {
    Tet4Rule r = make_rule();
    GSLS_CUDA(cudaMemcpyToSymbol(c_rule, &r, sizeof(r)));
    rule_set = true;
  }
  const int nNo = lhs->nNo;
  std::vector<int> ien((size_t)nEl * 4);
  for (size_t k = 0; k < ien.size(); k++) {
    ien[k] = IEN[k] - 1;
    if (ien[k] < 0 || ien[k] >= nNo) {
      set_error("gsls_mesh_create: element contains an out of bound node");
      return GSLS_ERR_ARG;
    }
  }
  // greedy colouring: elements sharing a node get different colours
  std::vector<uint64_t> used((size_t)nNo, 0ull);
  std::vector<std::vector<uint64_t>> used_hi;  // colours >= 64, rare
  std::vector<int> col(nEl);
  int ncol = 0;
  for (int e = 0; e < nEl; e++) {
    uint64_t forb = 0;
    for (int a = 0; a < 4; a++) forb |= used[ien[(size_t)e * 4 + a]];
    int c;
    if (~forb) {
      c = __builtin_ctzll(~forb);
    } else {
      // extend beyond 64 colours with explicit per-colour node sets
      c = 64;
      for (;; c++) {
        const int hi = c - 64;
        if ((int)used_hi.size() <= hi) used_hi.emplace_back((size_t)nNo, 0ull);
        bool ok = true;
        for (int a = 0; a < 4; a++)
          if (used_hi[hi][ien[(size_t)e * 4 + a]]) ok = false;
        if (ok) break;
      }
    }
    col[e] = c;
    if (c < 64) {
      for (int a = 0; a < 4; a++) used[ien[(size_t)e * 4 + a]] |= (1ull << c);
    } else {
      for (int a = 0; a < 4; a++) used_hi[c - 64][ien[(size_t)e * 4 + a]] = 1;
    }
    if (c + 1 > ncol) ncol = c + 1;
  }
  gsls_mesh *m = new gsls_mesh();
  m->lhs = lhs;
  m->nEl = nEl;
  m->nNo = nNo;
  m->ncolors = ncol;
  m->color_off.assign(ncol + 1, 0);
  for (int e = 0; e < nEl; e++) m->color_off[col[e] + 1]++;
  for (int c = 0; c < ncol; c++) m->color_off[c + 1] += m->color_off[c];
  m->perm.resize(nEl);
  {
    std::vector<int> fill(m->color_off.begin(), m->color_off.end() - 1);
    for (int e = 0; e < nEl; e++) m->perm[fill[col[e]]++] = e;
  }
  // colour-ordered IEN and element -> CSR map (DOASSEM's search, done once)
  m->h_ien.resize((size_t)nEl * 4);
  std::vector<int> map((size_t)nEl * 16);
  const std::vector<int> &rp = lhs->h_rowPtr, &cp = lhs->h_colPtr;
  for (int k = 0; k < nEl; k++) {
    const int e = m->perm[k];
    for (int a = 0; a < 4; a++) m->h_ien[(size_t)k * 4 + a] = ien[(size_t)e * 4 + a];
    for (int a = 0; a < 4; a++) {
      const int row = ien[(size_t)e * 4 + a];
      for (int b = 0; b < 4; b++) {
        const int colN = ien[(size_t)e * 4 + b];
        const int *lo = cp.data() + rp[row], *hi = cp.data() + rp[row + 1];
        const int *f = std::lower_bound(lo, hi, colN);
        if (f == hi || *f != colN) {
          set_error("gsls_mesh_create: element pair missing from the CSR pattern");
          delete m;
          return GSLS_ERR_ARG;
        }
        map[(size_t)k * 16 + a * 4 + b] = (int)(f - cp.data());
      }
    }
  }
  int rc;
  cudaStream_t st = lhs->stream;
  if ((rc = m->d_ien.alloc(sizeof(int) * 4 * (size_t)nEl)) ||
      (rc = m->d_map.alloc(sizeof(int) * 16 * (size_t)nEl)) ||
      (rc = m->d_x.alloc(sizeof(double) * 3 * (size_t)nNo)) || (rc = m->d_err.alloc(16))) {
    delete m;
    return rc;
  }
  cudaMemcpyAsync(m->d_ien.p, m->h_ien.data(), sizeof(int) * 4 * (size_t)nEl,
                  cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(m->d_map.p, map.data(), sizeof(int) * 16 * (size_t)nEl, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(m->d_x.p, x, sizeof(double) * 3 * (size_t)nNo, cudaMemcpyHostToDevice, st);
  cudaMemsetAsync(m->d_err.p, 0, 16, st);
  cudaError_t ce = cudaStreamSynchronize(st);
  if (ce != cudaSuccess) {
    delete m;
    return cuda_fail(ce, "mesh upload", __FILE__, __LINE__);
  }
  *out = m;
  return GSLS_OK;
}

int gsls_mesh_free(gsls_mesh *m) {
  if (!m) return GSLS_ERR_ARG;
  if (m->lhs) cudaStreamSynchronize(m->lhs->stream);
  delete m;
  return GSLS_OK;
}

int gsls_mesh_ncolors(const gsls_mesh *m) { return m ? m->ncolors : -1; }

int gsls_assemble_dev(gsls_mesh *m, const gsls_eq_params *p, const double *dAg,
                      const double *dYg, const double *dDg, double *dR, void *dVal,
                      int val_prec) {
  if (!m || !p || !dAg || !dYg || !dR || !dVal) return GSLS_ERR_ARG;
  GSLS_TRY(mesh_set_eparam(m, p->eparam));
  GSLS_TRY(assemble_dev(m, p, dAg, dYg, dDg, dR, dVal, val_prec));
  GSLS_CUDA(cudaStreamSynchronize(m->lhs->stream));
  return mesh_check_error(m);
}

int gsls_assemble(gsls_mesh *m, const gsls_eq_params *p, const double *Ag, const double *Yg,
                  const double *Dg, double *R, double *Val) {
  if (!m || !p || !Ag || !Yg || !R || !Val) return GSLS_ERR_ARG;
  gsls_lhs *lhs = m->lhs;
  const size_t ns = (size_t)lhs->nNo * p->tDof;
  const size_t nr = (size_t)lhs->nNo * p->dof, nv = (size_t)lhs->nnz * p->dof * p->dof;
  DevBuf a, y, d, r, v;
  GSLS_TRY(a.alloc(sizeof(double) * ns));
  GSLS_TRY(y.alloc(sizeof(double) * ns));
  GSLS_TRY(d.alloc(sizeof(double) * ns));
  GSLS_TRY(r.alloc(sizeof(double) * nr));
  GSLS_TRY(v.alloc(sizeof(double) * nv));
  cudaStream_t st = lhs->stream;
  GSLS_CUDA(cudaMemcpyAsync(a.p, Ag, sizeof(double) * ns, cudaMemcpyHostToDevice, st));
  GSLS_CUDA(cudaMemcpyAsync(y.p, Yg, sizeof(double) * ns, cudaMemcpyHostToDevice, st));
  if (Dg)
    GSLS_CUDA(cudaMemcpyAsync(d.p, Dg, sizeof(double) * ns, cudaMemcpyHostToDevice, st));
  else
    GSLS_CUDA(cudaMemsetAsync(d.p, 0, sizeof(double) * ns, st));
  int rc = gsls_assemble_dev(m, p, a.as<double>(), y.as<double>(), d.as<double>(), r.as<double>(),
                             v.p, GSLS_PREC_FP64);
  if (rc != GSLS_OK) return rc;
  GSLS_CUDA(cudaMemcpyAsync(R, r.p, sizeof(double) * nr, cudaMemcpyDeviceToHost, st));
  GSLS_CUDA(cudaMemcpyAsync(Val, v.p, sizeof(double) * nv, cudaMemcpyDeviceToHost, st));
  GSLS_CUDA(cudaStreamSynchronize(st));
  return GSLS_OK;
}

}  // extern "C"
