// STRUCT3D (Code/Source/svFSI/STRUCT.f:164-496) with the neo-Hookean
// isochoric model and the ST91 volumetric penalty (GETPK2CC stIso_nHook and
// GETSVOLP, Code/Source/svFSI/MATMODELS.f:136-150, 539-564) for one tet4
// per thread.  Included by gsls_assemble.cu (needs AsmArgs, c_rule,
// kAsmThreads).
//
// GB300 restatement (same quantities, fewer FP64 instructions):
//  * tet4 gradients are constant, so F, S, P and the tangent are computed
//    once per element; the Gauss-point sums only enter through the
//    constant tables sum_g N_a N_b and sum_g N_a (mass/inertia terms);
//  * inverses by adjugate with one division; J^(-2/3) by two Newton steps
//    of the inverse cube root z <- z (4 - J z^3)/3 from an FP32 start;
//  * the material tangent B_a^T Dm B_b is contracted in closed form: for
//    CC = -2/3 (Ci(x)S + S(x)Ci) + cA Ci(.)Ci + cB Ci(x)Ci (TEN_DYADPROD,
//    TEN_SYMMPROD) and B_a(r,I,J) = F(r,I) Nx(J,a),
//      K_ab(r,c) = -2/3 (u_a(r) s_b(c) + s_a(r) u_b(c))
//                  + cA/2 (d_rc Nx_a.Ci.Nx_b + u_b(r) u_a(c)) + cB u_a(r) u_b(c)
//    with u_a = F Ci Nx_a, s_a = F S_iso Nx_a (F Ci F^T = I);
//  * without viscosity the element matrix is symmetric (K_ba = K_ab^T),
//    so 10 of the 16 blocks are computed.
// Residual path (F, J, S, P, lR) is FP64; the tangent runs in VT.
#pragma once

namespace gsls {

template <class T>
__device__ __forceinline__ T adj_det3(const T A[3][3], T B[3][3]) {
  B[0][0] = A[1][1] * A[2][2] - A[1][2] * A[2][1];
  B[0][1] = A[0][2] * A[2][1] - A[0][1] * A[2][2];
  B[0][2] = A[0][1] * A[1][2] - A[0][2] * A[1][1];
  B[1][0] = A[1][2] * A[2][0] - A[1][0] * A[2][2];
  B[1][1] = A[0][0] * A[2][2] - A[0][2] * A[2][0];
  B[1][2] = A[0][2] * A[1][0] - A[0][0] * A[1][2];
  B[2][0] = A[1][0] * A[2][1] - A[1][1] * A[2][0];
  B[2][1] = A[0][1] * A[2][0] - A[0][0] * A[2][1];
  B[2][2] = A[0][0] * A[1][1] - A[0][1] * A[1][0];
  return A[0][0] * B[0][0] + A[0][1] * B[1][0] + A[0][2] * B[2][0];
}

// J^(-2/3) for J > 0: z = J^(-1/3) refined by Newton on f(z) = z^-3 - J
// (z <- z (4 - J z^3) / 3, quadratic convergence) from an FP32 estimate.
__device__ __forceinline__ double jm23(double J) {
  double z = (double)exp2f(-log2f((float)J) * (1.0f / 3.0f));
  z = z * (4.0 - J * z * z * z) * (1.0 / 3.0);
  z = z * (4.0 - J * z * z * z) * (1.0 / 3.0);
  return z * z;
}

// FP32 tangent: 3 blocks per SM fit in 168 registers (28 bytes of spill);
// the FP64 variant stays at its natural register count
template <class VT>
__global__ void __launch_bounds__(kAsmThreads, sizeof(VT) == 4 ? 3 : 1) k_asm_struct(AsmArgs A) {
  asm_colour_start();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= A.nColorEl) return;
  using AT = VT;
  const int e = A.el0 + t;
  const int4 nd = A.ien[e];
  const int n4[4] = {nd.x, nd.y, nd.z, nd.w};
  const int tD = A.tDof, s0 = A.s;

  // ---- geometry (GNN, FP64, precomputed per mesh)
  double Nx[3][4];
  const double w = c_rule.w * load_geo(A, e, Nx);

  // ---- kinematics (FP64)
  double F[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  double inert[4][3];  // rho*al + dmp*yl per node
  double vx[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  const double rho = A.rho, mu = A.visc, dmp = A.dmp;
  const bool visc = (mu != 0.0);
#pragma unroll
  for (int a = 0; a < 4; a++) {
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const size_t k = (size_t)n4[a] * tD + s0 + c;
      const double d = __ldg(A.Dg + k);
      const double y = __ldg(A.Yg + k);
      inert[a][c] = rho * __ldg(A.Ag + k) + dmp * y;
#pragma unroll
      for (int m = 0; m < 3; m++) F[c][m] += Nx[m][a] * d;
      if (visc) {
#pragma unroll
        for (int m = 0; m < 3; m++) vx[c][m] += Nx[m][a] * y;
      }
    }
  }
  double Fi[3][3];
  const double J = adj_det3(F, Fi);
  const double iJ = 1.0 / J;  // one FP64 division, also the ST91 pressure's 1/J
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) Fi[i][j] *= iJ;
  // Ci = C^-1 = Fi Fi^T, trC = |F|^2
  double Ci[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = i; j < 3; j++) {
      const double v = Fi[i][0] * Fi[j][0] + Fi[i][1] * Fi[j][1] + Fi[i][2] * Fi[j][2];
      Ci[i][j] = v;
      Ci[j][i] = v;
    }
  double trC = 0.0;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) trC += F[i][j] * F[i][j];
  const double C10 = A.eparam ? A.eparam[e] : A.C10;
  const double g1 = 2.0 * C10;
  const double J2d = jm23(J);
  double p = 0.0, pl = 0.0;
  if (A.Kpen != 0.0) {
    p = 0.5 * A.Kpen * (J - iJ);
    pl = A.Kpen * J;
  }
  const double r1 = J2d * g1 * trC / 3.0;
  double Siso[3][3], S[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      Siso[i][j] = (i == j ? J2d * g1 : 0.0) - r1 * Ci[i][j];
      S[i][j] = Siso[i][j] + p * J * Ci[i][j];
    }
  // viscous stress, Code/Source/svFSI/STRUCT.f:258-269
  double VxFi[3][3], ddev[3][3];
  if (visc) {
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) VxFi[i][j] = vx[i][0] * Fi[0][j] + vx[i][1] * Fi[1][j] + vx[i][2] * Fi[2][j];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) ddev[i][j] = 0.5 * (VxFi[i][j] + VxFi[j][i]);
    const double tr = (ddev[0][0] + ddev[1][1] + ddev[2][2]) / 3.0;
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

  // ---- residual (FP64): lR(a,c) = W Nx_a.P(c,:) + w sum_b M_ab inert_b - w rho fb N_a
  asm_colour_scatter();
  {
    double P[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) P[i][j] = F[i][0] * S[0][j] + F[i][1] * S[1][j] + F[i][2] * S[2][j];
    const double W = 4.0 * w;
#pragma unroll
    for (int a = 0; a < 4; a++) {
#pragma unroll
      for (int c = 0; c < 3; c++) {
        double m = -rho * A.fb[c] * c_rule.Ns[a];
#pragma unroll
        for (int b = 0; b < 4; b++) m += c_rule.M[a][b] * inert[b][c];
        const double v = W * (Nx[0][a] * P[c][0] + Nx[1][a] * P[c][1] + Nx[2][a] * P[c][2]) + w * m;
        A.R[(size_t)n4[a] * 3 + c] += v;
      }
    }
  }

  // ---- tangent (AT)
  const double afu = A.af * A.beta * A.dt * A.dt;
  const double afv = A.af * A.gam * A.dt;
  const double amd = A.am * rho + afv * dmp;
  const AT afuW = AT(afu * 4.0 * w);
  const AT kc1 = AT(-2.0 / 3.0);
  const AT kcA2 = AT(r1 - p * J);          // cA/2 with cA = 2 (r1 - p J)
  const AT kcB = AT(pl * J - 2.0 * r1 / 3.0);
  AT Fa[3][3], Cia[3][3], FCi[3][3], FSi[3][3], Sa[3][3], Nxa[3][4];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      Fa[i][j] = AT(F[i][j]);
      Cia[i][j] = AT(Ci[i][j]);
      Sa[i][j] = AT(S[i][j]);
    }
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int a = 0; a < 4; a++) Nxa[i][a] = AT(Nx[i][a]);
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      FCi[i][j] = Fa[i][0] * Cia[0][j] + Fa[i][1] * Cia[1][j] + Fa[i][2] * Cia[2][j];
      FSi[i][j] = Fa[i][0] * AT(Siso[0][j]) + Fa[i][1] * AT(Siso[1][j]) + Fa[i][2] * AT(Siso[2][j]);
    }
  AT u[4][3], sv[4][3], q[4][3], SN[4][3];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int r = 0; r < 3; r++) {
      u[a][r] = FCi[r][0] * Nxa[0][a] + FCi[r][1] * Nxa[1][a] + FCi[r][2] * Nxa[2][a];
      sv[a][r] = FSi[r][0] * Nxa[0][a] + FSi[r][1] * Nxa[1][a] + FSi[r][2] * Nxa[2][a];
      q[a][r] = Cia[r][0] * Nxa[0][a] + Cia[r][1] * Nxa[1][a] + Cia[r][2] * Nxa[2][a];
      SN[a][r] = Sa[r][0] * Nxa[0][a] + Sa[r][1] * Nxa[1][a] + Sa[r][2] * Nxa[2][a];
    }
  // viscous tangent quantities (STRUCT.f:336-356)
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
  const AT Wsum = AT(4.0 * w);
#pragma unroll
  for (int a = 0; a < 4; a++) {
    const int4 m4 = A.map[(size_t)e * 4 + a];
    const int pos[4] = {m4.x, m4.y, m4.z, m4.w};
#pragma unroll
    for (int b = 0; b < 4; b++) {
      if (!visc && b < a) continue;  // filled from the transposed (b,a) block
      const AT NCN = Nxa[0][a] * q[b][0] + Nxa[1][a] * q[b][1] + Nxa[2][a] * q[b][2];
      const AT NSN = Nxa[0][a] * SN[b][0] + Nxa[1][a] * SN[b][1] + Nxa[2][a] * SN[b][2];
      const AT diag = AT(amd * w * c_rule.M[a][b]) + afuW * (NSN + kcA2 * NCN);
      AT blk[9];
#pragma unroll
      for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
          AT v = kc1 * (u[a][r] * sv[b][c] + sv[a][r] * u[b][c]) + kcA2 * (u[b][r] * u[a][c]) +
                 kcB * (u[a][r] * u[b][c]);
          v = afuW * v + ((r == c) ? diag : AT(0));
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
      VT *dst = Val + (size_t)pos[b] * 9;
#pragma unroll
      for (int k = 0; k < 9; k++) dst[k] += VT(blk[k]);
      if (!visc && b > a) {
        // block (b,a) = block(a,b)^T
        const int4 mb = A.map[(size_t)e * 4 + b];
        const int pba = (a == 0) ? mb.x : (a == 1) ? mb.y : (a == 2) ? mb.z : mb.w;
        VT *dt = Val + (size_t)pba * 9;
#pragma unroll
        for (int r = 0; r < 3; r++)
#pragma unroll
          for (int c = 0; c < 3; c++) dt[r * 3 + c] += VT(blk[c * 3 + r]);
      }
    }
  }
}

}  // namespace gsls
