// FLUID3D_M + FLUID3D_C (Code/Source/svFSI/FLUID.f:192-560, 813-1084) for
// P1-P1 tet4 with VMS stabilisation, one element per thread, with the
// constant, Carreau-Yasuda or Casson viscosity of GETVISCOSITY
// (FLUID.f:1690-1739).  Included by gsls_assemble.cu (needs AsmArgs,
// c_rule, adj_det3, kAsmThreads).
//
// Same quantities as the reference, arranged for GB300:
//  * the momentum and continuity passes of CONSTRUCT_FLUID run over the same
//    four Gauss points with the same basis (GETTHOODFS, FS.f:270-286) and
//    write disjoint entries, so they are fused into one point loop;
//  * tet4 gradients are constant and the second derivatives vanish, so
//    uxx, d2u2, es_x, mu_x and rS are zero; the shear rate, mu and mu_g are
//    element constants, and the viscosity model adds
//    4 wl mu_g esNx_i(a) esNx_j(b) to Kuu (zero for constant viscosity);
//  * the residual (u, ud, p, tauM, tauC, tauB, up, rM, lR) is FP64 at every
//    Gauss point; the tangent runs in TT and is rebuilt per block (a,b) from
//    eleven per-point factors (tauM, tauC, tauB, u.Nx_a, up.Nx_a):
//      Kuu(i,j) = wl [4 mu Nx_i(b)Nx_j(a) + (sum tauC) Nx_i(a)Nx_j(b) + d_ij S_ab]
//      S_ab     = 4 mu Nx_a.Nx_b + rho amd M_ab
//                 + sum_g [rho^2 tauM uaNx_a (uNx_b + amd N_b)
//                          + rho N_a (uNx_b + upNx_b) + tauB upNx_a upNx_b]
//      Kup(i)   = -wl [Nx_i(a) Ns_b - rho Nx_i(b) sum_g tauM uaNx_a]
//      Kpu(j)   =  wl [Ns_a Nx_j(b) + rho Nx_j(a) sum_g tauM (uNx_b + amd N_b)]
//      Kpp      =  wl (sum tauM) Nx_a.Nx_b
//    which is the reference's per-point sum with updu = -rho uNx d_ij.
#pragma once

namespace gsls {

// GETVISCOSITY (FLUID.f:1690-1739) for the Carreau-Yasuda and Casson models:
// mu and mu_x = d mu / d gamma at shear rate gam (Casson raises gam to its
// threshold lam first)
__device__ __forceinline__ void visc_model(const AsmArgs &A, double &gam, double &mu,
                                           double &mu_x) {
  if (A.viscType == GSLS_VISC_CY) {
    const double mi = A.mu_f, mo = A.mu_o, lam = A.vlam, a = A.va, n = A.vn;
    double T1 = 1.0 + pow(lam * gam, a);
    double T2 = pow(T1, (n - 1.0) / a);
    mu = mi + (mo - mi) * T2;
    T1 = T2 / T1;
    T2 = pow(lam, a) * pow(gam, a - 1.0) * T1;
    mu_x = (mo - mi) * (n - 1.0) * T2;
  } else {
    const double mi = A.mu_f, lam = A.vlam;
    double mo;
    if (gam < lam) {
      mo = A.mu_o / sqrt(lam);
      gam = lam;
    } else {
      mo = A.mu_o / sqrt(gam);
    }
    mu = (mi + mo) * (mi + mo);
    mu_x = 2.0 * mo * (mo + mi) / gam;
  }
}

// NN: a shear-rate dependent viscosity (Carreau-Yasuda or Casson); the
// constant-viscosity kernel carries none of its terms
template <class TT, bool NN>
__global__ void __launch_bounds__(kAsmThreads) k_asm_fluid(AsmArgs A) {
  asm_colour_start();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= A.nColorEl) return;
  const int e = A.el0 + t;
  const int4 nd = A.ien[e];
  const int n4[4] = {nd.x, nd.y, nd.z, nd.w};
  const int tD = A.tDof, s0 = A.s;

  // ---- geometry (GNN with ks, FP64, precomputed per mesh): xiX(a,i) = Nx(i,a)
  double Nx[3][4], K[3][3];
  const double w = c_rule.w * load_geo(A, e, Nx);
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++)
      K[i][j] = Nx[i][0] * Nx[j][0] + Nx[i][1] * Nx[j][1] + Nx[i][2] * Nx[j][2];

  // ---- nodal values and element-constant gradients (FP64)
  double yl[4][4], al[4][3];
#pragma unroll
  for (int a = 0; a < 4; a++) {
    const size_t k = (size_t)n4[a] * tD + s0;
#pragma unroll
    for (int c = 0; c < 4; c++) yl[a][c] = __ldg(A.Yg + k + c);
#pragma unroll
    for (int c = 0; c < 3; c++) al[a][c] = __ldg(A.Ag + k + c);
  }
  double ux[3][3], px[3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
#pragma unroll
    for (int j = 0; j < 3; j++)
      ux[i][j] = Nx[i][0] * yl[0][j] + Nx[i][1] * yl[1][j] + Nx[i][2] * yl[2][j] + Nx[i][3] * yl[3][j];
    px[i] = Nx[i][0] * yl[0][3] + Nx[i][1] * yl[1][3] + Nx[i][2] * yl[2][3] + Nx[i][3] * yl[3][3];
  }
  const double divU = ux[0][0] + ux[1][1] + ux[2][2];
  double es[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) es[i][j] = ux[i][j] + ux[j][i];

  // shear rate (2 e_ij e_ij)^(1/2), FLUID.f:358-373, and the viscosity
  double mu = A.mu_f, mu_g = 0.0;
  if (NN) {
    double gam = 0.0;
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int i = 0; i < 3; i++) gam += es[i][j] * es[i][j];
    gam = sqrt(0.5 * gam);
    double mu_x;
    visc_model(A, gam, mu, mu_x);
    // ISZERO (MATFUN.f:763-780): |x| < eps^2
    mu_g = (fabs(gam) < 4.930380657631324e-32) ? 0.0 : mu_x / gam;
  }
  const double rho = A.rho;
  const double T1c = A.af * A.gam * A.dt;
  const double amd = A.am / T1c;
  const double wl = w * T1c, wr = w * rho;
  const double kT = 4.0 * (A.ctM / A.dt) * (A.ctM / A.dt);
  double kS = 0.0;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) kS += K[i][j] * K[i][j];
  kS = A.ctC * kS * (mu / rho) * (mu / rho);
  const double trK = K[0][0] + K[1][1] + K[2][2];

  double lR[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int c = 0; c < 4; c++) lR[a][c] = 0.0;
  // tangent factors accumulated over the Gauss points
  const TT rh = TT(rho), md = TT(amd);
  TT SC = TT(0), ST = TT(0), Q[4], Vc[4], G[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++) {
    Q[a] = Vc[a] = TT(0);
#pragma unroll
    for (int b = 0; b < 4; b++) G[a][b] = TT(0);
  }

#pragma unroll 1
  for (int g = 0; g < 4; g++) {
    double N[4];
#pragma unroll
    for (int a = 0; a < 4; a++) N[a] = c_rule.N[g][a];
    double u[3], ud[3], pr = 0.0;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      u[i] = N[0] * yl[0][i] + N[1] * yl[1][i] + N[2] * yl[2][i] + N[3] * yl[3][i];
      ud[i] = -A.fb[i] + N[0] * al[0][i] + N[1] * al[1][i] + N[2] * al[2][i] + N[3] * al[3][i];
    }
#pragma unroll
    for (int a = 0; a < 4; a++) pr += N[a] * yl[a][3];
    double kU = 0.0;
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int i = 0; i < 3; i++) kU += u[i] * u[j] * K[i][j];
    const double tauM = 1.0 / (rho * sqrt(kT + kU + kS));
    double rV[3], up[3];
#pragma unroll
    for (int j = 0; j < 3; j++) {
      rV[j] = ud[j] + u[0] * ux[0][j] + u[1] * ux[1][j] + u[2] * ux[2][j];
      up[j] = -tauM * (rho * rV[j] + px[j]);
    }
    const double tauC = 1.0 / (tauM * trK);
    double tauB = 0.0;
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int i = 0; i < 3; i++) tauB += up[i] * up[j] * K[i][j];
    // ISZERO (MATFUN.f:763-780): |x| < eps^2
    if (fabs(tauB) < 4.930380657631324e-32) tauB = 2.220446049250313e-16;
    tauB = rho / sqrt(tauB);
    double ua[3];
#pragma unroll
    for (int i = 0; i < 3; i++) ua[i] = u[i] + up[i];
    const double pa = pr - tauC * divU;
    double rB[3], rV2[3];
#pragma unroll
    for (int j = 0; j < 3; j++) {
      rB[j] = tauB * (up[0] * ux[0][j] + up[1] * ux[1][j] + up[2] * ux[2][j]);
      rV2[j] = ud[j] + ua[0] * ux[0][j] + ua[1] * ux[1][j] + ua[2] * ux[2][j];
    }
    // lR(a,j) += wr N_a rV2_j + w sum_i Nx_i(a) rM(i,j)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      double rM[3];
#pragma unroll
      for (int i = 0; i < 3; i++)
        rM[i] = mu * es[i][j] - rho * up[j] * ua[i] + rB[j] * up[i] - (i == j ? pa : 0.0);
#pragma unroll
      for (int a = 0; a < 4; a++)
        lR[a][j] += wr * N[a] * rV2[j] + w * (Nx[0][a] * rM[0] + Nx[1][a] * rM[1] + Nx[2][a] * rM[2]);
    }
    TT uN[4], upN[4], vN[4];
#pragma unroll
    for (int a = 0; a < 4; a++) {
      const double upNx = up[0] * Nx[0][a] + up[1] * Nx[1][a] + up[2] * Nx[2][a];
      lR[a][3] += w * (N[a] * divU - upNx);
      uN[a] = TT(u[0] * Nx[0][a] + u[1] * Nx[1][a] + u[2] * Nx[2][a]);
      upN[a] = TT(upNx);
      vN[a] = uN[a] + md * TT(N[a]);
    }
    const TT tM = TT(tauM), tB = TT(tauB);
    SC += TT(tauC);
    ST += tM;
#pragma unroll
    for (int a = 0; a < 4; a++) {
      const TT uaa = uN[a] + upN[a];
      Q[a] += tM * uaa;
      Vc[a] += tM * vN[a];
      const TT c1 = rh * rh * tM * uaa, c2 = rh * TT(N[a]), c3 = tB * upN[a];
#pragma unroll
      for (int b = 0; b < 4; b++) G[a][b] += c1 * vN[b] + c2 * (uN[b] + upN[b]) + c3 * upN[b];
    }
  }
  asm_colour_scatter();
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int c = 0; c < 4; c++) A.R[(size_t)n4[a] * 4 + c] += lR[a][c];

  // ---- tangent (TT)
  const TT mu4 = TT(4.0 * mu), wlt = TT(wl);
  TT Nxa[3][4];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int a = 0; a < 4; a++) Nxa[i][a] = TT(Nx[i][a]);
  TT *Val = reinterpret_cast<TT *>(A.Val);
  // esNx_i(a) = sum_k es(k,i) Nx_k(a) for the term 4 mu_g esNx_i(a) esNx_j(b)
  const TT g4 = TT(4.0 * mu_g);
  TT eN[3][4];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int a = 0; a < 4; a++)
      eN[i][a] = NN ? TT(es[0][i] * Nx[0][a] + es[1][i] * Nx[1][a] + es[2][i] * Nx[2][a]) : TT(0);
#pragma unroll
  for (int a = 0; a < 4; a++) {
    const int4 m4 = A.map[(size_t)e * 4 + a];
    const int pos[4] = {m4.x, m4.y, m4.z, m4.w};
#pragma unroll
    for (int b = 0; b < 4; b++) {
      const TT NxNx = Nxa[0][a] * Nxa[0][b] + Nxa[1][a] * Nxa[1][b] + Nxa[2][a] * Nxa[2][b];
      const TT S = mu4 * NxNx + rh * md * TT(c_rule.M[a][b]) + G[a][b];
      TT blk[16];
#pragma unroll
      for (int i = 0; i < 3; i++) {
#pragma unroll
        for (int j = 0; j < 3; j++)
          blk[i * 4 + j] = wlt * (mu4 * Nxa[i][b] * Nxa[j][a] + SC * Nxa[i][a] * Nxa[j][b] +
                                  (NN ? g4 * eN[i][a] * eN[j][b] : TT(0)) +
                                  (i == j ? S : TT(0)));
        blk[i * 4 + 3] = -wlt * (Nxa[i][a] * TT(c_rule.Ns[b]) - rh * Nxa[i][b] * Q[a]);
        blk[12 + i] = wlt * (TT(c_rule.Ns[a]) * Nxa[i][b] + rh * Nxa[i][a] * Vc[b]);
      }
      blk[15] = wlt * ST * NxNx;
      TT *dst = Val + (size_t)pos[b] * 16;
#pragma unroll
      for (int k = 0; k < 16; k++) dst[k] += blk[k];
    }
  }
}

}  // namespace gsls
