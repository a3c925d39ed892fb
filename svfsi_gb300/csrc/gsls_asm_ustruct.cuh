// USTRUCT (Code/Source/svFSI/USTRUCT.f): the velocity-pressure nonlinear
// solid for one tet4 per thread, equal-order velocity/pressure with VMS
// stabilisation (nFs = 1), the neo-Hookean isochoric stress of GETPK2CCdev
// (MATMODELS.f:568-1016, no fibres or active coupling), the volumetric
// penalty of GVOLPEN (MATMODELS.f:1020-1070) and tauM/tauC of GETTAU
// (MATMODELS.f:1073-1104).  Included by gsls_assemble.cu (needs AsmArgs,
// c_rule, load_geo, kAsmThreads, adj_det3).
//
// On a tet4 the kinematics (F, J, F^-1, the velocity gradient, Siso, Dm,
// the viscous stress) and tauM/tauC are element constants; only the
// point values of v', p, p' (and so rho(p), beta(p)) change between the
// four Gauss points.  USTRUCT3D_M and USTRUCT3D_C's point sums are taken
// block by block: for each node pair (a,b) the 16 entries of lK and the 12
// of lKd (the displacement tangent, USTRUCT_DOASSEM's Kd) are summed over
// the points and scattered, so no 4x4x16 element array is held.  Residual
// and the kinematics are formed in FP64; the 16 blocks of both tangents in
// the tangent's precision VT (FP64 for the drop-in; FP32 for the mixed path,
// whose FP32 tangent needs no FP64 arithmetic -- the FP64 form kept the
// FP64 pipe 88 % busy).  Kd is stored in FP64 either way: it enters
// USTRUCTR's FP64 residual correction on the first Newton iteration only,
// whose error the later iterations (Rd = 0, exact FP64 residual) remove.
#pragma once

namespace gsls {

// ISZERO of the reference (MATFUN.f:763-780): |a| / max(|a|, eps) < eps
__device__ __forceinline__ bool ust_iszero(double a) {
  const double eps = 2.220446049250313e-16;
  return fabs(a) / fmax(fabs(a), eps) < eps;
}

struct UstVol {
  double ro, bt, dro, dbt;
};
// GVOLPEN with Ja = 1
__device__ __forceinline__ UstVol ust_gvolpen(const AsmArgs &A, double p) {
  UstVol v{A.rho, 0.0, 0.0, 0.0};
  const double Kp = A.Kpen;
  if (ust_iszero(Kp)) return v;
  if (A.volType == 0) {  // quadratic
    const double r1 = 1.0 / (Kp - p);
    v.ro = v.ro * Kp * r1;
    v.bt = r1;
    v.dro = v.ro * r1;
    v.dbt = r1 * r1;
  } else if (A.volType == 1) {  // ST91
    const double r1 = v.ro / Kp, r2 = sqrt(p * p + Kp * Kp);
    v.ro = r1 * (p + r2);
    v.bt = 1.0 / r2;
    v.dro = v.ro * v.bt;
    v.dbt = -v.bt * p / (p * p + Kp * Kp);
  } else {  // M94
    const double r1 = v.ro / Kp, r2 = Kp + p;
    v.ro = r1 * r2;
    v.bt = 1.0 / r2;
    v.dro = r1;
    v.dbt = -v.bt * v.bt;
  }
  return v;
}

template <class VT>
__global__ void __launch_bounds__(kAsmThreads) k_asm_ustruct(AsmArgs A, double *Kd) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= A.nColorEl) return;
  const int e = A.el0 + t;
  const int4 nd = A.ien[e];
  const int n4[4] = {nd.x, nd.y, nd.z, nd.w};
  const int tD = A.tDof, s0 = A.s;
  double Nx[3][4];
  const double Je = load_geo(A, e, Nx);
  const double w = c_rule.w * Je;  // every point has the same weight
  const double mu = A.visc, am = A.am, af = A.af * A.gam * A.dt, afm = af / am;
  const double r13 = 1.0 / 3.0, r23 = 2.0 / 3.0;

  // ---- kinematics (element constants)
  double F[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}}, vx[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  double al[4][4], yl[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++) {
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const size_t k = (size_t)n4[a] * tD + s0 + c;
      al[a][c] = A.Ag[k];
      yl[a][c] = A.Yg[k];
    }
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const double d = A.Dg[(size_t)n4[a] * tD + s0 + i];
#pragma unroll
      for (int j = 0; j < 3; j++) {
        F[i][j] += Nx[j][a] * d;
        vx[i][j] += Nx[j][a] * yl[a][i];
      }
    }
  }
  double Fi[3][3];
  const double J = adj_det3(F, Fi);
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) Fi[i][j] /= J;
  // GETPK2CCdev, neo-Hookean: S = J^-2/3 2 C10 (I - tr(C)/3 C^-1),
  // CC = 2 r1 (Ci (.) Ci - 1/3 Ci x Ci) - 2/3 (Ci x S + S x Ci)
  double Ci[3][3], trC = 0.0;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      Ci[i][j] = Fi[i][0] * Fi[j][0] + Fi[i][1] * Fi[j][1] + Fi[i][2] * Fi[j][2];
      trC += F[i][j] * F[i][j];
    }
  const double J2d = pow(J, -2.0 / 3.0);
  const double g1 = 2.0 * A.C10;
  const double r1 = J2d * g1 * trC / 3.0;
  double S0[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) S0[i][j] = (i == j ? J2d * g1 : 0.0) - r1 * Ci[i][j];
  // Voigt pairs (11, 22, 33, 12, 23, 31), CCTOVOIGT's order
  const int vi[6] = {0, 1, 2, 0, 1, 2}, vj[6] = {0, 1, 2, 1, 2, 0};
  double Dm[6][6];
#pragma unroll
  for (int I = 0; I < 6; I++)
#pragma unroll
    for (int K = 0; K < 6; K++) {
      const int i = vi[I], j = vj[I], k = vi[K], l = vj[K];
      const double sym = 0.5 * (Ci[i][k] * Ci[j][l] + Ci[i][l] * Ci[j][k]);
      Dm[I][K] = 2.0 * r1 * (sym - r13 * Ci[i][j] * Ci[k][l]) -
                 r23 * (Ci[i][j] * S0[k][l] + S0[i][j] * Ci[k][l]);
    }
  // viscous stress, USTRUCT.f:298-307
  double VxFi[3][3], ddev[3][3], Siso[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) VxFi[i][j] = vx[i][0] * Fi[0][j] + vx[i][1] * Fi[1][j] + vx[i][2] * Fi[2][j];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) ddev[i][j] = 0.5 * (VxFi[i][j] + VxFi[j][i]);
  {
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
        Siso[i][j] = S0[i][j] + 2.0 * mu * J * (Fi[i][0] * tmp[0][j] + Fi[i][1] * tmp[1][j] + Fi[i][2] * tmp[2][j]);
  }
  double Pdev[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) Pdev[i][j] = F[i][0] * Siso[0][j] + F[i][1] * Siso[1][j] + F[i][2] * Siso[2][j];
  double NxFi[3][4], DdNx[3][4], VxNx[3][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int i = 0; i < 3; i++)
      NxFi[i][a] = Nx[0][a] * Fi[0][i] + Nx[1][a] * Fi[1][i] + Nx[2][a] * Fi[2][i];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int i = 0; i < 3; i++) {
      DdNx[i][a] = ddev[i][0] * NxFi[0][a] + ddev[i][1] * NxFi[1][a] + ddev[i][2] * NxFi[2][a];
      VxNx[i][a] = VxFi[0][i] * NxFi[0][a] + VxFi[1][i] * NxFi[1][a] + VxFi[2][i] * NxFi[2][a];
    }
  // GETTAU (element constants: detF and Je); tauM of the continuity pass
  // adds the viscous term with Kx = F^-T ksix F^-1, ksix from the tet4
  // gradients (xi_X(k, i) = Nx(i, k) for k < 3)
  double tauC, tauMc;
  {
    const double he = 0.5 * pow(Je, 1.0 / 3.0);
    const double rho0 = A.rho, nu = A.nu_s, Em = A.E_s;
    const double mue = 0.5 * Em / (1.0 + nu);
    double c;
    if (ust_iszero(nu - 0.5)) {
      c = sqrt(mue / rho0);
    } else {
      const double lam = 2.0 * mue * nu / (1.0 - 2.0 * nu);
      c = sqrt((lam + 2.0 * mue) / rho0);
    }
    const double tauM = A.ctM * (he / c) * (J / rho0);
    tauC = A.ctC * (he * c) * (rho0 / J);
    double ks[3][3], tmp[3][3], Kx2 = 0.0;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) ks[i][j] = Nx[i][0] * Nx[j][0] + Nx[i][1] * Nx[j][1] + Nx[i][2] * Nx[j][2];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) tmp[i][j] = ks[i][0] * Fi[0][j] + ks[i][1] * Fi[1][j] + ks[i][2] * Fi[2][j];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        const double k = Fi[0][i] * tmp[0][j] + Fi[1][i] * tmp[1][j] + Fi[2][i] * tmp[2][j];
        Kx2 += k * k;
      }
    const double tauV = 36.0 * mu * mu * Kx2;
    tauMc = 1.0 / sqrt(tauV + (1.0 / tauM) * (1.0 / tauM));
  }
  // pressure gradient (element constant) in the current configuration
  double px[3] = {0, 0, 0};
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int i = 0; i < 3; i++) px[i] += Nx[i][a] * yl[a][3];
  double PxFi[3];
#pragma unroll
  for (int i = 0; i < 3; i++) PxFi[i] = px[0] * Fi[0][i] + px[1] * Fi[1][i] + px[2] * Fi[2][i];
  const double divv = VxFi[0][0] + VxFi[1][1] + VxFi[2][2];

  // ---- point values
  double vd[4][3], pdg[4], rC[4], rCl[4], rM[4][3];
  UstVol vol[4];
#pragma unroll
  for (int g = 0; g < 4; g++) {
    double p = 0.0, pd = 0.0;
#pragma unroll
    for (int i = 0; i < 3; i++) vd[g][i] = -A.fb[i];
#pragma unroll
    for (int a = 0; a < 4; a++) {
      const double N = c_rule.N[g][a];
#pragma unroll
      for (int i = 0; i < 3; i++) vd[g][i] += N * al[a][i];
      p += N * yl[a][3];
      pd += N * al[a][3];
    }
    pdg[g] = pd;
    vol[g] = ust_gvolpen(A, p);
    rC[g] = vol[g].bt * pd + divv;
    rCl[g] = -p + tauC * rC[g];
#pragma unroll
    for (int i = 0; i < 3; i++) rM[g][i] = vol[g].ro * vd[g][i] + PxFi[i];
  }
  const double W = 4.0 * w;

  // ---- residual
#pragma unroll
  for (int a = 0; a < 4; a++) {
    double r[4];
#pragma unroll
    for (int i = 0; i < 3; i++) {
      double s = 0.0;
#pragma unroll
      for (int g = 0; g < 4; g++)
        s += w * (J * vol[g].ro * vd[g][i] * c_rule.N[g][a] + J * rCl[g] * NxFi[i][a]);
      r[i] = s + W * (Pdev[i][0] * Nx[0][a] + Pdev[i][1] * Nx[1][a] + Pdev[i][2] * Nx[2][a]);
    }
    double s = 0.0;
#pragma unroll
    for (int g = 0; g < 4; g++) {
      const double rMN = rM[g][0] * NxFi[0][a] + rM[g][1] * NxFi[1][a] + rM[g][2] * NxFi[2][a];
      s += w * J * (c_rule.N[g][a] * rC[g] + tauMc * rMN);
    }
    r[3] = s;
#pragma unroll
    for (int i = 0; i < 4; i++) A.R[(size_t)n4[a] * 4 + i] += r[i];
  }

  // ---- tangents, block by block, in the tangent's precision
  using TT = VT;
  TT tN[4][4], tNx[3][4], tNxFi[3][4], tDdNx[3][4], tVxNx[3][4];
  TT tF[3][3], tSiso[3][3], tVxFi[3][3], tDm[6][6];
  TT tro[4], tbt[4], tdro[4], tdbt[4], tvd[4][3], tpdg[4], tRc[4], trCl[4], trM[4][3];
#pragma unroll
  for (int g = 0; g < 4; g++) {
#pragma unroll
    for (int a = 0; a < 4; a++) tN[g][a] = TT(c_rule.N[g][a]);
    tro[g] = TT(vol[g].ro);
    tbt[g] = TT(vol[g].bt);
    tdro[g] = TT(vol[g].dro);
    tdbt[g] = TT(vol[g].dbt);
    tpdg[g] = TT(pdg[g]);
    tRc[g] = TT(rC[g]);
    trCl[g] = TT(rCl[g]);
#pragma unroll
    for (int i = 0; i < 3; i++) {
      tvd[g][i] = TT(vd[g][i]);
      trM[g][i] = TT(rM[g][i]);
    }
  }
#pragma unroll
  for (int i = 0; i < 3; i++) {
#pragma unroll
    for (int a = 0; a < 4; a++) {
      tNx[i][a] = TT(Nx[i][a]);
      tNxFi[i][a] = TT(NxFi[i][a]);
      tDdNx[i][a] = TT(DdNx[i][a]);
      tVxNx[i][a] = TT(VxNx[i][a]);
    }
#pragma unroll
    for (int j = 0; j < 3; j++) {
      tF[i][j] = TT(F[i][j]);
      tSiso[i][j] = TT(Siso[i][j]);
      tVxFi[i][j] = TT(VxFi[i][j]);
    }
  }
#pragma unroll
  for (int I = 0; I < 6; I++)
#pragma unroll
    for (int K = 0; K < 6; K++) tDm[I][K] = TT(Dm[I][K]);
  const TT tw = TT(w), tW = TT(W), tJ = TT(J), tmu = TT(mu), tam = TT(am), taf = TT(af);
  const TT tafm = TT(afm), ttauC = TT(tauC), ttauMc = TT(tauMc);
  const TT tr13 = TT(r13), tr23 = TT(r23), one = TT(1);
  TT tPxFi[3];
#pragma unroll
  for (int i = 0; i < 3; i++) tPxFi[i] = TT(PxFi[i]);

  VT *Val = reinterpret_cast<VT *>(A.Val);
  for (int a = 0; a < 4; a++) {
    const int4 m4 = A.map[(size_t)e * 4 + a];
    const int pos[4] = {m4.x, m4.y, m4.z, m4.w};
    for (int b = 0; b < 4; b++) {
      TT k16[16], k12[12];
      TT NxSNx = TT(0);
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) NxSNx += tNx[i][a] * tSiso[i][j] * tNx[j][b];
      const TT NxNx = tNxFi[0][a] * tNxFi[0][b] + tNxFi[1][a] * tNxFi[1][b] + tNxFi[2][a] * tNxFi[2][b];
      // point sums that recur below (each includes the weight w)
      TT sRoNN = TT(0), sRo = TT(0), sRcl = TT(0), sRoVdN[3] = {TT(0), TT(0), TT(0)};
#pragma unroll
      for (int g = 0; g < 4; g++) {
        const TT Na = tN[g][a], Nb = tN[g][b];
        sRoNN += tw * tro[g] * Na * Nb;
        sRo += tw * tro[g];
        sRcl += tw * trCl[g];
#pragma unroll
        for (int r = 0; r < 3; r++) sRoVdN[r] += tw * tro[g] * tvd[g][r] * Na;
      }
      // Bm(:, :, a), Bm(:, :, b) and DBm = Dm Bm(:, :, b)
      TT Bb[6][3], Ba[6][3];
#pragma unroll
      for (int c = 0; c < 3; c++) {
        Bb[0][c] = tNx[0][b] * tF[c][0];
        Bb[1][c] = tNx[1][b] * tF[c][1];
        Bb[2][c] = tNx[2][b] * tF[c][2];
        Bb[3][c] = tNx[0][b] * tF[c][1] + tF[c][0] * tNx[1][b];
        Bb[4][c] = tNx[1][b] * tF[c][2] + tF[c][1] * tNx[2][b];
        Bb[5][c] = tNx[2][b] * tF[c][0] + tF[c][2] * tNx[0][b];
        Ba[0][c] = tNx[0][a] * tF[c][0];
        Ba[1][c] = tNx[1][a] * tF[c][1];
        Ba[2][c] = tNx[2][a] * tF[c][2];
        Ba[3][c] = tNx[0][a] * tF[c][1] + tF[c][0] * tNx[1][a];
        Ba[4][c] = tNx[1][a] * tF[c][2] + tF[c][1] * tNx[2][a];
        Ba[5][c] = tNx[2][a] * tF[c][0] + tF[c][2] * tNx[0][a];
      }
      TT DBm[6][3];
#pragma unroll
      for (int I = 0; I < 6; I++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
          TT sm = TT(0);
#pragma unroll
          for (int K = 0; K < 6; K++) sm += tDm[I][K] * Bb[K][c];
          DBm[I][c] = sm;
        }
      // momentum rows, USTRUCT3D_M
#pragma unroll
      for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
          TT BtDB = TT(0);
#pragma unroll
          for (int I = 0; I < 6; I++) BtDB += Ba[I][r] * DBm[I][c];
          const TT T1 = tJ * sRoVdN[r] * tNxFi[c][b];
          const TT T2 = -ttauC * tJ * tNxFi[r][a] * tVxNx[c][b];
          const TT T3 = (r == c) ? TT(0)
                                 : tJ * sRcl * (tNxFi[r][a] * tNxFi[c][b] - tNxFi[c][a] * tNxFi[r][b]);
          const TT Tv = (TT(2) * (tDdNx[r][a] * tNxFi[c][b] - tDdNx[r][b] * tNxFi[c][a]) -
                         (NxNx * tVxFi[r][c] + tNxFi[r][b] * tVxNx[c][a] -
                          tr23 * tNxFi[r][a] * tVxNx[c][b])) *
                        tmu * tJ;
          const TT Ku = taf * (T1 + T3 + tW * (T2 + Tv + BtDB + ((r == c) ? NxSNx : TT(0))));
          k12[3 * r + c] = Ku;
          TT kv;
          if (r == c)
            kv = tam * tJ * sRoNN + taf * tJ * ttauC * sRo * tNxFi[r][a] * tNxFi[r][b] +
                 tW * taf * tmu * tJ * (tr13 * tNxFi[r][a] * tNxFi[r][b] + NxNx);
          else
            kv = taf * tJ * ttauC * sRo * tNxFi[r][a] * tNxFi[c][b] +
                 tW * taf * tmu * tJ * (tNxFi[c][a] * tNxFi[r][b] - tr23 * tNxFi[r][a] * tNxFi[c][b]);
          k16[4 * r + c] = kv + tafm * Ku;
        }
      // dM/dP
#pragma unroll
      for (int r = 0; r < 3; r++) {
        TT sm = TT(0);
#pragma unroll
        for (int g = 0; g < 4; g++) {
          const TT T1 = tam * ttauC * tbt[g] + taf * (ttauC * tdbt[g] * tpdg[g] - one);
          sm += tw * tJ * (T1 * tNxFi[r][a] * tN[g][b] + taf * tdro[g] * tvd[g][r] * tN[g][a] * tN[g][b]);
        }
        k16[4 * r + 3] = sm;
      }
      // continuity row, USTRUCT3D_C
#pragma unroll
      for (int c = 0; c < 3; c++) {
        TT Ku = TT(0), kv = TT(0);
#pragma unroll
        for (int g = 0; g < 4; g++) {
          const TT Na = tN[g][a], Nb = tN[g][b];
          const TT rMNqa = trM[g][0] * tNxFi[0][a] + trM[g][1] * tNxFi[1][a] + trM[g][2] * tNxFi[2][a];
          const TT rMNwb = trM[g][0] * tNxFi[0][b] + trM[g][1] * tNxFi[1][b] + trM[g][2] * tNxFi[2][b];
          const TT T1 = Na * (tRc[g] * tNxFi[c][b] - tVxNx[c][b]);
          const TT T2 = ttauMc * (rMNqa * tNxFi[c][b] - rMNwb * tNxFi[c][a]);
          const TT T3 = -ttauMc * NxNx * tPxFi[c];
          Ku += tw * taf * tJ * (T1 + T2 + T3);
          kv += tw * tJ * ((tam * ttauMc * tro[g]) * tNxFi[c][a] * Nb + taf * Na * tNxFi[c][b]);
        }
        k12[9 + c] = Ku;
        k16[12 + c] = kv + tafm * Ku;
      }
      {
        TT sm = TT(0);
#pragma unroll
        for (int g = 0; g < 4; g++) {
          const TT Na = tN[g][a], Nb = tN[g][b];
          const TT T1 = (tam * tbt[g] + taf * tdbt[g] * tpdg[g]) * Na * Nb;
          const TT T2 = tNxFi[0][a] * tvd[g][0] + tNxFi[1][a] * tvd[g][1] + tNxFi[2][a] * tvd[g][2];
          sm += tw * tJ * (T1 + taf * ttauMc * (NxNx + tdro[g] * T2 * Nb));
        }
        k16[15] = sm;
      }
      VT *dv = Val + (size_t)pos[b] * 16;
#pragma unroll
      for (int k = 0; k < 16; k++) dv[k] += VT(k16[k]);
      double *dk = Kd + (size_t)pos[b] * 12;
#pragma unroll
      for (int k = 0; k < 12; k++) dk[k] += double(k12[k]);
    }
  }
}

}  // namespace gsls
