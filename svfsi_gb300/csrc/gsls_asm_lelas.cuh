// LELAS3D (Code/Source/svFSI/LELAS.f:130-238): linear elasticity for one
// tet4 per thread, lambda = E nu/((1+nu)(1-2nu)), mu = E/(2(1+nu)), no
// prestress and no nodal body force (the domain force f is fb).  Included
// by gsls_assemble.cu (needs AsmArgs, c_rule, load_geo, kAsmThreads).
//
// With constant gradients the Gauss-point sums reduce to the rule tables
// (W = sum_g w = 4 w, M_ab = sum_g N_a N_b, Ns_a = sum_g N_a):
//   lR(a,c)    = w rho (sum_b M_ab al(b,c) - f_c Ns_a) + W (Nx_a . S)(c)
//   lK_ab(r,c) = d_rc (w am rho M_ab + W T1 mu Nx_a.Nx_b)
//                + W T1 (lambda Nx(r,a) Nx(c,b) + mu Nx(c,a) Nx(r,b))
// with T1 = af beta dt^2 (the reference's wl (amd N_a N_b / mu + ...) with
// wl = w T1 mu and amd = am rho / T1, summed over the points).  The element
// matrix is symmetric (lK_ba = lK_ab^T): 10 of the 16 blocks are computed.
// Strain and stress (and so the residual) in FP64, tangent in VT.
#pragma once

namespace gsls {

template <class VT>
__global__ void __launch_bounds__(kAsmThreads) k_asm_lelas(AsmArgs A) {
  asm_colour_start();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= A.nColorEl) return;
  const int e = A.el0 + t;
  const int4 nd = A.ien[e];
  const int n4[4] = {nd.x, nd.y, nd.z, nd.w};
  const int tD = A.tDof, s0 = A.s;
  double Nx[3][4];
  const double w = c_rule.w * load_geo(A, e, Nx), W = 4.0 * w;
  const double lam = A.lam_le, mu = A.mu_le, rho = A.rho;

  // ---- strain (Voigt, engineering shear: xy, yz, xz) and stress (FP64)
  double al[4][3], ed[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
  for (int a = 0; a < 4; a++) {
    double d[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const size_t k = (size_t)n4[a] * tD + s0 + c;
      d[c] = __ldg(A.Dg + k);
      al[a][c] = __ldg(A.Ag + k);
    }
    ed[0] += Nx[0][a] * d[0];
    ed[1] += Nx[1][a] * d[1];
    ed[2] += Nx[2][a] * d[2];
    ed[3] += Nx[1][a] * d[0] + Nx[0][a] * d[1];
    ed[4] += Nx[2][a] * d[1] + Nx[1][a] * d[2];
    ed[5] += Nx[0][a] * d[2] + Nx[2][a] * d[0];
  }
  const double divD = lam * (ed[0] + ed[1] + ed[2]);
  const double Sxx = divD + 2.0 * mu * ed[0], Syy = divD + 2.0 * mu * ed[1];
  const double Szz = divD + 2.0 * mu * ed[2];
  const double Sxy = mu * ed[3], Syz = mu * ed[4], Sxz = mu * ed[5];

  // ---- residual (FP64)
  asm_colour_scatter();
#pragma unroll
  for (int a = 0; a < 4; a++) {
    double m[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      m[c] = -A.fb[c] * c_rule.Ns[a];
#pragma unroll
      for (int b = 0; b < 4; b++) m[c] += c_rule.M[a][b] * al[b][c];
    }
    double *R = A.R + (size_t)n4[a] * 3;
    R[0] += w * rho * m[0] + W * (Nx[0][a] * Sxx + Nx[1][a] * Sxy + Nx[2][a] * Sxz);
    R[1] += w * rho * m[1] + W * (Nx[0][a] * Sxy + Nx[1][a] * Syy + Nx[2][a] * Syz);
    R[2] += w * rho * m[2] + W * (Nx[0][a] * Sxz + Nx[1][a] * Syz + Nx[2][a] * Szz);
  }

  // ---- tangent (VT), symmetric blocks
  const double T1 = A.af * A.beta * A.dt * A.dt;
  const VT kM = VT(w * A.am * rho), kL = VT(W * T1 * lam), kU = VT(W * T1 * mu);
  VT Nxa[3][4];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int a = 0; a < 4; a++) Nxa[i][a] = VT(Nx[i][a]);
  VT *Val = reinterpret_cast<VT *>(A.Val);
#pragma unroll
  for (int a = 0; a < 4; a++) {
    const int4 m4 = A.map[(size_t)e * 4 + a];
    const int pos[4] = {m4.x, m4.y, m4.z, m4.w};
#pragma unroll
    for (int b = a; b < 4; b++) {
      const VT dd = Nxa[0][a] * Nxa[0][b] + Nxa[1][a] * Nxa[1][b] + Nxa[2][a] * Nxa[2][b];
      const VT diag = kM * VT(c_rule.M[a][b]) + kU * dd;
      VT blk[9];
#pragma unroll
      for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++)
          blk[r * 3 + c] = kL * Nxa[r][a] * Nxa[c][b] + kU * Nxa[c][a] * Nxa[r][b] +
                           ((r == c) ? diag : VT(0));
      VT *dst = Val + (size_t)pos[b] * 9;
#pragma unroll
      for (int k = 0; k < 9; k++) dst[k] += blk[k];
      if (b > a) {
        // block (b,a) = block(a,b)^T
        const int4 mb = A.map[(size_t)e * 4 + b];
        const int pba = (a == 0) ? mb.x : (a == 1) ? mb.y : (a == 2) ? mb.z : mb.w;
        VT *dt = Val + (size_t)pba * 9;
#pragma unroll
        for (int r = 0; r < 3; r++)
#pragma unroll
          for (int c = 0; c < 3; c++) dt[r * 3 + c] += blk[c * 3 + r];
      }
    }
  }
}

}  // namespace gsls
