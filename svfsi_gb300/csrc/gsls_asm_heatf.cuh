// HEATF3D (Code/Source/svFSI/HEATF.f:116-205): advection-diffusion of the
// temperature (state component s) by the velocity in components 0..2, one
// tet4 per thread, no mesh motion.  Included by gsls_assemble.cu (needs
// AsmArgs, c_rule, load_geo, kAsmThreads).
//
// Per Gauss point, as the reference: u = sum_a N_a y_a, Td = sum_a N_a T'_a
// - s, Tx = grad T (constant on a tet4), the discontinuity-capturing
// diffusivity nu_g = nu + |Td + u.Tx| / (2 sqrt(Tx.ks.Tx)) (ISZERO -> eps),
// tauM = 1/sqrt(4/dt^2 + u.ks.u + 3 nu_g^2 ks:ks) and
//   lR_a += w (N_a (Td + u.Tx) + nu_g Nx_a.Tx + tauM (u.Nx_a)(Td + u.Tx))
//   lK_ab += w T1 (nu_g Nx_a.Nx_b + (N_a + tauM u.Nx_a)(amd N_b + u.Nx_b))
// with ks = xiX^T xiX from the geometry table and T1 = af gam dt.  The
// point quantities are FP64 (the residual), the 16 tangent entries are
// accumulated in VT.
#pragma once

namespace gsls {

template <class VT>
__global__ void __launch_bounds__(kAsmThreads) k_asm_heatf(AsmArgs A) {
  asm_colour_start();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= A.nColorEl) return;
  const int e = A.el0 + t;
  const int4 nd = A.ien[e];
  const int n4[4] = {nd.x, nd.y, nd.z, nd.w};
  const int tD = A.tDof, s0 = A.s;
  double Nx[3][4], K[3][3];
  const double w = c_rule.w * load_geo(A, e, Nx);
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++)
      K[i][j] = Nx[i][0] * Nx[j][0] + Nx[i][1] * Nx[j][1] + Nx[i][2] * Nx[j][2];
  double y[4][3], Ty[4], Ta[4];
#pragma unroll
  for (int a = 0; a < 4; a++) {
    const size_t b = (size_t)n4[a] * tD;
#pragma unroll
    for (int i = 0; i < 3; i++) y[a][i] = __ldg(A.Yg + b + i);
    Ty[a] = __ldg(A.Yg + b + s0);
    Ta[a] = __ldg(A.Ag + b + s0);
  }
  double Tx[3];
#pragma unroll
  for (int i = 0; i < 3; i++) Tx[i] = Nx[i][0] * Ty[0] + Nx[i][1] * Ty[1] + Nx[i][2] * Ty[2] + Nx[i][3] * Ty[3];
  double kS = 0.0;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) kS += K[i][j] * K[i][j];
  double nTx = K[0][0] * Tx[0] * Tx[0] + K[1][1] * Tx[1] * Tx[1] + K[2][2] * Tx[2] * Tx[2] +
               (K[0][1] + K[1][0]) * Tx[0] * Tx[1] + (K[0][2] + K[2][0]) * Tx[0] * Tx[2] +
               (K[1][2] + K[2][1]) * Tx[1] * Tx[2];
  // ISZERO (MATFUN.f:763-780): |x| < eps^2
  if (fabs(nTx) < 4.930380657631324e-32) nTx = 2.220446049250313e-16;
  const double rnTx = 0.5 / sqrt(nTx);
  const double dt = A.dt, T1 = A.af * A.gam * dt, amd = A.am / T1;
  const double kT = 4.0 / (dt * dt);
  double lR[4] = {0, 0, 0, 0};
  VT lK[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) lK[a][b] = VT(0);
  VT NxN[4][4];  // Nx_a . Nx_b
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++)
      NxN[a][b] = VT(Nx[0][a] * Nx[0][b] + Nx[1][a] * Nx[1][b] + Nx[2][a] * Nx[2][b]);
  const double wl = w * T1;
#pragma unroll 1
  for (int g = 0; g < 4; g++) {
    double N[4];
#pragma unroll
    for (int a = 0; a < 4; a++) N[a] = c_rule.N[g][a];
    double u[3], Td = -A.src;
#pragma unroll
    for (int i = 0; i < 3; i++) u[i] = N[0] * y[0][i] + N[1] * y[1][i] + N[2] * y[2][i] + N[3] * y[3][i];
#pragma unroll
    for (int a = 0; a < 4; a++) Td += N[a] * Ta[a];
    double kU = 0.0;
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int i = 0; i < 3; i++) kU += u[i] * u[j] * K[i][j];
    const double udTx = u[0] * Tx[0] + u[1] * Tx[1] + u[2] * Tx[2];
    const double r = Td + udTx;
    const double nu = A.cond + fabs(r) * rnTx;
    const double tauM = 1.0 / sqrt(kT + kU + 3.0 * nu * nu * kS);
    double udNx[4];
#pragma unroll
    for (int a = 0; a < 4; a++) udNx[a] = u[0] * Nx[0][a] + u[1] * Nx[1][a] + u[2] * Nx[2][a];
#pragma unroll
    for (int a = 0; a < 4; a++)
      lR[a] += w * (N[a] * r + (Nx[0][a] * Tx[0] + Nx[1][a] * Tx[1] + Nx[2][a] * Tx[2]) * nu +
                    udNx[a] * tauM * r);
    const VT wn = VT(wl * nu);
    VT ta[4], tb[4];
#pragma unroll
    for (int a = 0; a < 4; a++) {
      ta[a] = VT(wl * (N[a] + tauM * udNx[a]));
      tb[a] = VT(N[a] * amd + udNx[a]);
    }
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
      for (int b = 0; b < 4; b++) lK[a][b] += wn * NxN[a][b] + ta[a] * tb[b];
  }
  VT *Val = reinterpret_cast<VT *>(A.Val);
  asm_colour_scatter();
#pragma unroll
  for (int a = 0; a < 4; a++) {
    A.R[n4[a]] += lR[a];
    const int4 mp = A.map[(size_t)e * 4 + a];
    const int pos[4] = {mp.x, mp.y, mp.z, mp.w};
#pragma unroll
    for (int b = 0; b < 4; b++) Val[pos[b]] += lK[a][b];
  }
}

}  // namespace gsls
