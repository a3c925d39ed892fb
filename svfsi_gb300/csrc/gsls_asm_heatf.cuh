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
// point quantities are FP64 (the residual); the tangent's factors are
// rounded to VT and its 16 entries formed and accumulated in VT.
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
  double Nx[3][4];
  const double w = c_rule.w * load_geo(A, e, Nx);
  double y[4][3], Ty[4], Ta[4];
#pragma unroll
  for (int a = 0; a < 4; a++) {
    const size_t b = (size_t)n4[a] * tD;
#pragma unroll
    for (int i = 0; i < 3; i++) y[a][i] = __ldg(A.Yg + b + i);
    Ty[a] = __ldg(A.Yg + b + s0);
    Ta[a] = __ldg(A.Ag + b + s0);
  }
  // ks = xiX^T xiX (GNN, NN.f:1539-1547); on a tet4 the rows of xiX are the
  // gradients of the first three shape functions, so ks = sum_{a<3} Nx_a
  // Nx_a^T.  The element runs on the FP64 pipe, so its quadratic forms are
  // taken through those gradients, x.ks.x = sum_{a<3} (Nx_a.x)^2 (u.ks.u
  // and Tx.ks.Tx), and ks:ks from the six distinct entries of the symmetric
  // ks: the reference's quantities, rounded differently.
  double k00 = 0, k01 = 0, k02 = 0, k11 = 0, k12 = 0, k22 = 0;
#pragma unroll
  for (int a = 0; a < 3; a++) {
    k00 += Nx[0][a] * Nx[0][a];
    k01 += Nx[0][a] * Nx[1][a];
    k02 += Nx[0][a] * Nx[2][a];
    k11 += Nx[1][a] * Nx[1][a];
    k12 += Nx[1][a] * Nx[2][a];
    k22 += Nx[2][a] * Nx[2][a];
  }
  const double kS = k00 * k00 + k11 * k11 + k22 * k22 + 2.0 * (k01 * k01 + k02 * k02 + k12 * k12);
  double Tx[3];
#pragma unroll
  for (int i = 0; i < 3; i++) Tx[i] = Nx[i][0] * Ty[0] + Nx[i][1] * Ty[1] + Nx[i][2] * Ty[2] + Nx[i][3] * Ty[3];
  double NxTx[4];  // Nx_a . Tx (constant on a tet4)
#pragma unroll
  for (int a = 0; a < 4; a++) NxTx[a] = Nx[0][a] * Tx[0] + Nx[1][a] * Tx[1] + Nx[2][a] * Tx[2];
  double nTx = NxTx[0] * NxTx[0] + NxTx[1] * NxTx[1] + NxTx[2] * NxTx[2];  // Tx.ks.Tx
  // ISZERO (MATFUN.f:763-780): |x| < eps^2
  if (fabs(nTx) < 4.930380657631324e-32) nTx = 2.220446049250313e-16;
  const double rnTx = 0.5 * rsqrt(nTx);
  const double T1 = A.af * A.gam * A.dt, amd = A.hf_amd, kT = A.hf_kT;
  VT lK[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) lK[a][b] = VT(0);
  // Nx_a . Nx_b in the tangent's precision (symmetric: 10 entries)
  VT NxN[4][4];
  {
    VT nx[3][4];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int a = 0; a < 4; a++) nx[i][a] = VT(Nx[i][a]);
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
      for (int b = a; b < 4; b++) {
        NxN[a][b] = nx[0][a] * nx[0][b] + nx[1][a] * nx[1][b] + nx[2][a] * nx[2][b];
        NxN[b][a] = NxN[a][b];
      }
  }
  // The tet4 rule's shape values are N_a(g) = t + (s - t) delta_ag (NN.f:
  // 268-275), so the point values are u_g = t sum_a y_a + (s - t) y_g (and
  // Td likewise), and the N_a r_g part of lR_a sums to t sum_g r_g +
  // (s - t) r_a: the reference's sums, regrouped.
  const double rt = c_rule.N[0][1], rd = c_rule.N[0][0] - c_rule.N[0][1];
  double ys[3], Tas = 0.0;
#pragma unroll
  for (int i = 0; i < 3; i++) ys[i] = rt * (y[0][i] + y[1][i] + y[2][i] + y[3][i]);
  Tas = rt * (Ta[0] + Ta[1] + Ta[2] + Ta[3]) - A.src;
  const double wl = w * T1;
  const VT wlv = VT(wl), amdv = VT(amd), ntv = VT(rt), nsv = VT(c_rule.N[0][0]);
  double rg[4], rsum = 0.0, nusum = 0.0, lRu[4] = {0, 0, 0, 0};
#pragma unroll
  for (int g = 0; g < 4; g++) {
    double u[3];
#pragma unroll
    for (int i = 0; i < 3; i++) u[i] = ys[i] + rd * y[g][i];
    const double Td = Tas + rd * Ta[g];
    double udNx[4];  // u . Nx_a
#pragma unroll
    for (int a = 0; a < 4; a++) udNx[a] = u[0] * Nx[0][a] + u[1] * Nx[1][a] + u[2] * Nx[2][a];
    const double kU = udNx[0] * udNx[0] + udNx[1] * udNx[1] + udNx[2] * udNx[2];  // u.ks.u
    const double udTx = u[0] * Tx[0] + u[1] * Tx[1] + u[2] * Tx[2];
    const double r = Td + udTx;
    const double nu = A.cond + fabs(r) * rnTx;
    const double tauM = rsqrt(kT + kU + 3.0 * nu * nu * kS);
    const double tr = tauM * r;
    rg[g] = r;
    rsum += r;
    nusum += nu;
#pragma unroll
    for (int a = 0; a < 4; a++) lRu[a] += udNx[a] * tr;
    const VT wn = VT(wl * nu), tv = VT(tauM);
    VT ta[4], tb[4];
#pragma unroll
    for (int a = 0; a < 4; a++) {
      const VT un = VT(udNx[a]), na = a == g ? nsv : ntv;
      ta[a] = wlv * (na + tv * un);
      tb[a] = na * amdv + un;
    }
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
      for (int b = 0; b < 4; b++) lK[a][b] += wn * NxN[a][b] + ta[a] * tb[b];
  }
  double lR[4];
#pragma unroll
  for (int a = 0; a < 4; a++) lR[a] = rt * rsum + rd * rg[a] + NxTx[a] * nusum + lRu[a];
  VT *Val = reinterpret_cast<VT *>(A.Val);
  asm_colour_scatter();
#pragma unroll
  for (int a = 0; a < 4; a++) {
    A.R[n4[a]] += w * lR[a];
    const int4 mp = A.map[(size_t)e * 4 + a];
    const int pos[4] = {mp.x, mp.y, mp.z, mp.w};
#pragma unroll
    for (int b = 0; b < 4; b++) Val[pos[b]] += lK[a][b];
  }
}

}  // namespace gsls
