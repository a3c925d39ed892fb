// Element assembly for tet4 meshes: HEATS (Code/Source/svFSI/HEATS.f:39-159),
// isotropic CEP (CEP.f:136-266), FLUID with VMS stabilisation
// (FLUID.f:40-1084) and STRUCT with the neo-Hookean + ST91 material
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
  gsls::DevBuf d_geo;             // per-element Nx (12) and Jacobian, SoA: geo[k * nEl + e]
  bool bad_jac = false;           // a zero or non-finite element Jacobian
  const double *eparam_src = nullptr;
  bool has_eparam = false;
  gsls::DevBuf d_fib;             // CEP fibres, SoA: fib[(i*3 + k) * nEl + e] (colour order)
  int nFn = 0;                    // fibre families in d_fib (0: none)
  // HEATS/CEP operators (built on the first heat/CEP assembly, rebuilt after
  // a new per-element parameter): the assembled mass sum_e w M_ab, the
  // assembled conduction sum_e W nu_e Nx_a.Nx_b (nu_e = 1 without a
  // per-element parameter) as FP64 scalar CSR, and sum_e w Ns_a per node
  gsls::DevBuf d_linM, d_linK, d_linB;
  gsls::DevBuf d_linM32, d_linK32;  // FP32 copies for the mixed-precision tangent
  bool lin_ready = false;
  unsigned lin_serial = 0;  // bumped by every build of the operators
  double lin_key[5] = {0, 0, 0, 0, 0};  // the diffusivities the conduction operator holds
};

namespace gsls {

constexpr int kAsmThreads = 128;

// tet4 Gauss rule and shape functions (Code/Source/svFSI/NN.f:268-275,
// 654-671): 4 points, w = 1/24.
struct Tet4Rule {
  double N[4][4];  // N[g][a]
  double w;
  double M[4][4];  // sum_g N_a(g) N_b(g)
  double Ns[4];    // sum_g N_a(g)
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
  for (int a = 0; a < 4; a++) {
    r.Ns[a] = 0.0;
    for (int b = 0; b < 4; b++) {
      r.M[a][b] = 0.0;
      for (int g = 0; g < 4; g++) r.M[a][b] += r.N[g][a] * r.N[g][b];
    }
    for (int g = 0; g < 4; g++) r.Ns[a] += r.N[g][a];
  }
  return r;
}

struct AsmArgs {
  int nColorEl, el0;
  int tDof, s;
  double am, af, beta, gam, dt;
  double rho, cond, src;
  double C10, Kpen, visc, dmp;
  double fb[3];
  double mu_f, ctM, ctC;
  double lam_le, mu_le;  // LELAS Lame parameters
  int viscType;          // FLUID viscosity model (GSLS_VISC_*)
  double mu_o, vlam, va, vn;
  double E_s, nu_s;      // USTRUCT elasticity modulus and Poisson ratio (GETTAU)
  int volType;           // USTRUCT volumetric penalty (GVOLPEN)
  double hf_amd, hf_kT;  // HEATF am / (af gam dt) and 4 / dt^2, formed once on the host
  const double *fib;     // CEP fibre table (SoA, colour order) or null
  int nFn;               // fibre families in fib
  double Dani[3];        // their anisotropic diffusivities
  const int4 *ien;
  const int4 *map;  // 4 int4 per element: map[e*4 + a] = (b0..b3)
  const double *x;
  const double *Ag, *Yg, *Dg;
  const double *geo;     // kGeo x nEl (structure of arrays, colour order)
  int nElAll;            // leading dimension of geo
  const double *eparam;
  double *R;
  void *Val;
  int *err;
};

// ---------------------------------------------------------------------------
// Static tet4 geometry (GNN, Code/Source/svFSI/NN.f:1469-1565): the shape-
// function gradients Nx(3,4) and the Jacobian depend on the mesh only, so
// they are computed once per mesh (adjugate, one division) and read by every
// assembly as 13 coalesced streams instead of 12 gathered coordinates.
constexpr int kGeo = 13;  // Nx[i][a] at k = i*4 + a, Jac at k = 12
__device__ __forceinline__ double load_geo(const AsmArgs &A, int e, double Nx[3][4]) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int a = 0; a < 4; a++) Nx[i][a] = __ldg(A.geo + (size_t)(i * 4 + a) * A.nElAll + e);
  return __ldg(A.geo + (size_t)12 * A.nElAll + e);
}

// Colour launches overlap: each colour kernel lets the next one be
// scheduled as soon as its blocks run, and waits for the previous colour
// (programmatic dependent launch) only before its read-modify-write
// scatter, so element loads and element math of colour c+1 overlap the
// tail of colour c (heat in a fluid: 2.38 -> 1.46 ms per assembly of the
// cylinder; neo-Hookean beam 3.92 -> 3.79 ms).  Without the launch
// attribute both calls are no-ops.
__device__ __forceinline__ void asm_colour_start() { cudaTriggerProgrammaticLaunchCompletion(); }
__device__ __forceinline__ void asm_colour_scatter() { cudaGridDependencySynchronize(); }

}  // namespace gsls

#include "gsls_asm_struct.cuh"

namespace gsls {

__global__ void k_geo_tet4(int nEl, const int4 *__restrict__ ien, const double *__restrict__ x,
                           double *geo, int *err) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nEl) return;
  const int4 nd = ien[e];
  const int n4[4] = {nd.x, nd.y, nd.z, nd.w};
  double xXi[3][3], x3[3];
#pragma unroll
  for (int i = 0; i < 3; i++) x3[i] = x[(size_t)n4[3] * 3 + i];
#pragma unroll
  for (int k = 0; k < 3; k++)
#pragma unroll
    for (int i = 0; i < 3; i++) xXi[i][k] = x[(size_t)n4[k] * 3 + i] - x3[i];
  double adj[3][3];
  const double Jac = adj_det3(xXi, adj);
  if (!(Jac != 0.0) || !isfinite(Jac)) atomicOr(err, 1);
  const double iJ = 1.0 / Jac;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const double n0 = adj[0][i] * iJ, n1 = adj[1][i] * iJ, n2 = adj[2][i] * iJ;
    geo[(size_t)(i * 4 + 0) * nEl + e] = n0;
    geo[(size_t)(i * 4 + 1) * nEl + e] = n1;
    geo[(size_t)(i * 4 + 2) * nEl + e] = n2;
    geo[(size_t)(i * 4 + 3) * nEl + e] = -(n0 + n1 + n2);
  }
  geo[(size_t)12 * nEl + e] = Jac;
}

// ---------------------------------------------------------------------------
// HEATS3D (Code/Source/svFSI/HEATS.f:116-159) and isotropic CEP3D, one tet per
// thread.  tet4 gradients are constant, so the Gauss-point sums reduce to
// the rule's tables: with W = sum_g w and M_ab = sum_g N_a N_b,
//   lR(a)   = w rho (sum_b M_ab al_b - s Ns_a) + W nu Nx_a . grad T
//   lK(a,b) = wl (amd M_ab + 4 nu Nx_a . Nx_b)
// (the reference's per-point sums, reordered).  Geometry from the per-mesh
// table; residual FP64, tangent in VT.
// CEP fibres (CEP3D, CEP.f:221-233): with D_e = nu I + sum_i Dani_i f_i f_i^T,
// Nx_a . D_e Nx_b = nu Nx_a.Nx_b + sum_i Dani_i (f_i.Nx_a)(f_i.Nx_b).  fNx
// receives f_i.Nx_a pre-scaled by Dani_i (zero past nFn).
__device__ __forceinline__ void fibre_proj(const AsmArgs &A, int e, const double Nx[3][4],
                                           double dfNx[3][4], double fNx[3][4]) {
#pragma unroll
  for (int i = 0; i < 3; i++) {
    double f[3] = {0.0, 0.0, 0.0};
    const double d = i < A.nFn ? A.Dani[i] : 0.0;
    if (i < A.nFn) {
#pragma unroll
      for (int k = 0; k < 3; k++) f[k] = __ldg(A.fib + (size_t)(i * 3 + k) * A.nElAll + e);
    }
#pragma unroll
    for (int a = 0; a < 4; a++) {
      fNx[i][a] = f[0] * Nx[0][a] + f[1] * Nx[1][a] + f[2] * Nx[2][a];
      dfNx[i][a] = d * fNx[i][a];
    }
  }
}

template <class VT>
__global__ void __launch_bounds__(kAsmThreads) k_asm_heats(AsmArgs A) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= A.nColorEl) return;
  const int e = A.el0 + t;
  const int4 nd = A.ien[e];
  const int n4[4] = {nd.x, nd.y, nd.z, nd.w};
  double al[4], yl[4];
#pragma unroll
  for (int a = 0; a < 4; a++) {
    al[a] = __ldg(A.Ag + (size_t)n4[a] * A.tDof + A.s);
    yl[a] = __ldg(A.Yg + (size_t)n4[a] * A.tDof + A.s);
  }
  double Nx[3][4];
  const double Jac = load_geo(A, e, Nx);
  const double nu = A.eparam ? A.eparam[e] : A.cond;
  const double w = c_rule.w * Jac, W = 4.0 * w;
  const double T1 = A.af * A.gam * A.dt;
  const double amd = A.am * A.rho / T1;
  double Tx[3];
#pragma unroll
  for (int i = 0; i < 3; i++) Tx[i] = Nx[i][0] * yl[0] + Nx[i][1] * yl[1] + Nx[i][2] * yl[2] + Nx[i][3] * yl[3];
  VT *Val = reinterpret_cast<VT *>(A.Val);
  const VT wl = VT(w * T1), kM = VT(amd), kS = VT(4.0 * nu);
  VT Nxa[3][4];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int a = 0; a < 4; a++) Nxa[i][a] = VT(Nx[i][a]);
  double dfNx[3][4], fNx[3][4], fTx[3] = {0.0, 0.0, 0.0};
  if (A.nFn > 0) {
    fibre_proj(A, e, Nx, dfNx, fNx);
#pragma unroll
    for (int i = 0; i < 3; i++)
      fTx[i] = fNx[i][0] * yl[0] + fNx[i][1] * yl[1] + fNx[i][2] * yl[2] + fNx[i][3] * yl[3];
  }
#pragma unroll
  for (int a = 0; a < 4; a++) {
    double m = -A.src * c_rule.Ns[a];
#pragma unroll
    for (int b = 0; b < 4; b++) m += c_rule.M[a][b] * al[b];
    double dx = nu * (Nx[0][a] * Tx[0] + Nx[1][a] * Tx[1] + Nx[2][a] * Tx[2]);
    if (A.nFn > 0) dx += dfNx[0][a] * fTx[0] + dfNx[1][a] * fTx[1] + dfNx[2][a] * fTx[2];
    A.R[n4[a]] += w * A.rho * m + W * dx;
    const int4 mp = A.map[(size_t)e * 4 + a];
    const int pos[4] = {mp.x, mp.y, mp.z, mp.w};
#pragma unroll
    for (int b = 0; b < 4; b++) {
      const VT dd = Nxa[0][a] * Nxa[0][b] + Nxa[1][a] * Nxa[1][b] + Nxa[2][a] * Nxa[2][b];
      VT v = kM * VT(c_rule.M[a][b]) + kS * dd;
      if (A.nFn > 0)
        v += VT(4.0 * (dfNx[0][a] * fNx[0][b] + dfNx[1][a] * fNx[1][b] + dfNx[2][a] * fNx[2][b]));
      Val[pos[b]] += wl * v;
    }
  }
}

// ---------------------------------------------------------------------------
// HEATS3D and isotropic CEP3D are linear in the state with mesh-constant
// element matrices: with m_e(a,b) = w M_ab (mass) and k_e(a,b) = W Nx_a.Nx_b
// (conduction; W = 4w), the element terms above are
//   lR(a)   = rho sum_b m_e(a,b) al_b + nu sum_b k_e(a,b) yl_b - rho s w Ns_a
//   lK(a,b) = am rho m_e(a,b) + T1 nu k_e(a,b)            (T1 = af gam dt)
// so DOASSEM's sums over elements are the assembled operators Mg = sum m_e,
// Kg = sum nu_e k_e and b = sum w Ns, built once per mesh (one colour launch
// each, k_lin_build), and every Newton assembly is one row-parallel pass:
//   R = rho Mg Ag + nu Kg Yg - rho s b,   Val = am rho Mg + T1 nu Kg
// (k_asm_lin).  The sums are regrouped, not changed: FP64 results agree
// with the element-by-element loop to rounding.  With CEP fibres the
// conduction operator holds the whole tensor, Kg = sum_e W Nx_a . D_e Nx_b
// with D_e = nu_e I + sum_i Dani_i f_i f_i^T (nu_e the element's parameter
// or Diso), and the assembly passes nu = 1.
__global__ void __launch_bounds__(kAsmThreads) k_lin_build(AsmArgs A, double *Mg, double *Kg,
                                                           double *Bg) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= A.nColorEl) return;
  const int e = A.el0 + t;
  const int4 nd = A.ien[e];
  const int n4[4] = {nd.x, nd.y, nd.z, nd.w};
  double Nx[3][4];
  const double Jac = load_geo(A, e, Nx);
  const double w = c_rule.w * Jac;
  const double Wn = 4.0 * w * (A.eparam ? A.eparam[e] : (A.nFn > 0 ? A.cond : 1.0));
  double dfNx[3][4], fNx[3][4];
  if (A.nFn > 0) fibre_proj(A, e, Nx, dfNx, fNx);
#pragma unroll
  for (int a = 0; a < 4; a++) {
    Bg[n4[a]] += w * c_rule.Ns[a];
    const int4 mp = A.map[(size_t)e * 4 + a];
    const int pos[4] = {mp.x, mp.y, mp.z, mp.w};
#pragma unroll
    for (int b = 0; b < 4; b++) {
      Mg[pos[b]] += w * c_rule.M[a][b];
      double k = Wn * (Nx[0][a] * Nx[0][b] + Nx[1][a] * Nx[1][b] + Nx[2][a] * Nx[2][b]);
      if (A.nFn > 0)
        k += 4.0 * w * (dfNx[0][a] * fNx[0][b] + dfNx[1][a] * fNx[1][b] + dfNx[2][a] * fNx[2][b]);
      Kg[pos[b]] += k;
    }
  }
}

// 2 lanes per CSR row (tet4 rows hold ~15 entries), entries strided by 2,
// the row sums by one fixed shuffle step: deterministic.  GB300 runs FP64
// at ~1/74 of the FP32 rate, so a pass over the operators is FP64-bound
// before it is HBM-bound: the residual takes two FP64 FMAs per entry
// (rM = sum m Ag, rK = sum k Yg; R = rho rM + nu rK - rs b) and the lane
// sums 2 FP64 adds per lane (4 lanes spent 4 per lane, 30 % more FP64 work
// per row, and took 63.8 against 53.0 us per pass on the CEP slab; 16 lanes
// ran 4x slower), and the FP32 tangent is formed from FP32 copies of the
// operators (Val = cM m + cK k in VT; the FP64 tangent from the FP64
// operators).
constexpr int kLinLanes = 2;
template <class VT, bool kVal = true>
__global__ void __launch_bounds__(256) k_asm_lin(int nNo, const int *__restrict__ rowPtr,
                                                 const int *__restrict__ colPtr,
                                                 const double *__restrict__ Mg,
                                                 const double *__restrict__ Kg,
                                                 const VT *__restrict__ Mt,
                                                 const VT *__restrict__ Kt,
                                                 const double *__restrict__ Bg,
                                                 const double *__restrict__ Ag,
                                                 const double *__restrict__ Yg, int tDof, int s,
                                                 double rho, double nu, double rs, VT cM, VT cK,
                                                 double *__restrict__ R, VT *__restrict__ Val) {
  const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int row = (int)(g / kLinLanes), l = (int)(g % kLinLanes);
  double rM = 0.0, rK = 0.0;
  if (row < nNo) {
    const int j0 = __ldg(rowPtr + row), j1 = __ldg(rowPtr + row + 1);
    // a lane's entries j, j+4, ... are loaded kU at a time (columns and
    // operator values, then the gathers) so that one pass over a tet4 row
    // of ~15 entries is one memory round trip; the sums keep the entry order
    constexpr int kU = 4;
    for (int j = j0 + l; j < j1; j += kU * kLinLanes) {
      double m[kU], k[kU], a[kU], y[kU];
      size_t c[kU];
#pragma unroll
      for (int u = 0; u < kU; u++) {
        const int jj = j + u * kLinLanes;
        const bool ok = jj < j1;
        m[u] = ok ? __ldcs(Mg + jj) : 0.0;
        k[u] = ok ? __ldcs(Kg + jj) : 0.0;
        c[u] = ok ? (size_t)__ldcs(colPtr + jj) * tDof + s : (size_t)s;
        if constexpr (kVal)
          if (ok) __stcs(Val + jj, cM * __ldcs(Mt + jj) + cK * __ldcs(Kt + jj));
      }
#pragma unroll
      for (int u = 0; u < kU; u++) {
        const bool ok = j + u * kLinLanes < j1;
        a[u] = ok ? __ldg(Ag + c[u]) : 0.0;
        y[u] = ok ? __ldg(Yg + c[u]) : 0.0;
      }
#pragma unroll
      for (int u = 0; u < kU; u++) {
        if (j + u * kLinLanes < j1) {
          rM = fma(m[u], a[u], rM);
          rK = fma(k[u], y[u], rK);
        }
      }
    }
  }
#pragma unroll
  for (int o = kLinLanes / 2; o > 0; o >>= 1) {
    rM += __shfl_xor_sync(0xffffffffu, rM, o, kLinLanes);
    rK += __shfl_xor_sync(0xffffffffu, rK, o, kLinLanes);
  }
  if (row < nNo && l == 0) R[row] = rho * rM + nu * rK - rs * Bg[row];
}

__global__ void k_f64_to_f32(size_t n, const double *__restrict__ a, float *__restrict__ b) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x)
    b[k] = (float)a[k];
}

static int lin_prepare(gsls_mesh *m, AsmArgs A) {
  // the diffusivities the conduction operator holds: none without fibres
  // (Kg = sum W nu_e k_e, nu_e = 1 or the element parameter), the fibre
  // diffusivities and, without an element parameter, Diso with fibres
  const double key[5] = {(double)A.nFn, A.Dani[0], A.Dani[1], A.Dani[2],
                         (A.nFn > 0 && !A.eparam) ? A.cond : 0.0};
  if (m->lin_ready && memcmp(key, m->lin_key, sizeof(key)) != 0) m->lin_ready = false;
  if (m->lin_ready) return GSLS_OK;
  memcpy(m->lin_key, key, sizeof(key));
  gsls_lhs *lhs = m->lhs;
  cudaStream_t st = lhs->stream;
  GSLS_TRY(m->d_linM.alloc(sizeof(double) * (size_t)lhs->nnz));
  GSLS_TRY(m->d_linK.alloc(sizeof(double) * (size_t)lhs->nnz));
  GSLS_TRY(m->d_linB.alloc(sizeof(double) * (size_t)lhs->nNo));
  GSLS_CUDA(cudaMemsetAsync(m->d_linM.p, 0, sizeof(double) * (size_t)lhs->nnz, st));
  GSLS_CUDA(cudaMemsetAsync(m->d_linK.p, 0, sizeof(double) * (size_t)lhs->nnz, st));
  GSLS_CUDA(cudaMemsetAsync(m->d_linB.p, 0, sizeof(double) * (size_t)lhs->nNo, st));
  for (int c = 0; c < m->ncolors; c++) {
    A.el0 = m->color_off[c];
    A.nColorEl = m->color_off[c + 1] - m->color_off[c];
    if (A.nColorEl <= 0) continue;
    k_lin_build<<<(A.nColorEl + kAsmThreads - 1) / kAsmThreads, kAsmThreads, 0, st>>>(
        A, m->d_linM.as<double>(), m->d_linK.as<double>(), m->d_linB.as<double>());
    GSLS_CHECK_LAUNCH();
  }
  GSLS_TRY(m->d_linM32.alloc(sizeof(float) * (size_t)lhs->nnz));
  GSLS_TRY(m->d_linK32.alloc(sizeof(float) * (size_t)lhs->nnz));
  const int nb = 4 * num_sms();
  k_f64_to_f32<<<nb, 256, 0, st>>>(lhs->nnz, m->d_linM.as<double>(), m->d_linM32.as<float>());
  GSLS_CHECK_LAUNCH();
  k_f64_to_f32<<<nb, 256, 0, st>>>(lhs->nnz, m->d_linK.as<double>(), m->d_linK32.as<float>());
  GSLS_CHECK_LAUNCH();
  m->lin_ready = true;
  m->lin_serial++;
  return GSLS_OK;
}

// GSLS_HEATS_ASM=element keeps the per-Newton element loop (k_asm_heats)
static bool lin_on() {
  static const bool on = [] {
    const char *e = getenv("GSLS_HEATS_ASM");
    return !(e && strcmp(e, "element") == 0);
  }();
  return on;
}

}  // namespace gsls

#include "gsls_asm_fluid.cuh"
#include "gsls_asm_lelas.cuh"
#include "gsls_asm_heatf.cuh"
#include "gsls_asm_ustruct.cuh"

namespace gsls {

// Colour launch, with programmatic dependent launch after the first colour
// (GSLS_ASM_PDL=0 launches the colours plainly)
static bool asm_pdl() {
  static const bool on = [] {
    const char *e = getenv("GSLS_ASM_PDL");
    return !(e && strcmp(e, "0") == 0);
  }();
  return on;
}
template <class K>
static int asm_launch(K kern, int nb, cudaStream_t st, const AsmArgs &A, bool pdl) {
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = pdl ? 1 : 0;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nb);
  cfg.blockDim = dim3(kAsmThreads);
  cfg.stream = st;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  GSLS_CUDA(cudaLaunchKernelEx(&cfg, kern, A));
  return GSLS_OK;
}

// ---------------------------------------------------------------------------
static int launch_assembly(gsls_mesh *m, const gsls_eq_params *p, const double *Ag,
                           const double *Yg, const double *Dg, double *R, void *Val,
                           int val_prec, double *Kd = nullptr, LinAsm *la = nullptr) {
  gsls_lhs *lhs = m->lhs;
  cudaStream_t st = lhs->stream;
  const int dof = p->dof;
  const size_t vbytes = (size_t)lhs->nnz * dof * dof * (val_prec == GSLS_PREC_MIXED ? 4 : 8);
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
  if (p->phys == GSLS_PHYS_CEP) {
    // isotropic CEP3D (Code/Source/svFSI/CEP.f:136-266) is HEATS3D with
    // unit density, no source and conductivity Diso
    A.rho = 1.0;
    A.src = 0.0;
    A.cond = p->Diso;
  }
  A.C10 = p->C10;
  A.Kpen = p->Kpen;
  A.visc = p->visc;
  A.dmp = p->dmp;
  for (int i = 0; i < 3; i++) A.fb[i] = p->fb[i];
  A.mu_f = p->mu_f;
  A.ctM = p->ctM;
  A.ctC = p->ctC;
  if (p->phys == GSLS_PHYS_FLUID &&
      (p->viscType < GSLS_VISC_CONST || p->viscType > GSLS_VISC_CASSON ||
       (p->viscType == GSLS_VISC_CY && !(p->va > 0.0)) ||
       (p->viscType == GSLS_VISC_CASSON && !(p->vlam > 0.0)))) {
    set_error("assembly: unknown viscosity model or a <= 0 (Carreau-Yasuda) / "
              "threshold <= 0 (Casson)");
    return GSLS_ERR_ARG;
  }
  A.viscType = p->viscType;
  A.mu_o = p->mu_o;
  A.vlam = p->vlam;
  A.va = p->va;
  A.vn = p->vn;
  A.E_s = p->elM;
  A.nu_s = p->nu;
  A.volType = p->volType;
  A.hf_amd = p->am / (p->af * p->gam * p->dt);
  A.hf_kT = 4.0 / (p->dt * p->dt);
  A.nFn = (p->phys == GSLS_PHYS_CEP) ? m->nFn : 0;  // only CEP reads the mesh's fibres
  A.fib = A.nFn > 0 ? m->d_fib.as<double>() : nullptr;
  for (int i = 0; i < 3; i++) A.Dani[i] = i < A.nFn ? p->Dani[i] : 0.0;
  if (p->phys == GSLS_PHYS_USTRUCT &&
      (p->dof != 4 || p->s + 4 > p->tDof || !Dg || !Kd || !(p->am > 0.0) ||
       !(p->rho > 0.0) || !(p->elM > 0.0) || p->volType < 0 || p->volType > 2 ||
       !(p->ctM > 0.0))) {
    set_error("assembly: USTRUCT needs dof 4, Dg, the Kd output, am, rho, elM > 0, "
              "ctM > 0 and volType 0..2");
    return GSLS_ERR_ARG;
  }
  if (p->phys == GSLS_PHYS_LELAS) {
    // F/LELAS.f:166-167
    A.lam_le = p->elM * p->nu / (1.0 + p->nu) / (1.0 - 2.0 * p->nu);
    A.mu_le = p->elM * 0.5 / (1.0 + p->nu);
  }
  A.ien = m->d_ien.as<int4>();
  A.map = m->d_map.as<int4>();
  A.x = m->d_x.as<double>();
  A.geo = m->d_geo.as<double>();
  A.nElAll = m->nEl;
  A.Ag = Ag;
  A.Yg = Yg;
  A.Dg = Dg;
  A.eparam = m->has_eparam ? m->d_eparam.as<double>() : nullptr;
  A.R = R;
  A.Val = Val;
  A.err = m->d_err.as<int>();
  const bool mixed = (val_prec == GSLS_PREC_MIXED);
  if ((p->phys == GSLS_PHYS_HEATS || p->phys == GSLS_PHYS_CEP) && lin_on()) {
    if (dof != 1) return GSLS_ERR_ARG;
    GSLS_TRY(lin_prepare(m, A));
    const double T1 = A.af * A.gam * A.dt;
    // a per-element nu, or the whole tensor with fibres, is inside Kg
    const double nu = (A.eparam || A.nFn > 0) ? 1.0 : A.cond;
    const long long nt = (long long)lhs->nNo * kLinLanes;
    const int nb = (int)((nt + 255) / 256);
    const int *rp = lhs->d_rowPtr.as<int>(), *cp = lhs->d_colPtr.as<int>();
    const double *M = m->d_linM.as<double>(), *K = m->d_linK.as<double>();
    const double cM = A.am * A.rho, cK = T1 * nu;
    // the caller's Val already holds this tangent (preconditioned): R only
    const bool skip = la && la->skip_val && la->serial == m->lin_serial && la->cM == cM &&
                      la->cK == cK;
#define GSLS_LIN(VT, KV, MT, KT)                                                               \
  k_asm_lin<VT, KV><<<nb, 256, 0, st>>>(lhs->nNo, rp, cp, M, K, MT, KT, m->d_linB.as<double>(), \
                                        Ag, Yg, A.tDof, A.s, A.rho, nu, A.rho * A.src, VT(cM),  \
                                        VT(cK), R, static_cast<VT *>(Val))
    if (mixed) {
      if (skip)
        GSLS_LIN(float, false, m->d_linM32.as<float>(), m->d_linK32.as<float>());
      else
        GSLS_LIN(float, true, m->d_linM32.as<float>(), m->d_linK32.as<float>());
    } else {
      if (skip)
        GSLS_LIN(double, false, M, K);
      else
        GSLS_LIN(double, true, M, K);
    }
#undef GSLS_LIN
    GSLS_CHECK_LAUNCH();
    if (la) {
      la->used = true;
      la->skipped = skip;
      la->serial = m->lin_serial;
      la->cM = cM;
      la->cK = cK;
    }
    return GSLS_OK;
  }
  GSLS_CUDA(cudaMemsetAsync(R, 0, sizeof(double) * (size_t)lhs->nNo * dof, st));
  GSLS_CUDA(cudaMemsetAsync(Val, 0, vbytes, st));
  if (p->phys == GSLS_PHYS_USTRUCT)
    GSLS_CUDA(cudaMemsetAsync(Kd, 0, sizeof(double) * 12 * (size_t)lhs->nnz, st));
  for (int c = 0; c < m->ncolors; c++) {
    A.el0 = m->color_off[c];
    A.nColorEl = m->color_off[c + 1] - m->color_off[c];
    if (A.nColorEl <= 0) continue;
    const int nb = (A.nColorEl + kAsmThreads - 1) / kAsmThreads;
    // the heat element is light: its colours gain nothing from overlapping
    const bool pdl = c > 0 && asm_pdl() && p->phys != GSLS_PHYS_HEATS && p->phys != GSLS_PHYS_CEP;
    if (p->phys == GSLS_PHYS_HEATS || p->phys == GSLS_PHYS_CEP) {
      if (dof != 1) return GSLS_ERR_ARG;
      if (mixed)
        GSLS_TRY(asm_launch(k_asm_heats<float>, nb, st, A, pdl));
      else
        GSLS_TRY(asm_launch(k_asm_heats<double>, nb, st, A, pdl));
    } else if (p->phys == GSLS_PHYS_STRUCT) {
      if (dof != 3 || p->s + 3 > p->tDof || !Dg) return GSLS_ERR_ARG;
      if (mixed)
        GSLS_TRY(asm_launch(k_asm_struct<float>, nb, st, A, pdl));
      else
        GSLS_TRY(asm_launch(k_asm_struct<double>, nb, st, A, pdl));
    } else if (p->phys == GSLS_PHYS_FLUID) {
      if (dof != 4 || p->s + 4 > p->tDof || !(p->rho > 0.0) || !(p->dt > 0.0)) return GSLS_ERR_ARG;
      const bool nn = (p->viscType != GSLS_VISC_CONST);
      if (mixed)
        GSLS_TRY(asm_launch(nn ? k_asm_fluid<float, true> : k_asm_fluid<float, false>, nb, st, A,
                            pdl));
      else
        GSLS_TRY(asm_launch(nn ? k_asm_fluid<double, true> : k_asm_fluid<double, false>, nb, st,
                            A, pdl));
    } else if (p->phys == GSLS_PHYS_HEATF) {
      if (dof != 1 || p->tDof < 4 || p->s < 3 || p->s >= p->tDof || !(p->dt > 0.0))
        return GSLS_ERR_ARG;
      if (mixed)
        GSLS_TRY(asm_launch(k_asm_heatf<float>, nb, st, A, pdl));
      else
        GSLS_TRY(asm_launch(k_asm_heatf<double>, nb, st, A, pdl));
    } else if (p->phys == GSLS_PHYS_USTRUCT) {
      if (mixed)
        k_asm_ustruct<float><<<nb, kAsmThreads, 0, st>>>(A, Kd);
      else
        k_asm_ustruct<double><<<nb, kAsmThreads, 0, st>>>(A, Kd);
    } else if (p->phys == GSLS_PHYS_LELAS) {
      if (dof != 3 || p->s + 3 > p->tDof || !Dg || !(p->elM > 0.0) || !(p->nu > -1.0) ||
          !(p->nu < 0.5) || !(p->dt > 0.0))
        return GSLS_ERR_ARG;
      if (mixed)
        GSLS_TRY(asm_launch(k_asm_lelas<float>, nb, st, A, pdl));
      else
        GSLS_TRY(asm_launch(k_asm_lelas<double>, nb, st, A, pdl));
    } else {
      set_error("assembly: physics not built in this version of the library");
      return GSLS_ERR_UNSUPPORTED;
    }
    GSLS_CHECK_LAUNCH();
  }
  return GSLS_OK;
}

// ---------------------------------------------------------------------------
// Parameter sensitivity of the element residual (adjoint dR/dp), one element
// per thread, no scatter: out[e] += scale * lambda_e . d(lR_e)/d(p_e) with
// p_e the per-element parameter of the physics (STRUCT: C10 = mu/2;
// HEATS/CEP: conductivity/diffusivity), evaluated at (Ag, Yg, Dg).
//   STRUCT: S_iso = J^-2/3 (2 C10 I - (2 C10 trC / 3) C^-1) is linear in C10,
//           so d lR(a,c)/d C10 = W Nx_a . (F S_iso / C10)(c,:)
//           (STRUCT.f:276-296, MATMODELS.f:136-150; W = sum_g w).
//   HEATS:  d lR(a)/d nu = W Nx_a . grad T (HEATS.f:146-154).
__global__ void __launch_bounds__(kAsmThreads) k_dRdp_struct(AsmArgs A, int nEl,
                                                             const double *__restrict__ lam,
                                                             double *out, double scale) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nEl) return;
  const int4 nd = A.ien[e];
  const int n4[4] = {nd.x, nd.y, nd.z, nd.w};
  double Nx[3][4];
  const double W = 4.0 * c_rule.w * load_geo(A, e, Nx);
  double F[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const double d = A.Dg[(size_t)n4[a] * A.tDof + A.s + c];
#pragma unroll
      for (int m = 0; m < 3; m++) F[c][m] += Nx[m][a] * d;
    }
  double Fi[3][3];
  const double J = adj_det3(F, Fi);
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) Fi[i][j] /= J;
  double Ci[3][3], trC = 0.0;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      Ci[i][j] = Fi[i][0] * Fi[j][0] + Fi[i][1] * Fi[j][1] + Fi[i][2] * Fi[j][2];
      trC += F[i][j] * F[i][j];
    }
  const double J2d = jm23(J);
  double St[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) St[i][j] = 2.0 * J2d * ((i == j ? 1.0 : 0.0) - trC / 3.0 * Ci[i][j]);
  double acc = 0.0;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    double Pt[3];
#pragma unroll
    for (int k = 0; k < 3; k++) Pt[k] = F[c][0] * St[0][k] + F[c][1] * St[1][k] + F[c][2] * St[2][k];
#pragma unroll
    for (int a = 0; a < 4; a++)
      acc += lam[(size_t)n4[a] * 3 + c] * W * (Nx[0][a] * Pt[0] + Nx[1][a] * Pt[1] + Nx[2][a] * Pt[2]);
  }
  out[e] += scale * acc;
}

__global__ void __launch_bounds__(kAsmThreads) k_dRdp_heats(AsmArgs A, int nEl,
                                                            const double *__restrict__ lam,
                                                            double *out, double scale) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nEl) return;
  const int4 nd = A.ien[e];
  const int n4[4] = {nd.x, nd.y, nd.z, nd.w};
  double yl[4];
#pragma unroll
  for (int a = 0; a < 4; a++) yl[a] = A.Yg[(size_t)n4[a] * A.tDof + A.s];
  double Nx[3][4];
  const double Jac = load_geo(A, e, Nx);
  double Tx[3];
#pragma unroll
  for (int i = 0; i < 3; i++) Tx[i] = Nx[i][0] * yl[0] + Nx[i][1] * yl[1] + Nx[i][2] * yl[2] + Nx[i][3] * yl[3];
  const double W = 4.0 * c_rule.w * Jac;
  double acc = 0.0;
#pragma unroll
  for (int a = 0; a < 4; a++)
    acc += lam[n4[a]] * W * (Nx[0][a] * Tx[0] + Nx[1][a] * Tx[1] + Nx[2][a] * Tx[2]);
  out[e] += scale * acc;
}

// out (colour order, nEl) += scale * (dR/dp)^T lambda
int mesh_dRdp(gsls_mesh *m, const gsls_eq_params *p, const double *Yg, const double *Dg,
              const double *lam, double *out, double scale) {
  AsmArgs A;
  memset(&A, 0, sizeof(A));
  A.tDof = p->tDof;
  A.s = p->s;
  A.ien = m->d_ien.as<int4>();
  A.x = m->d_x.as<double>();
  A.geo = m->d_geo.as<double>();
  A.nElAll = m->nEl;
  A.Yg = Yg;
  A.Dg = Dg;
  cudaStream_t st = m->lhs->stream;
  const int nb = (m->nEl + kAsmThreads - 1) / kAsmThreads;
  if (p->phys == GSLS_PHYS_STRUCT) {
    if (p->dof != 3 || !Dg) return GSLS_ERR_ARG;
    k_dRdp_struct<<<nb, kAsmThreads, 0, st>>>(A, m->nEl, lam, out, scale);
  } else if (p->phys == GSLS_PHYS_HEATS || p->phys == GSLS_PHYS_CEP) {
    k_dRdp_heats<<<nb, kAsmThreads, 0, st>>>(A, m->nEl, lam, out, scale);
  } else {
    set_error("dR/dp: physics without a per-element parameter sensitivity");
    return GSLS_ERR_UNSUPPORTED;
  }
  GSLS_CHECK_LAUNCH();
  return GSLS_OK;
}

// Consistent mass matrix M_ab = sum_g w N_a N_b as a scalar CSR (the HEATS
// element with unit density, no conduction and unit gen-alpha factors).
int mesh_mass(gsls_mesh *m, const double *zeros, double *R, double *Val) {
  gsls_lhs *lhs = m->lhs;
  cudaStream_t st = lhs->stream;
  GSLS_CUDA(cudaMemsetAsync(R, 0, sizeof(double) * (size_t)lhs->nNo, st));
  GSLS_CUDA(cudaMemsetAsync(Val, 0, sizeof(double) * (size_t)lhs->nnz, st));
  AsmArgs A;
  memset(&A, 0, sizeof(A));
  A.tDof = 1;
  A.am = A.af = A.gam = A.dt = 1.0;
  A.rho = 1.0;
  A.ien = m->d_ien.as<int4>();
  A.map = m->d_map.as<int4>();
  A.x = m->d_x.as<double>();
  A.geo = m->d_geo.as<double>();
  A.nElAll = m->nEl;
  A.Ag = A.Yg = A.Dg = zeros;
  A.R = R;
  A.Val = Val;
  A.err = m->d_err.as<int>();
  for (int c = 0; c < m->ncolors; c++) {
    A.el0 = m->color_off[c];
    A.nColorEl = m->color_off[c + 1] - m->color_off[c];
    if (A.nColorEl <= 0) continue;
    k_asm_heats<double><<<(A.nColorEl + kAsmThreads - 1) / kAsmThreads, kAsmThreads, 0, st>>>(A);
    GSLS_CHECK_LAUNCH();
  }
  return GSLS_OK;
}

// host copies for boundary-face setup: IEN (0-based, colour order, 4 per
// element) and the coordinates (3 per node)
int mesh_host_geometry(gsls_mesh *m, const int **ien, int *nEl, std::vector<double> &x) {
  *ien = m->h_ien.data();
  *nEl = m->nEl;
  x.resize((size_t)m->nNo * 3);
  GSLS_CUDA(cudaMemcpy(x.data(), m->d_x.p, sizeof(double) * x.size(), cudaMemcpyDeviceToHost));
  return GSLS_OK;
}

// colour-order index -> original element index
const int *mesh_perm(gsls_mesh *m, int *nEl) {
  *nEl = m->nEl;
  return m->perm.data();
}

int mesh_set_eparam(gsls_mesh *m, const double *eparam) {
  m->lin_ready = false;  // the heat/CEP conduction operator holds the parameter
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

// CEP fibres in original element order (3*nFn per element) -> the colour-
// ordered SoA table; nFn = 0 clears them
int mesh_set_fibers(gsls_mesh *m, int nFn, const double *fN) {
  if (nFn < 0 || nFn > 3 || (nFn > 0 && !fN)) {
    set_error("fibres: nFn must be 0..3 with 3*nFn directions per element");
    return GSLS_ERR_ARG;
  }
  m->lin_ready = false;  // the conduction operator holds the fibres
  m->nFn = nFn;
  if (nFn == 0) return GSLS_OK;
  const size_t nE = (size_t)m->nEl;
  std::vector<double> v(nE * 3 * nFn);
  for (size_t i = 0; i < nE; i++) {
    const double *f = fN + (size_t)m->perm[i] * 3 * nFn;
    for (int k = 0; k < 3 * nFn; k++) {
      if (!std::isfinite(f[k])) {
        m->nFn = 0;
        set_error("fibres: a non-finite fibre direction");
        return GSLS_ERR_ARG;
      }
      v[(size_t)k * nE + i] = f[k];
    }
  }
  GSLS_TRY(m->d_fib.alloc(sizeof(double) * v.size()));
  GSLS_CUDA(cudaMemcpyAsync(m->d_fib.p, v.data(), sizeof(double) * v.size(),
                            cudaMemcpyHostToDevice, m->lhs->stream));
  GSLS_CUDA(cudaStreamSynchronize(m->lhs->stream));
  return GSLS_OK;
}

int assemble_dev(gsls_mesh *m, const gsls_eq_params *p, const double *Ag, const double *Yg,
                 const double *Dg, double *R, void *Val, int val_prec, double *Kd,
                 LinAsm *la = nullptr) {
  return launch_assembly(m, p, Ag, Yg, Dg, R, Val, val_prec, Kd, la);
}

gsls_lhs *mesh_lhs(gsls_mesh *m) { return m->lhs; }

int mesh_coords_host(gsls_mesh *m, double *x) {
  GSLS_CUDA(cudaMemcpy(x, m->d_x.p, sizeof(double) * 3 * (size_t)m->nNo, cudaMemcpyDeviceToHost));
  return GSLS_OK;
}

int mesh_check_error(gsls_mesh *m) {
  if (m->bad_jac) {
    set_error("assembly: zero or non-finite element Jacobian");
    return GSLS_ERR_JAC;
  }
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
  lhs_attach(lhs, &m->lhs);
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
  if ((rc = m->d_geo.alloc(sizeof(double) * kGeo * (size_t)nEl))) {
    delete m;
    return rc;
  }
  k_geo_tet4<<<(nEl + 127) / 128, 128, 0, st>>>(nEl, m->d_ien.as<int4>(), m->d_x.as<double>(),
                                                m->d_geo.as<double>(), m->d_err.as<int>());
  count_launch();
  int herr = 0;
  cudaMemcpyAsync(&herr, m->d_err.p, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaError_t ce = cudaStreamSynchronize(st);
  if (ce != cudaSuccess) {
    delete m;
    return cuda_fail(ce, "mesh upload", __FILE__, __LINE__);
  }
  m->bad_jac = herr != 0;
  cudaMemsetAsync(m->d_err.p, 0, 16, st);
  *out = m;
  return GSLS_OK;
}

int gsls_mesh_free(gsls_mesh *m) {
  if (!m) return GSLS_ERR_ARG;
  if (m->lhs) {
    cudaStreamSynchronize(m->lhs->stream);
    lhs_detach(m->lhs, &m->lhs);
  } else {
    cudaDeviceSynchronize();  // its lhs (and stream) is gone already
  }
  delete m;
  return GSLS_OK;
}

int gsls_mesh_ncolors(const gsls_mesh *m) { return m ? m->ncolors : -1; }

int gsls_assemble_dev(gsls_mesh *m, const gsls_eq_params *p, const double *dAg,
                      const double *dYg, const double *dDg, double *dR, void *dVal,
                      int val_prec) {
  if (!m || !p || !dAg || !dYg || !dR || !dVal) return GSLS_ERR_ARG;
  if (p->nFn != 0 && p->phys != GSLS_PHYS_CEP) {
    set_error("assembly: fibres are read by CEP only");
    return GSLS_ERR_ARG;
  }
  GSLS_TRY(mesh_set_eparam(m, p->eparam));
  if (p->phys == GSLS_PHYS_CEP) GSLS_TRY(mesh_set_fibers(m, p->nFn, p->fN));
  GSLS_TRY(assemble_dev(m, p, dAg, dYg, dDg, dR, dVal, val_prec, nullptr));
  GSLS_CUDA(cudaStreamSynchronize(m->lhs->stream));
  return mesh_check_error(m);
}

int gsls_assemble_ustruct_dev(gsls_mesh *m, const gsls_eq_params *p, const double *dAg,
                              const double *dYg, const double *dDg, double *dR, void *dVal,
                              double *dKd, int val_prec) {
  if (!m || !p || !dAg || !dYg || !dDg || !dR || !dVal || !dKd ||
      p->phys != GSLS_PHYS_USTRUCT || p->nFn != 0)
    return GSLS_ERR_ARG;
  GSLS_TRY(assemble_dev(m, p, dAg, dYg, dDg, dR, dVal, val_prec, dKd));
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
