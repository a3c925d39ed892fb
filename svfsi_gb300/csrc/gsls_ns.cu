// Row-column scaling preconditioner (PRECONDRCS,
// Code/Source/svFSILS/PRECOND.f:150-368) and the NS block solver for
// incompressible flow (NSSOLVER, Code/Source/svFSILS/NSSOLVER.f:52-305, with
// CGRAD_SCHUR, CGRAD.f:51-123, GE, GE.f:51-151, and the GMRES of
// GMRES.f:51-169).
//
// GB300 layout:
//  * both need the CSR position of the transposed block; it is built once
//    per LHS on the host (the sparsity of a mesh is structurally symmetric);
//  * RCS keeps the Dirichlet-masked matrix and two scaling vectors W1 (rows)
//    and W2 (columns); each of its <= 10 passes takes the row and column
//    maxima of |Val| W1 W2 on the fly (column maxima gathered through the
//    transpose map, no atomics) and only the final pass rewrites Val;
//  * NSSOLVER's DEPART split (mK 3x3, mG 3x1, mD 1x3, mL, Gt = -mG^T) is one
//    kernel; the rectangular products SPARMULVS/SV/SS use 4 lanes per block
//    row; the Schur CG runs device-resident with the host polling a scalar
//    block every 8 iterations; the <= 20 x 20 least-squares system of each
//    outer iteration is solved on the host (GE).
// Vectors are in the Krylov type XT (FP32 in mixed mode), scalars in FP64.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "gsls_internal.cuh"
#include "gsls_gridbar.cuh"
#include "gsls_spmv.cuh"

namespace gsls {

constexpr int kNT = 256;

static inline int grid_for(size_t n, int cap) {
  size_t b = (n + kNT - 1) / kNT;
  if (b > (size_t)cap) b = cap;
  if (b < 1) b = 1;
  return (int)b;
}

// ---------------------------------------------------------------------------
// transpose map: tpos[j] = position of block (col(j), row(j))
static int build_tpos(gsls_lhs *lhs) {
  if (lhs->tpos_ok) return GSLS_OK;
  const int nNo = lhs->nNo, nnz = lhs->nnz;
  const std::vector<int> &rp = lhs->h_rowPtr, &cp = lhs->h_colPtr;
  std::vector<int> tp(nnz > 0 ? nnz : 1, -1);
  for (int i = 0; i < nNo; i++)
    for (int j = rp[i]; j < rp[i + 1]; j++) {
      const int k = cp[j];
      auto b = cp.begin() + rp[k], e = cp.begin() + rp[k + 1];
      auto it = std::lower_bound(b, e, i);
      if (it == e || *it != i) {
        set_error("RCS/NS: the sparsity pattern must be structurally symmetric with sorted "
                  "columns");
        return GSLS_ERR_ARG;
      }
      tp[j] = (int)(it - cp.begin());
    }
  GSLS_TRY(lhs->d_tpos.alloc(sizeof(int) * tp.size()));
  GSLS_CUDA(cudaMemcpy(lhs->d_tpos.p, tp.data(), sizeof(int) * tp.size(),
                       cudaMemcpyHostToDevice));
  lhs->tpos_ok = true;
  return GSLS_OK;
}

// ---------------------------------------------------------------------------
// RCS
struct RcsCtl {
  unsigned long long mx_r, mx_c;  // max |1 - W| of the pass (bits of a non-negative double)
  int active[16];                 // pass k runs iff active[k]
};

__device__ __forceinline__ double rcs_renorm(double w) { return w > 0.5 ? 1.0 : 0.0; }

// PRECONDRCS Dirichlet step (PRECOND.f:175-234): Wr = renormalised product
// of the face values; Val = diag(Wr) Val diag(Wr); R = Wr R; the diagonal of
// a masked row becomes 1.  D lanes per block row.
template <int D, class VT>
__global__ void __launch_bounds__(kNT) k_rcs_mask(int nNo, const int *__restrict__ rowPtr,
                                                  const int *__restrict__ colPtr,
                                                  const int *__restrict__ diagPtr, VT *Val,
                                                  const double *__restrict__ mask, double *R) {
  constexpr int RPW = 32 / D, DD = D * D;
  const int lane = threadIdx.x & 31, grp = lane / D, r = lane - grp * D;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int base = warp * RPW; base < nNo; base += nwarps * RPW) {
    const int i = base + grp;
    if (grp >= RPW || i >= nNo) continue;
    const double mr = rcs_renorm(mask[(size_t)i * D + r]);
    for (int j = rowPtr[i]; j < rowPtr[i + 1]; j++) {
      const int col = colPtr[j];
      VT *v = Val + (size_t)j * DD + r * D;
#pragma unroll
      for (int c = 0; c < D; c++) v[c] = VT(double(v[c]) * mr * rcs_renorm(mask[(size_t)col * D + c]));
    }
    R[(size_t)i * D + r] *= mr;
    VT *dg = Val + (size_t)diagPtr[i] * DD + r * D + r;
    *dg = VT(mr * (double(*dg) - 1.0) + 1.0);
  }
}

__global__ void k_fill(size_t n, double *a, double v) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x)
    a[k] = v;
}

__device__ __forceinline__ double block_max(double v, double *sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  const int nw = blockDim.x >> 5;
  v = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
  if (wid == 0)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// One RCS pass k (PRECOND.f:238-334): Wr(i,r) = max |Val(r,:)| over row i,
// Wc(i,c) = max |Val(:,c)| over column i (gathered through the transposed
// blocks of row i), with Val = Val_masked * W1(row) * W2(col).
template <int D, class VT>
__global__ void __launch_bounds__(kNT) k_rcs_rowcol(int k, int nNo, const int *__restrict__ rowPtr,
                                                    const int *__restrict__ colPtr,
                                                    const int *__restrict__ tpos,
                                                    const VT *__restrict__ Val,
                                                    const double *__restrict__ W1,
                                                    const double *__restrict__ W2, double *Wr,
                                                    double *Wc, RcsCtl *ctl) {
  if (!ctl->active[k]) return;
  __shared__ double sh[32];
  constexpr int RPW = 32 / D, DD = D * D;
  const int lane = threadIdx.x & 31, grp = lane / D, r = lane - grp * D;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  double dr = 0.0, dc = 0.0;
  for (int base = warp * RPW; base < nNo; base += nwarps * RPW) {
    const int i = base + grp;
    if (grp >= RPW || i >= nNo) continue;
    const double w1 = W1[(size_t)i * D + r], w2 = W2[(size_t)i * D + r];
    double rmax = 0.0, cmax = 0.0;
    for (int j = rowPtr[i]; j < rowPtr[i + 1]; j++) {
      const int col = colPtr[j];
      const VT *v = Val + (size_t)j * DD + r * D;
#pragma unroll
      for (int c = 0; c < D; c++)
        rmax = fmax(rmax, fabs(double(v[c])) * w1 * W2[(size_t)col * D + c]);
      // block (col, i): its column r belongs to column i of the matrix
      const VT *t = Val + (size_t)tpos[j] * DD + r;
#pragma unroll
      for (int rr = 0; rr < D; rr++)
        cmax = fmax(cmax, fabs(double(t[rr * D])) * W1[(size_t)col * D + rr] * w2);
    }
    Wr[(size_t)i * D + r] = rmax;
    Wc[(size_t)i * D + r] = cmax;
    dr = fmax(dr, fabs(1.0 - rmax));
    dc = fmax(dc, fabs(1.0 - cmax));
  }
  dr = block_max(dr, sh);
  __syncthreads();
  dc = block_max(dc, sh);
  if (threadIdx.x == 0) {
    atomicMax(&ctl->mx_r, (unsigned long long)__double_as_longlong(dr));
    atomicMax(&ctl->mx_c, (unsigned long long)__double_as_longlong(dc));
  }
}

// W1 *= Wr^-1/2, W2 *= Wc^-1/2 (PRECOND.f:334-341); decides whether pass
// k+1 runs (PRECOND.f:243-248, 331-332).
__global__ void k_rcs_apply(int k, size_t n, double *W1, double *W2, const double *Wr,
                            const double *Wc, RcsCtl *ctl, double tol, int maxiter) {
  if (!ctl->active[k]) return;
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n;
       q += (size_t)gridDim.x * blockDim.x) {
    W1[q] *= 1.0 / sqrt(Wr[q]);
    W2[q] *= 1.0 / sqrt(Wc[q]);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const double mr = __longlong_as_double((long long)ctl->mx_r);
    const double mc = __longlong_as_double((long long)ctl->mx_c);
    const bool stop = (k + 1 >= maxiter) || (mr < tol && mc < tol);
    ctl->active[k + 1] = stop ? 0 : 1;
    ctl->mx_r = 0ull;
    ctl->mx_c = 0ull;
  }
}

// Val = diag(W1) Val diag(W2), R = W1 R
template <int D, class VT>
__global__ void __launch_bounds__(kNT) k_rcs_final(int nNo, const int *__restrict__ rowPtr,
                                                   const int *__restrict__ colPtr, VT *Val,
                                                   const double *__restrict__ W1,
                                                   const double *__restrict__ W2, double *R) {
  constexpr int RPW = 32 / D, DD = D * D;
  const int lane = threadIdx.x & 31, grp = lane / D, r = lane - grp * D;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int base = warp * RPW; base < nNo; base += nwarps * RPW) {
    const int i = base + grp;
    if (grp >= RPW || i >= nNo) continue;
    const double w1 = W1[(size_t)i * D + r];
    for (int j = rowPtr[i]; j < rowPtr[i + 1]; j++) {
      const int col = colPtr[j];
      VT *v = Val + (size_t)j * DD + r * D;
#pragma unroll
      for (int c = 0; c < D; c++) v[c] = VT(double(v[c]) * w1 * W2[(size_t)col * D + c]);
    }
    R[(size_t)i * D + r] *= w1;
  }
}

template <int D, class VT>
static int precond_rcs_t(gsls_lhs *lhs, VT *Val, double *R, double *W) {
  GSLS_TRY(build_tpos(lhs));
  cudaStream_t st = lhs->stream;
  Workspace &ws = lhs->ws;
  const int nNo = lhs->nNo;
  const size_t n = (size_t)nNo * D;
  const size_t nal = (n + 31) & ~(size_t)31;
  GSLS_TRY(ws.rcs.alloc(sizeof(double) * 3 * nal + sizeof(RcsCtl) + 64));
  double *W1 = ws.rcs.as<double>(), *Wr = W1 + nal, *Wc = Wr + nal;
  RcsCtl *ctl = reinterpret_cast<RcsCtl *>(Wc + nal);
  const int G = lhs->grid;
  const int maxiter = 10;
  const double tol = 2.0;
  RcsCtl h;
  memset(&h, 0, sizeof(h));
  h.active[0] = 1;
  GSLS_CUDA(cudaMemcpyAsync(ctl, &h, sizeof(h), cudaMemcpyHostToDevice, st));
  k_fill<<<grid_for(n, G), kNT, 0, st>>>(n, W1, 1.0);
  GSLS_CHECK_LAUNCH();
  k_fill<<<grid_for(n, G), kNT, 0, st>>>(n, W, 1.0);
  GSLS_CHECK_LAUNCH();
  const int *rp = lhs->d_rowPtr.as<int>(), *cp = lhs->d_colPtr.as<int>();
  k_rcs_mask<D, VT><<<G, kNT, 0, st>>>(nNo, rp, cp, lhs->d_diagPtr.as<int>(), Val,
                                        ws.mask.as<double>(), R);
  GSLS_CHECK_LAUNCH();
  for (int k = 0; k < maxiter; k++) {
    k_rcs_rowcol<D, VT><<<G, kNT, 0, st>>>(k, nNo, rp, cp, lhs->d_tpos.as<int>(), Val, W1, W, Wr,
                                            Wc, ctl);
    GSLS_CHECK_LAUNCH();
    k_rcs_apply<<<grid_for(n, G), kNT, 0, st>>>(k, n, W1, W, Wr, Wc, ctl, tol, maxiter);
    GSLS_CHECK_LAUNCH();
  }
  k_rcs_final<D, VT><<<G, kNT, 0, st>>>(nNo, rp, cp, Val, W1, W, R);
  GSLS_CHECK_LAUNCH();
  return GSLS_OK;
}

int precond_rcs_run(gsls_lhs *lhs, int D, bool mixed, void *Val, double *R, double *W) {
  switch (D) {
#define GSLS_RCS_CASE(DV)                                                           \
  case DV:                                                                          \
    return mixed ? precond_rcs_t<DV, float>(lhs, (float *)Val, R, W)                \
                 : precond_rcs_t<DV, double>(lhs, (double *)Val, R, W);
    GSLS_RCS_CASE(1)
    GSLS_RCS_CASE(2)
    GSLS_RCS_CASE(3)
    GSLS_RCS_CASE(4)
#undef GSLS_RCS_CASE
    default:
      return GSLS_ERR_UNSUPPORTED;
  }
}

// ---------------------------------------------------------------------------
// NS solver kernels (nsd = 3, dof = 4)

// Rmi = Rm = R(1:3,:), Rci = Rc = R(4,:); |Rm|^2, |Rc|^2
template <class XT>
__global__ void __launch_bounds__(kNT) k_ns_split(int nNo, const double *__restrict__ R, XT *Rmi,
                                                  XT *Rci, XT *Rm, XT *Rc, double *partials,
                                                  unsigned *ticket, double *out) {
  __shared__ double sh[32];
  double am = 0.0, ac = 0.0;
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < nNo; a += gridDim.x * blockDim.x) {
#pragma unroll
    for (int m = 0; m < 3; m++) {
      const double v = R[(size_t)a * 4 + m];
      Rmi[(size_t)a * 3 + m] = XT(v);
      Rm[(size_t)a * 3 + m] = XT(v);
      am += v * v;
    }
    const double v = R[(size_t)a * 4 + 3];
    Rci[a] = XT(v);
    Rc[a] = XT(v);
    ac += v * v;
  }
  double bs[2];
  bs[0] = block_sum(am, sh);
  __syncthreads();
  bs[1] = block_sum(ac, sh);
  double tot[2];
  if (grid_reduce_last<2>(bs, partials, ticket, tot, sh) && threadIdx.x == 0) {
    out[0] = tot[0];
    out[1] = tot[1];
  }
}

// DEPART (NSSOLVER.f:237-305) for nsd = 3.  Also writes the Schur operands
// packed four to a block for the persistent CG: A1 = (mG, 0), A2 = (Gt, mL).
template <class VT>
__global__ void k_depart(int nnz, const VT *__restrict__ Val, const int *__restrict__ tpos, VT *mK,
                         VT *mG, VT *mD, VT *mL, VT *Gt, VT *A1, VT *A2) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < nnz; j += gridDim.x * blockDim.x) {
    const VT *t = Val + (size_t)j * 16;
    VT *k = mK + (size_t)j * 9;
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
      for (int c = 0; c < 3; c++) k[r * 3 + c] = t[r * 4 + c];
    const int l = tpos[j];
#pragma unroll
    for (int m = 0; m < 3; m++) {
      const VT g = t[m * 4 + 3];
      mG[(size_t)j * 3 + m] = g;
      mD[(size_t)j * 3 + m] = t[12 + m];
      Gt[(size_t)l * 3 + m] = -g;
      A1[(size_t)j * 4 + m] = g;
      A2[(size_t)l * 4 + m] = -g;
    }
    A1[(size_t)j * 4 + 3] = VT(0);
    mL[j] = t[15];
    A2[(size_t)j * 4 + 3] = t[15];
  }
}

// 16-byte (FP32) / 2 x 16-byte (FP64) vector access to 4 packed values
template <class T> struct V4;
template <> struct V4<float> {
  static __device__ __forceinline__ void ldg(const float *p, float o[4]) {
    const float4 v = __ldg(reinterpret_cast<const float4 *>(p));
    o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
  }
  static __device__ __forceinline__ void ldcg(const float *p, float o[4]) {
    const float4 v = __ldcg(reinterpret_cast<const float4 *>(p));
    o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
  }
  static __device__ __forceinline__ void stcg(float *p, float a, float b, float c, float d) {
    __stcg(reinterpret_cast<float4 *>(p), make_float4(a, b, c, d));
  }
};
template <> struct V4<double> {
  static __device__ __forceinline__ void ldg(const double *p, double o[4]) {
    const double2 a = __ldg(reinterpret_cast<const double2 *>(p));
    const double2 b = __ldg(reinterpret_cast<const double2 *>(p) + 1);
    o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
  }
  static __device__ __forceinline__ void ldcg(const double *p, double o[4]) {
    const double2 a = __ldcg(reinterpret_cast<const double2 *>(p));
    const double2 b = __ldcg(reinterpret_cast<const double2 *>(p) + 1);
    o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
  }
  static __device__ __forceinline__ void stcg(double *p, double a, double b, double c, double d) {
    __stcg(reinterpret_cast<double2 *>(p), make_double2(a, b));
    __stcg(reinterpret_cast<double2 *>(p) + 1, make_double2(c, d));
  }
};

// 4 lanes per block row, 8 rows per warp; lane q takes blocks rs+q, rs+q+4, ...
constexpr int kRL = 4;
template <class T>
__device__ __forceinline__ T quad_sum(T v) {
  v += __shfl_xor_sync(0xffffffffu, v, 1);
  v += __shfl_xor_sync(0xffffffffu, v, 2);
  return v;
}

// SPARMULVS (SPARMUL.f:135-200): y = K(1x3 blocks) . x3; y = sub - y when
// sub is given.  Skipped when *done is set.
template <class VT, class XT>
__global__ void __launch_bounds__(kNT) k_ns_vs(int nNo, const int *__restrict__ rowPtr,
                                               const int *__restrict__ colPtr,
                                               const VT *__restrict__ K, const XT *__restrict__ x,
                                               const XT *__restrict__ sub, XT *y,
                                               const int *done) {
  if (done && *(volatile const int *)done) return;
  using AT = typename AccOf<VT>::T;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int q = t & (kRL - 1);
  for (int i = t / kRL; i < (nNo + 7) / 8 * 8; i += (gridDim.x * blockDim.x) / kRL) {
    AT acc = AT(0);
    if (i < nNo)
      for (int j = rowPtr[i] + q; j < rowPtr[i + 1]; j += kRL) {
        const int col = colPtr[j];
#pragma unroll
        for (int m = 0; m < 3; m++) acc = fma(AT(K[(size_t)j * 3 + m]), AT(x[(size_t)col * 3 + m]), acc);
      }
    acc = quad_sum(acc);
    if (q == 0 && i < nNo) y[i] = sub ? XT(AT(sub[i]) - acc) : XT(acc);
  }
}

// SPARMULSV (SPARMUL.f:202-271): y3 = K(3x1 blocks) x; optionally
// y3b = sub3 - y3.  Skipped when *done is set.
template <class VT, class XT>
__global__ void __launch_bounds__(kNT) k_ns_sv(int nNo, const int *__restrict__ rowPtr,
                                               const int *__restrict__ colPtr,
                                               const VT *__restrict__ K, const XT *__restrict__ x,
                                               XT *y3, const XT *__restrict__ sub3, XT *y3b,
                                               const int *done) {
  if (done && *(volatile const int *)done) return;
  using AT = typename AccOf<VT>::T;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int q = t & (kRL - 1);
  for (int i = t / kRL; i < (nNo + 7) / 8 * 8; i += (gridDim.x * blockDim.x) / kRL) {
    AT a0 = AT(0), a1 = AT(0), a2 = AT(0);
    if (i < nNo)
      for (int j = rowPtr[i] + q; j < rowPtr[i + 1]; j += kRL) {
        const AT xv = AT(x[colPtr[j]]);
        a0 = fma(AT(K[(size_t)j * 3 + 0]), xv, a0);
        a1 = fma(AT(K[(size_t)j * 3 + 1]), xv, a1);
        a2 = fma(AT(K[(size_t)j * 3 + 2]), xv, a2);
      }
    a0 = quad_sum(a0);
    a1 = quad_sum(a1);
    a2 = quad_sum(a2);
    if (q == 0 && i < nNo) {
      y3[(size_t)i * 3 + 0] = XT(a0);
      y3[(size_t)i * 3 + 1] = XT(a1);
      y3[(size_t)i * 3 + 2] = XT(a2);
      if (y3b) {
        y3b[(size_t)i * 3 + 0] = XT(AT(sub3[(size_t)i * 3 + 0]) - a0);
        y3b[(size_t)i * 3 + 1] = XT(AT(sub3[(size_t)i * 3 + 1]) - a1);
        y3b[(size_t)i * 3 + 2] = XT(AT(sub3[(size_t)i * 3 + 2]) - a2);
      }
    }
  }
}

// MP(iB) = SPARMULSS(mL, P), MP(iBB) = SPARMULVS(mD, U)
template <class VT, class XT>
__global__ void __launch_bounds__(kNT) k_ns_ss_vs(int nNo, const int *__restrict__ rowPtr,
                                                  const int *__restrict__ colPtr,
                                                  const VT *__restrict__ L,
                                                  const XT *__restrict__ p,
                                                  const VT *__restrict__ K,
                                                  const XT *__restrict__ u, XT *ys, XT *yv) {
  using AT = typename AccOf<VT>::T;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int q = t & (kRL - 1);
  for (int i = t / kRL; i < (nNo + 7) / 8 * 8; i += (gridDim.x * blockDim.x) / kRL) {
    AT as = AT(0), av = AT(0);
    if (i < nNo)
      for (int j = rowPtr[i] + q; j < rowPtr[i + 1]; j += kRL) {
        const int col = colPtr[j];
        as = fma(AT(L[j]), AT(p[col]), as);
#pragma unroll
        for (int m = 0; m < 3; m++) av = fma(AT(K[(size_t)j * 3 + m]), AT(u[(size_t)col * 3 + m]), av);
      }
    as = quad_sum(as);
    av = quad_sum(av);
    if (q == 0 && i < nNo) {
      ys[i] = XT(as);
      yv[i] = XT(av);
    }
  }
}

// Schur CG scalar block (CGRAD_SCHUR, CGRAD.f:51-123)
struct SchurScal {
  double err, errO, eps, dot, iNorm2;
  int done, suc, itr, mItr;
};

// X = 0, Rs = Ps = P (in), |P|^2 -> err; decides the first stop test
template <class XT>
__global__ void __launch_bounds__(kNT) k_schur_init(int n, XT *Pio, XT *Rs, XT *Ps,
                                                    double *partials, unsigned *ticket,
                                                    SchurScal *sc, double absTol, double relTol,
                                                    int mItr) {
  __shared__ double sh[32];
  double acc = 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const XT v = Pio[k];
    Rs[k] = v;
    Ps[k] = v;
    Pio[k] = XT(0);
    acc += double(v) * double(v);
  }
  double bs = block_sum(acc, sh);
  double tot;
  if (grid_reduce_last<1>(&bs, partials, ticket, &tot, sh) && threadIdx.x == 0) {
    const double in = sqrt(tot);
    double e = fmax(absTol, relTol * in);
    e = e * e;
    sc->iNorm2 = tot;
    sc->err = in * in;
    sc->errO = in * in;
    sc->eps = e;
    sc->itr = 0;
    sc->mItr = mItr;
    sc->suc = (sc->err < e) ? 1 : 0;
    sc->done = (sc->suc || mItr < 1) ? 1 : 0;
  }
}

// SP = mL P - Gt GP (SPARMULSS, SPARMULVS, OMPSUMS(-1)); dot = P.SP
template <class VT, class XT>
__global__ void __launch_bounds__(kNT) k_schur_sp(int nNo, const int *__restrict__ rowPtr,
                                                  const int *__restrict__ colPtr,
                                                  const VT *__restrict__ L,
                                                  const VT *__restrict__ Gt,
                                                  const XT *__restrict__ P,
                                                  const XT *__restrict__ GP, XT *SP,
                                                  double *partials, unsigned *ticket,
                                                  SchurScal *sc) {
  if (*(volatile const int *)&sc->done) return;
  __shared__ double sh[32];
  using AT = typename AccOf<VT>::T;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int q = t & (kRL - 1);
  AT dot = AT(0);
  for (int i = t / kRL; i < (nNo + 7) / 8 * 8; i += (gridDim.x * blockDim.x) / kRL) {
    AT sl = AT(0), sd = AT(0);
    if (i < nNo)
      for (int j = rowPtr[i] + q; j < rowPtr[i + 1]; j += kRL) {
        const int col = colPtr[j];
        sl = fma(AT(L[j]), AT(P[col]), sl);
#pragma unroll
        for (int m = 0; m < 3; m++) sd = fma(AT(Gt[(size_t)j * 3 + m]), AT(GP[(size_t)col * 3 + m]), sd);
      }
    sl = quad_sum(sl);
    sd = quad_sum(sd);
    if (q == 0 && i < nNo) {
      const XT v = XT(sl + AT(-1) * sd);
      SP[i] = v;
      dot = fma(AT(P[i]), AT(v), dot);
    }
  }
  double bs = block_sum(double(dot), sh);
  double tot;
  if (grid_reduce_last<1>(&bs, partials, ticket, &tot, sh) && threadIdx.x == 0) sc->dot = tot;
}

// alpha = errO/dot; X += alpha P; R -= alpha SP; err = |R|^2; stop tests
template <class XT>
__global__ void __launch_bounds__(kNT) k_schur_update(int n, XT *X, const XT *__restrict__ P,
                                                      XT *R, const XT *__restrict__ SP,
                                                      double *partials, unsigned *ticket,
                                                      SchurScal *sc) {
  if (*(volatile const int *)&sc->done) return;
  __shared__ double sh[32];
  const double errO = sc->err;
  const double alpha = errO / sc->dot;
  const XT a = XT(alpha), ma = XT(-alpha);
  double acc = 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    X[k] = X[k] + a * P[k];
    const XT r = R[k] + ma * SP[k];
    R[k] = r;
    acc += double(r) * double(r);
  }
  double bs = block_sum(acc, sh);
  double tot;
  if (grid_reduce_last<1>(&bs, partials, ticket, &tot, sh) && threadIdx.x == 0) {
    double e = sqrt(tot);
    e = e * e;
    sc->errO = errO;
    sc->err = e;
    sc->itr += 1;
    if (!isfinite(e)) {
      sc->done = 3;
    } else if (sc->itr >= sc->mItr) {
      sc->done = 2;  // no stop test after the last iteration
    } else if (e < sc->eps) {
      sc->suc = 1;
      sc->done = 1;
    }
  }
}

// P = P + (errO/err) R; P = (err/errO) P
template <class XT>
__global__ void k_schur_pupdate(int n, XT *P, const XT *__restrict__ R, const SchurScal *sc) {
  const double err = sc->err, errO = sc->errO;
  const XT c1 = XT(errO / err), c2 = XT(err / errO);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    P[k] = c2 * (P[k] + c1 * R[k]);
}

// NS least-squares dots for column k: out[j] = MU_j.MUk + MP_j.MPk
// (j < nvec), out[nvec] = MUk.Rmi + MPk.Rci; one FP64 partial per (j, block)
template <class XT>
__global__ void __launch_bounds__(kNT) k_ns_multidot(int nNo, int nvec, const XT *__restrict__ MU,
                                                     size_t ldv, const XT *__restrict__ MP,
                                                     size_t lds, const XT *__restrict__ MUk,
                                                     const XT *__restrict__ MPk,
                                                     const XT *__restrict__ Rmi,
                                                     const XT *__restrict__ Rci,
                                                     double *partials) {
  const int per = (nNo + gridDim.x - 1) / gridDim.x;
  const int s = blockIdx.x * per;
  const int e = min(s + per, nNo);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int j = wid; j <= nvec; j += nw) {
    const XT *u = (j < nvec) ? MU + ldv * j : Rmi;
    const XT *p = (j < nvec) ? MP + lds * j : Rci;
    XT acc = XT(0);
    for (int a = s + lane; a < e; a += 32) {
      acc = fma(u[(size_t)a * 3 + 0], MUk[(size_t)a * 3 + 0], acc);
      acc = fma(u[(size_t)a * 3 + 1], MUk[(size_t)a * 3 + 1], acc);
      acc = fma(u[(size_t)a * 3 + 2], MUk[(size_t)a * 3 + 2], acc);
      acc = fma(p[a], MPk[a], acc);
    }
    double v = warp_sum(double(acc));
    if (lane == 0) partials[(size_t)j * gridDim.x + blockIdx.x] = v;
  }
}

__global__ void k_ns_colsum(int grid, const double *partials, double *out) {
  __shared__ double sh[32];
  const int j = blockIdx.x;
  double s = 0.0;
  for (int b = threadIdx.x; b < grid; b += blockDim.x) s += partials[(size_t)j * grid + b];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) out[j] = s;
}

// out = (base ? base : 0) + sign * sum_j c_j V_j, sequential in j
struct NsCoef {
  double c[40];
};
template <class XT>
__global__ void k_ns_comb(size_t n, XT *out, const XT *__restrict__ base, const XT *__restrict__ V,
                          size_t ld, int stride, int first, int nc, NsCoef cf, double sign) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    XT acc = base ? base[k] : XT(0);
    for (int j = 0; j < nc; j++) {
      const XT cj = XT(sign * cf.c[j]);
      acc = acc + cj * V[ld * (size_t)(first + j * stride) + k];
    }
    out[k] = acc;
  }
}

// |v|^2
template <class XT>
__global__ void __launch_bounds__(kNT) k_ns_norm2(int n, const XT *__restrict__ v,
                                                  double *partials, unsigned *ticket,
                                                  double *out) {
  __shared__ double sh[32];
  double acc = 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    acc += double(v[k]) * double(v[k]);
  double bs = block_sum(acc, sh);
  double tot;
  if (grid_reduce_last<1>(&bs, partials, ticket, &tot, sh) && threadIdx.x == 0) *out = tot;
}

// Ri(1:3) = Rmi, Ri(4) = Rci, then SOLVE's R = Wc R
template <class XT>
__global__ void k_ns_out(int nNo, double *R, const XT *__restrict__ Rm, const XT *__restrict__ Rc,
                         const double *__restrict__ W) {
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < nNo; a += gridDim.x * blockDim.x) {
#pragma unroll
    for (int m = 0; m < 3; m++)
      R[(size_t)a * 4 + m] = W[(size_t)a * 4 + m] * double(Rm[(size_t)a * 3 + m]);
    R[(size_t)a * 4 + 3] = W[(size_t)a * 4 + 3] * double(Rc[a]);
  }
}

// GE (GE.f:51-151): symmetric diagonal scaling then Gaussian elimination
// with partial pivoting on the leading N x N block of A (leading dim nV,
// column-major).  Returns false (B = 0) when singular.
static bool ge_solve(int nV, int N, const std::vector<double> &A, std::vector<double> &B) {
  const double kEps = 2.220446049250313e-16, kTiny = 2.2250738585072014e-308;
  auto AA = [&](int i, int j) { return A[(size_t)j * nV + i]; };
  std::vector<double> W(N > 0 ? N : 1);
  for (int i = 0; i < N; i++) {
    if (fabs(AA(i, i)) < kTiny) {
      std::fill(B.begin(), B.begin() + N, 0.0);
      return false;
    }
    W[i] = 1.0 / sqrt(fabs(AA(i, i)));
  }
  if (N <= 0) return false;
  std::vector<double> C((size_t)N * (N + 1));
  auto CC = [&](int i, int j) -> double & { return C[(size_t)j * N + i]; };
  for (int i = 0; i < N; i++) {
    for (int j = 0; j < N; j++) CC(i, j) = W[i] * W[j] * AA(i, j);
    CC(i, N) = W[i] * B[i];
  }
  if (N == 1) {
    B[0] = CC(0, 1) / CC(0, 0);
    B[0] = B[0] * W[0];
    return true;
  }
  if (N == 2) {
    const double pivot = CC(0, 0) * CC(1, 1) - CC(1, 0) * CC(0, 1);
    if (fabs(pivot) < kEps) {
      B[0] = B[1] = 0.0;
      return false;
    }
    B[0] = (CC(0, 2) * CC(1, 1) - CC(1, 2) * CC(0, 1)) / pivot;
    B[1] = (CC(1, 2) * CC(0, 0) - CC(0, 2) * CC(1, 0)) / pivot;
    B[0] = W[0] * B[0];
    B[1] = W[1] * B[1];
    return true;
  }
  for (int m = 0; m < N - 1; m++) {
    int ipv = m;
    double pivot = fabs(CC(m, m));
    for (int i = m + 1; i < N; i++)
      if (fabs(CC(i, m)) > pivot) {
        ipv = i;
        pivot = fabs(CC(i, m));
      }
    if (fabs(pivot) < kEps) {
      std::fill(B.begin(), B.begin() + N, 0.0);
      return false;
    }
    if (ipv != m)
      for (int j = m; j <= N; j++) std::swap(CC(m, j), CC(ipv, j));
    for (int i = m + 1; i < N; i++) {
      const double f = CC(i, m) / CC(m, m);
      CC(i, m) = 0.0;
      for (int j = m + 1; j <= N; j++) CC(i, j) = CC(i, j) - f * CC(m, j);
    }
  }
  for (int j = N - 1; j >= 0; j--) {
    for (int i = j + 1; i < N; i++) CC(j, N) = CC(j, N) - CC(j, i) * CC(i, N);
    CC(j, N) = CC(j, N) / CC(j, j);
  }
  for (int i = 0; i < N; i++) B[i] = W[i] * CC(i, N);
  return true;
}

// ---------------------------------------------------------------------------
// Persistent Schur CG: every iteration of CGRAD_SCHUR in one cooperative
// launch.  Phases are separated by a grid barrier (generation counter; each
// wait is bounded and sets an error word when it gives up, after which
// every block returns).  Data written by other blocks is read through L2
// (__ldcg); the matrix blocks are read-only.  Reductions: one FP64 partial
// per block, summed in block order by every block (identical result in all
// blocks, reproducible for a fixed grid).
template <class VT, class XT>
struct SchurArgs {
  int nNo;
  const int *rowPtr, *colPtr;
  const VT *A1, *A2;              // (mG, 0) and (Gt, mL) per CSR block
  XT *X, *Pa, *Pb, *R, *SP, *GP;  // Pa holds the initial direction; GP 4 per node
  double *part;                   // 2 * gridDim.x
  GridBar *bar;
  SchurScal *sc;
  int K;                          // rows per 4-lane group (row slots)
  int zz;                         // reverse the row-slot order on odd iterations
  unsigned spin;                  // poll limit of the grid barrier
};

constexpr int kPT = 1024;
constexpr int kPQ = kPT / kRL;  // 4-lane groups per block

// Row slots of a block: slot (k, g) is row blockIdx.x*kPQ + g + k*gridDim.x*kPQ.
// The K segments of a block are contiguous in the CSR; their column
// indices and row ranges are staged in shared memory once per launch:
//   srp[k*kPQ + g] = (first, end) of the row in scol, sdel[k] = global - local
__device__ __forceinline__ void schur_stage(const int *__restrict__ rowPtr,
                                            const int *__restrict__ colPtr, int nNo, int K,
                                            int2 *srp, int *sdel, int *scol) {
  const int nq = gridDim.x * kPQ;
  int off = 0;
  for (int k = 0; k < K; k++) {
    const int base = blockIdx.x * kPQ + k * nq;
    if (base >= nNo) {
      if (threadIdx.x < kPQ) srp[k * kPQ + threadIdx.x] = make_int2(0, 0);
      if (threadIdx.x == 0) sdel[k] = 0;
      continue;
    }
    const int hi = min(base + kPQ, nNo);
    const int s0 = __ldg(rowPtr + base), s1 = __ldg(rowPtr + hi);
    for (int j = threadIdx.x; j < s1 - s0; j += blockDim.x) scol[off + j] = __ldg(colPtr + s0 + j);
    if (threadIdx.x < kPQ) {
      const int i = base + threadIdx.x;
      srp[k * kPQ + threadIdx.x] =
          (i < nNo) ? make_int2(__ldg(rowPtr + i) - s0 + off, __ldg(rowPtr + i + 1) - s0 + off)
                    : make_int2(0, 0);
    }
    if (threadIdx.x == 0) sdel[k] = s0 - off;
    off += s1 - s0;
  }
  __syncthreads();
}

// Iteration k of CGRAD_SCHUR (CGRAD.f:86-110), three phases:
//  1. P_k = (err/errO) (P_{k-1} + (errO/err) R) formed on the fly from the
//     previous direction (the reference's two OMPSUMS/OMPMULS steps; P_1 = R
//     exactly with errO/err = 0, err/errO = 1) and GP = mG P_k; the owner of
//     row i stores P_k(i) in the other buffer;
//  2. SP = mL P_k - Gt GP and the block partials of P_k.SP;
//  3. alpha = errO/dot, X += alpha P_k, R -= alpha SP and the partials of |R|^2.
// With zz set, odd iterations visit the row slots last to first, so the
// operator blocks read at the end of one pass are the first read by the
// next and are still in L2 when the operator does not fit there whole.
template <class VT, class XT>
__global__ void __launch_bounds__(kPT, 1) k_schur_persistent(SchurArgs<VT, XT> A) {
  using AT = typename AccOf<VT>::T;
  constexpr int kPU = sizeof(AT) == 4 ? 4 : 2;  // blocks per lane issued together
  extern __shared__ int4 smem_raw[];
  int2 *srp = reinterpret_cast<int2 *>(smem_raw);
  int *sdel = reinterpret_cast<int *>(srp + A.K * kPQ);
  int *scol = sdel + ((A.K + 3) & ~3);
  __shared__ double sh[32];
  const unsigned nblk = gridDim.x;
  const int nNo = A.nNo, K = A.K;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nthr = gridDim.x * blockDim.x;
  const int q = t & (kRL - 1), g = threadIdx.x / kRL;
  const int nq = gridDim.x * kPQ;
  double err = A.sc->err;
  const double eps = A.sc->eps;
  const int mItr = A.sc->mItr;
  int done = A.sc->done, suc = A.sc->suc, itr = 0;
  double errO = A.sc->errO;
  XT c1 = XT(0), c2 = XT(1);
  XT *Pold = A.Pa, *Pnew = A.Pb;
  bool ok = true;
  unsigned epoch = 0;
  schur_stage(A.rowPtr, A.colPtr, nNo, K, srp, sdel, scol);
  while (!done) {
    const bool rev = A.zz && (itr & 1);
    // phase 1: P_k on the fly, GP = mG P_k
    for (int kk = 0; kk < K; kk++) {
      const int k = rev ? K - 1 - kk : kk;
      const int i = blockIdx.x * kPQ + g + k * nq;
      if ((i & ~7) >= nNo) continue;  // warp-uniform: a warp covers 8 consecutive rows
      const int2 rr = srp[k * kPQ + g];
      const int dl = sdel[k];
      // the owner's own entry of P_k, loaded before the gathers
      XT pown = XT(0);
      if (q == 0 && i < nNo) pown = XT(c2 * (__ldcg(Pold + i) + c1 * __ldcg(A.R + i)));
      AT a0 = AT(0), a1 = AT(0), a2 = AT(0);
      for (int j0 = rr.x + q; j0 < rr.y; j0 += kPU * kRL) {
        AT pv[kPU], gv[kPU][3];
#pragma unroll
        for (int u = 0; u < kPU; u++) {
          const int jl = j0 + u * kRL;
          if (jl < rr.y) {
            const int col = scol[jl];
            const size_t j = (size_t)(jl + dl);
            pv[u] = AT(c2 * (__ldcg(Pold + col) + c1 * __ldcg(A.R + col)));
            VT a4[4];
            V4<VT>::ldg(A.A1 + j * 4, a4);
#pragma unroll
            for (int m = 0; m < 3; m++) gv[u][m] = AT(a4[m]);
          } else {
            pv[u] = AT(0);
#pragma unroll
            for (int m = 0; m < 3; m++) gv[u][m] = AT(0);
          }
        }
#pragma unroll
        for (int u = 0; u < kPU; u++) {
          a0 = fma(gv[u][0], pv[u], a0);
          a1 = fma(gv[u][1], pv[u], a1);
          a2 = fma(gv[u][2], pv[u], a2);
        }
      }
      a0 = quad_sum(a0);
      a1 = quad_sum(a1);
      a2 = quad_sum(a2);
      if (q == 0 && i < nNo) {
        V4<XT>::stcg(A.GP + (size_t)i * 4, XT(a0), XT(a1), XT(a2), XT(0));
        __stcg(Pnew + i, pown);
      }
    }
    if (!(ok = grid_bar(A.bar, nblk, epoch, A.spin))) break;
    // phase 2: SP = mL P - Gt GP; dot = P.SP
    AT dloc = AT(0);
    for (int kk = 0; kk < K; kk++) {
      const int k = rev ? K - 1 - kk : kk;
      const int i = blockIdx.x * kPQ + g + k * nq;
      if ((i & ~7) >= nNo) continue;
      const int2 rr = srp[k * kPQ + g];
      const int dl = sdel[k];
      const AT pown = (q == 0 && i < nNo) ? AT(__ldcg(Pnew + i)) : AT(0);
      AT sl = AT(0), sd = AT(0);
      for (int j0 = rr.x + q; j0 < rr.y; j0 += kPU * kRL) {
        AT lv[kPU], pv[kPU], gt[kPU][3], gp[kPU][3];
#pragma unroll
        for (int u = 0; u < kPU; u++) {
          const int jl = j0 + u * kRL;
          if (jl < rr.y) {
            const int col = scol[jl];
            const size_t j = (size_t)(jl + dl);
            VT a4[4];
            V4<VT>::ldg(A.A2 + j * 4, a4);
            XT g4[4];
            V4<XT>::ldcg(A.GP + (size_t)col * 4, g4);
            lv[u] = AT(a4[3]);
            pv[u] = AT(__ldcg(Pnew + col));
#pragma unroll
            for (int m = 0; m < 3; m++) {
              gt[u][m] = AT(a4[m]);
              gp[u][m] = AT(g4[m]);
            }
          } else {
            lv[u] = pv[u] = AT(0);
#pragma unroll
            for (int m = 0; m < 3; m++) gt[u][m] = gp[u][m] = AT(0);
          }
        }
#pragma unroll
        for (int u = 0; u < kPU; u++) {
          sl = fma(lv[u], pv[u], sl);
#pragma unroll
          for (int m = 0; m < 3; m++) sd = fma(gt[u][m], gp[u][m], sd);
        }
      }
      sl = quad_sum(sl);
      sd = quad_sum(sd);
      if (q == 0 && i < nNo) {
        const XT v = XT(sl + AT(-1) * sd);
        __stcg(A.SP + i, v);
        dloc = fma(pown, AT(v), dloc);
      }
    }
    {
      const double bs = block_sum(double(dloc), sh);
      if (threadIdx.x == 0) __stcg(A.part + blockIdx.x, bs);
    }
    if (!(ok = grid_bar(A.bar, nblk, epoch, A.spin))) break;
    // phase 3: X, R and |R|^2
    const double dot = sum_partials(A.part, nblk, sh);
    errO = err;
    const double alpha = errO / dot;
    const XT al = XT(alpha), mal = XT(-alpha);
    double eloc = 0.0;
    for (int k = t; k < nNo; k += nthr) {
      __stcg(A.X + k, XT(__ldcg(A.X + k) + al * __ldcg(Pnew + k)));
      const XT r = XT(__ldcg(A.R + k) + mal * __ldcg(A.SP + k));
      __stcg(A.R + k, r);
      eloc += double(r) * double(r);
    }
    {
      const double bs = block_sum(eloc, sh);
      if (threadIdx.x == 0) __stcg(A.part + nblk + blockIdx.x, bs);
    }
    if (!(ok = grid_bar(A.bar, nblk, epoch, A.spin))) break;
    double e = sqrt(sum_partials(A.part + nblk, nblk, sh));
    e = e * e;
    err = e;
    itr++;
    c1 = XT(errO / err);
    c2 = XT(err / errO);
    XT *tmp = Pold;
    Pold = Pnew;
    Pnew = tmp;
    if (!isfinite(err)) {
      done = 3;
    } else if (itr >= mItr) {
      done = 2;  // no stop test after the last iteration
    } else if (err < eps) {
      suc = 1;
      done = 1;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    SchurScal *sc = A.sc;
    sc->err = err;
    sc->errO = errO;
    sc->itr = itr;
    sc->suc = suc;
    sc->done = ok ? done : 4;
  }
}

// Launch geometry of the persistent Schur CG: one block per SM, K row slots
// per 4-lane group, shared memory for the staged rows of the largest block
// (0 when it does not fit: the caller then uses the per-kernel path).
static size_t schur_geometry(const gsls_lhs *lhs, int nblk, int *K_out) {
  const int nNo = lhs->nNo, nq = nblk * kPQ;
  const int K = (nNo + nq - 1) / nq;
  const std::vector<int> &rp = lhs->h_rowPtr;
  long long mx = 0;
  for (int b = 0; b < nblk; b++) {
    long long tot = 0;
    for (int k = 0; k < K; k++) {
      const int base = b * kPQ + k * nq;
      if (base >= nNo) break;
      const int hi = std::min(base + kPQ, nNo);
      tot += rp[hi] - rp[base];
    }
    mx = std::max(mx, tot);
  }
  *K_out = K;
  const size_t bytes = (size_t)K * kPQ * sizeof(int2) + (size_t)((K + 3) & ~3) * sizeof(int) +
                       (size_t)mx * sizeof(int);
  return bytes <= 200 * 1024 ? bytes : 0;
}

// CGRAD_SCHUR on P (in: right-hand side, out: solution)
template <class VT, class XT>
static int schur_cg(gsls_lhs *lhs, gsls_sub_ls *ls, const VT *mG, const VT *Gt, const VT *mL,
                    const VT *A1, const VT *A2, XT *P, XT *Rs, XT *Ps, XT *Pb, XT *SP, XT *GP,
                    XT *GP4, SchurScal *sc, SchurScal *h_sc, GridBar *db) {
  cudaStream_t st = lhs->stream;
  const int nNo = lhs->nNo, G = lhs->grid;
  double *part = lhs->ws.partials.as<double>();
  unsigned *tk = lhs->ws.ticket.as<unsigned>();
  const int *rp = lhs->d_rowPtr.as<int>(), *cp = lhs->d_colPtr.as<int>();
  auto t0 = std::chrono::steady_clock::now();
  ls->suc = 0;
  k_schur_init<XT><<<G, kNT, 0, st>>>(nNo, P, Rs, Ps, part, tk, sc, ls->absTol, ls->relTol, ls->mItr);
  GSLS_CHECK_LAUNCH();
  static const bool kernels = [] {
    const char *e = getenv("GSLS_SCHUR");
    return e && strcmp(e, "kernels") == 0;
  }();
  // the coupled-face PRE term needs a global dot between the two Schur
  // products: the per-kernel path carries it
  bool use_kernels = kernels || lhs->ws.cpl_on;
  if (!use_kernels) {
    // persistent cooperative kernel: one block per SM
    const int nblk = num_sms();
    int K = 0;
    const size_t smem = schur_geometry(lhs, nblk, &K);
    int nb = 0;
    if (smem) {
      GSLS_CUDA(cudaFuncSetAttribute(k_schur_persistent<VT, XT>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      GSLS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_schur_persistent<VT, XT>, kPT,
                                                              smem));
    }
    if (nb < 1) {
      use_kernels = true;  // rows of a block do not fit in shared memory
    } else {
      GSLS_TRY(lhs->ws.partials.alloc(sizeof(double) * ((size_t)2 * nblk + 64) + 64));
      GSLS_CUDA(cudaMemsetAsync(db, 0, sizeof(GridBar), st));
      SchurArgs<VT, XT> a{nNo, rp, cp, A1, A2, P, Ps, Pb, Rs, SP, GP4,
                          lhs->ws.partials.as<double>(), db, sc, K, zigzag_on(),
                          wait_limit()};
      void *args[] = {&a};
      const bool prof = prof_on();
      cudaEvent_t pe0 = nullptr, pe1 = nullptr;
      if (prof) {
        GSLS_CUDA(cudaEventCreate(&pe0));
        GSLS_CUDA(cudaEventCreate(&pe1));
        GSLS_CUDA(cudaEventRecord(pe0, st));
      }
      GSLS_CUDA(cudaLaunchCooperativeKernel((const void *)k_schur_persistent<VT, XT>, dim3(nblk),
                                            dim3(kPT), args, smem, st));
      GSLS_CHECK_LAUNCH();
      if (prof) GSLS_CUDA(cudaEventRecord(pe1, st));
      GSLS_CUDA(cudaMemcpyAsync(h_sc, sc, sizeof(SchurScal), cudaMemcpyDeviceToHost, st));
      GSLS_CUDA(cudaStreamSynchronize(st));
      if (prof) {
        // per CG iteration: count = iterations of this call
        float ms = 0.f;
        GSLS_CUDA(cudaEventElapsedTime(&ms, pe0, pe1));
        prof_add("schur", h_sc->itr, ms);
        prof_add("schur_calls", 1, ms);
        cudaEventDestroy(pe0);
        cudaEventDestroy(pe1);
      }
      if (h_sc->done == 4) {
        set_error("NS: grid barrier of the Schur-complement CG timed out");
        return GSLS_ERR_CUDA;
      }
    }
  }
  const int batch = 8;
  for (; use_kernels;) {
    GSLS_CUDA(cudaMemcpyAsync(h_sc, sc, sizeof(SchurScal), cudaMemcpyDeviceToHost, st));
    GSLS_CUDA(cudaStreamSynchronize(st));
    if (h_sc->done) break;
    for (int b = 0; b < batch; b++) {
      k_ns_sv<VT, XT><<<G, kNT, 0, st>>>(nNo, rp, cp, mG, Ps, GP, nullptr, nullptr, &sc->done);
      GSLS_CHECK_LAUNCH();
      launch_addbcmul<XT>(lhs, 1, 3, GP, GP, &sc->done);
      k_schur_sp<VT, XT><<<G, kNT, 0, st>>>(nNo, rp, cp, mL, Gt, Ps, GP, SP, part, tk, sc);
      GSLS_CHECK_LAUNCH();
      k_schur_update<XT><<<G, kNT, 0, st>>>(nNo, P, Ps, Rs, SP, part, tk, sc);
      GSLS_CHECK_LAUNCH();
      k_schur_pupdate<XT><<<G, kNT, 0, st>>>(nNo, Ps, Rs, sc);
      GSLS_CHECK_LAUNCH();
    }
  }
  if (h_sc->done == 3) {
    set_error("NS: NaN/Inf in the Schur-complement CG");
    return GSLS_ERR_NAN;
  }
  ls->iNorm = sqrt(h_sc->iNorm2);
  ls->suc = h_sc->suc;
  ls->fNorm = sqrt(h_sc->err);
  ls->itr += h_sc->itr;
  ls->dB = (h_sc->errO < 2.220446049250313e-16) ? 0.0 : 5.0 * log(h_sc->err / h_sc->errO);
  ls->callD += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return GSLS_OK;
}

template <class VT, class XT>
static int ns_t(gsls_lhs *lhs, gsls_ls *ls, const VT *Val, double *R, const double *W) {
  GSLS_TRY(build_tpos(lhs));
  cudaStream_t st = lhs->stream;
  Workspace &ws = lhs->ws;
  const int nNo = lhs->nNo, nnz = lhs->nnz, G = lhs->grid;
  const int mI = ls->RI.mItr;
  if (mI < 1 || mI > 20) {
    set_error("NS: RI.mItr must be in [1, 20]");
    return GSLS_ERR_ARG;
  }
  const int nB = 2 * mI;
  auto t0 = std::chrono::steady_clock::now();
  // vectors: Rmi Rm GP MU(nB) U(mI) (3-vectors); Rci Rc Rs Ps SP Pb MP(nB) P(mI) (scalars)
  const size_t l3 = ((size_t)nNo * 3 + 63) & ~(size_t)63, l1 = ((size_t)nNo + 63) & ~(size_t)63;
  const size_t nvec3 = 5 + (size_t)nB + mI, nvec1 = 6 + (size_t)nB + mI;
  GSLS_TRY(ws.ns_vec.alloc(sizeof(XT) * (nvec3 * l3 + nvec1 * l1) + 2048 + 2 * sizeof(SchurScal)));
  XT *v3 = ws.ns_vec.as<XT>();
  XT *Rmi = v3, *Rm = v3 + l3, *GP = v3 + 2 * l3, *GP4 = v3 + 3 * l3;  // GP4: 4 per node
  XT *MU = v3 + 5 * l3, *U = MU + (size_t)nB * l3;
  XT *v1 = v3 + nvec3 * l3;
  XT *Rci = v1, *Rc = v1 + l1, *Rs = v1 + 2 * l1, *Ps = v1 + 3 * l1, *SP = v1 + 4 * l1;
  XT *Pb = v1 + 5 * l1, *MP = v1 + 6 * l1, *P = MP + (size_t)nB * l1;
  SchurScal *sc = reinterpret_cast<SchurScal *>(
      (reinterpret_cast<uintptr_t>(v1 + nvec1 * l1) + 127) & ~(uintptr_t)127);
  double *dsc = reinterpret_cast<double *>(sc + 2);  // 96 doubles: norms and dots
  GridBar *bar = reinterpret_cast<GridBar *>(dsc + 96);
  const size_t m9 = (size_t)nnz * 9, m3 = (size_t)nnz * 3;
  const size_t m1 = ((size_t)nnz + 15) & ~(size_t)15;
  GSLS_TRY(ws.ns_mat.alloc(sizeof(VT) * (m9 + 4 * m3 + m1 + 8 * (size_t)nnz) + 256));
  VT *mK = ws.ns_mat.as<VT>(), *mG = mK + m9, *mD = mG + m3, *Gt = mD + m3, *mL = Gt + m3;
  VT *A1 = reinterpret_cast<VT *>((reinterpret_cast<uintptr_t>(mL + m1) + 63) & ~(uintptr_t)63);
  VT *A2 = A1 + 4 * (size_t)nnz;
  // the GMRES workspace may grow ws.partials: size it for both up front
  const int Gd = num_sms() * 2;
  const int sD = ls->GM.sD > 0 ? ls->GM.sD : 1;
  GSLS_TRY(ws.partials.alloc(sizeof(double) * (size_t)(std::max(sD, nB) + 2) * std::max(Gd, G) * 2 +
                             64));
  double *part = ws.partials.as<double>();
  unsigned *tk = ws.ticket.as<unsigned>();
  SchurScal h_sc;
  const int *rp = lhs->d_rowPtr.as<int>(), *cp = lhs->d_colPtr.as<int>();

  k_ns_split<XT><<<G, kNT, 0, st>>>(nNo, R, Rmi, Rci, Rm, Rc, part, tk, dsc);
  GSLS_CHECK_LAUNCH();
  k_depart<VT><<<grid_for(nnz, G * 4), kNT, 0, st>>>(nnz, Val, lhs->d_tpos.as<int>(), mK, mG, mD, mL,
                                                      Gt, A1, A2);
  GSLS_CHECK_LAUNCH();
  double n2[2];
  GSLS_CUDA(cudaMemcpyAsync(n2, dsc, sizeof(n2), cudaMemcpyDeviceToHost, st));
  GSLS_CUDA(cudaStreamSynchronize(st));
  if (!std::isfinite(n2[0]) || !std::isfinite(n2[1])) {
    set_error("NS: NaN/Inf in the right-hand side");
    return GSLS_ERR_NAN;
  }
  double eps = sqrt(sqrt(n2[0]) * sqrt(n2[0]) + sqrt(n2[1]) * sqrt(n2[1]));
  ls->RI.iNorm = eps;
  ls->RI.fNorm = eps * eps;
  ls->CG.callD = 0.0;
  ls->GM.callD = 0.0;
  ls->CG.itr = 0;
  ls->GM.itr = 0;
  ls->RI.suc = 0;
  eps = fmax(ls->RI.absTol, ls->RI.relTol * eps);

  std::vector<double> A((size_t)nB * nB, 0.0), Bv(nB, 0.0), xB(nB, 0.0), oldxB(nB, 0.0);
  std::vector<double> tmp((size_t)2 * (nB + 1));
  int i, iB = 0, iBB = 0;
  const size_t n3 = (size_t)nNo * 3;
  for (i = 1; i <= mI; i++) {
    iB = 2 * i - 1;
    iBB = 2 * i;
    ls->RI.dB = ls->RI.fNorm;
    XT *Ui = U + (size_t)(i - 1) * l3, *Pi = P + (size_t)(i - 1) * l1;
    XT *MUiB = MU + (size_t)(iB - 1) * l3, *MUiBB = MU + (size_t)(iBB - 1) * l3;
    XT *MPiB = MP + (size_t)(iB - 1) * l1, *MPiBB = MP + (size_t)(iBB - 1) * l1;
    GSLS_TRY((gmres_ns<3, VT, XT>(lhs, &ls->GM, mK, Rm, Ui)));
    part = ws.partials.as<double>();
    k_ns_vs<VT, XT><<<G, kNT, 0, st>>>(nNo, rp, cp, mD, Ui, Rc, Pi, nullptr);
    GSLS_CHECK_LAUNCH();
    GSLS_TRY((schur_cg<VT, XT>(lhs, &ls->CG, mG, Gt, mL, A1, A2, Pi, Rs, Ps, Pb, SP, GP, GP4, sc,
                               &h_sc, bar)));
    k_ns_sv<VT, XT><<<G, kNT, 0, st>>>(nNo, rp, cp, mG, Pi, MUiB, Rm, MUiBB, nullptr);
    GSLS_CHECK_LAUNCH();
    GSLS_TRY((gmres_ns<3, VT, XT>(lhs, &ls->GM, mK, MUiBB, Ui)));
    part = ws.partials.as<double>();
    k_spmv<3, VT, XT, XT><<<G, kNT, 0, st>>>(nNo, rp, cp, mK, Ui, MUiBB);
    GSLS_CHECK_LAUNCH();
    launch_addbcmul<XT>(lhs, 0, 3, Ui, MUiBB, nullptr);
    k_ns_ss_vs<VT, XT><<<G, kNT, 0, st>>>(nNo, rp, cp, mL, Pi, mD, Ui, MPiB, MPiBB);
    GSLS_CHECK_LAUNCH();
    // least-squares dots for columns iB and iBB (NSSOLVER.f:131-143)
    int c = 0;
    for (int k = iB; k <= iBB; k++) {
      const XT *MUk = MU + (size_t)(k - 1) * l3, *MPk = MP + (size_t)(k - 1) * l1;
      k_ns_multidot<XT><<<Gd, kNT, 0, st>>>(nNo, k, MU, l3, MP, l1, MUk, MPk, Rmi, Rci, part);
      GSLS_CHECK_LAUNCH();
      k_ns_colsum<<<k + 1, kNT, 0, st>>>(Gd, part, dsc + 8 + c);
      GSLS_CHECK_LAUNCH();
      c += k + 1;
    }
    GSLS_CUDA(cudaMemcpyAsync(tmp.data(), dsc + 8, sizeof(double) * c, cudaMemcpyDeviceToHost, st));
    GSLS_CUDA(cudaStreamSynchronize(st));
    c = 0;
    for (int k = iB; k <= iBB; k++) {
      for (int j = 1; j <= k; j++) {
        A[(size_t)(k - 1) * nB + (j - 1)] = tmp[c];
        A[(size_t)(j - 1) * nB + (k - 1)] = tmp[c];
        c++;
      }
      Bv[k - 1] = tmp[c++];
    }
    xB = Bv;
    if (ge_solve(nB, iBB, A, xB)) {
      oldxB = xB;
    } else {
      xB = oldxB;
      if (i > 1) {
        iB -= 2;
        iBB -= 2;
      }
      break;
    }
    double sxb = 0.0;
    for (int k = 0; k < iBB; k++) sxb += xB[k] * Bv[k];
    ls->RI.fNorm = ls->RI.iNorm * ls->RI.iNorm - sxb;
    if (!std::isfinite(ls->RI.fNorm)) {
      set_error("NS: NaN/Inf in the least-squares step");
      return GSLS_ERR_NAN;
    }
    if (ls->RI.fNorm < eps * eps) {
      ls->RI.suc = 1;
      break;
    }
    NsCoef cf;
    for (int j = 0; j < iBB; j++) cf.c[j] = xB[j];
    k_ns_comb<XT><<<grid_for(n3, G), kNT, 0, st>>>(n3, Rm, Rmi, MU, l3, 1, 0, iBB, cf, -1.0);
    GSLS_CHECK_LAUNCH();
    k_ns_comb<XT><<<grid_for(nNo, G), kNT, 0, st>>>(nNo, Rc, Rci, MP, l1, 1, 0, iBB, cf, -1.0);
    GSLS_CHECK_LAUNCH();
  }
  NsCoef cf;
  if (i > mI) {
    ls->RI.itr = mI;
  } else {
    ls->RI.itr = i;
    for (int j = 0; j < iBB; j++) cf.c[j] = xB[j];
    k_ns_comb<XT><<<grid_for(nNo, G), kNT, 0, st>>>(nNo, Rc, Rci, MP, l1, 1, 0, iBB, cf, -1.0);
    GSLS_CHECK_LAUNCH();
  }
  k_ns_norm2<XT><<<G, kNT, 0, st>>>(nNo, Rc, part, tk, dsc);
  GSLS_CHECK_LAUNCH();
  double rc2;
  GSLS_CUDA(cudaMemcpyAsync(&rc2, dsc, sizeof(double), cudaMemcpyDeviceToHost, st));
  GSLS_CUDA(cudaStreamSynchronize(st));
  {
    const double rc = sqrt(rc2);
    const double q = 100.0 * rc * rc / ls->RI.fNorm;
    ls->Resc = (std::isfinite(q) && fabs(q) < 2e9) ? (int)llround(q) : -1;
    ls->Resm = 100 - ls->Resc;
  }
  // Rmi = sum_i xB(2i) U_i, Rci = sum_i xB(2i-1) P_i
  const int itr = ls->RI.itr;
  NsCoef cu, cpv;
  for (int k = 0; k < itr; k++) {
    cu.c[k] = xB[2 * k + 1];
    cpv.c[k] = xB[2 * k];
  }
  k_ns_comb<XT><<<grid_for(n3, G), kNT, 0, st>>>(n3, Rmi, nullptr, U, l3, 1, 0, itr, cu, 1.0);
  GSLS_CHECK_LAUNCH();
  k_ns_comb<XT><<<grid_for(nNo, G), kNT, 0, st>>>(nNo, Rci, nullptr, P, l1, 1, 0, itr, cpv, 1.0);
  GSLS_CHECK_LAUNCH();
  k_ns_out<XT><<<grid_for(nNo, G), kNT, 0, st>>>(nNo, R, Rmi, Rci, W);
  GSLS_CHECK_LAUNCH();
  GSLS_CUDA(cudaStreamSynchronize(st));
  ls->RI.callD = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  ls->RI.dB = 5.0 * log(ls->RI.fNorm / ls->RI.dB);
  if (ls->Resc < 0 || ls->Resm < 0) {
    ls->Resc = 0;
    ls->Resm = 0;
    ls->RI.dB = 0.0;
    ls->RI.fNorm = 0.0;
  }
  ls->RI.fNorm = sqrt(ls->RI.fNorm);
  return GSLS_OK;
}

int ns_run(gsls_lhs *lhs, gsls_ls *ls, int D, bool mixed, const void *Val, double *R,
           const double *W) {
  if (D != 4) {
    set_error("NS solver: dof must be nsd + 1 = 4");
    return GSLS_ERR_UNSUPPORTED;
  }
  return mixed ? ns_t<float, float>(lhs, ls, (const float *)Val, R, W)
               : ns_t<double, double>(lhs, ls, (const double *)Val, R, W);
}

}  // namespace gsls
