// Restarted GMRES (GMRESS/GMRESV, Code/Source/svFSILS/GMRES.f:171-431, and
// the GMRES of the NS solver, GMRES.f:51-169):
// classical Gram-Schmidt with one batched multi-dot per Arnoldi step and the
// Pythagorean norm (GMRES.f:116-126), Givens rotations (GMRES.f:130-141),
// back-substitution (GMRES.f:149-155).  Basis vectors in the Krylov vector
// type (FP32 in mixed mode); Hessenberg matrix, Givens data and every
// cross-block sum in FP64.  The Arnoldi loop runs device-resident: the
// Givens kernel sets a device flag and the host polls it once per batch.
// FP32 basis vectors take the norm of the orthogonalised vector explicitly
// (k_gm_orth_nrm) instead of the Pythagorean difference |v|^2 - sum h_j^2,
// which cancels catastrophically in FP32 once the new vector lies nearly in
// the span of the basis.
#include <chrono>
#include <cmath>
#include <cstring>

#include "gsls_internal.cuh"
#include "gsls_spmv.cuh"

namespace gsls {

constexpr int kT = 256;

struct GmresCtl {
  double eps;   // max(absTol, relTol*iNorm)
  double pad;
  int i;        // next Arnoldi column (1-based)
  int done;     // inner loop finished
  int conv;     // converged (suc)
  int last_i;   // last column built in this restart
  int nan;
  int pad2;
};

// u1 = R - u1 (sub) or R, norm -> *outNorm
template <class XT>
__global__ void __launch_bounds__(kT) k_gm_residual(size_t n, const XT *__restrict__ R,
                                                    XT *__restrict__ u1, int sub, double *partials,
                                                    unsigned *ticket, double *outNorm) {
  __shared__ double sh[32];
  __shared__ XT sha[32];
  XT acc = XT(0);
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    const XT v = sub ? XT(R[k] - u1[k]) : R[k];
    u1[k] = v;
    acc = fma(v, v, acc);
  }
  double bs = double(block_sum_t<XT>(acc, sha));
  double tot;
  if (grid_reduce_last<1>(&bs, partials, ticket, &tot, sh) && threadIdx.x == 0)
    *outNorm = sqrt(tot);
}

// err = |u| (after the coupled-face PRE term)
template <class XT>
__global__ void __launch_bounds__(kT) k_gm_norm(size_t n, const XT *__restrict__ u,
                                                double *partials, unsigned *ticket,
                                                double *outNorm) {
  __shared__ double sh[32];
  double acc = 0.0;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x)
    acc += double(u[k]) * double(u[k]);
  double bs = block_sum(acc, sh);
  double tot;
  if (grid_reduce_last<1>(&bs, partials, ticket, &tot, sh) && threadIdx.x == 0)
    *outNorm = sqrt(tot);
}

template <class XT>
__global__ void k_gm_scale(size_t n, XT *__restrict__ u, const double *normp) {
  const XT inv = XT(1.0 / *normp);
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x)
    u[k] = u[k] * inv;
}

// SpMV that is skipped once the Arnoldi loop is done; rev: rows walked from
// the end (zig-zag order across Arnoldi steps, zigzag_on)
template <int D, class VT, class XT>
__global__ void __launch_bounds__(kT) k_gm_spmv(int nNo, const int *__restrict__ rowPtr,
                                                const int *__restrict__ colPtr,
                                                const VT *__restrict__ Val,
                                                const XT *__restrict__ x, XT *__restrict__ y,
                                                const GmresCtl *ctl, int rev) {
  if (*(volatile const int *)&ctl->done) return;
  using AT = typename AccOf<VT>::T;
  constexpr int RPW = 32 / D;
  const int lane = threadIdx.x & 31, grp = lane / D, r = lane - grp * D;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  GatherX<D, XT, AT> g{x};
  for (int base = warp * RPW; base < nNo; base += nwarps * RPW) {
    const int i = rev ? nNo - 1 - (base + grp) : base + grp;
    if (grp < RPW && i >= 0 && i < nNo)
      y[(size_t)i * D + r] = XT(spmv_row_comp<D, VT, AT>(i, r, rowPtr, colPtr, Val, g));
  }
}

// 16-byte vectors of the Krylov type: four FP32 or two FP64 values.  Basis
// vectors start on 32-element boundaries (ld), so every vector's 16-byte
// groups are aligned; the n % L tail is handled element by element.
template <class XT> struct Vec16;
template <> struct Vec16<float> {
  using T = float4;
  static constexpr int L = 4;
  static __device__ __forceinline__ float dot(const float4 a, const float4 b, float acc) {
    acc = fmaf(a.x, b.x, acc);
    acc = fmaf(a.y, b.y, acc);
    acc = fmaf(a.z, b.z, acc);
    return fmaf(a.w, b.w, acc);
  }
  static __device__ __forceinline__ void axpy(float h, const float4 u, float4 &acc) {
    acc.x = fmaf(h, u.x, acc.x);
    acc.y = fmaf(h, u.y, acc.y);
    acc.z = fmaf(h, u.z, acc.z);
    acc.w = fmaf(h, u.w, acc.w);
  }
  static __device__ __forceinline__ void scale(float4 &a, float s) {
    a.x *= s;
    a.y *= s;
    a.z *= s;
    a.w *= s;
  }
};
template <> struct Vec16<double> {
  using T = double2;
  static constexpr int L = 2;
  static __device__ __forceinline__ double dot(const double2 a, const double2 b, double acc) {
    acc = fma(a.x, b.x, acc);
    return fma(a.y, b.y, acc);
  }
  static __device__ __forceinline__ void axpy(double h, const double2 u, double2 &acc) {
    acc.x = fma(h, u.x, acc.x);
    acc.y = fma(h, u.y, acc.y);
  }
  static __device__ __forceinline__ void scale(double2 &a, double s) {
    a.x *= s;
    a.y *= s;
  }
};

// h_j = u_j . v, j = 0..nvec-1; one FP64 partial per (j, block).  Block b
// owns a contiguous range of 16-byte groups; warp w of a block takes the
// vector pairs (2w, 2w+1), (2w+16, 2w+17), ..., so that one load of v
// serves two basis vectors and every lane keeps two independent loads and
// FMA chains in flight.  The last block adds the n % L tail.
template <class XT>
__global__ void __launch_bounds__(kT) k_gm_multidot(size_t n, const XT *__restrict__ basis,
                                                    size_t ld, int nvec, const XT *__restrict__ v,
                                                    double *partials, const GmresCtl *ctl) {
  if (*(volatile const int *)&ctl->done) return;
  using V = Vec16<XT>;
  using VT4 = typename V::T;
  constexpr int L = V::L;
  const size_t nq = n / L;
  const size_t per = (nq + gridDim.x - 1) / gridDim.x;
  const size_t s = (size_t)blockIdx.x * per;
  const size_t e = s + per < nq ? s + per : nq;
  const bool tail = blockIdx.x == gridDim.x - 1;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const VT4 *__restrict__ v4 = reinterpret_cast<const VT4 *>(v);
  for (int j = 2 * wid; j < nvec; j += 2 * nw) {
    const bool two = j + 1 < nvec;
    const VT4 *__restrict__ ua = reinterpret_cast<const VT4 *>(basis + ld * j);
    const VT4 *__restrict__ ub = reinterpret_cast<const VT4 *>(basis + ld * (two ? j + 1 : j));
    XT acc_a = XT(0), acc_b = XT(0);
#pragma unroll 4
    for (size_t k = s + lane; k < e; k += 32) {
      const VT4 x = v4[k];
      acc_a = V::dot(ua[k], x, acc_a);
      if (two) acc_b = V::dot(ub[k], x, acc_b);
    }
    if (tail) {
      for (size_t k = nq * L + lane; k < n; k += 32) {
        acc_a = fma(basis[ld * j + k], v[k], acc_a);
        if (two) acc_b = fma(basis[ld * (j + 1) + k], v[k], acc_b);
      }
    }
    const double a = warp_sum(double(acc_a));
    const double b = warp_sum(double(acc_b));
    if (lane == 0) {
      partials[(size_t)j * gridDim.x + blockIdx.x] = a;
      if (two) partials[(size_t)(j + 1) * gridDim.x + blockIdx.x] = b;
    }
  }
}

// Column sums of the multi-dot partials: one block per j (deterministic).
__global__ void k_gm_colsum(int grid, const double *partials, double *h, const GmresCtl *ctl) {
  if (*(volatile const int *)&ctl->done) return;
  __shared__ double sh[32];
  const int j = blockIdx.x;
  double s = 0.0;
  for (int b = threadIdx.x; b < grid; b += blockDim.x) s += partials[(size_t)j * grid + b];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) h[j] = s;
}

// Norm + Givens rotation for column i (1-based), one thread.  pyth: hcol[i]
// holds v.v and the norm is the Pythagorean sqrt|v.v - sum h_j^2|; else
// hcol[i] already holds |v - sum h_j u_j|^2.  hraw[0..i] receives the
// unrotated column for the Gram-Schmidt update.
__global__ void k_gm_givens(int sD, double *H, const double *hcol, double *hraw, double *c,
                            double *s, double *err, GmresCtl *ctl, int pyth) {
  if (ctl->done) return;
  const int i = ctl->i;
  double *h = H + (size_t)(i - 1) * (sD + 1);
  for (int j = 0; j <= i; j++) h[j] = hcol[j];
  for (int j = 0; j < i; j++) {
    hraw[j] = h[j];
    if (pyth) h[i] = h[i] - h[j] * h[j];
  }
  h[i] = sqrt(fabs(h[i]));
  hraw[i] = h[i];
  for (int j = 1; j <= i - 1; j++) {
    const double tmp = c[j - 1] * h[j - 1] + s[j - 1] * h[j];
    h[j] = -s[j - 1] * h[j - 1] + c[j - 1] * h[j];
    h[j - 1] = tmp;
  }
  const double tmp = sqrt(h[i - 1] * h[i - 1] + h[i] * h[i]);
  c[i - 1] = h[i - 1] / tmp;
  s[i - 1] = h[i] / tmp;
  h[i - 1] = tmp;
  h[i] = 0.0;
  err[i] = -s[i - 1] * err[i - 1];
  err[i - 1] = c[i - 1] * err[i - 1];
  ctl->last_i = i;
  if (!isfinite(err[i]) || !isfinite(hraw[i]) || hraw[i] == 0.0) {
    // breakdown: h(i+1,i) = 0 or non-finite
    ctl->nan = (!isfinite(err[i]) || !isfinite(hraw[i])) ? 1 : 0;
    ctl->conv = ctl->nan ? 0 : 1;
    ctl->done = 1;
  } else if (fabs(err[i]) < ctl->eps) {
    ctl->conv = 1;
    ctl->done = 1;
  }
  ctl->i = i + 1;
  if (i >= sD) ctl->done = 1;
}

// u_{i+1} = (u_{i+1} - sum_j hraw_j u_j) / hraw_i, one 16-byte group per
// thread and step (the same per-element FMA sequence as an element loop)
template <class XT>
__global__ void __launch_bounds__(kT) k_gm_orth(size_t n, XT *__restrict__ basis, size_t ld,
                                                const double *__restrict__ hraw,
                                                const GmresCtl *ctl, int i_expected) {
  if (ctl->last_i != i_expected || ctl->nan || hraw[i_expected] == 0.0) return;
  using V = Vec16<XT>;
  using VT4 = typename V::T;
  constexpr int L = V::L;
  const int i = i_expected;
  __shared__ XT hs[512];
  for (int j = threadIdx.x; j < i && j < 512; j += blockDim.x) hs[j] = XT(-hraw[j]);
  __syncthreads();
  XT *__restrict__ v = basis + ld * i;
  const XT inv = XT(1.0 / hraw[i]);
  const size_t nq = n / L;
  const size_t t0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t nt = (size_t)gridDim.x * blockDim.x;
  for (size_t q = t0; q < nq; q += nt) {
    VT4 acc = reinterpret_cast<const VT4 *>(v)[q];
#pragma unroll 4
    for (int j = 0; j < i; j++) V::axpy(hs[j], reinterpret_cast<const VT4 *>(basis + ld * j)[q], acc);
    V::scale(acc, inv);
    reinterpret_cast<VT4 *>(v)[q] = acc;
  }
  for (size_t k = nq * L + t0; k < n; k += nt) {
    XT acc = v[k];
    for (int j = 0; j < i; j++) acc = fma(hs[j], basis[ld * j + k], acc);
    v[k] = acc * inv;
  }
}

// FP32 basis: u_{i+1} -= sum_{j<i} h_j u_j (h_j from the multi-dot, before
// the Givens kernel of the step) and |u_{i+1}|^2 -> hcol[i], a deterministic
// grid sum; each 16-byte group's squares are summed in FP32 and added in
// FP64.  k_gm_scale_i then divides by the norm once the Givens kernel has
// accepted the column.
template <class XT>
__global__ void __launch_bounds__(kT) k_gm_orth_nrm(size_t n, XT *__restrict__ basis, size_t ld,
                                                    double *__restrict__ hcol, const GmresCtl *ctl,
                                                    int i, double *partials, unsigned *ticket) {
  if (*(volatile const int *)&ctl->done) return;
  using V = Vec16<XT>;
  using VT4 = typename V::T;
  constexpr int L = V::L;
  __shared__ XT hs[512];
  __shared__ double sh[32];
  for (int j = threadIdx.x; j < i && j < 512; j += blockDim.x) hs[j] = XT(-hcol[j]);
  __syncthreads();
  XT *__restrict__ v = basis + ld * i;
  const size_t nq = n / L;
  const size_t t0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t nt = (size_t)gridDim.x * blockDim.x;
  double nrm = 0.0;
  for (size_t q = t0; q < nq; q += nt) {
    VT4 acc = reinterpret_cast<const VT4 *>(v)[q];
#pragma unroll 4
    for (int j = 0; j < i; j++) V::axpy(hs[j], reinterpret_cast<const VT4 *>(basis + ld * j)[q], acc);
    reinterpret_cast<VT4 *>(v)[q] = acc;
    nrm += double(V::dot(acc, acc, XT(0)));
  }
  for (size_t k = nq * L + t0; k < n; k += nt) {
    XT acc = v[k];
    for (int j = 0; j < i; j++) acc = fma(hs[j], basis[ld * j + k], acc);
    v[k] = acc;
    nrm += double(acc) * double(acc);
  }
  const double bs = block_sum(nrm, sh);
  double tot;
  if (grid_reduce_last<1>(&bs, partials, ticket, &tot, sh) && threadIdx.x == 0) hcol[i] = tot;
}

// u_{i+1} /= h_{i+1,i} after the Givens kernel of step i (FP32 basis)
template <class XT>
__global__ void k_gm_scale_i(size_t n, XT *__restrict__ basis, size_t ld,
                             const double *__restrict__ hraw, const GmresCtl *ctl, int i) {
  if (ctl->last_i != i || ctl->nan || hraw[i] == 0.0) return;
  XT *__restrict__ v = basis + ld * i;
  const XT inv = XT(1.0 / hraw[i]);
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x)
    v[k] = v[k] * inv;
}

// Back substitution y = H(1:i,1:i)^-1 err(1:i), one thread.
__global__ void k_gm_backsub(int sD, const double *H, const double *err, double *y,
                             const GmresCtl *ctl) {
  int i = ctl->last_i;
  if (i > sD) i = sD;
  for (int j = 0; j < i; j++) y[j] = err[j];
  for (int j = i; j >= 1; j--) {
    for (int k = j + 1; k <= i; k++) y[j - 1] -= H[(size_t)(k - 1) * (sD + 1) + (j - 1)] * y[k - 1];
    y[j - 1] /= H[(size_t)(j - 1) * (sD + 1) + (j - 1)];
  }
}

// X += sum_j y_j u_j
template <class XT>
__global__ void __launch_bounds__(kT) k_gm_update_x(size_t n, XT *__restrict__ X,
                                                    const XT *__restrict__ basis, size_t ld,
                                                    const double *__restrict__ y,
                                                    const GmresCtl *ctl) {
  const int i = ctl->last_i;
  __shared__ XT ys[512];
  for (int j = threadIdx.x; j < i && j < 512; j += blockDim.x) ys[j] = XT(y[j]);
  __syncthreads();
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    XT acc = X[k];
    for (int j = 0; j < i; j++) acc = fma(ys[j], basis[ld * j + k], acc);
    X[k] = acc;
  }
}

template <class XT>
__global__ void k_to_xt(size_t n, const double *__restrict__ a, XT *__restrict__ b) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x)
    b[k] = XT(a[k]);
}

template <class XT>
__global__ void k_scale_out_g(size_t n, double *__restrict__ Rout, const XT *__restrict__ X,
                              const double *__restrict__ W) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x)
    Rout[k] = W[k] * double(X[k]);
}

__global__ void __launch_bounds__(kT) k_norm2(size_t n, const double *__restrict__ u,
                                              double *out, double *partials, unsigned *ticket) {
  __shared__ double sh[32];
  double acc = 0.0;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x)
    acc += u[k] * u[k];
  double bs = block_sum(acc, sh);
  double tot;
  if (grid_reduce_last<1>(&bs, partials, ticket, &tot, sh) && threadIdx.x == 0) *out = tot;
}

__global__ void k_vmul(size_t n, double *__restrict__ R, const double *__restrict__ W) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x)
    R[k] *= W[k];
}

// Restart loop shared by GMRESV (GMRES.f:273-431) and the GMRES that the NS
// solver calls (GMRES.f:51-169) on device vectors: Rk (right-hand side, not
// modified) and X (solution, zeroed here).  ns selects the latter's
// bookkeeping: no iteration counted for the first restart, eps and iNorm set
// from the first residual, and an initial residual at or below absTol
// returns X = 0 (*early = true).  Otherwise eps is the caller's.
template <int D, class VT, class XT>
static int gmres_loop(gsls_lhs *lhs, gsls_sub_ls *ls, const VT *Val, const XT *Rk, XT *X,
                      bool ns, double eps, bool *early) {
  cudaStream_t st = lhs->stream;
  Workspace &ws = lhs->ws;
  const int nNo = lhs->nNo, sD = ls->sD;
  if (sD < 1 || sD > 512) {
    set_error("GMRES: Krylov space dimension must be in [1, 512]");
    return GSLS_ERR_ARG;
  }
  const size_t nv = (size_t)nNo * D;
  const size_t ld = (nv + 31) & ~(size_t)31;
  constexpr bool kExplicitNorm = sizeof(XT) == 4;
  GSLS_TRY(ws.basis.alloc(sizeof(XT) * ld * (size_t)(sD + 1)));
  const int G = lhs->grid;
  // multi-dot grid: 4 co-resident blocks per SM for vectors of >= 2^20
  // unknowns (USTRUCT beam, 1.43M: 0.324 -> 0.282 ms per Arnoldi step),
  // else 2: shorter vectors, e.g. the NS solver's momentum block of the
  // cylinder (645k), are bound by the per-block reductions, and 4 per SM
  // made that fluid step 5 % slower
  const int Gd = num_sms() * (nv >= ((size_t)1 << 20) ? 4 : 2);
  const size_t hbytes = sizeof(double) * ((size_t)(sD + 1) * sD + 6 * (sD + 2)) + 64;
  GSLS_TRY(ws.hcol.alloc(hbytes + sizeof(GmresCtl) + 64));
  GSLS_TRY(ws.partials.alloc(sizeof(double) * (size_t)(sD + 2) * (Gd > G ? Gd : G) + 64));
  double *H = ws.hcol.as<double>();
  double *hcol = H + (size_t)(sD + 1) * sD;
  double *hraw = hcol + (sD + 2);
  double *cc = hraw + (sD + 2);
  double *ss = cc + (sD + 2);
  double *err = ss + (sD + 2);
  double *y = err + (sD + 2);
  GmresCtl *ctl = reinterpret_cast<GmresCtl *>(y + (sD + 2));
  XT *basis = ws.basis.as<XT>();
  double *part = ws.partials.as<double>();
  unsigned *tk = ws.ticket.as<unsigned>();
  *early = false;
  GSLS_CUDA(cudaMemsetAsync(X, 0, sizeof(XT) * nv, st));
  GmresCtl hc;
  for (int l = 1; l <= ls->mItr; l++) {
    if (!ns || l > 1) ls->itr++;
    XT *u1 = basis;
    memset(&hc, 0, sizeof(hc));
    hc.eps = eps;
    hc.i = 1;
    GSLS_CUDA(cudaMemcpyAsync(ctl, &hc, sizeof(hc), cudaMemcpyHostToDevice, st));
    if (l > 1) {
      k_gm_spmv<D, VT, XT><<<G, kT, 0, st>>>(nNo, lhs->d_rowPtr.as<int>(),
                                             lhs->d_colPtr.as<int>(), Val, X, u1, ctl, 0);
      GSLS_CHECK_LAUNCH();
      launch_addbcmul<XT>(lhs, 0, D, X, u1, &ctl->done);
    }
    k_gm_residual<XT><<<G, kT, 0, st>>>(nv, Rk, u1, l > 1 ? 1 : 0, part, tk, err);
    GSLS_CHECK_LAUNCH();
    if (ns && ws.cpl_on) {
      // u1 = PRE(u1), then its norm (GMRES.f:88-91)
      launch_addbcmul<XT>(lhs, 1, D, u1, u1, &ctl->done);
      k_gm_norm<XT><<<G, kT, 0, st>>>(nv, u1, part, tk, err);
      GSLS_CHECK_LAUNCH();
    }
    if (ns && l == 1) {
      double e0;
      GSLS_CUDA(cudaMemcpyAsync(&e0, err, sizeof(double), cudaMemcpyDeviceToHost, st));
      GSLS_CUDA(cudaStreamSynchronize(st));
      if (!std::isfinite(e0)) {
        set_error("GMRES: NaN/Inf in the right-hand side");
        return GSLS_ERR_NAN;
      }
      if (e0 <= ls->absTol) {
        ls->callD = 2.220446049250313e-16;
        ls->dB = 0.0;
        *early = true;
        return GSLS_OK;
      }
      ls->iNorm = e0;
      ls->fNorm = e0;
      eps = fmax(ls->absTol, ls->relTol * e0);
      hc.eps = eps;
      GSLS_CUDA(cudaMemcpyAsync(ctl, &hc, sizeof(hc), cudaMemcpyHostToDevice, st));
    }
    ls->dB = ls->fNorm;
    k_gm_scale<XT><<<G, kT, 0, st>>>(nv, u1, err);
    GSLS_CHECK_LAUNCH();
    // profiling runs time every Arnoldi SpMV with events and poll after
    // each step, so that no skipped launch is counted
    const bool prof = prof_on();
    int i_next = 1, batch = prof ? 1 : 4;
    bool inner_done = false;
    while (!inner_done) {
      for (int b = 0; b < batch && i_next <= sD; b++, i_next++) {
        const int i = i_next;
        XT *ui = basis + ld * (i - 1), *ui1 = basis + ld * i;
        if (prof) cudaEventRecord(prof_event(0), st);
        k_gm_spmv<D, VT, XT><<<G, kT, 0, st>>>(nNo, lhs->d_rowPtr.as<int>(),
                                               lhs->d_colPtr.as<int>(), Val, ui, ui1, ctl,
                                               zigzag_on() & i);
        GSLS_CHECK_LAUNCH();
        if (prof) cudaEventRecord(prof_event(1), st);
        if (ws.cpl_on) {
          launch_addbcmul<XT>(lhs, 0, D, ui, ui1, &ctl->done);
          if (ns) launch_addbcmul<XT>(lhs, 1, D, ui1, ui1, &ctl->done);
        }
        if (kExplicitNorm) {
          // h_j for j < i, then the orthogonalised vector and its norm
          k_gm_multidot<XT><<<Gd, kT, 0, st>>>(nv, basis, ld, i, ui1, part, ctl);
          GSLS_CHECK_LAUNCH();
          k_gm_colsum<<<i, kT, 0, st>>>(Gd, part, hcol, ctl);
          GSLS_CHECK_LAUNCH();
          k_gm_orth_nrm<XT><<<G, kT, 0, st>>>(nv, basis, ld, hcol, ctl, i, part, tk);
          GSLS_CHECK_LAUNCH();
          k_gm_givens<<<1, 1, 0, st>>>(sD, H, hcol, hraw, cc, ss, err, ctl, 0);
          GSLS_CHECK_LAUNCH();
          k_gm_scale_i<XT><<<G, kT, 0, st>>>(nv, basis, ld, hraw, ctl, i);
          GSLS_CHECK_LAUNCH();
        } else {
          k_gm_multidot<XT><<<Gd, kT, 0, st>>>(nv, basis, ld, i + 1, ui1, part, ctl);
          GSLS_CHECK_LAUNCH();
          k_gm_colsum<<<i + 1, kT, 0, st>>>(Gd, part, hcol, ctl);
          GSLS_CHECK_LAUNCH();
          k_gm_givens<<<1, 1, 0, st>>>(sD, H, hcol, hraw, cc, ss, err, ctl, 1);
          GSLS_CHECK_LAUNCH();
          k_gm_orth<XT><<<G, kT, 0, st>>>(nv, basis, ld, hraw, ctl, i);
          GSLS_CHECK_LAUNCH();
        }
        if (prof) cudaEventRecord(prof_event(2), st);
      }
      GSLS_CUDA(cudaMemcpyAsync(&hc, ctl, sizeof(hc), cudaMemcpyDeviceToHost, st));
      GSLS_CUDA(cudaStreamSynchronize(st));
      if (prof) {
        float t = 0.f;
        cudaEventElapsedTime(&t, prof_event(0), prof_event(1));
        prof_add(D == 3 ? "gm_spmv_d3" : "gm_spmv", 1, t);
        // multi-dot, Givens and Gram-Schmidt update of the same step
        cudaEventElapsedTime(&t, prof_event(1), prof_event(2));
        prof_add("gm_orth", 1, t);
      }
      if (hc.done || i_next > sD) inner_done = true;
      if (!prof && batch < 16) batch *= 2;
    }
    if (hc.nan) {
      set_error("GMRES: NaN/Inf in the Arnoldi process");
      return GSLS_ERR_NAN;
    }
    ls->itr += hc.last_i;
    k_gm_backsub<<<1, 1, 0, st>>>(sD, H, err, y, ctl);
    GSLS_CHECK_LAUNCH();
    k_gm_update_x<XT><<<G, kT, 0, st>>>(nv, X, basis, ld, y, ctl);
    GSLS_CHECK_LAUNCH();
    double errv;
    GSLS_CUDA(cudaMemcpyAsync(&errv, err + hc.last_i, sizeof(double), cudaMemcpyDeviceToHost, st));
    GSLS_CUDA(cudaStreamSynchronize(st));
    ls->fNorm = fabs(errv);
    if (hc.conv) {
      ls->suc = 1;
      break;
    }
  }
  return GSLS_OK;
}

template <int D, class VT, class XT>
static int gmres_t(gsls_lhs *lhs, gsls_sub_ls *ls, const VT *Val, double *R, const double *Wc) {
  cudaStream_t st = lhs->stream;
  Workspace &ws = lhs->ws;
  const int nNo = lhs->nNo;
  const size_t nv = (size_t)nNo * D;
  const int G = lhs->grid;
  GSLS_TRY(ws.partials.alloc(sizeof(double) * (size_t)G * 4 + 64));
  XT *X = ws.vec[0].as<XT>(), *Rk = ws.vec[3].as<XT>();
  double *part = ws.partials.as<double>();
  unsigned *tk = ws.ticket.as<unsigned>();
  double *dnorm = ws.scal.as<double>();

  auto t0 = std::chrono::steady_clock::now();
  ls->suc = 0;
  k_norm2<<<G, kT, 0, st>>>(nv, R, dnorm, part, tk);
  GSLS_CHECK_LAUNCH();
  double n2;
  GSLS_CUDA(cudaMemcpyAsync(&n2, dnorm, sizeof(double), cudaMemcpyDeviceToHost, st));
  GSLS_CUDA(cudaStreamSynchronize(st));
  double eps = sqrt(n2);
  ls->iNorm = eps;
  ls->fNorm = eps;
  eps = fmax(ls->absTol, ls->relTol * eps);
  ls->itr = 0;
  if (!std::isfinite(n2)) {
    set_error("GMRES: NaN/Inf in the right-hand side");
    return GSLS_ERR_NAN;
  }
  if (ls->iNorm <= ls->absTol) {
    // the reference returns with R untouched (GMRES.f:310-314); SOLVE then
    // applies R = Wc*R
    ls->callD = 2.220446049250313e-16;
    ls->dB = 0.0;
    k_vmul<<<G, kT, 0, st>>>(nv, R, Wc);
    GSLS_CHECK_LAUNCH();
    GSLS_CUDA(cudaStreamSynchronize(st));
    return GSLS_OK;
  }
  k_to_xt<XT><<<G, kT, 0, st>>>(nv, R, Rk);
  GSLS_CHECK_LAUNCH();
  bool early = false;
  GSLS_TRY((gmres_loop<D, VT, XT>(lhs, ls, Val, Rk, X, false, eps, &early)));
  k_scale_out_g<XT><<<G, kT, 0, st>>>(nv, R, X, Wc);
  GSLS_CHECK_LAUNCH();
  GSLS_CUDA(cudaStreamSynchronize(st));
  ls->dB = 10.0 * log(ls->fNorm / ls->dB);
  ls->callD = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return GSLS_OK;
}

// GMRES of the NS solver (GMRES.f:51-169) on the K block: X = K^-1 Rk
// approximately; itr and callD accumulate in ls.
template <int D, class VT, class XT>
int gmres_ns(gsls_lhs *lhs, gsls_sub_ls *ls, const VT *Val, const XT *Rk, XT *X) {
  auto t0 = std::chrono::steady_clock::now();
  ls->suc = 0;
  bool early = false;
  GSLS_TRY((gmres_loop<D, VT, XT>(lhs, ls, Val, Rk, X, true, 0.0, &early)));
  if (early) return GSLS_OK;
  ls->callD += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  ls->dB = 10.0 * log(ls->fNorm / ls->dB);
  return GSLS_OK;
}
template int gmres_ns<3, float, float>(gsls_lhs *, gsls_sub_ls *, const float *, const float *,
                                       float *);
template int gmres_ns<3, double, double>(gsls_lhs *, gsls_sub_ls *, const double *,
                                         const double *, double *);

int gmres_run(gsls_lhs *lhs, gsls_sub_ls *ls, int D, bool mixed, const void *Val, double *R,
              const double *Wc) {
#define GSLS_GM_CASE(DV)                                                                   \
  case DV:                                                                                 \
    return mixed ? gmres_t<DV, float, float>(lhs, ls, (const float *)Val, R, Wc)           \
                 : gmres_t<DV, double, double>(lhs, ls, (const double *)Val, R, Wc);
  switch (D) {
    GSLS_GM_CASE(1)
    GSLS_GM_CASE(2)
    GSLS_GM_CASE(3)
    GSLS_GM_CASE(4)
    default:
      return GSLS_ERR_UNSUPPORTED;
  }
#undef GSLS_GM_CASE
}

}  // namespace gsls
