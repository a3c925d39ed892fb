// Block-CSR SpMV, reductions, preconditioners and Krylov solvers (CG,
// restarted GMRES) with the semantics of svFSILS (Code/Source/svFSILS:
// SPARMUL.f, DOT.f, NORM.f, PRECOND.f, CGRAD.f, GMRES.f, SOLVE.f).
//
// Design: all Krylov scalars live in device memory (KrylovScalars); every
// kernel of an iteration first checks the device "done" flag, so the host
// can enqueue batches of iterations without reading anything back and only
// polls the flag once per batch.  Reductions use a fixed grid and a
// last-block pass, so every sum is bitwise reproducible.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "gsls_internal.cuh"

namespace gsls {

constexpr int kThreads = 256;

// ---------------------------------------------------------------------------
// SpMV core: a group of LPR lanes owns one block row.  The row's values are
// read as one flat, contiguous range (coalesced), each lane accumulates the
// component r of its value, then the group reduces with shuffles.
template <class VT> struct AccOf { using T = double; };
template <> struct AccOf<float> { using T = float; };

template <int D, int LPR, class VT, class XT>
__device__ __forceinline__ void spmv_row(int i, bool valid, int lane, const int *__restrict__ rowPtr,
                                         const int *__restrict__ colPtr,
                                         const VT *__restrict__ Val, const XT *__restrict__ x,
                                         typename AccOf<VT>::T acc[D]) {
  using AT = typename AccOf<VT>::T;
  constexpr int DD = D * D;
#pragma unroll
  for (int r = 0; r < D; r++) acc[r] = AT(0);
  if (valid) {
    const int rs = __ldg(rowPtr + i), re = __ldg(rowPtr + i + 1);
    const int L = (re - rs) * DD;
    const VT *__restrict__ v = Val + (size_t)rs * DD;
    const int *__restrict__ cp = colPtr + rs;
#pragma unroll 4
    for (int t = lane; t < L; t += LPR) {
      const int blk = t / DD;
      const int rem = t - blk * DD;
      const int r = rem / D;
      const int c = rem - r * D;
      const int col = __ldg(cp + blk);
      const AT prod = AT(__ldg(v + t)) * AT(__ldg(x + (size_t)col * D + c));
#pragma unroll
      for (int rr = 0; rr < D; rr++) acc[rr] += (r == rr) ? prod : AT(0);
    }
  }
#pragma unroll
  for (int r = 0; r < D; r++)
#pragma unroll
    for (int o = LPR / 2; o > 0; o >>= 1) acc[r] += __shfl_xor_sync(0xffffffffu, acc[r], o, LPR);
}

template <int D> struct Lpr { static constexpr int v = 32; };
template <> struct Lpr<1> { static constexpr int v = 16; };
template <> struct Lpr<2> { static constexpr int v = 32; };

// y = K x (plain)
template <int D, class VT, class XT, class YT>
__global__ void __launch_bounds__(kThreads) k_spmv(int nNo, const int *__restrict__ rowPtr,
                                                   const int *__restrict__ colPtr,
                                                   const VT *__restrict__ Val,
                                                   const XT *__restrict__ x, YT *__restrict__ y) {
  using AT = typename AccOf<VT>::T;
  constexpr int LPR = Lpr<D>::v, GPW = 32 / LPR;
  const int lane = threadIdx.x % LPR, grp = (threadIdx.x & 31) / LPR;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int base = warp * GPW; base < nNo; base += nwarps * GPW) {
    const int i = base + grp;
    const bool valid = i < nNo;
    AT acc[D];
    spmv_row<D, LPR, VT, XT>(i, valid, lane, rowPtr, colPtr, Val, x, acc);
    if (valid && lane == 0)
#pragma unroll
      for (int r = 0; r < D; r++) y[(size_t)i * D + r] = YT(acc[r]);
  }
}

// ---------------------------------------------------------------------------
// CG kernels (CGRADS/CGRADV, Code/Source/svFSILS/CGRAD.f:125-242)

// R_k = R; P = R; X = 0; iNorm = ||R||; eps; errO = err = iNorm^2
template <class XT>
__global__ void __launch_bounds__(kThreads) k_cg_init(size_t n, const double *__restrict__ R,
                                                      XT *__restrict__ Rk, XT *__restrict__ P,
                                                      XT *__restrict__ X, KrylovScalars *S,
                                                      double absTol, double relTol, int mItr,
                                                      double *partials, unsigned *ticket) {
  __shared__ double sh[32];
  double acc = 0.0;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    const double r = R[k];
    acc += r * r;
    Rk[k] = XT(r);
    P[k] = XT(r);
    X[k] = XT(0);
  }
  double bs = block_sum(acc, sh);
  double tot;
  if (grid_reduce_last<1>(&bs, partials, ticket, &tot, sh) && threadIdx.x == 0) {
    const double iNorm = sqrt(tot);
    S->iNorm = iNorm;
    double e = fmax(absTol, relTol * iNorm);
    S->eps = e * e;
    S->errO = iNorm * iNorm;
    S->err = S->errO;
    S->itr = 0;
    S->mItr = mItr;
    S->suc = 0;
    S->done = 0;
    if (mItr < 1) S->done = 2;
    else if (S->err < S->eps) {
      S->done = 1;
      S->suc = 1;
    }
    if (!isfinite(tot)) S->done = 3;
  }
}

// KP = K P, alpha = errO / (P . KP)
template <int D, class VT, class XT>
__global__ void __launch_bounds__(kThreads) k_cg_spmv(int nNo, const int *__restrict__ rowPtr,
                                                      const int *__restrict__ colPtr,
                                                      const VT *__restrict__ Val,
                                                      const XT *__restrict__ P, XT *__restrict__ KP,
                                                      KrylovScalars *S, double *partials,
                                                      unsigned *ticket) {
  if (*(volatile int *)&S->done) return;
  using AT = typename AccOf<VT>::T;
  __shared__ double sh[32];
  constexpr int LPR = Lpr<D>::v, GPW = 32 / LPR;
  const int lane = threadIdx.x % LPR, grp = (threadIdx.x & 31) / LPR;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  double dot = 0.0;
  for (int base = warp * GPW; base < nNo; base += nwarps * GPW) {
    const int i = base + grp;
    const bool valid = i < nNo;
    AT acc[D];
    spmv_row<D, LPR, VT, XT>(i, valid, lane, rowPtr, colPtr, Val, P, acc);
    if (valid && lane == 0) {
#pragma unroll
      for (int r = 0; r < D; r++) {
        const XT kp = XT(acc[r]);
        KP[(size_t)i * D + r] = kp;
        dot += double(P[(size_t)i * D + r]) * double(kp);
      }
    }
  }
  double bs = block_sum(dot, sh);
  double tot;
  if (grid_reduce_last<1>(&bs, partials, ticket, &tot, sh) && threadIdx.x == 0) {
    S->errO = S->err;
    S->dot = tot;
    S->alpha = S->errO / tot;
    if (!isfinite(S->alpha)) S->done = 3;
  }
}

// X += alpha P; R -= alpha KP; err = ||R||^2; convergence test
template <class XT>
__global__ void __launch_bounds__(kThreads) k_cg_update(size_t n, XT *__restrict__ X,
                                                        XT *__restrict__ R,
                                                        const XT *__restrict__ P,
                                                        const XT *__restrict__ KP,
                                                        KrylovScalars *S, double *partials,
                                                        unsigned *ticket) {
  if (*(volatile int *)&S->done) return;
  __shared__ double sh[32];
  const double alpha = S->alpha;
  double acc = 0.0;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    X[k] = XT(double(X[k]) + alpha * double(P[k]));
    const double r = double(R[k]) + (-alpha) * double(KP[k]);
    const XT rk = XT(r);
    R[k] = rk;
    acc += double(rk) * double(rk);
  }
  double bs = block_sum(acc, sh);
  double tot;
  if (grid_reduce_last<1>(&bs, partials, ticket, &tot, sh) && threadIdx.x == 0) {
    S->err = tot;
    S->itr += 1;
    if (!isfinite(tot)) S->done = 3;
    else if (S->itr >= S->mItr) S->done = 2;
    else if (S->err < S->eps) {
      S->done = 1;
      S->suc = 1;
    }
  }
}

// P = (P + (errO/err) R) * (err/errO), the reference's OMPSUMS + OMPMULS
template <class XT>
__global__ void __launch_bounds__(kThreads) k_cg_pupdate(size_t n, XT *__restrict__ P,
                                                         const XT *__restrict__ R,
                                                         const KrylovScalars *S) {
  if (*(volatile const int *)&S->done) return;
  const double a = S->errO / S->err, b = S->err / S->errO;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x)
    P[k] = XT((double(P[k]) + a * double(R[k])) * b);
}

// R_out = W * X
template <class XT>
__global__ void k_scale_out(size_t n, double *__restrict__ Rout, const XT *__restrict__ X,
                            const double *__restrict__ W) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x)
    Rout[k] = W[k] * double(X[k]);
}

// ---------------------------------------------------------------------------
// Diagonal preconditioner (PRECONDDIAG, Code/Source/svFSILS/PRECOND.f:50-145)
template <int D, class VT>
__global__ void k_diag_w(int nNo, const int *__restrict__ diagPtr, const VT *__restrict__ Val,
                         const double *__restrict__ mask, double *__restrict__ W) {
  constexpr int DD = D * D;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nNo; i += gridDim.x * blockDim.x) {
    const int d = diagPtr[i];
#pragma unroll
    for (int k = 0; k < D; k++) {
      double w = double(Val[(size_t)d * DD + k * D + k]);
      if (w == 0.0) w = 1.0;
      w = 1.0 / sqrt(fabs(w));
      W[(size_t)i * D + k] = w * mask[(size_t)i * D + k];
    }
  }
}

// Val = diag(Wr) Val diag(Wc) (PREMUL then POSMUL), R = Wr R
template <int D, class VT>
__global__ void __launch_bounds__(kThreads) k_scale_val(size_t nflat, const int *__restrict__ rowOf,
                                                        const int *__restrict__ colPtr,
                                                        VT *__restrict__ Val,
                                                        const double *__restrict__ Wr,
                                                        const double *__restrict__ Wc) {
  constexpr int DD = D * D;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < nflat;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t j = t / DD;
    const int rem = (int)(t - j * DD);
    const int r = rem / D, c = rem - (rem / D) * D;
    const int row = __ldg(rowOf + j), col = __ldg(colPtr + j);
    if (sizeof(VT) == 8) {
      double v = double(Val[t]) * Wr[(size_t)row * D + r];
      v = v * Wc[(size_t)col * D + c];
      Val[t] = VT(v);
    } else {
      const float wr = float(Wr[(size_t)row * D + r]), wc = float(Wc[(size_t)col * D + c]);
      Val[t] = VT(float(Val[t]) * wr * wc);
    }
  }
}

__global__ void k_vec_mul(size_t n, double *__restrict__ R, const double *__restrict__ W) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x)
    R[k] *= W[k];
}

// ---------------------------------------------------------------------------
// Plain reductions for the public dot/norm entry points.
__global__ void __launch_bounds__(kThreads) k_dot(size_t n, const double *__restrict__ u,
                                                  const double *__restrict__ v, double *out,
                                                  double *partials, unsigned *ticket) {
  __shared__ double sh[32];
  double acc = 0.0;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x)
    acc += u[k] * v[k];
  double bs = block_sum(acc, sh);
  double tot;
  if (grid_reduce_last<1>(&bs, partials, ticket, &tot, sh) && threadIdx.x == 0) *out = tot;
}

// ---------------------------------------------------------------------------
// GMRES kernels (GMRESS/GMRESV, Code/Source/svFSILS/GMRES.f:171-431).
// Basis vectors u_j (XT), Hessenberg and Givens data in FP64.

struct GmresCtl {
  double eps;      // max(absTol, relTol*iNorm)
  double errNorm;  // err(1) of the current restart
  int i;           // current Arnoldi column (1-based) being built
  int done;        // inner loop finished (converged or breakdown)
  int conv;        // converged flag (suc)
  int last_i;      // last column built in this restart
  int nan;
  int pad;
};

// u1 = R - u1 (u1 holds K X on entry when sub == 1), norm partials
template <class XT>
__global__ void __launch_bounds__(kThreads) k_gm_residual(size_t n, const XT *__restrict__ R,
                                                          XT *__restrict__ u1, int sub,
                                                          double *partials, unsigned *ticket,
                                                          double *outNorm) {
  __shared__ double sh[32];
  double acc = 0.0;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    const XT v = sub ? XT(double(R[k]) - double(u1[k])) : R[k];
    u1[k] = v;
    acc += double(v) * double(v);
  }
  double bs = block_sum(acc, sh);
  double tot;
  if (grid_reduce_last<1>(&bs, partials, ticket, &tot, sh) && threadIdx.x == 0)
    *outNorm = sqrt(tot);
}

template <class XT>
__global__ void k_gm_scale(size_t n, XT *__restrict__ u, const double *normp) {
  const double inv = *normp;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x)
    u[k] = XT(double(u[k]) / inv);
}

// Multi-dot h_j = u_j . v for j = 0..nv-1: each warp owns a subset of j,
// partials[j*grid + block] (one value per block and j, no block syncs).
template <class XT>
__global__ void __launch_bounds__(kThreads) k_gm_multidot(size_t n, const XT *__restrict__ basis,
                                                          size_t ld, int nvec,
                                                          const XT *__restrict__ v,
                                                          double *partials, const GmresCtl *ctl) {
  if (ctl->done) return;
  const size_t per = (n + gridDim.x - 1) / gridDim.x;
  const size_t s = (size_t)blockIdx.x * per;
  const size_t e = s + per < n ? s + per : n;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int j = wid; j < nvec; j += nw) {
    const XT *__restrict__ u = basis + ld * j;
    double acc = 0.0;
    for (size_t k = s + lane; k < e; k += 32) acc += double(u[k]) * double(v[k]);
    acc = warp_sum(acc);
    if (lane == 0) partials[(size_t)j * gridDim.x + blockIdx.x] = acc;
  }
}

// Column sums of the multi-dot partials: one block per j (deterministic).
__global__ void k_gm_colsum(int grid, const double *partials, double *h, const GmresCtl *ctl) {
  if (ctl->done) return;
  __shared__ double sh[32];
  const int j = blockIdx.x;
  double s = 0.0;
  for (int b = threadIdx.x; b < grid; b += blockDim.x) s += partials[(size_t)j * grid + b];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) h[j] = s;
}

// Pythagorean norm + Givens rotation for column i (1-based), one thread.
// hraw[0..i] receives the unrotated column for the Gram-Schmidt update.
__global__ void k_gm_givens(int sD, double *H /*(sD+1) x sD, col-major*/, double *hcol,
                            double *hraw, double *c, double *s, double *err, GmresCtl *ctl) {
  if (ctl->done) return;
  const int i = ctl->i;
  double *h = H + (size_t)(i - 1) * (sD + 1);
  for (int j = 0; j <= i; j++) h[j] = hcol[j];
  for (int j = 0; j < i; j++) {
    hraw[j] = h[j];
    h[i] = h[i] - h[j] * h[j];
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
  if (!isfinite(err[i]) || !isfinite(hraw[i])) {
    ctl->nan = 1;
    ctl->done = 1;
  } else if (fabs(err[i]) < ctl->eps) {
    ctl->conv = 1;
    ctl->done = 1;
  }
  ctl->i = i + 1;
  if (i >= sD) ctl->done = 1;
}

// u_{i+1} = (u_{i+1} - sum_j hraw_j u_j) / hraw_{i}  (classical GS, then
// normalisation), hraw written by k_gm_givens for the column just built.
template <class XT>
__global__ void __launch_bounds__(kThreads) k_gm_orth(size_t n, XT *__restrict__ basis, size_t ld,
                                                      const double *__restrict__ hraw,
                                                      const GmresCtl *ctl, int i_expected) {
  // runs after k_gm_givens of column i_expected; skip if that column was not built
  if (ctl->last_i != i_expected || ctl->nan) return;
  const int i = i_expected;
  XT *__restrict__ v = basis + ld * i;
  const double inv = 1.0 / hraw[i];
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    double acc = double(v[k]);
    for (int j = 0; j < i; j++) acc += -hraw[j] * double(basis[ld * j + k]);
    v[k] = XT(acc * inv);
  }
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
__global__ void __launch_bounds__(kThreads) k_gm_update_x(size_t n, XT *__restrict__ X,
                                                          const XT *__restrict__ basis, size_t ld,
                                                          const double *__restrict__ y,
                                                          const GmresCtl *ctl) {
  const int i = ctl->last_i;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    double acc = double(X[k]);
    for (int j = 0; j < i; j++) acc += y[j] * double(basis[ld * j + k]);
    X[k] = XT(acc);
  }
}

template <class XT>
__global__ void k_convert(size_t n, const double *__restrict__ a, XT *__restrict__ b) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x)
    b[k] = XT(a[k]);
}

// ---------------------------------------------------------------------------
// host side

static inline int blocks_for(size_t n, int cap) {
  size_t b = (n + kThreads - 1) / kThreads;
  if (b > (size_t)cap) b = cap;
  if (b < 1) b = 1;
  return (int)b;
}

template <int D, class VT>
static int precond_diag_t(gsls_lhs *lhs, VT *Val, double *R, double *W) {
  cudaStream_t st = lhs->stream;
  const int nNo = lhs->nNo;
  const size_t nv = (size_t)nNo * D;
  k_diag_w<D, VT><<<blocks_for(nNo, num_sms() * 8), kThreads, 0, st>>>(
      nNo, lhs->d_diagPtr.as<int>(), Val, lhs->ws.mask.as<double>(), W);
  GSLS_CHECK_LAUNCH();
  const size_t nflat = (size_t)lhs->nnz * D * D;
  k_scale_val<D, VT><<<blocks_for(nflat, num_sms() * 16), kThreads, 0, st>>>(
      nflat, lhs->d_rowOf.as<int>(), lhs->d_colPtr.as<int>(), Val, W, W);
  GSLS_CHECK_LAUNCH();
  k_vec_mul<<<blocks_for(nv, num_sms() * 8), kThreads, 0, st>>>(nv, R, W);
  GSLS_CHECK_LAUNCH();
  return GSLS_OK;
}

static int wait_scalars(gsls_lhs *lhs) {
  GSLS_CUDA(cudaMemcpyAsync(lhs->ws.h_scal, lhs->ws.scal.p, sizeof(KrylovScalars),
                            cudaMemcpyDeviceToHost, lhs->stream));
  GSLS_CUDA(cudaStreamSynchronize(lhs->stream));
  return GSLS_OK;
}

// CG on the preconditioned system; R (double, device) in: rhs, out: W*X.
template <int D, class VT, class XT>
static int cg_t(gsls_lhs *lhs, gsls_sub_ls *ls, const VT *Val, double *R, const double *Wc) {
  cudaStream_t st = lhs->stream;
  Workspace &ws = lhs->ws;
  const int nNo = lhs->nNo;
  const size_t nv = (size_t)nNo * D;
  XT *X = ws.vec[0].as<XT>(), *P = ws.vec[1].as<XT>(), *KP = ws.vec[2].as<XT>(),
     *Rk = ws.vec[3].as<XT>();
  KrylovScalars *S = ws.scal.as<KrylovScalars>();
  double *part = ws.partials.as<double>();
  unsigned *tk = ws.ticket.as<unsigned>();
  const int G = lhs->grid;
  auto t0 = std::chrono::steady_clock::now();
  k_cg_init<XT><<<G, kThreads, 0, st>>>(nv, R, Rk, P, X, S, ls->absTol, ls->relTol, ls->mItr,
                                        part, tk);
  GSLS_CHECK_LAUNCH();
  GSLS_TRY(wait_scalars(lhs));
  int batch = 4;
  const bool prof = prof_on();
  while (ws.h_scal->done == 0) {
    const int itr_before = ws.h_scal->itr;
    for (int b = 0; b < batch; b++) {
      if (prof) cudaEventRecord(prof_event(2 * b), st);
      k_cg_spmv<D, VT, XT><<<G, kThreads, 0, st>>>(nNo, lhs->d_rowPtr.as<int>(),
                                                   lhs->d_colPtr.as<int>(), Val, P, KP, S, part,
                                                   tk);
      GSLS_CHECK_LAUNCH();
      if (prof) cudaEventRecord(prof_event(2 * b + 1), st);
      k_cg_update<XT><<<G, kThreads, 0, st>>>(nv, X, Rk, P, KP, S, part, tk);
      GSLS_CHECK_LAUNCH();
      k_cg_pupdate<XT><<<G, kThreads, 0, st>>>(nv, P, Rk, S);
      GSLS_CHECK_LAUNCH();
    }
    GSLS_TRY(wait_scalars(lhs));
    if (prof) {
      // only the launches that did work (one per completed iteration)
      const int worked = ws.h_scal->itr - itr_before;
      double ms = 0.0;
      for (int b = 0; b < worked && b < batch; b++) {
        float t = 0.f;
        cudaEventElapsedTime(&t, prof_event(2 * b), prof_event(2 * b + 1));
        ms += t;
      }
      prof_add("cg_spmv", worked, ms);
    }
    if (batch < 32) batch *= 2;
  }
  k_scale_out<XT><<<G, kThreads, 0, st>>>(nv, R, X, Wc);
  GSLS_CHECK_LAUNCH();
  GSLS_CUDA(cudaStreamSynchronize(st));
  const KrylovScalars &h = *ws.h_scal;
  ls->iNorm = h.iNorm;
  ls->itr = h.itr;
  ls->suc = h.suc;
  ls->fNorm = sqrt(h.err);
  ls->dB = (h.errO < 2.220446049250313e-16) ? 0.0 : 5.0 * log(h.err / h.errO);
  ls->callD = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (h.done == 3) {
    set_error("CG: NaN/Inf or breakdown in Krylov scalars");
    return GSLS_ERR_NAN;
  }
  return GSLS_OK;
}

// Restarted GMRES on the preconditioned system (GMRESS/GMRESV).
// Rhs R (double, device); on exit R = Wc * X, or Wc * R unchanged when
// ||R|| <= absTol (the reference returns early leaving R untouched,
// Code/Source/svFSILS/GMRES.f:310-314).
template <int D, class VT, class XT>
static int gmres_t(gsls_lhs *lhs, gsls_sub_ls *ls, const VT *Val, double *R, const double *Wc) {
  cudaStream_t st = lhs->stream;
  Workspace &ws = lhs->ws;
  const int nNo = lhs->nNo, sD = ls->sD;
  if (sD < 1) {
    set_error("GMRES: Krylov space dimension must be >= 1");
    return GSLS_ERR_ARG;
  }
  const size_t nv = (size_t)nNo * D;
  const size_t ld = (nv + 31) & ~(size_t)31;
  GSLS_TRY(ws.basis.alloc(sizeof(XT) * ld * (size_t)(sD + 1)));
  const int G = lhs->grid;
  const int Gd = num_sms() * 2;  // multi-dot grid
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
  XT *X = ws.vec[0].as<XT>(), *Rk = ws.vec[3].as<XT>();
  double *part = ws.partials.as<double>();
  unsigned *tk = ws.ticket.as<unsigned>();
  double *dnorm = ws.scal.as<double>();  // scratch scalar

  auto t0 = std::chrono::steady_clock::now();
  ls->suc = 0;
  // eps = ||R||, iNorm = fNorm = eps, eps = max(absTol, relTol*eps)
  k_dot<<<G, kThreads, 0, st>>>(nv, R, R, dnorm, part, tk);
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
    ls->callD = 2.220446049250313e-16;
    ls->dB = 0.0;
    k_vec_mul<<<G, kThreads, 0, st>>>(nv, R, Wc);
    GSLS_CHECK_LAUNCH();
    GSLS_CUDA(cudaStreamSynchronize(st));
    return GSLS_OK;
  }
  k_convert<XT><<<G, kThreads, 0, st>>>(nv, R, Rk);
  GSLS_CHECK_LAUNCH();
  GSLS_CUDA(cudaMemsetAsync(X, 0, sizeof(XT) * nv, st));
  GmresCtl hc;
  for (int l = 1; l <= ls->mItr; l++) {
    ls->dB = ls->fNorm;
    ls->itr++;
    XT *u1 = basis;
    if (l > 1) {
      k_spmv<D, VT, XT, XT><<<G, kThreads, 0, st>>>(nNo, lhs->d_rowPtr.as<int>(),
                                                   lhs->d_colPtr.as<int>(), Val, X, u1);
      GSLS_CHECK_LAUNCH();
    }
    k_gm_residual<XT><<<G, kThreads, 0, st>>>(nv, Rk, u1, l > 1 ? 1 : 0, part, tk, err);
    GSLS_CHECK_LAUNCH();
    k_gm_scale<XT><<<G, kThreads, 0, st>>>(nv, u1, err);
    GSLS_CHECK_LAUNCH();
    memset(&hc, 0, sizeof(hc));
    hc.eps = eps;
    hc.i = 1;
    GSLS_CUDA(cudaMemcpyAsync(ctl, &hc, sizeof(hc), cudaMemcpyHostToDevice, st));
    int i_next = 1, batch = 4;
    bool inner_done = false;
    while (!inner_done) {
      for (int b = 0; b < batch && i_next <= sD; b++, i_next++) {
        const int i = i_next;
        XT *ui = basis + ld * (i - 1), *ui1 = basis + ld * i;
        k_spmv<D, VT, XT, XT><<<G, kThreads, 0, st>>>(nNo, lhs->d_rowPtr.as<int>(),
                                                     lhs->d_colPtr.as<int>(), Val, ui, ui1);
        GSLS_CHECK_LAUNCH();
        k_gm_multidot<XT><<<Gd, kThreads, 0, st>>>(nv, basis, ld, i + 1, ui1, part, ctl);
        GSLS_CHECK_LAUNCH();
        k_gm_colsum<<<i + 1, kThreads, 0, st>>>(Gd, part, hcol, ctl);
        GSLS_CHECK_LAUNCH();
        k_gm_givens<<<1, 1, 0, st>>>(sD, H, hcol, hraw, cc, ss, err, ctl);
        GSLS_CHECK_LAUNCH();
        k_gm_orth<XT><<<G, kThreads, 0, st>>>(nv, basis, ld, hraw, ctl, i);
        GSLS_CHECK_LAUNCH();
      }
      GSLS_CUDA(cudaMemcpyAsync(&hc, ctl, sizeof(hc), cudaMemcpyDeviceToHost, st));
      GSLS_CUDA(cudaStreamSynchronize(st));
      if (hc.done || i_next > sD) inner_done = true;
      if (batch < 16) batch *= 2;
    }
    if (hc.nan) {
      set_error("GMRES: NaN/Inf or breakdown in the Arnoldi process");
      return GSLS_ERR_NAN;
    }
    ls->itr += hc.last_i;
    k_gm_backsub<<<1, 1, 0, st>>>(sD, H, err, y, ctl);
    GSLS_CHECK_LAUNCH();
    k_gm_update_x<XT><<<G, kThreads, 0, st>>>(nv, X, basis, ld, y, ctl);
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
  k_scale_out<XT><<<G, kThreads, 0, st>>>(nv, R, X, Wc);
  GSLS_CHECK_LAUNCH();
  GSLS_CUDA(cudaStreamSynchronize(st));
  ls->dB = 10.0 * log(ls->fNorm / ls->dB);
  ls->callD = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return GSLS_OK;
}

template <int D, class VT, class XT>
static int solve_t(gsls_lhs *lhs, gsls_ls *ls, double *dRi, VT *Val, int prec) {
  Workspace &ws = lhs->ws;
  double *W = ws.W.as<double>();
  if (prec == GSLS_PRECOND_FSILS) {
    GSLS_TRY(precond_diag_t<D, VT>(lhs, Val, dRi, W));
  } else if (prec == GSLS_PRECOND_RCS) {
    set_error("PRECOND_RCS is not built in this version of the library");
    return GSLS_ERR_UNSUPPORTED;
  } else {
    set_error("This linear solver and preconditioner combination is not supported.");
    return GSLS_ERR_ARG;
  }
  switch (ls->LS_type) {
    case GSLS_LS_TYPE_CG:
      return cg_t<D, VT, XT>(lhs, &ls->RI, Val, dRi, W);
    case GSLS_LS_TYPE_GMRES:
      return gmres_t<D, VT, XT>(lhs, &ls->RI, Val, dRi, W);
    case GSLS_LS_TYPE_NS:
      set_error("LS_TYPE_NS is not built in this version of the library");
      return GSLS_ERR_UNSUPPORTED;
    default:
      set_error("LS_type not defined");
      return GSLS_ERR_ARG;
  }
}

int solve_dev(gsls_lhs *lhs, gsls_ls *ls, int dof, double *dRi, void *dVal, int val_prec,
              int prec) {
  GSLS_TRY(lhs_prepare_ws(lhs, dof));
  GSLS_TRY(build_dir_mask(lhs, dof));
  const bool mixed = (val_prec == GSLS_PREC_MIXED);
#define GSLS_SOLVE_CASE(DV)                                                              \
  case DV:                                                                               \
    return mixed ? solve_t<DV, float, float>(lhs, ls, dRi, (float *)dVal, prec)          \
                 : solve_t<DV, double, double>(lhs, ls, dRi, (double *)dVal, prec);
  switch (dof) {
    GSLS_SOLVE_CASE(1)
    GSLS_SOLVE_CASE(2)
    GSLS_SOLVE_CASE(3)
    GSLS_SOLVE_CASE(4)
    default:
      set_error("dof must be 1..4");
      return GSLS_ERR_UNSUPPORTED;
  }
#undef GSLS_SOLVE_CASE
}

int spmv_launch(gsls_lhs *lhs, int dof, const void *dVal, int val_prec, const void *dx, void *dy,
                int xprec) {
  (void)xprec;
  cudaStream_t st = lhs->stream;
  const int G = lhs->grid;
  const bool mixed = (val_prec == GSLS_PREC_MIXED);
#define GSLS_SPMV_CASE(DV)                                                                    \
  case DV:                                                                                    \
    if (mixed)                                                                                \
      k_spmv<DV, float, double, double><<<G, kThreads, 0, st>>>(                              \
          lhs->nNo, lhs->d_rowPtr.as<int>(), lhs->d_colPtr.as<int>(), (const float *)dVal,     \
          (const double *)dx, (double *)dy);                                                  \
    else                                                                                      \
      k_spmv<DV, double, double, double><<<G, kThreads, 0, st>>>(                             \
          lhs->nNo, lhs->d_rowPtr.as<int>(), lhs->d_colPtr.as<int>(), (const double *)dVal,    \
          (const double *)dx, (double *)dy);                                                  \
    break;
  switch (dof) {
    GSLS_SPMV_CASE(1)
    GSLS_SPMV_CASE(2)
    GSLS_SPMV_CASE(3)
    GSLS_SPMV_CASE(4)
    default:
      return GSLS_ERR_UNSUPPORTED;
  }
#undef GSLS_SPMV_CASE
  GSLS_CHECK_LAUNCH();
  return GSLS_OK;
}

}  // namespace gsls

using namespace gsls;

extern "C" {

int gsls_solve_dev(gsls_lhs *lhs, gsls_ls *ls, int dof, double *dRi, void *dVal, int val_prec,
                   int prec, const int *incL, const double *res) {
  if (!lhs || !ls || !ls->foC || !dRi || !dVal) {
    set_error("gsls_solve_dev: bad arguments");
    return GSLS_ERR_ARG;
  }
  GSLS_TRY(lhs_update_faces(lhs, incL, res));
  return solve_dev(lhs, ls, dof, dRi, dVal, val_prec, prec);
}

int gsls_solve(gsls_lhs *lhs, gsls_ls *ls, int dof, double *Ri, double *Val, int prec,
               const int *incL, const double *res) {
  if (!lhs || !ls || !ls->foC || !Ri || !Val || dof < 1) {
    set_error("gsls_solve: bad arguments");
    return GSLS_ERR_ARG;
  }
  GSLS_TRY(lhs_update_faces(lhs, incL, res));
  const size_t nr = (size_t)lhs->nNo * dof, nval = (size_t)lhs->nnz * dof * dof;
  GSLS_TRY(lhs->ws.io.alloc(sizeof(double) * nr));
  GSLS_TRY(lhs->ws.io2.alloc(sizeof(double) * nval));
  cudaStream_t st = lhs->stream;
  GSLS_CUDA(cudaMemcpyAsync(lhs->ws.io.p, Ri, sizeof(double) * nr, cudaMemcpyHostToDevice, st));
  GSLS_CUDA(cudaMemcpyAsync(lhs->ws.io2.p, Val, sizeof(double) * nval, cudaMemcpyHostToDevice, st));
  int rc = solve_dev(lhs, ls, dof, lhs->ws.io.as<double>(), lhs->ws.io2.p, GSLS_PREC_FP64, prec);
  if (rc != GSLS_OK && rc != GSLS_ERR_NAN) return rc;
  GSLS_CUDA(cudaMemcpyAsync(Ri, lhs->ws.io.p, sizeof(double) * nr, cudaMemcpyDeviceToHost, st));
  GSLS_CUDA(cudaMemcpyAsync(Val, lhs->ws.io2.p, sizeof(double) * nval, cudaMemcpyDeviceToHost, st));
  GSLS_CUDA(cudaStreamSynchronize(st));
  return rc;
}

int gsls_spmv_dev(gsls_lhs *lhs, int dof, const void *dVal, int val_prec, const double *dx,
                  double *dy) {
  if (!lhs || !dVal || !dx || !dy) return GSLS_ERR_ARG;
  GSLS_TRY(spmv_launch(lhs, dof, dVal, val_prec, dx, dy, 0));
  GSLS_CUDA(cudaStreamSynchronize(lhs->stream));
  return GSLS_OK;
}

int gsls_dot_dev(gsls_lhs *lhs, int dof, const double *du, const double *dv, double *result) {
  if (!lhs || !du || !dv || !result || dof < 1) return GSLS_ERR_ARG;
  GSLS_TRY(lhs_prepare_ws(lhs, dof));
  cudaStream_t st = lhs->stream;
  double *out = lhs->ws.scal.as<double>();
  k_dot<<<lhs->grid, kThreads, 0, st>>>((size_t)lhs->nNo * dof, du, dv, out,
                                        lhs->ws.partials.as<double>(),
                                        lhs->ws.ticket.as<unsigned>());
  GSLS_CHECK_LAUNCH();
  GSLS_CUDA(cudaMemcpyAsync(result, out, sizeof(double), cudaMemcpyDeviceToHost, st));
  GSLS_CUDA(cudaStreamSynchronize(st));
  return GSLS_OK;
}

int gsls_norm_dev(gsls_lhs *lhs, int dof, const double *du, double *result) {
  int rc = gsls_dot_dev(lhs, dof, du, du, result);
  if (rc == GSLS_OK) *result = sqrt(*result);
  return rc;
}

}  // extern "C"
