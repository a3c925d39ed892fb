// BiCGStab (BICGSS/BICGSV, Code/Source/svFSILS/BICGS.f:51-230) on the
// preconditioned system.  Device-resident like CG: the scalars live in a
// device block, every kernel checks its done flag and the host polls it
// once per batch of 8 iterations.  Per iteration: V = K P with Rh.V fused,
// S = R - alpha V, T = K S with T.T and T.S fused, the X/R update with |R|
// and R.Rh, and P = R + beta (P - omega V).  Vectors in the Krylov type XT,
// scalars and every cross-block sum in FP64.
#include <chrono>
#include <cmath>

#include "gsls_internal.cuh"
#include "gsls_spmv.cuh"

namespace gsls {

constexpr int kBT = 256;

struct BiScal {
  double err, errO, eps, rho, rhoO, alpha, omega, beta, iNorm;
  int done, suc, itr, mItr;
};

template <class XT>
__global__ void __launch_bounds__(kBT) k_bi_init(size_t n, const double *__restrict__ R, XT *Rk,
                                                 XT *P, XT *Rh, XT *X, double *partials,
                                                 unsigned *ticket, BiScal *S, double absTol,
                                                 double relTol, int mItr) {
  __shared__ double sh[32];
  double acc = 0.0;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    const double r = R[k];
    Rk[k] = XT(r);
    P[k] = XT(r);
    Rh[k] = XT(r);
    X[k] = XT(0);
    acc += r * r;
  }
  double bs = block_sum(acc, sh);
  double tot;
  if (grid_reduce_last<1>(&bs, partials, ticket, &tot, sh) && threadIdx.x == 0) {
    const double err = sqrt(tot);
    S->err = err;
    S->errO = err;
    S->iNorm = err;
    S->eps = fmax(absTol, relTol * err);
    S->rho = err * err;
    S->beta = S->rho;
    S->itr = 0;
    S->mItr = mItr;
    S->suc = (err < S->eps) ? 1 : 0;
    S->done = (S->suc || mItr < 1) ? 1 : 0;
    if (!isfinite(tot)) S->done = 3;
  }
}

// Y = K Xin; one or two fused dot products of Y with (A, B)
template <int D, class VT, class XT, int NDOT>
__global__ void __launch_bounds__(kBT) k_bi_spmv(int nNo, const int *__restrict__ rowPtr,
                                                 const int *__restrict__ colPtr,
                                                 const VT *__restrict__ Val,
                                                 const XT *__restrict__ Xin, XT *Y,
                                                 const XT *__restrict__ Adot, double *partials,
                                                 unsigned *ticket, BiScal *S) {
  if (*(volatile int *)&S->done) return;
  using AT = typename AccOf<VT>::T;
  __shared__ double sh[32];
  constexpr int RPW = 32 / D;
  const int lane = threadIdx.x & 31, grp = lane / D, r = lane - grp * D;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  GatherX<D, XT, AT> g{Xin};
  double d0 = 0.0, d1 = 0.0;
  for (int base = warp * RPW; base < nNo; base += nwarps * RPW) {
    const int i = base + grp;
    if (grp < RPW && i < nNo) {
      const size_t k = (size_t)i * D + r;
      const AT y = spmv_row_comp<D, VT, AT>(i, r, rowPtr, colPtr, Val, g);
      Y[k] = XT(y);
      if (NDOT == 1) {
        d0 += double(Adot[k]) * double(y);
      } else {
        d0 += double(y) * double(y);
        d1 += double(y) * double(Adot[k]);
      }
    }
  }
  double bs[2];
  bs[0] = block_sum(d0, sh);
  __syncthreads();
  bs[1] = block_sum(d1, sh);
  double tot[2];
  if (grid_reduce_last<2>(bs, partials, ticket, tot, sh) && threadIdx.x == 0) {
    if (NDOT == 1) {
      S->alpha = S->rho / tot[0];  // alpha = rho / (Rh . V)
      if (!isfinite(S->alpha)) S->done = 3;
    } else {
      double om = sqrt(tot[0]);     // omega = |T| ; omega = (T . S) / omega^2
      om = tot[1] / (om * om);
      S->omega = om;
      if (!isfinite(om)) S->done = 3;
    }
  }
}

// S = R - alpha V
template <class XT>
__global__ void k_bi_s(size_t n, const XT *__restrict__ R, const XT *__restrict__ V, XT *Sv,
                       const BiScal *S) {
  if (*(volatile const int *)&S->done) return;
  const XT a = XT(S->alpha);
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x)
    Sv[k] = R[k] - a * V[k];
}

// X += alpha P + omega S; R = S - omega T; err = |R|; rho = R . Rh; beta
template <class XT>
__global__ void __launch_bounds__(kBT) k_bi_update(size_t n, XT *X, const XT *__restrict__ P,
                                                   const XT *__restrict__ Sv,
                                                   const XT *__restrict__ T, XT *R,
                                                   const XT *__restrict__ Rh, double *partials,
                                                   unsigned *ticket, BiScal *S) {
  if (*(volatile int *)&S->done) return;
  __shared__ double sh[32];
  const XT a = XT(S->alpha), o = XT(S->omega);
  double e = 0.0, rh = 0.0;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    X[k] = X[k] + a * P[k] + o * Sv[k];
    const XT r = Sv[k] - o * T[k];
    R[k] = r;
    e += double(r) * double(r);
    rh += double(r) * double(Rh[k]);
  }
  double bs[2];
  bs[0] = block_sum(e, sh);
  __syncthreads();
  bs[1] = block_sum(rh, sh);
  double tot[2];
  if (grid_reduce_last<2>(bs, partials, ticket, tot, sh) && threadIdx.x == 0) {
    S->errO = S->err;
    S->err = sqrt(tot[0]);
    S->rhoO = S->rho;
    S->rho = tot[1];
    S->beta = S->rho * S->alpha / (S->rhoO * S->omega);
    S->itr += 1;
    if (!isfinite(S->err) || !isfinite(S->beta))
      S->done = 3;
    else if (S->itr >= S->mItr)
      S->done = 2;  // no stop test after the last iteration
    else if (S->err < S->eps) {
      S->suc = 1;
      S->done = 1;
    }
  }
}

// P = R + beta (P - omega V)
template <class XT>
__global__ void k_bi_pupdate(size_t n, XT *P, const XT *__restrict__ R, const XT *__restrict__ V,
                             const BiScal *S) {
  if (*(volatile const int *)&S->done) return;
  const XT b = XT(S->beta), o = XT(S->omega);
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x)
    P[k] = R[k] + b * (P[k] - o * V[k]);
}

template <class XT>
__global__ void k_bi_out(size_t n, double *R, const XT *__restrict__ X, const double *__restrict__ W) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x)
    R[k] = W[k] * double(X[k]);
}

template <int D, class VT, class XT>
static int bicgs_t(gsls_lhs *lhs, gsls_sub_ls *ls, const VT *Val, double *R, const double *W) {
  cudaStream_t st = lhs->stream;
  Workspace &ws = lhs->ws;
  const int nNo = lhs->nNo, G = lhs->grid;
  const size_t n = (size_t)nNo * D, ld = (n + 31) & ~(size_t)31;
  GSLS_TRY(ws.basis.alloc(sizeof(XT) * ld * 7 + 256 + sizeof(BiScal)));
  XT *X = ws.basis.as<XT>(), *Rk = X + ld, *P = Rk + ld, *Rh = P + ld, *V = Rh + ld, *Sv = V + ld,
     *T = Sv + ld;
  BiScal *S = reinterpret_cast<BiScal *>((reinterpret_cast<uintptr_t>(T + ld) + 127) & ~(uintptr_t)127);
  GSLS_TRY(ws.partials.alloc(sizeof(double) * (size_t)G * 6 + 64));
  double *part = ws.partials.as<double>();
  unsigned *tk = ws.ticket.as<unsigned>();
  const int *rp = lhs->d_rowPtr.as<int>(), *cp = lhs->d_colPtr.as<int>();
  auto t0 = std::chrono::steady_clock::now();
  ls->suc = 0;
  k_bi_init<XT><<<G, kBT, 0, st>>>(n, R, Rk, P, Rh, X, part, tk, S, ls->absTol, ls->relTol, ls->mItr);
  GSLS_CHECK_LAUNCH();
  BiScal h;
  for (;;) {
    GSLS_CUDA(cudaMemcpyAsync(&h, S, sizeof(h), cudaMemcpyDeviceToHost, st));
    GSLS_CUDA(cudaStreamSynchronize(st));
    if (h.done) break;
    for (int b = 0; b < 8; b++) {
      k_bi_spmv<D, VT, XT, 1><<<G, kBT, 0, st>>>(nNo, rp, cp, Val, P, V, Rh, part, tk, S);
      GSLS_CHECK_LAUNCH();
      k_bi_s<XT><<<G, kBT, 0, st>>>(n, Rk, V, Sv, S);
      GSLS_CHECK_LAUNCH();
      k_bi_spmv<D, VT, XT, 2><<<G, kBT, 0, st>>>(nNo, rp, cp, Val, Sv, T, Sv, part, tk, S);
      GSLS_CHECK_LAUNCH();
      k_bi_update<XT><<<G, kBT, 0, st>>>(n, X, P, Sv, T, Rk, Rh, part, tk, S);
      GSLS_CHECK_LAUNCH();
      k_bi_pupdate<XT><<<G, kBT, 0, st>>>(n, P, Rk, V, S);
      GSLS_CHECK_LAUNCH();
    }
  }
  k_bi_out<XT><<<G, kBT, 0, st>>>(n, R, X, W);
  GSLS_CHECK_LAUNCH();
  GSLS_CUDA(cudaStreamSynchronize(st));
  ls->iNorm = h.iNorm;
  ls->itr = h.itr;
  ls->suc = h.suc;
  ls->fNorm = h.err;
  ls->dB = (h.errO < 2.220446049250313e-16) ? 0.0 : 10.0 * log(h.err / h.errO);
  ls->callD = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (h.done == 3) {
    set_error("BiCGStab: NaN/Inf or breakdown in the Krylov scalars");
    return GSLS_ERR_NAN;
  }
  return GSLS_OK;
}

int bicgs_run(gsls_lhs *lhs, gsls_sub_ls *ls, int D, bool mixed, const void *Val, double *R,
              const double *W) {
#define GSLS_BI_CASE(DV)                                                                   \
  case DV:                                                                                 \
    return mixed ? bicgs_t<DV, float, float>(lhs, ls, (const float *)Val, R, W)            \
                 : bicgs_t<DV, double, double>(lhs, ls, (const double *)Val, R, W);
  switch (D) {
    GSLS_BI_CASE(1)
    GSLS_BI_CASE(2)
    GSLS_BI_CASE(3)
    GSLS_BI_CASE(4)
    default:
      return GSLS_ERR_UNSUPPORTED;
  }
#undef GSLS_BI_CASE
}

}  // namespace gsls
