// Preconditioning, CG and FSILS_SOLVE dispatch with the semantics of
// svFSILS (Code/Source/svFSILS: PRECOND.f, CGRAD.f, DOT.f, NORM.f, SOLVE.f).
//
// Design: all Krylov scalars live in device memory (KrylovScalars); every
// kernel of an iteration first checks the device "done" flag, so the host
// enqueues fixed batches of iterations (replayed as one CUDA graph) and
// polls the flag once per batch.  The CG direction update P = R + beta*P is
// fused into the next SpMV (double-buffered P), so one CG iteration is two
// kernels: SpMV+dot and update+norm.  Reductions use a fixed grid and a
// last-block pass: every sum is bitwise reproducible.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "gsls_internal.cuh"
#include "gsls_spmv.cuh"

namespace gsls {

constexpr int kThreads = 256;

// ---------------------------------------------------------------------------
// CG kernels (CGRADS/CGRADV, Code/Source/svFSILS/CGRAD.f:125-242)
struct CgVecs {
  void *X, *R, *P0, *P1, *KP;
};

// R_k = R; P0 = 0; X = 0; iNorm = ||R||; eps; errO = err = iNorm^2; beta = 0
template <class XT>
__global__ void __launch_bounds__(kThreads) k_cg_init(size_t n, const double *__restrict__ R,
                                                      CgVecs v, KrylovScalars *S, double absTol,
                                                      double relTol, int mItr, double *partials,
                                                      unsigned *ticket) {
  __shared__ double sh[32];
  XT *Rk = (XT *)v.R, *P0 = (XT *)v.P0, *X = (XT *)v.X;
  double acc = 0.0;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    const double r = R[k];
    acc += r * r;
    Rk[k] = XT(r);
    P0[k] = XT(0);
    X[k] = XT(0);
  }
  double bs = block_sum(acc, sh);
  double tot;
  if (grid_reduce_last<1>(&bs, partials, ticket, &tot, sh) && threadIdx.x == 0) {
    const double iNorm = sqrt(tot);
    S->iNorm = iNorm;
    const double e = fmax(absTol, relTol * iNorm);
    S->eps = e * e;
    S->errO = iNorm * iNorm;
    S->err = S->errO;
    S->beta = 0.0;
    S->itr = 0;
    S->mItr = mItr;
    S->suc = 0;
    S->done = 0;
    if (mItr < 1)
      S->done = 2;
    else if (S->err < S->eps) {
      S->done = 1;
      S->suc = 1;
    }
    if (!isfinite(tot)) S->done = 3;
  }
}

// P_new = R + beta P_old (own rows), KP = K P_new with P_new gathered on the
// fly, dot = P_new . KP, alpha = errO / dot.
template <int D, class VT, class XT>
__global__ void __launch_bounds__(kThreads) k_cg_spmv(int nNo, const int *__restrict__ rowPtr,
                                                      const int *__restrict__ colPtr,
                                                      const VT *__restrict__ Val, CgVecs v,
                                                      KrylovScalars *S, double *partials,
                                                      unsigned *ticket) {
  if (*(volatile int *)&S->done) return;
  using AT = typename AccOf<VT>::T;
  __shared__ double sh[32];
  __shared__ AT sha[32];
  constexpr int RPW = 32 / D;
  const int par = S->itr & 1;
  const XT *__restrict__ Pold = (const XT *)(par ? v.P1 : v.P0);
  XT *__restrict__ Pnew = (XT *)(par ? v.P0 : v.P1);
  const XT *__restrict__ R = (const XT *)v.R;
  XT *__restrict__ KP = (XT *)v.KP;
  const AT beta = AT(S->beta);
  GatherDir<D, XT, AT> g{R, Pold, beta};
  const int lane = threadIdx.x & 31, grp = lane / D, r = lane - grp * D;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  AT dot = AT(0);
  for (int base = warp * RPW; base < nNo; base += nwarps * RPW) {
    const int i = base + grp;
    if (grp < RPW && i < nNo) {
      const AT y = spmv_row_comp<D, VT, AT>(i, r, rowPtr, colPtr, Val, g);
      const size_t k = (size_t)i * D + r;
      const AT pn = AT(R[k]) + beta * AT(Pold[k]);
      Pnew[k] = XT(pn);
      KP[k] = XT(y);
      dot = fma(pn, y, dot);
    }
  }
  const AT bsa = block_sum_t<AT>(dot, sha);
  double bs = double(bsa);
  double tot;
  if (grid_reduce_last<1>(&bs, partials, ticket, &tot, sh) && threadIdx.x == 0) {
    S->errO = S->err;
    S->dot = tot;
    S->alpha = S->errO / tot;
    if (!isfinite(S->alpha)) S->done = 3;
  }
}

// X += alpha P_new; R -= alpha KP; err = ||R||^2; beta; convergence test
template <class XT>
__global__ void __launch_bounds__(kThreads) k_cg_update(size_t n, CgVecs v, KrylovScalars *S,
                                                        double *partials, unsigned *ticket) {
  if (*(volatile int *)&S->done) return;
  using AT = XT;
  __shared__ double sh[32];
  __shared__ AT sha[32];
  const int par = S->itr & 1;
  const XT *__restrict__ P = (const XT *)(par ? v.P0 : v.P1);
  XT *__restrict__ X = (XT *)v.X;
  XT *__restrict__ R = (XT *)v.R;
  const XT *__restrict__ KP = (const XT *)v.KP;
  const AT alpha = AT(S->alpha);
  AT acc = AT(0);
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    X[k] = fma(alpha, P[k], X[k]);
    const AT r = fma(-alpha, KP[k], R[k]);
    R[k] = r;
    acc = fma(r, r, acc);
  }
  const AT bsa = block_sum_t<AT>(acc, sha);
  double bs = double(bsa);
  double tot;
  if (grid_reduce_last<1>(&bs, partials, ticket, &tot, sh) && threadIdx.x == 0) {
    S->err = tot;
    S->beta = tot / S->errO;
    S->itr += 1;
    if (!isfinite(tot))
      S->done = 3;
    else if (S->itr >= S->mItr)
      S->done = 2;
    else if (S->err < S->eps) {
      S->done = 1;
      S->suc = 1;
    }
  }
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
                         const double *__restrict__ mask, double *__restrict__ W,
                         float *__restrict__ Wf, double *__restrict__ R) {
  constexpr int DD = D * D;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nNo; i += gridDim.x * blockDim.x) {
    const int d = diagPtr[i];
#pragma unroll
    for (int k = 0; k < D; k++) {
      double w = double(Val[(size_t)d * DD + k * D + k]);
      if (w == 0.0) w = 1.0;
      w = 1.0 / sqrt(fabs(w));
      w = w * mask[(size_t)i * D + k];
      W[(size_t)i * D + k] = w;
      Wf[(size_t)i * D + k] = float(w);
      R[(size_t)i * D + k] *= w;  // R = W R
    }
  }
}

// Val = diag(W) Val diag(W) (PREMUL then POSMUL), block row per D-lane group
template <int D, class VT, class WT>
__global__ void __launch_bounds__(kThreads) k_scale_val(int nNo, const int *__restrict__ rowPtr,
                                                        const int *__restrict__ colPtr,
                                                        VT *__restrict__ Val,
                                                        const WT *__restrict__ W) {
  constexpr int RPW = 32 / D, DD = D * D;
  const int lane = threadIdx.x & 31, grp = lane / D, r = lane - grp * D;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int base = warp * RPW; base < nNo; base += nwarps * RPW) {
    const int i = base + grp;
    if (grp >= RPW || i >= nNo) continue;
    const WT wr = W[(size_t)i * D + r];
    const int rs = rowPtr[i], re = rowPtr[i + 1];
    for (int j = rs; j < re; j++) {
      const int col = colPtr[j];
      VT *v = Val + (size_t)j * DD + r * D;
#pragma unroll
      for (int c = 0; c < D; c++) {
        WT t = WT(v[c]) * wr;
        t = t * W[(size_t)col * D + c];
        v[c] = VT(t);
      }
    }
  }
}

__global__ void k_vec_mul(size_t n, double *__restrict__ R, const double *__restrict__ W) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x)
    R[k] *= W[k];
}

// plain dot product for the public entry point
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
  float *Wf = lhs->ws.Wf.as<float>();
  k_diag_w<D, VT><<<blocks_for(nNo, num_sms() * 8), kThreads, 0, st>>>(
      nNo, lhs->d_diagPtr.as<int>(), Val, lhs->ws.mask.as<double>(), W, Wf, R);
  GSLS_CHECK_LAUNCH();
  if (sizeof(VT) == 4)
    k_scale_val<D, VT, float><<<lhs->grid, kThreads, 0, st>>>(
        nNo, lhs->d_rowPtr.as<int>(), lhs->d_colPtr.as<int>(), Val, Wf);
  else
    k_scale_val<D, VT, double><<<lhs->grid, kThreads, 0, st>>>(
        nNo, lhs->d_rowPtr.as<int>(), lhs->d_colPtr.as<int>(), Val, W);
  GSLS_CHECK_LAUNCH();
  return GSLS_OK;
}

static int wait_scalars(gsls_lhs *lhs) {
  GSLS_CUDA(cudaMemcpyAsync(lhs->ws.h_scal, lhs->ws.scal.p, sizeof(KrylovScalars),
                            cudaMemcpyDeviceToHost, lhs->stream));
  GSLS_CUDA(cudaStreamSynchronize(lhs->stream));
  return GSLS_OK;
}

// Grid of a grid-stride kernel: exactly the resident blocks on all SMs (one
// wave), capped by the lhs reduction grid; fixed per kernel and device, so
// its reductions stay reproducible.
template <class K>
static int resident_grid(K kernel, int cap) {
  int nb = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, kThreads, 0);
  if (nb < 1) nb = 1;
  int g = nb * num_sms();
  return g < cap ? g : cap;
}

template <int D, class VT, class XT>
static int cg_enqueue(gsls_lhs *lhs, const VT *Val, const CgVecs &v, int n_iter, bool prof,
                      int ev_base) {
  cudaStream_t st = lhs->stream;
  Workspace &ws = lhs->ws;
  const int nNo = lhs->nNo;
  static const int Gs = resident_grid(k_cg_spmv<D, VT, XT>, 1 << 30);
  static const int Gu = resident_grid(k_cg_update<XT>, 1 << 30);
  const int G1 = Gs < lhs->grid ? Gs : lhs->grid, G2 = Gu < lhs->grid ? Gu : lhs->grid;
  const size_t nv = (size_t)nNo * D;
  KrylovScalars *S = ws.scal.as<KrylovScalars>();
  double *part = ws.partials.as<double>();
  unsigned *tk = ws.ticket.as<unsigned>();
  for (int b = 0; b < n_iter; b++) {
    if (prof) cudaEventRecord(prof_event(ev_base + 2 * b), st);
    k_cg_spmv<D, VT, XT><<<G1, kThreads, 0, st>>>(nNo, lhs->d_rowPtr.as<int>(),
                                                  lhs->d_colPtr.as<int>(), Val, v, S, part, tk);
    GSLS_CHECK_LAUNCH();
    if (prof) cudaEventRecord(prof_event(ev_base + 2 * b + 1), st);
    k_cg_update<XT><<<G2, kThreads, 0, st>>>(nv, v, S, part, tk);
    GSLS_CHECK_LAUNCH();
  }
  return GSLS_OK;
}

// CG on the preconditioned system; R (double, device) in: rhs, out: W*X.
template <int D, class VT, class XT>
static int cg_t(gsls_lhs *lhs, gsls_sub_ls *ls, const VT *Val, double *R, const double *Wc) {
  cudaStream_t st = lhs->stream;
  Workspace &ws = lhs->ws;
  const int nNo = lhs->nNo;
  const size_t nv = (size_t)nNo * D;
  CgVecs v{ws.vec[0].p, ws.vec[1].p, ws.vec[2].p, ws.vec[3].p, ws.vec[4].p};
  KrylovScalars *S = ws.scal.as<KrylovScalars>();
  double *part = ws.partials.as<double>();
  unsigned *tk = ws.ticket.as<unsigned>();
  const int G = lhs->grid;
  auto t0 = std::chrono::steady_clock::now();
  k_cg_init<XT><<<G, kThreads, 0, st>>>(nv, R, v, S, ls->absTol, ls->relTol, ls->mItr, part, tk);
  GSLS_CHECK_LAUNCH();
  GSLS_TRY(wait_scalars(lhs));
  const bool prof = prof_on();
  const int B = nv < (1u << 20) ? 8 : 16;
  // CUDA graph of B iterations, cached per (D, types, Val, workspace)
  GraphKey key{D, (int)sizeof(VT), (int)sizeof(XT), (const void *)Val, v.X, B, nNo};
  if (!prof && !(ws.cg_graph && ws.cg_key == key)) {
    if (ws.cg_graph) {
      cudaGraphExecDestroy(ws.cg_graph);
      ws.cg_graph = nullptr;
    }
    cudaGraph_t g;
    GSLS_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    int rc = cg_enqueue<D, VT, XT>(lhs, Val, v, B, false, 0);
    cudaError_t e = cudaStreamEndCapture(st, &g);
    if (rc != GSLS_OK) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture", __FILE__, __LINE__);
    GSLS_CUDA(cudaGraphInstantiate(&ws.cg_graph, g, 0));
    cudaGraphDestroy(g);
    ws.cg_key = key;
  }
  while (ws.h_scal->done == 0) {
    const int itr_before = ws.h_scal->itr;
    if (prof) {
      GSLS_TRY(cg_enqueue<D, VT, XT>(lhs, Val, v, B, true, 0));
    } else {
      GSLS_CUDA(cudaGraphLaunch(ws.cg_graph, st));
      count_launch_n(2 * B - 1);
    }
    GSLS_TRY(wait_scalars(lhs));
    if (prof) {
      // only the launches that did work (one per completed iteration)
      const int worked = ws.h_scal->itr - itr_before;
      double ms = 0.0;
      for (int b = 0; b < worked && b < B; b++) {
        float t = 0.f;
        cudaEventElapsedTime(&t, prof_event(2 * b), prof_event(2 * b + 1));
        ms += t;
      }
      prof_add("cg_spmv", worked, ms);
    }
  }
  k_scale_out<XT><<<G, kThreads, 0, st>>>(nv, R, (const XT *)v.X, Wc);
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
      return gmres_run(lhs, &ls->RI, D, sizeof(VT) == 4, Val, dRi, W);
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
