// Sliced block-ELL copy of the matrix for the CG SpMV.
//
// The CSR SpMV (gsls_spmv.cuh) gives each warp 32/D block rows; one value
// load instruction then touches 32/D unrelated segments of the matrix
// stream (one or two 32-byte sectors each), so the kernel is bound by L1
// sector lookups rather than by HBM.  The sliced copy stores, for each
// slice s of RPW = 32/D rows and each step t below the slice's longest
// row, the t-th block of every row of the slice side by side:
//   value (r, c) of slot g:  sval[(off[s] + t) * RPW*D*D + c * RPW*D + g * D + r]
//   its column:              scol[(off[s] + t) * RPW + g]
// so that load c of a step is RPW*D consecutive values (four sectors for
// D = 3 in FP32) and the columns of a step are RPW consecutive ints.  Rows
// shorter than their slice are padded with zero blocks on their own column;
// a padded step adds fma(0, x, acc) = acc, so every row's product is the
// CSR kernel's bit for bit.  Rows are assigned to slots by decreasing
// length within windows of 32 slices, which keeps the padding small on
// unstructured meshes while the gathers stay local.
#pragma once

#include "gsls_spmv.cuh"

namespace gsls {

struct SellArgs {
  int nS;                 // slices
  const int *off;         // nS + 1 step offsets
  const int *slotRow;     // nS * RPW rows (-1: empty slot)
  const int *scol;        // steps * RPW columns
  const void *sval;       // steps * RPW * D * D values (VT)
};

// sval[slot layout] = Val[CSR block j], from pos[j] = (off[s] + t) * RPW + g
template <int D, class VT>
__global__ void k_sell_pack(size_t n, const int *__restrict__ pos, const VT *__restrict__ Val,
                            VT *__restrict__ sval) {
  constexpr int RPW = 32 / D, DD = D * D;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    const size_t j = k / DD;
    const int rc = (int)(k - j * DD), r = rc / D, c = rc - r * D;
    const int P = __ldg(pos + j);
    const int st = P / RPW, g = P - st * RPW;
    sval[(size_t)st * (RPW * DD) + c * (RPW * D) + g * D + r] = Val[k];
  }
}

// KP = K P over the sliced copy, dot = P . KP, alpha = errO / dot (the
// split CG form of k_cg_spmv; same per-row arithmetic).  zz: odd
// iterations walk the slices from the end.
template <int D, class VT, class XT, int U>
__global__ void __launch_bounds__(kThreads, sizeof(VT) == 4 ? (U > 4 ? 4 : 6) : 1)
    k_cg_spmv_sell(SellArgs A, CgVecs v, KrylovScalars *S, double *partials, unsigned *ticket,
                   int zz) {
  cudaGridDependencySynchronize();  // launched with programmatic serialization
  if (*(volatile int *)&S->done) return;
  using AT = typename AccOf<VT>::T;
  constexpr int VD = VStride<D, XT>::v, RPW = 32 / D, DD = D * D, CH = RPW * DD;
  __shared__ double sh[32];
  __shared__ AT sha[32];
  const VT *__restrict__ sval = (const VT *)A.sval;
  const XT *__restrict__ P = (const XT *)v.P0;
  XT *__restrict__ KP = (XT *)v.KP;
  GatherX<D, XT, AT, VD> gx{P};
  const int lane = threadIdx.x & 31, g = lane / D, r = lane - g * D;
  const bool act = g < RPW;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  AT dot = AT(0);
  const bool rev = zz && (S->itr & 1);
  for (int s0 = warp; s0 < A.nS; s0 += nwarps) {
    const int s = rev ? A.nS - 1 - s0 : s0;
    const int t0 = __ldg(A.off + s), t1 = __ldg(A.off + s + 1);
    const int row = act ? __ldg(A.slotRow + s * RPW + g) : -1;
    AT acc0 = AT(0), acc1 = AT(0);
    // columns run one group of U steps ahead, so that a group's gathers,
    // its values and the next group's columns are in flight together (one
    // memory round trip per group instead of two)
    int cn[U];
#pragma unroll
    for (int u = 0; u < U; u++)
      cn[u] = (act && t0 + u < t1) ? __ldg(A.scol + (size_t)(t0 + u) * RPW + g) : -1;
    for (int t = t0; t < t1; t += U) {
      int cc[U];
#pragma unroll
      for (int u = 0; u < U; u++) {
        cc[u] = cn[u];
        cn[u] = (act && t + U + u < t1) ? __ldg(A.scol + (size_t)(t + U + u) * RPW + g) : -1;
      }
      AT a[U][D], xg[U][D];
#pragma unroll
      for (int u = 0; u < U; u++) {
        if (cc[u] >= 0) {
          const VT *p = sval + (size_t)(t + u) * CH + g * D + r;
#pragma unroll
          for (int c = 0; c < D; c++) a[u][c] = AT(__ldg(p + c * (RPW * D)));
          gx.get(cc[u], xg[u]);
        } else {
#pragma unroll
          for (int c = 0; c < D; c++) a[u][c] = xg[u][c] = AT(0);
        }
      }
#pragma unroll
      for (int u = 0; u < U; u++)
#pragma unroll
        for (int c = 0; c < D; c++) {
          if (u & 1)
            acc1 = fma(a[u][c], xg[u][c], acc1);
          else
            acc0 = fma(a[u][c], xg[u][c], acc0);
        }
    }
    if (row >= 0) {
      const AT y = acc0 + acc1;
      const size_t k = (size_t)row * VD + r;
      KP[k] = XT(y);
      dot = fma(AT(P[k]), y, dot);
    }
  }
  const AT bsa = block_sum_t<AT>(dot, sha);
  double bs = double(bsa);
  double tot;
  if (grid_reduce_last1<1>(&bs, partials, ticket, &tot, sh) && threadIdx.x == 0) {
    S->errO = S->err;
    S->dot = tot;
    S->alpha = S->errO / tot;
    if (!isfinite(S->alpha)) S->done = 3;
  }
}

}  // namespace gsls
