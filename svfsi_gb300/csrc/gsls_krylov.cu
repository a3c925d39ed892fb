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
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "gsls_gridbar.cuh"
#include "gsls_internal.cuh"
#include "gsls_spmv.cuh"

namespace gsls {

constexpr int kThreads = 256;

// ---------------------------------------------------------------------------
// CG kernels (CGRADS/CGRADV, Code/Source/svFSILS/CGRAD.f:125-242)
struct CgVecs {
  void *X, *R, *P0, *P1, *KP;
};

// R_k = R; P0 = P1 = KP = 0; X = 0; iNorm = ||R||; eps; errO = err =
// iNorm^2; beta = 0.  Work vectors use node stride VD (pads stay zero).
template <int D, class XT, bool FUSED>
__global__ void __launch_bounds__(kThreads) k_cg_init(int nNo, const double *__restrict__ R,
                                                      CgVecs v, KrylovScalars *S, double absTol,
                                                      double relTol, int mItr, double *partials,
                                                      unsigned *ticket) {
  constexpr int VD = VStride<D, XT>::v;
  __shared__ double sh[32];
  XT *Rk = (XT *)v.R, *P0 = (XT *)v.P0, *P1 = (XT *)v.P1, *X = (XT *)v.X, *KP = (XT *)v.KP;
  double acc = 0.0;
  const size_t n = (size_t)nNo * VD;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    const size_t a = k / VD;
    const int c = (int)(k - a * VD);
    const double r = (c < D) ? R[a * D + c] : 0.0;
    acc += r * r;
    Rk[k] = XT(r);
    P0[k] = FUSED ? XT(0) : XT(r);  // fused: P built from R in the first SpMV
    P1[k] = XT(0);
    KP[k] = XT(0);
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
// FUSED = false: the direction P (= P0) is updated by k_cg_pupdate and the
// SpMV gathers P alone (half the gather traffic of the fused form).
// zz: odd iterations walk the rows from the end (see zigzag_rev).
template <int D, class VT, class XT, bool FUSED>
__global__ void __launch_bounds__(kThreads) k_cg_spmv(int nNo, const int *__restrict__ rowPtr,
                                                      const int *__restrict__ colPtr,
                                                      const VT *__restrict__ Val, CgVecs v,
                                                      KrylovScalars *S, double *partials,
                                                      unsigned *ticket, int zz) {
  cudaGridDependencySynchronize();  // launched with programmatic serialization
  if (*(volatile int *)&S->done) return;
  using AT = typename AccOf<VT>::T;
  constexpr int VD = VStride<D, XT>::v;
  __shared__ double sh[32];
  __shared__ AT sha[32];
  constexpr int RPW = 32 / D;
  const int par = S->itr & 1;
  const XT *__restrict__ Pold = (const XT *)(par ? v.P1 : v.P0);
  XT *__restrict__ Pnew = (XT *)(par ? v.P0 : v.P1);
  const XT *__restrict__ R = (const XT *)v.R;
  XT *__restrict__ KP = (XT *)v.KP;
  const AT beta = AT(S->beta);
  GatherDir<D, XT, AT, VD> gd{R, Pold, beta};
  GatherX<D, XT, AT, VD> gx{(const XT *)v.P0};
  const int lane = threadIdx.x & 31, grp = lane / D, r = lane - grp * D;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  AT dot = AT(0);
  const bool rev = zz && (S->itr & 1);
  for (int base = warp * RPW; base < nNo; base += nwarps * RPW) {
    const int i = rev ? nNo - 1 - (base + grp) : base + grp;
    if (grp < RPW && i >= 0 && i < nNo) {
      const size_t k = (size_t)i * VD + r;
      AT y, pn;
      if constexpr (FUSED) {
        y = spmv_row_comp<D, VT, AT>(i, r, rowPtr, colPtr, Val, gd);
        pn = AT(R[k]) + beta * AT(Pold[k]);
        Pnew[k] = XT(pn);
      } else {
        y = spmv_row_comp<D, VT, AT>(i, r, rowPtr, colPtr, Val, gx);
        pn = AT(((const XT *)v.P0)[k]);
      }
      KP[k] = XT(y);
      dot = fma(pn, y, dot);
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

#include "gsls_sell.cuh"

namespace gsls {

// ---------------------------------------------------------------------------
// TMA-staged variant of k_cg_spmv.  A tile is NW*(32/D) consecutive block
// rows; its matrix values and column indices are one contiguous range each,
// copied global -> shared by cp.async.bulk (one elected thread, completion on
// an mbarrier), double-buffered so the copy of tile k+2 overlaps the math of
// tile k.  Lanes then read values/columns from shared memory and only gather
// the vector from L2.  Copies start on a 16-byte boundary (ranges rounded
// outwards), so Val and colPtr must be allocated with >= 16 bytes of slack.
struct TmaTiles {
  int ntiles, tile_rows;
  int val_buf, col_buf;  // bytes per buffer (multiples of 16)
  int *err;              // device error word (bit 1: barrier wait timed out)
};

__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
// Bounded wait on an mbarrier phase; false if the limit was hit.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity) {
  for (int it = 0; it < (1 << 22); it++) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

template <int D, class VT>
__device__ __forceinline__ void tma_issue_tile(int t, int nNo, const TmaTiles &tt,
                                               const int *__restrict__ rowPtr,
                                               const int *__restrict__ colPtr,
                                               const VT *__restrict__ Val, unsigned char *buf,
                                               uint64_t *bar) {
  constexpr int DD = D * D, A = 16 / sizeof(VT);
  const int r0 = t * tt.tile_rows;
  const int r1 = min(r0 + tt.tile_rows, nNo);
  const int c0 = __ldg(rowPtr + r0), c1 = __ldg(rowPtr + r1);
  const long long e0 = (long long)c0 * DD, e1 = (long long)c1 * DD;
  const long long e0a = e0 & ~(long long)(A - 1), e1a = (e1 + A - 1) & ~(long long)(A - 1);
  const int c0a = c0 & ~3, c1a = (c1 + 3) & ~3;
  const unsigned vb = (unsigned)((e1a - e0a) * sizeof(VT)), cb = (unsigned)((c1a - c0a) * 4);
  mbar_expect_tx(bar, vb + cb);
  bulk_g2s(buf, Val + e0a, vb, bar);
  bulk_g2s(buf + tt.val_buf, colPtr + c0a, cb, bar);
}

template <int D, class VT, class XT, int NW, bool FUSED>
__global__ void __launch_bounds__(NW * 32) k_cg_spmv_tma(int nNo, const int *__restrict__ rowPtr,
                                                         const int *__restrict__ colPtr,
                                                         const VT *__restrict__ Val, CgVecs v,
                                                         KrylovScalars *S, double *partials,
                                                         unsigned *ticket, TmaTiles tt) {
  if (*(volatile int *)&S->done) return;
  using AT = typename AccOf<VT>::T;
  constexpr int VD = VStride<D, XT>::v;
  constexpr int RPW = 32 / D, DD = D * D, A = 16 / sizeof(VT);
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ double sh[32];
  __shared__ AT sha[32];
  const int bufsz = tt.val_buf + tt.col_buf;
  unsigned char *buf0 = smem, *buf1 = smem + bufsz;
  const int par = S->itr & 1;
  const XT *__restrict__ Pold = (const XT *)(par ? v.P1 : v.P0);
  XT *__restrict__ Pnew = (XT *)(par ? v.P0 : v.P1);
  const XT *__restrict__ R = (const XT *)v.R;
  XT *__restrict__ KP = (XT *)v.KP;
  const AT beta = AT(S->beta);
  using G = typename std::conditional<FUSED, GatherDir<D, XT, AT, VD>, GatherX<D, XT, AT, VD>>::type;
  G g;
  if constexpr (FUSED)
    g = G{R, Pold, beta};
  else
    g = G{(const XT *)v.P0};
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, grp = lane / D, r = lane - grp * D;
  constexpr int SP = 2, RW = RPW / SP;  // lane groups per row, rows per warp
  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const int t0 = blockIdx.x, stride = gridDim.x;
  if (threadIdx.x == 0) {
    if (t0 < tt.ntiles) tma_issue_tile<D, VT>(t0, nNo, tt, rowPtr, colPtr, Val, buf0, &bars[0]);
    if (t0 + stride < tt.ntiles)
      tma_issue_tile<D, VT>(t0 + stride, nNo, tt, rowPtr, colPtr, Val, buf1, &bars[1]);
  }
  AT dot = AT(0);
  bool ok = true;
  int k = 0;
  for (int t = t0; t < tt.ntiles; t += stride, k++) {
    const int b = k & 1;
    unsigned char *buf = b ? buf1 : buf0;
    const bool waited = mbar_wait(&bars[b], (k >> 1) & 1);
    if (!__syncthreads_and(waited)) {
      // a copy did not land: stop, drain what is in flight (bounded), flag
      ok = false;
      if (threadIdx.x == 0) {
        mbar_wait(&bars[b], (k >> 1) & 1);
        if (t + stride < tt.ntiles) mbar_wait(&bars[b ^ 1], ((k + 1) >> 1) & 1);
      }
      break;
    }
    const int r0 = t * tt.tile_rows;
    const long long e0a = ((long long)__ldg(rowPtr + r0) * DD) & ~(long long)(A - 1);
    const int c0a = __ldg(rowPtr + r0) & ~3;
    const VT *__restrict__ sv = reinterpret_cast<const VT *>(buf);
    const int *__restrict__ sc = reinterpret_cast<const int *>(buf + tt.val_buf);
    // SP lane groups share a block row (blocks j = s, s+SP, ...) so that a
    // tile keeps 2x the warps busy for the same shared-memory footprint
    const int slot = grp / SP, s = grp - slot * SP;
    const int i = r0 + wid * RW + slot;
    const bool valid = grp < RPW && slot < RW && i < nNo && i < r0 + tt.tile_rows;
    AT y = AT(0);
    if (valid) {
      const int rs = __ldg(rowPtr + i), re = __ldg(rowPtr + i + 1);
      const VT *vrow = sv + ((long long)rs * DD - e0a) + r * D;
      const int *crow = sc + (rs - c0a);
      AT acc0 = AT(0), acc1 = AT(0);
      const int nb = re - rs;
      // all gathers of U blocks in flight before the first FMA (the L2
      // gather latency is what bounds this kernel, not the staged stream)
      constexpr int U = 8;
      for (int j = s; j < nb; j += U * SP) {
        AT xg[U][D];
#pragma unroll
        for (int u = 0; u < U; u++) {
          if (j + u * SP < nb) {
            g.get(crow[j + u * SP], xg[u]);
          } else {
#pragma unroll
            for (int c = 0; c < D; c++) xg[u][c] = AT(0);
          }
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
          if (j + u * SP < nb) {
#pragma unroll
            for (int c = 0; c < D; c++) {
              if (u & 1)
                acc1 = fma(AT(vrow[(j + u * SP) * DD + c]), xg[u][c], acc1);
              else
                acc0 = fma(AT(vrow[(j + u * SP) * DD + c]), xg[u][c], acc0);
            }
          }
        }
      }
      y = acc0 + acc1;
    }
#pragma unroll
    for (int o = 1; o < SP; o <<= 1) y += __shfl_down_sync(0xffffffffu, y, o * D);
    if (valid && s == 0) {
      const size_t kk = (size_t)i * VD + r;
      AT pn;
      if constexpr (FUSED) {
        pn = AT(R[kk]) + beta * AT(Pold[kk]);
        Pnew[kk] = XT(pn);
      } else {
        pn = AT(((const XT *)v.P0)[kk]);
      }
      KP[kk] = XT(y);
      dot = fma(pn, y, dot);
    }
    __syncthreads();  // everyone is done with this buffer
    if (threadIdx.x == 0 && t + 2 * stride < tt.ntiles)
      tma_issue_tile<D, VT>(t + 2 * stride, nNo, tt, rowPtr, colPtr, Val, buf, &bars[b]);
  }
  if (!ok && threadIdx.x == 0) atomicOr(tt.err, 2);
  const AT bsa = block_sum_t<AT>(dot, sha);
  double bs = double(bsa);
  double tot;
  if (grid_reduce_last<1>(&bs, partials, ticket, &tot, sh) && threadIdx.x == 0) {
    S->errO = S->err;
    S->dot = tot;
    S->alpha = S->errO / tot;
    if (!isfinite(S->alpha)) S->done = 3;
    if (*(volatile int *)tt.err) S->done = 3;
  }
}

// X += alpha P_new; R -= alpha KP; err = ||R||^2; beta; convergence test.
// Fat blocks (kUpdThreads) keep the grid -- and the last-block ticket chain
// -- short; FP32 vectors are streamed as float4.
constexpr int kUpdThreads = 512;
template <class XT, bool FUSED>
__global__ void __launch_bounds__(kUpdThreads, 2) k_cg_update(size_t n, CgVecs v, KrylovScalars *S,
                                                           double *partials, unsigned *ticket) {
  cudaGridDependencySynchronize();
  using AT = XT;
  __shared__ double sh[32];
  __shared__ AT sha[32];
  XT *__restrict__ X = (XT *)v.X;
  XT *__restrict__ R = (XT *)v.R;
  const XT *__restrict__ KP = (const XT *)v.KP;
  AT acc = AT(0);
  size_t k0 = 0;
  constexpr bool kEarly = sizeof(XT) == 4 && !FUSED;
  if constexpr (kEarly) {
    // the first float4 of each vector is requested before the done flag and
    // alpha, so that the loads' latency overlaps the scalar reads
    const size_t n4 = n / 4, t0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t nt = (size_t)gridDim.x * blockDim.x;
    float4 *__restrict__ X4 = reinterpret_cast<float4 *>(X);
    float4 *__restrict__ R4 = reinterpret_cast<float4 *>(R);
    const float4 *__restrict__ P4 = reinterpret_cast<const float4 *>(v.P0);
    const float4 *__restrict__ K4 = reinterpret_cast<const float4 *>(KP);
    float4 xa = make_float4(0.f, 0.f, 0.f, 0.f), ra = xa, pa = xa, qa = xa;
    if (t0 < n4) {
      xa = X4[t0];
      ra = R4[t0];
      pa = P4[t0];
      qa = K4[t0];
    }
    if (*(volatile int *)&S->done) return;
    const AT alpha = AT(S->alpha);
    for (size_t k = t0; k < n4; k += nt) {
      float4 x, r, p, q;
      if (k == t0) {
        x = xa;
        r = ra;
        p = pa;
        q = qa;
      } else {
        x = X4[k];
        r = R4[k];
        p = P4[k];
        q = K4[k];
      }
      x.x = fmaf(alpha, p.x, x.x);
      x.y = fmaf(alpha, p.y, x.y);
      x.z = fmaf(alpha, p.z, x.z);
      x.w = fmaf(alpha, p.w, x.w);
      r.x = fmaf(-alpha, q.x, r.x);
      r.y = fmaf(-alpha, q.y, r.y);
      r.z = fmaf(-alpha, q.z, r.z);
      r.w = fmaf(-alpha, q.w, r.w);
      X4[k] = x;
      R4[k] = r;
      acc = fmaf(r.x, r.x, acc);
      acc = fmaf(r.y, r.y, acc);
      acc = fmaf(r.z, r.z, acc);
      acc = fmaf(r.w, r.w, acc);
    }
    k0 = n4 * 4;
  } else {
    if (*(volatile int *)&S->done) return;
  }
  const int par = S->itr & 1;
  const XT *__restrict__ P = (const XT *)(FUSED ? (par ? v.P0 : v.P1) : v.P0);
  const AT alpha = AT(S->alpha);
  if constexpr (sizeof(XT) == 4 && FUSED) {
    const size_t n4 = n / 4;
    float4 *__restrict__ X4 = reinterpret_cast<float4 *>(X);
    float4 *__restrict__ R4 = reinterpret_cast<float4 *>(R);
    const float4 *__restrict__ P4 = reinterpret_cast<const float4 *>(P);
    const float4 *__restrict__ K4 = reinterpret_cast<const float4 *>(KP);
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n4;
         k += (size_t)gridDim.x * blockDim.x) {
      float4 x = X4[k], r = R4[k];
      const float4 p = P4[k], q = K4[k];
      x.x = fmaf(alpha, p.x, x.x);
      x.y = fmaf(alpha, p.y, x.y);
      x.z = fmaf(alpha, p.z, x.z);
      x.w = fmaf(alpha, p.w, x.w);
      r.x = fmaf(-alpha, q.x, r.x);
      r.y = fmaf(-alpha, q.y, r.y);
      r.z = fmaf(-alpha, q.z, r.z);
      r.w = fmaf(-alpha, q.w, r.w);
      X4[k] = x;
      R4[k] = r;
      acc = fmaf(r.x, r.x, acc);
      acc = fmaf(r.y, r.y, acc);
      acc = fmaf(r.z, r.z, acc);
      acc = fmaf(r.w, r.w, acc);
    }
    k0 = n4 * 4;
  }
  for (size_t k = k0 + (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    X[k] = fma(alpha, P[k], X[k]);
    const AT r = fma(-alpha, KP[k], R[k]);
    R[k] = r;
    acc = fma(r, r, acc);
  }
  const AT bsa = block_sum_t<AT>(acc, sha);
  double bs = double(bsa);
  double tot;
  if (grid_reduce_last1<1>(&bs, partials, ticket, &tot, sh) && threadIdx.x == 0) {
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

// P = R + beta P (the reference's OMPSUMS/OMPMULS pair, CGRAD.f:172-175),
// non-fused mode; vectors are L2-resident between the CG kernels.
template <class XT>
__global__ void __launch_bounds__(kUpdThreads, 2) k_cg_pupdate(size_t n, CgVecs v,
                                                            const KrylovScalars *S) {
  cudaGridDependencySynchronize();
  XT *__restrict__ P = (XT *)v.P0;
  const XT *__restrict__ R = (const XT *)v.R;
  size_t k0 = 0;
  if constexpr (sizeof(XT) == 4) {
    // first float4 requested before the done flag and beta (as k_cg_update)
    const size_t n4 = n / 4, t0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t nt = (size_t)gridDim.x * blockDim.x;
    float4 *__restrict__ P4 = reinterpret_cast<float4 *>(P);
    const float4 *__restrict__ R4 = reinterpret_cast<const float4 *>(R);
    float4 pa = make_float4(0.f, 0.f, 0.f, 0.f), ra = pa;
    if (t0 < n4) {
      pa = P4[t0];
      ra = R4[t0];
    }
    if (*(volatile const int *)&S->done) return;
    const XT beta = XT(S->beta);
    for (size_t k = t0; k < n4; k += nt) {
      float4 p = (k == t0) ? pa : P4[k];
      const float4 r = (k == t0) ? ra : R4[k];
      p.x = fmaf(beta, p.x, r.x);
      p.y = fmaf(beta, p.y, r.y);
      p.z = fmaf(beta, p.z, r.z);
      p.w = fmaf(beta, p.w, r.w);
      P4[k] = p;
    }
    k0 = n4 * 4;
  } else {
    if (*(volatile const int *)&S->done) return;
  }
  const XT beta = XT(S->beta);
  for (size_t k = k0 + (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x)
    P[k] = fma(beta, P[k], R[k]);
}

// ---------------------------------------------------------------------------
// Persistent CG for systems whose matrix sits in L2 (the heat cube, the CEP
// slab): a solve of a few thousand to a few hundred thousand rows spends a
// three-kernel iteration mostly on launch and drain latency, so every
// iteration runs inside one cooperative launch.  Iteration k:
//  1. P_k = R + beta P_{k-1} formed on the fly at every column (and stored
//     by the owner of each row into the other buffer), KP = K P_k and the
//     block partials of P_k.KP;
//  2. after a grid barrier every block sums the partials in block order:
//     alpha = errO / dot; X += alpha P_k, R -= alpha KP and the partials of
//     |R|^2;
//  3. after the second barrier: err, beta = err / errO and CGRAD's stopping
//     tests in k_cg_update's order.
// The arithmetic of each entry is that of k_cg_spmv (fused form) and
// k_cg_update; vectors written inside the launch are read through L2
// (ld.cg), the matrix through the read-only path.
template <int D, class XT, class AT, int VD>
struct GatherDirL2 {
  const XT *__restrict__ R;
  const XT *__restrict__ Pold;
  AT beta;
  __device__ __forceinline__ void get(int col, AT out[D]) const {
#pragma unroll
    for (int c = 0; c < D; c++)
      out[c] = fma(beta, AT(__ldcg(Pold + (size_t)col * VD + c)), AT(__ldcg(R + (size_t)col * VD + c)));
  }
};

constexpr int kCpThreads = 512;
// LN: lanes per scalar row (D = 1 only; 4 when the co-resident grid covers
// every row in one pass, so a row is one round of dependent loads; 1 for
// larger systems, where the passes dominate and fewer registers keep more
// blocks resident)
template <int D, class VT, class XT, int LN = 1>
__global__ void __launch_bounds__(kCpThreads) k_cg_persistent(int nNo,
                                                              const int *__restrict__ rowPtr,
                                                              const int *__restrict__ colPtr,
                                                              const VT *__restrict__ Val, CgVecs v,
                                                              KrylovScalars *S, double *part,
                                                              GridBar *bar, unsigned spin) {
  using AT = typename AccOf<VT>::T;
  constexpr int VD = VStride<D, XT>::v, RPW = 32 / D;
  __shared__ double sh[32];
  __shared__ AT sha[32];
  __shared__ XT shx[32];
  const unsigned nblk = gridDim.x;
  XT *__restrict__ X = (XT *)v.X;
  XT *__restrict__ R = (XT *)v.R;
  XT *__restrict__ KP = (XT *)v.KP;
  double err = S->err, errO = S->errO, alpha = S->alpha, beta = S->beta;
  const double eps = S->eps;
  const int mItr = S->mItr;
  int done = S->done, suc = S->suc, itr = S->itr;
  unsigned epoch = 0;
  bool ok = true;
  const int lane = threadIdx.x & 31, grp = lane / D, r = lane - grp * D;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const size_t n = (size_t)nNo * VD;
  const size_t t0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t nt = (size_t)gridDim.x * blockDim.x;
  while (!done) {
    XT *__restrict__ Pold = (XT *)((itr & 1) ? v.P1 : v.P0);
    XT *__restrict__ Pnew = (XT *)((itr & 1) ? v.P0 : v.P1);
    const AT b = AT(beta);
    GatherDirL2<D, XT, AT, VD> gd{R, Pold, b};
    AT dot = AT(0);
    if constexpr (D == 1 && LN == 4) {
      // scalar rows (~15 entries on tet4 meshes): 4 lanes per row, entries
      // strided by 4 and loaded 4 at a time, so a row is one round of
      // dependent loads; the lane sums by a fixed shuffle tree
      constexpr int RW = 32 / LN, UL = 4;
      const int sub = lane & (LN - 1), rg = lane / LN;
      for (int base = warp * RW; base < nNo; base += nwarps * RW) {
        const int i = base + rg;
        AT y = AT(0);
        if (i < nNo) {
          const int j0 = __ldg(rowPtr + i), j1 = __ldg(rowPtr + i + 1);
          for (int j = j0 + sub; j < j1; j += LN * UL) {
            int cc[UL];
            AT a[UL], x[UL];
#pragma unroll
            for (int u = 0; u < UL; u++) {
              const int jj = j + u * LN;
              cc[u] = jj < j1 ? __ldg(colPtr + jj) : -1;
              a[u] = jj < j1 ? AT(__ldg(Val + jj)) : AT(0);
            }
#pragma unroll
            for (int u = 0; u < UL; u++) {
              AT xv[1] = {AT(0)};
              if (cc[u] >= 0) gd.get(cc[u], xv);
              x[u] = xv[0];
            }
#pragma unroll
            for (int u = 0; u < UL; u++) y = fma(a[u], x[u], y);
          }
        }
        y += __shfl_xor_sync(0xffffffffu, y, 1);
        y += __shfl_xor_sync(0xffffffffu, y, 2);
        if (i < nNo && sub == 0) {
          const size_t k = (size_t)i * VD;
          const AT pn = fma(b, AT(__ldcg(Pold + k)), AT(__ldcg(R + k)));
          __stcg(Pnew + k, XT(pn));
          __stcg(KP + k, XT(y));
          dot = fma(pn, y, dot);
        }
      }
    } else {
      for (int base = warp * RPW; base < nNo; base += nwarps * RPW) {
        const int i = base + grp;
        if (grp < RPW && i < nNo) {
          const size_t k = (size_t)i * VD + r;
          const AT y = spmv_row_comp<D, VT, AT>(i, r, rowPtr, colPtr, Val, gd);
          const AT pn = fma(b, AT(__ldcg(Pold + k)), AT(__ldcg(R + k)));
          __stcg(Pnew + k, XT(pn));
          __stcg(KP + k, XT(y));
          dot = fma(pn, y, dot);
        }
      }
    }
    {
      const double bs = double(block_sum_t<AT>(dot, sha));
      if (threadIdx.x == 0) __stcg(part + blockIdx.x, bs);
    }
    if (!(ok = grid_bar(bar, nblk, epoch, spin))) break;
    const double dsum = sum_partials(part, nblk, sh);
    errO = err;
    alpha = errO / dsum;
    if (!isfinite(alpha)) {
      done = 3;
      break;
    }
    const XT al = XT(alpha);
    XT acc = XT(0);
    for (size_t k = t0; k < n; k += nt) {
      __stcg(X + k, XT(fma(al, __ldcg(Pnew + k), __ldcg(X + k))));
      const XT rr = XT(fma(-al, __ldcg(KP + k), __ldcg(R + k)));
      __stcg(R + k, rr);
      acc = fma(rr, rr, acc);
    }
    {
      const double bs = double(block_sum_t<XT>(acc, shx));
      if (threadIdx.x == 0) __stcg(part + nblk + blockIdx.x, bs);
    }
    if (!(ok = grid_bar(bar, nblk, epoch, spin))) break;
    err = sum_partials(part + nblk, nblk, sh);
    beta = err / errO;
    itr++;
    if (!isfinite(err))
      done = 3;
    else if (itr >= mItr)
      done = 2;
    else if (err < eps) {
      done = 1;
      suc = 1;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    S->err = err;
    S->errO = errO;
    S->alpha = alpha;
    S->beta = beta;
    S->itr = itr;
    S->suc = suc;
    S->done = ok ? done : 4;
  }
}

// R_out = W * X (X in node stride VD, R_out packed)
template <int D, class XT>
__global__ void k_scale_out(int nNo, double *__restrict__ Rout, const XT *__restrict__ X,
                            const double *__restrict__ W) {
  constexpr int VD = VStride<D, XT>::v;
  const size_t n = (size_t)nNo * D;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    const size_t a = k / D, c = k - a * D;
    Rout[k] = W[k] * double(X[a * VD + c]);
  }
}

// ---------------------------------------------------------------------------
// Diagonal preconditioner (PRECONDDIAG, Code/Source/svFSILS/PRECOND.f:50-145)

// 1/sqrt(a) for a > 0 in FP64 by Newton-Raphson on f(y) = 1/y^2 - a
// (y <- y (3 - a y^2) / 2, quadratic convergence) from the FP32 estimate:
// two steps take the ~1e-7 start to the FP64 rounding level with 8 FP64
// operations, where a division and a square root cost several times that on
// GB300's FP64 pipe (~1/74 of the FP32 rate).  Outside the FP32 normal range
// the plain FP64 expression is used.
__device__ __forceinline__ double rsqrt_nr(double a) {
  if (!(a > 1e-36 && a < 1e36)) return 1.0 / sqrt(a);
  double y = (double)rsqrtf((float)a);
  const double h = 0.5 * a;
  y = y * fma(-h * y, y, 1.5);
  y = y * fma(-h * y, y, 1.5);
  return y;
}

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
      // the FP64 drop-in keeps the reference's expression (rounding-
      // sensitive Krylov counts follow it); the mixed path takes the
      // Newton form
      if constexpr (sizeof(VT) == 8)
        w = 1.0 / sqrt(fabs(w));
      else
        w = rsqrt_nr(fabs(w));
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

// The same for scalar rows (D = 1): 4 lanes per row, entries strided by 4
// (a lane per row walked 32 rows at once with uncoalesced loads: 4x slower)
template <class VT, class WT>
__global__ void __launch_bounds__(kThreads) k_scale_val1(int nNo, const int *__restrict__ rowPtr,
                                                         const int *__restrict__ colPtr,
                                                         VT *__restrict__ Val,
                                                         const WT *__restrict__ W) {
  const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t nt = (size_t)gridDim.x * blockDim.x;
  for (size_t t = g; t < (size_t)nNo * 4; t += nt) {
    const int i = (int)(t >> 2), l = (int)(t & 3);
    const WT wr = W[i];
    const int re = rowPtr[i + 1];
    for (int j = rowPtr[i] + l; j < re; j += 4) Val[j] = VT((WT(Val[j]) * wr) * W[colPtr[j]]);
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
  if (D == 1) {
    const int nb = blocks_for((size_t)nNo * 4, num_sms() * 8);
    if (sizeof(VT) == 4)
      k_scale_val1<VT, float><<<nb, kThreads, 0, st>>>(nNo, lhs->d_rowPtr.as<int>(),
                                                       lhs->d_colPtr.as<int>(), Val, Wf);
    else
      k_scale_val1<VT, double><<<nb, kThreads, 0, st>>>(nNo, lhs->d_rowPtr.as<int>(),
                                                        lhs->d_colPtr.as<int>(), Val, W);
  } else if (sizeof(VT) == 4) {
    k_scale_val<D, VT, float><<<lhs->grid, kThreads, 0, st>>>(
        nNo, lhs->d_rowPtr.as<int>(), lhs->d_colPtr.as<int>(), Val, Wf);
  } else {
    k_scale_val<D, VT, double><<<lhs->grid, kThreads, 0, st>>>(
        nNo, lhs->d_rowPtr.as<int>(), lhs->d_colPtr.as<int>(), Val, W);
  }
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
static int resident_grid(K kernel, int cap, int threads = kThreads) {
  int nb = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, threads, 0);
  if (nb < 1) nb = 1;
  int g = nb * num_sms();
  return g < cap ? g : cap;
}

constexpr int kTmaWarps = 16;

// Tile geometry of the staged SpMV for block size D and value type VT,
// from the host copy of rowPtr; cached per lhs.  Returns false when the
// staged kernel does not apply (tiles too large for shared memory).
template <int D, class VT>
static bool tma_setup(gsls_lhs *lhs, TmaTiles &tt, int &smem, int &grid) {
  Workspace &ws = lhs->ws;
  const int key = D * 16 + (int)sizeof(VT);
  if (ws.tma_key == key) {
    tt = *reinterpret_cast<TmaTiles *>(&ws.tma_info);
    smem = ws.tma_smem;
    grid = ws.tma_grid;
    return ws.tma_ok;
  }
  constexpr int DD = D * D, A = 16 / sizeof(VT);
  const int rows = kTmaWarps * ((32 / D) / 2);  // SP = 2 lane groups per row
  const int nNo = lhs->nNo;
  const std::vector<int> &rp = lhs->h_rowPtr;
  long long vmax = 0, cmax = 0;
  const int ntiles = (nNo + rows - 1) / rows;
  for (int t = 0; t < ntiles; t++) {
    const int r0 = t * rows, r1 = std::min(r0 + rows, nNo);
    const long long e0 = (long long)rp[r0] * DD, e1 = (long long)rp[r1] * DD;
    const long long e0a = e0 & ~(long long)(A - 1), e1a = (e1 + A - 1) & ~(long long)(A - 1);
    const long long c0a = rp[r0] & ~3, c1a = (rp[r1] + 3) & ~3;
    vmax = std::max(vmax, (e1a - e0a) * (long long)sizeof(VT));
    cmax = std::max(cmax, (c1a - c0a) * 4LL);
  }
  tt.ntiles = ntiles;
  tt.tile_rows = rows;
  tt.val_buf = (int)((vmax + 127) & ~127LL);
  tt.col_buf = (int)((cmax + 127) & ~127LL);
  tt.err = ws.err.as<int>();
  smem = 2 * (tt.val_buf + tt.col_buf);
  bool ok = smem <= 200 * 1024;
  grid = 0;
  if (ok) {
    auto kern = k_cg_spmv_tma<D, VT, VT, kTmaWarps, true>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_cg_spmv_tma<D, VT, VT, kTmaWarps, false>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, kTmaWarps * 32, smem);
    if (nb < 1) ok = false;
    grid = std::min(ntiles, nb * num_sms());
    grid = std::min(grid, lhs->grid);
  }
  ws.tma_key = key;
  *reinterpret_cast<TmaTiles *>(&ws.tma_info) = tt;
  ws.tma_smem = smem;
  ws.tma_grid = grid;
  ws.tma_ok = ok;
  return ok;
}

// Programmatic dependent launch of the CG batch (default on; GSLS_PDL=0
// serialises the launches plainly).
static bool use_pdl() {
  static const bool on = [] {
    const char *e = getenv("GSLS_PDL");
    return !(e && strcmp(e, "0") == 0);
  }();
  return on;
}

// Sliced copy of the matrix (structure per lhs and block size, built on the
// host once): rows sorted by decreasing length within windows of 32 slices.
template <int D>
static int sell_setup(gsls_lhs *lhs) {
  Workspace &ws = lhs->ws;
  if (ws.sell_D == D) return GSLS_OK;
  constexpr int RPW = 32 / D, WIN = 32 * RPW;
  const int nNo = lhs->nNo;
  const std::vector<int> &rp = lhs->h_rowPtr, &cp = lhs->h_colPtr;
  const int nS = (nNo + RPW - 1) / RPW;
  std::vector<int> slotRow((size_t)nS * RPW, -1), idx;
  for (int w0 = 0; w0 < nNo; w0 += WIN) {
    const int w1 = std::min(nNo, w0 + WIN);
    idx.resize(w1 - w0);
    for (int i = w0; i < w1; i++) idx[i - w0] = i;
    std::stable_sort(idx.begin(), idx.end(),
                     [&](int a, int b) { return rp[a + 1] - rp[a] > rp[b + 1] - rp[b]; });
    for (int k = 0; k < w1 - w0; k++) slotRow[(size_t)w0 + k] = idx[k];
  }
  std::vector<int> off((size_t)nS + 1, 0);
  for (int s = 0; s < nS; s++) {
    int m = 0;
    for (int g = 0; g < RPW; g++) {
      const int i = slotRow[(size_t)s * RPW + g];
      if (i >= 0) m = std::max(m, rp[i + 1] - rp[i]);
    }
    if ((long long)off[s] + m > (1LL << 31) / RPW - 1) {
      set_error("sliced matrix copy: too many blocks");
      return GSLS_ERR_UNSUPPORTED;
    }
    off[s + 1] = off[s] + m;
  }
  const long long steps = off[nS];
  std::vector<int> scol((size_t)steps * RPW, 0), pos((size_t)lhs->nnz, 0);
  for (int s = 0; s < nS; s++)
    for (int g = 0; g < RPW; g++) {
      const int i = slotRow[(size_t)s * RPW + g];
      if (i < 0) continue;
      const int len = rp[i + 1] - rp[i];
      for (int t = 0; t < off[s + 1] - off[s]; t++) {
        const int P = (off[s] + t) * RPW + g;
        if (t < len) {
          scol[P] = cp[rp[i] + t];
          pos[rp[i] + t] = P;
        } else {
          scol[P] = i;  // zero block on the row's own column
        }
      }
    }
  GSLS_TRY(ws.sell_off.alloc(sizeof(int) * off.size()));
  GSLS_TRY(ws.sell_row.alloc(sizeof(int) * slotRow.size()));
  GSLS_TRY(ws.sell_col.alloc(sizeof(int) * scol.size()));
  GSLS_TRY(ws.sell_pos.alloc(sizeof(int) * pos.size()));
  cudaStream_t st = lhs->stream;
  GSLS_CUDA(cudaMemcpyAsync(ws.sell_off.p, off.data(), sizeof(int) * off.size(),
                            cudaMemcpyHostToDevice, st));
  GSLS_CUDA(cudaMemcpyAsync(ws.sell_row.p, slotRow.data(), sizeof(int) * slotRow.size(),
                            cudaMemcpyHostToDevice, st));
  GSLS_CUDA(cudaMemcpyAsync(ws.sell_col.p, scol.data(), sizeof(int) * scol.size(),
                            cudaMemcpyHostToDevice, st));
  GSLS_CUDA(cudaMemcpyAsync(ws.sell_pos.p, pos.data(), sizeof(int) * pos.size(),
                            cudaMemcpyHostToDevice, st));
  GSLS_CUDA(cudaStreamSynchronize(st));  // host vectors go out of scope
  ws.sell_D = D;
  ws.sell_nS = nS;
  ws.sell_steps = steps;
  ws.sell_vkey = 0;
  return GSLS_OK;
}

// Copy the (preconditioned) values into the sliced layout; padding blocks
// are zeroed when the buffer is (re)laid out and never written after.
template <int D, class VT>
static int sell_pack(gsls_lhs *lhs, const VT *Val, SellArgs &sa) {
  Workspace &ws = lhs->ws;
  GSLS_TRY(sell_setup<D>(lhs));
  constexpr int RPW = 32 / D, DD = D * D;
  const size_t vbytes = sizeof(VT) * (size_t)ws.sell_steps * RPW * DD;
  const int vkey = D * 16 + (int)sizeof(VT);
  cudaStream_t st = lhs->stream;
  if (ws.sell_vkey != vkey) {
    GSLS_TRY(ws.sell_val.alloc(vbytes));
    GSLS_CUDA(cudaMemsetAsync(ws.sell_val.p, 0, vbytes, st));
    ws.sell_vkey = vkey;
  }
  const size_t n = (size_t)lhs->nnz * DD;
  k_sell_pack<D, VT><<<lhs->grid, kThreads, 0, st>>>(n, ws.sell_pos.as<int>(), Val,
                                                     ws.sell_val.as<VT>());
  GSLS_CHECK_LAUNCH();
  sa.nS = ws.sell_nS;
  sa.off = ws.sell_off.as<int>();
  sa.slotRow = ws.sell_row.as<int>();
  sa.scol = ws.sell_col.as<int>();
  sa.sval = ws.sell_val.p;
  return GSLS_OK;
}

template <int D, class VT, class XT, bool FUSED>
static int cg_enqueue(gsls_lhs *lhs, const VT *Val, const CgVecs &v, int n_iter, bool prof,
                      int ev_base, const TmaTiles *tt = nullptr, int tma_smem = 0,
                      int tma_grid = 0, const SellArgs *sa = nullptr) {
  cudaStream_t st = lhs->stream;
  Workspace &ws = lhs->ws;
  const int nNo = lhs->nNo;
  static const int Gs = resident_grid(k_cg_spmv<D, VT, XT, FUSED>, 1 << 30);
  // sliced SpMV: 8 steps per group in FP32 (64 registers, 4 blocks per SM),
  // 4 in FP64
  constexpr int SU = sizeof(VT) == 4 ? 8 : 4;
  static const int Gsl = resident_grid(k_cg_spmv_sell<D, VT, XT, SU>, 1 << 30);
  static const int Gu = resident_grid(k_cg_update<XT, FUSED>, 1 << 30, kUpdThreads);
  static const int Gp = resident_grid(k_cg_pupdate<XT>, 1 << 30, kUpdThreads);
  const int G1 = Gs < lhs->grid ? Gs : lhs->grid, G2 = Gu < lhs->grid ? Gu : lhs->grid;
  const int G3 = Gp < lhs->grid ? Gp : lhs->grid;
  const size_t nv = (size_t)nNo * VStride<D, XT>::v;
  KrylovScalars *S = ws.scal.as<KrylovScalars>();
  double *part = ws.partials.as<double>();
  unsigned *tk = ws.ticket.as<unsigned>();
  const int zz = zigzag_on();
  for (int b = 0; b < n_iter; b++) {
    if (prof) cudaEventRecord(prof_event(ev_base + 4 * b), st);
    // programmatic dependent launch: each kernel's blocks may be scheduled
    // while its predecessor drains; they wait (cudaGridDependencySynchronize)
    // for its completion before reading anything it wrote
    cudaLaunchAttribute pdl[1];
    pdl[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    pdl[0].val.programmaticStreamSerializationAllowed = (prof || !use_pdl()) ? 0 : 1;
    cudaLaunchConfig_t cfg = {};
    cfg.stream = st;
    cfg.attrs = pdl;
    cfg.numAttrs = 1;
    if (tt) {
      k_cg_spmv_tma<D, VT, XT, kTmaWarps, FUSED><<<tma_grid, kTmaWarps * 32, tma_smem, st>>>(
          nNo, lhs->d_rowPtr.as<int>(), lhs->d_colPtr.as<int>(), Val, v, S, part, tk, *tt);
    } else if (sa && !FUSED) {
      cfg.gridDim = dim3(Gsl < lhs->grid ? Gsl : lhs->grid);
      cfg.blockDim = dim3(kThreads);
      GSLS_CUDA(
          cudaLaunchKernelEx(&cfg, k_cg_spmv_sell<D, VT, XT, SU>, *sa, v, S, part, tk, zz));
    } else {
      cfg.gridDim = dim3(G1);
      cfg.blockDim = dim3(kThreads);
      GSLS_CUDA(cudaLaunchKernelEx(&cfg, k_cg_spmv<D, VT, XT, FUSED>, nNo,
                                   (const int *)lhs->d_rowPtr.as<int>(),
                                   (const int *)lhs->d_colPtr.as<int>(), Val, v, S, part, tk,
                                   zz));
    }
    GSLS_CHECK_LAUNCH();
    if (prof) cudaEventRecord(prof_event(ev_base + 4 * b + 1), st);
    cfg.gridDim = dim3(G2);
    cfg.blockDim = dim3(kUpdThreads);
    GSLS_CUDA(cudaLaunchKernelEx(&cfg, k_cg_update<XT, FUSED>, nv, v, S, part, tk));
    GSLS_CHECK_LAUNCH();
    if (prof) cudaEventRecord(prof_event(ev_base + 4 * b + 2), st);
    if (!FUSED) {
      cfg.gridDim = dim3(G3);
      GSLS_CUDA(cudaLaunchKernelEx(&cfg, k_cg_pupdate<XT>, nv, v, (const KrylovScalars *)S));
      GSLS_CHECK_LAUNCH();
    }
    if (prof) cudaEventRecord(prof_event(ev_base + 4 * b + 3), st);
  }
  return GSLS_OK;
}

// CG on the preconditioned system; R (double, device) in: rhs, out: W*X.
template <int D, class VT, class XT, bool FUSED>
static int cg_t(gsls_lhs *lhs, gsls_sub_ls *ls, const VT *Val, double *R, const double *Wc,
                bool val_padded) {
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
  // Persistent CG (one cooperative launch per solve) when the matrix fits in
  // L2 with room to spare; GSLS_CG_PERSISTENT=0 never, =1 always
  static const int cp_mode = [] {
    const char *e = getenv("GSLS_CG_PERSISTENT");
    return e ? (strcmp(e, "0") == 0 ? 0 : 1) : -1;
  }();
  static const bool env_tma = [] {
    const char *e = getenv("GSLS_SPMV");
    return e && strcmp(e, "tma") == 0;
  }();
  const size_t vbytes = (size_t)lhs->nnz * D * D * sizeof(VT);
  const bool persistent =
      !env_tma && (cp_mode == 1 || (cp_mode == -1 && vbytes <= ((size_t)64 << 20)));
  if (persistent)
    k_cg_init<D, XT, true><<<G, kThreads, 0, st>>>(nNo, R, v, S, ls->absTol, ls->relTol,
                                                    ls->mItr, part, tk);
  else
    k_cg_init<D, XT, FUSED><<<G, kThreads, 0, st>>>(nNo, R, v, S, ls->absTol, ls->relTol,
                                                     ls->mItr, part, tk);
  GSLS_CHECK_LAUNCH();
  if (persistent) {
    // co-resident grid: enough warps for one pass over the rows, at most
    // what the SMs hold at once
    static const int per_sm = [] {
      int nb = 0;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_cg_persistent<D, VT, XT>, kCpThreads,
                                                    0);
      return nb;
    }();
    static const int per_sm4 = [] {
      int nb = 0;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_cg_persistent<D, VT, XT, 4>,
                                                    kCpThreads, 0);
      return nb;
    }();
    constexpr int WPB = kCpThreads / 32;
    // scalar rows: 4 lanes per row when one pass covers them all
    const bool four = D == 1 && (long long)per_sm4 * num_sms() * WPB * 8 >= nNo;
    const int RPW = four ? 8 : 32 / D;  // rows per warp
    const long long warps = ((long long)nNo + RPW - 1) / RPW;
    long long gp = (warps + WPB - 1) / WPB;
    const long long gmax = (long long)(four ? per_sm4 : per_sm) * num_sms();
    if (gp > gmax) gp = gmax;
    if (gp < 1) gp = 1;
    if ((four ? per_sm4 : per_sm) < 1) {
      set_error("CG: the persistent kernel does not fit on an SM");
      return GSLS_ERR_CUDA;
    }
    GSLS_TRY(ws.cgbar.alloc(sizeof(GridBar)));
    GSLS_CUDA(cudaMemsetAsync(ws.cgbar.p, 0, sizeof(GridBar), st));
    int nNo_ = nNo;
    const int *rp = lhs->d_rowPtr.as<int>(), *cp = lhs->d_colPtr.as<int>();
    GridBar *gb = ws.cgbar.as<GridBar>();
    unsigned spin = wait_limit();
    void *args[] = {&nNo_, (void *)&rp, (void *)&cp, (void *)&Val, &v, &S, &part, &gb, &spin};
    const bool prof_p = prof_on();
    if (prof_p) cudaEventRecord(prof_event(0), st);
    const void *kfn = four ? (const void *)k_cg_persistent<D, VT, XT, 4>
                           : (const void *)k_cg_persistent<D, VT, XT>;
    GSLS_CUDA(cudaLaunchCooperativeKernel(kfn, dim3((int)gp), dim3(kCpThreads), args, 0, st));
    GSLS_CHECK_LAUNCH();
    if (prof_p) cudaEventRecord(prof_event(1), st);
  }
  GSLS_TRY(wait_scalars(lhs));
  if (persistent && prof_on()) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, prof_event(0), prof_event(1));
    prof_add("cg_persistent", ws.h_scal->itr, ms);
  }
  const bool prof = prof_on() && !persistent;
  const int B = nv < (1u << 20) ? 8 : 16;
  // TMA-staged SpMV for FP32 values in a buffer with copy slack
  TmaTiles tt{};
  int tsmem = 0, tgrid = 0;
  static const bool want_tma = [] {
    const char *e = getenv("GSLS_SPMV");
    return e && strcmp(e, "tma") == 0;
  }();
  const bool use_tma =
      want_tma && val_padded && sizeof(VT) == 4 && tma_setup<D, VT>(lhs, tt, tsmem, tgrid);
  const TmaTiles *ttp = use_tma ? &tt : nullptr;
  if (use_tma) GSLS_CUDA(cudaMemsetAsync(ws.err.p, 0, sizeof(int), st));
  // Sliced SpMV: a solve that is still running after its first batch packs
  // the matrix into the sliced layout (one pass over Val) and continues on
  // it; short solves (a few iterations) never pay for the copy.
  // GSLS_SPMV=csr keeps the CSR kernel throughout.
  static const bool want_sell = [] {
    const char *e = getenv("GSLS_SPMV");
    return !(e && (strcmp(e, "csr") == 0 || strcmp(e, "tma") == 0));
  }();
  const bool sell_ok = want_sell && !FUSED && !use_tma;
  SellArgs sa{};
  bool sell_on = false;
  // First batch: the smallest power of two that holds the previous solve's
  // iteration count on this lhs (2..B), so that the short solves of a
  // Newton sequence (CEP, heat: 3-30 iterations) do not launch a full batch
  // of iterations that only test the done flag; later batches (sliced copy)
  // take B.  Powers of two keep the cached graph of the first batch stable.
  int B1 = B;
  if (sell_ok && ws.cg_last_itr > 0) {
    B1 = 2;
    while (B1 < ws.cg_last_itr && B1 < B) B1 *= 2;
  }
  // CUDA graph of a batch of iterations, cached per (D, types, Val,
  // workspace, layout, batch); one slot for the CSR batch and one for the
  // sliced batch
  auto graph_for = [&](bool sl, int nb, cudaGraphExec_t *&ge) -> int {
    cudaGraphExec_t &gx = sl ? ws.cg_graph_s : ws.cg_graph;
    GraphKey &gk = sl ? ws.cg_key_s : ws.cg_key;
    GraphKey key{D,  (int)sizeof(VT), (int)sizeof(XT), (const void *)Val, v.X, nb, nNo, use_tma,
                 FUSED, ws.partials.p, ws.scal.p, ws.Wf.p, sl ? sa.sval : nullptr};
    ge = &gx;
    if (gx && gk == key) return GSLS_OK;
    if (gx) {
      cudaGraphExecDestroy(gx);
      gx = nullptr;
    }
    cudaGraph_t g;
    GSLS_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    int rc = cg_enqueue<D, VT, XT, FUSED>(lhs, Val, v, nb, false, 0, ttp, tsmem, tgrid,
                                          sl ? &sa : nullptr);
    cudaError_t e = cudaStreamEndCapture(st, &g);
    if (rc != GSLS_OK) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture", __FILE__, __LINE__);
    GSLS_CUDA(cudaGraphInstantiate(&gx, g, 0));
    cudaGraphDestroy(g);
    gk = key;
    return GSLS_OK;
  };
  int nbatch = 0;
  while (!persistent && ws.h_scal->done == 0) {
    const int itr_before = ws.h_scal->itr;
    if (sell_ok && !sell_on && nbatch >= 1) {
      GSLS_TRY(sell_pack<D, VT>(lhs, Val, sa));
      count_launch();
      sell_on = true;
    }
    const int nb = nbatch == 0 ? B1 : B;
    nbatch++;
    if (prof) {
      GSLS_TRY(cg_enqueue<D, VT, XT, FUSED>(lhs, Val, v, nb, true, 0, ttp, tsmem, tgrid,
                                            sell_on ? &sa : nullptr));
    } else {
      cudaGraphExec_t *ge = nullptr;
      GSLS_TRY(graph_for(sell_on, nb, ge));
      GSLS_CUDA(cudaGraphLaunch(*ge, st));
      count_launch_n((FUSED ? 2 : 3) * nb - 1);
    }
    GSLS_TRY(wait_scalars(lhs));
    if (prof) {
      // only the launches that did work (one per completed iteration)
      const int worked = ws.h_scal->itr - itr_before;
      double ms = 0.0, mu = 0.0, mp = 0.0;
      for (int b = 0; b < worked && b < nb; b++) {
        float t = 0.f;
        cudaEventElapsedTime(&t, prof_event(4 * b), prof_event(4 * b + 1));
        ms += t;
        cudaEventElapsedTime(&t, prof_event(4 * b + 1), prof_event(4 * b + 2));
        mu += t;
        cudaEventElapsedTime(&t, prof_event(4 * b + 2), prof_event(4 * b + 3));
        mp += t;
      }
      prof_add("cg_spmv", worked, ms);
      prof_add("cg_update", worked, mu);
      prof_add("cg_pupdate", worked, mp);
    }
  }
  k_scale_out<D, XT><<<G, kThreads, 0, st>>>(nNo, R, (const XT *)v.X, Wc);
  GSLS_CHECK_LAUNCH();
  GSLS_CUDA(cudaStreamSynchronize(st));
  const KrylovScalars &h = *ws.h_scal;
  ws.cg_last_itr = h.itr;
  ls->iNorm = h.iNorm;
  ls->itr = h.itr;
  ls->suc = h.suc;
  ls->fNorm = sqrt(h.err);
  ls->dB = (h.errO < 2.220446049250313e-16) ? 0.0 : 5.0 * log(h.err / h.errO);
  ls->callD = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (use_tma) {
    int herr = 0;
    GSLS_CUDA(cudaMemcpy(&herr, ws.err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (herr) {
      set_error("CG: a staged copy did not complete (bounded mbarrier wait expired)");
      return GSLS_ERR_CUDA;
    }
  }
  if (h.done == 4) {
    set_error("CG: grid barrier of the persistent CG timed out");
    return GSLS_ERR_CUDA;
  }
  if (h.done == 3) {
    set_error("CG: NaN/Inf or breakdown in Krylov scalars");
    return GSLS_ERR_NAN;
  }
  return GSLS_OK;
}

template <int D, class VT, class XT>
static int solve_t(gsls_lhs *lhs, gsls_ls *ls, double *dRi, VT *Val, int prec, bool padded,
                   bool prescaled) {
  Workspace &ws = lhs->ws;
  double *W = ws.W.as<double>();
  if (prescaled && prec == GSLS_PRECOND_FSILS) {
    // R = W R with the W that scaled Val (the R update of k_diag_w)
    const size_t n = (size_t)lhs->nNo * D;
    k_vec_mul<<<blocks_for(n, num_sms() * 8), kThreads, 0, lhs->stream>>>(n, dRi, W);
    GSLS_CHECK_LAUNCH();
  } else if (prec == GSLS_PRECOND_FSILS) {
    GSLS_TRY(precond_diag_t<D, VT>(lhs, Val, dRi, W));
    ws.pre_serial++;
  } else if (prec == GSLS_PRECOND_RCS) {
    GSLS_TRY(precond_rcs_run(lhs, D, sizeof(VT) == 4, Val, dRi, W));
    ws.pre_serial++;
  } else {
    set_error("This linear solver and preconditioner combination is not supported.");
    return GSLS_ERR_ARG;
  }
  // coupled faces: ADDBCMUL enters GMRES and NS (CGRADS/V do not call it)
  GSLS_TRY(cpl_prepare(lhs, D, W, prec));
  switch (ls->LS_type) {
    case GSLS_LS_TYPE_CG:
    {
      static const bool fused = [] {
        const char *e = getenv("GSLS_CG");
        return e && strcmp(e, "fused") == 0;
      }();
      return fused ? cg_t<D, VT, XT, true>(lhs, &ls->RI, Val, dRi, W, padded)
                   : cg_t<D, VT, XT, false>(lhs, &ls->RI, Val, dRi, W, padded);
    }
    case GSLS_LS_TYPE_GMRES:
      return gmres_run(lhs, &ls->RI, D, sizeof(VT) == 4, Val, dRi, W);
    case GSLS_LS_TYPE_NS:
      return ns_run(lhs, ls, D, sizeof(VT) == 4, Val, dRi, W);
    case GSLS_LS_TYPE_BICGS:
      return bicgs_run(lhs, &ls->RI, D, sizeof(VT) == 4, Val, dRi, W);
    default:
      set_error("LS_type not defined");
      return GSLS_ERR_ARG;
  }
}

int solve_dev(gsls_lhs *lhs, gsls_ls *ls, int dof, double *dRi, void *dVal, int val_prec,
              int prec, bool padded, bool prescaled) {
  GSLS_TRY(lhs_prepare_ws(lhs, dof));
  const unsigned mser = lhs->ws.mask_serial;
  GSLS_TRY(build_dir_mask(lhs, dof));
  if (prescaled && lhs->ws.mask_serial != mser) {
    set_error("solve: the Dirichlet mask changed under a preconditioned matrix");
    return GSLS_ERR_ARG;
  }
  const bool mixed = (val_prec == GSLS_PREC_MIXED);
#define GSLS_SOLVE_CASE(DV)                                                                   \
  case DV:                                                                                    \
    return mixed ? solve_t<DV, float, float>(lhs, ls, dRi, (float *)dVal, prec, padded,       \
                                             prescaled)                                       \
                 : solve_t<DV, double, double>(lhs, ls, dRi, (double *)dVal, prec, padded,    \
                                               prescaled);
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
  return solve_dev(lhs, ls, dof, dRi, dVal, val_prec, prec, false);
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
  GSLS_TRY(lhs->ws.io2.alloc(sizeof(double) * nval + 64));
  cudaStream_t st = lhs->stream;
  GSLS_CUDA(cudaMemcpyAsync(lhs->ws.io.p, Ri, sizeof(double) * nr, cudaMemcpyHostToDevice, st));
  GSLS_CUDA(cudaMemcpyAsync(lhs->ws.io2.p, Val, sizeof(double) * nval, cudaMemcpyHostToDevice, st));
  int rc = solve_dev(lhs, ls, dof, lhs->ws.io.as<double>(), lhs->ws.io2.p, GSLS_PREC_FP64, prec,
                     true);
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
