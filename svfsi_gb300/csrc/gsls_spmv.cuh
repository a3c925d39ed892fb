// Block-CSR SpMV core shared by the Krylov kernels (FSILS_SPARMULVV,
// Code/Source/svFSILS/SPARMUL.f:51-133: KU(:,i) = sum_j K(:,:,j) U(:,col(j)),
// blocks stored row-major).
//
// Mapping: D lanes own one block row; lane r accumulates output component r
// over the row's blocks, reading row r of each block (D contiguous values)
// and the D components of the gathered vector.  One FMA per matrix value,
// no shuffles and no selects -- on GB300 every FP64 warp instruction costs
// ~64 SMSP cycles, so the FP64 path must not spend anything beyond the DFMA
// per value, and the FP32 path must not touch the FP64 pipe per value.
// 32/D block rows per warp (lanes >= D*(32/D) idle for D = 3).
#pragma once

#include "gsls_internal.cuh"

namespace gsls {

template <class VT> struct AccOf { using T = double; };
template <> struct AccOf<float> { using T = float; };

template <int D, class VT, class AT>
__device__ __forceinline__ void load_row_seg(const VT *__restrict__ p, AT out[D]) {
#pragma unroll
  for (int c = 0; c < D; c++) out[c] = AT(__ldg(p + c));
}
template <>
__device__ __forceinline__ void load_row_seg<4, float, float>(const float *__restrict__ p,
                                                              float out[4]) {
  const float4 v = __ldg(reinterpret_cast<const float4 *>(p));
  out[0] = v.x;
  out[1] = v.y;
  out[2] = v.z;
  out[3] = v.w;
}
template <>
__device__ __forceinline__ void load_row_seg<2, double, double>(const double *__restrict__ p,
                                                                double out[2]) {
  const double2 v = __ldg(reinterpret_cast<const double2 *>(p));
  out[0] = v.x;
  out[1] = v.y;
}
template <>
__device__ __forceinline__ void load_row_seg<2, float, float>(const float *__restrict__ p,
                                                              float out[2]) {
  const float2 v = __ldg(reinterpret_cast<const float2 *>(p));
  out[0] = v.x;
  out[1] = v.y;
}

// Node stride of the Krylov work vectors: FP32 3-vectors are padded to 4
// floats so that one 16-byte load gathers a node (the gather, not the matrix
// stream, dominates the L1 sector lookups of the block SpMV).
template <int D, class XT> struct VStride { static constexpr int v = D; };
template <> struct VStride<3, float> { static constexpr int v = 4; };

template <int D, int VD, class XT, class AT>
__device__ __forceinline__ void load_node(const XT *__restrict__ p, AT out[D]) {
  if constexpr (VD == 4 && D == 3 && sizeof(XT) == 4) {
    const float4 v = __ldg(reinterpret_cast<const float4 *>(p));
    out[0] = v.x;
    out[1] = v.y;
    out[2] = v.z;
  } else {
    load_row_seg<D, XT, AT>(p, out);
  }
}

// Gathered vector access: either x itself, or x = R + beta*Pold computed on
// the fly (CG direction update fused into the SpMV).
template <int D, class XT, class AT, int VD = D>
struct GatherX {
  const XT *__restrict__ x;
  __device__ __forceinline__ void get(int col, AT out[D]) const {
    load_node<D, VD, XT, AT>(x + (size_t)col * VD, out);
  }
};
template <int D, class XT, class AT, int VD = D>
struct GatherDir {
  const XT *__restrict__ R;
  const XT *__restrict__ Pold;
  AT beta;
  __device__ __forceinline__ void get(int col, AT out[D]) const {
    AT r[D], p[D];
    load_node<D, VD, XT, AT>(R + (size_t)col * VD, r);
    load_node<D, VD, XT, AT>(Pold + (size_t)col * VD, p);
#pragma unroll
    for (int c = 0; c < D; c++) out[c] = r[c] + beta * p[c];
  }
};

// y_r of block row i for lane component r
template <int D, class VT, class AT, class G>
__device__ __forceinline__ AT spmv_row_comp(int i, int r, const int *__restrict__ rowPtr,
                                            const int *__restrict__ colPtr,
                                            const VT *__restrict__ Val, const G &g) {
  constexpr int DD = D * D;
  const int rs = __ldg(rowPtr + i), re = __ldg(rowPtr + i + 1);
  const VT *__restrict__ v = Val + (size_t)rs * DD + r * D;
  AT acc0 = AT(0), acc1 = AT(0);
  // U blocks per step: column loads, value loads and gathers of all U
  // blocks are issued before the first FMA
  constexpr int U = 4;
  for (int j = rs; j < re; j += U) {
    int cc[U];
#pragma unroll
    for (int u = 0; u < U; u++) cc[u] = (j + u < re) ? __ldg(colPtr + j + u) : -1;
    AT a[U][D], xg[U][D];
#pragma unroll
    for (int u = 0; u < U; u++) {
      if (cc[u] >= 0) {
        load_row_seg<D, VT, AT>(v + (size_t)(j + u - rs) * DD, a[u]);
        g.get(cc[u], xg[u]);
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
  return acc0 + acc1;
}

// plain y = K x (grid-stride over groups of 32/D block rows per warp)
template <int D, class VT, class XT, class YT>
__global__ void __launch_bounds__(256) k_spmv(int nNo, const int *__restrict__ rowPtr,
                                              const int *__restrict__ colPtr,
                                              const VT *__restrict__ Val,
                                              const XT *__restrict__ x, YT *__restrict__ y) {
  using AT = typename AccOf<VT>::T;
  constexpr int RPW = 32 / D;
  const int lane = threadIdx.x & 31, grp = lane / D, r = lane - grp * D;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  GatherX<D, XT, AT> g{x};
  for (int base = warp * RPW; base < nNo; base += nwarps * RPW) {
    const int i = base + grp;
    if (grp < RPW && i < nNo)
      y[(size_t)i * D + r] = YT(spmv_row_comp<D, VT, AT>(i, r, rowPtr, colPtr, Val, g));
  }
}

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block sum in the accumulation type; result valid in thread 0.
template <class AT>
__device__ __forceinline__ AT block_sum_t(AT v, AT *sh /*[32]*/) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if constexpr (sizeof(AT) == 4)
    v = warp_sum_f(v);
  else
    v = warp_sum(v);
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  const int nw = blockDim.x >> 5;
  v = (threadIdx.x < nw) ? sh[threadIdx.x] : AT(0);
  if (wid == 0) {
    if constexpr (sizeof(AT) == 4)
      v = warp_sum_f(v);
    else
      v = warp_sum(v);
  }
  return v;
}

}  // namespace gsls
