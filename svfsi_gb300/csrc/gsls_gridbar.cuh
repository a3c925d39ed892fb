// Grid-wide barrier and reductions of the persistent (cooperative) Krylov
// kernels.  Every wait is bounded: after kBarSpin polls (each a 20 ns sleep
// plus an L2 round trip: seconds at most) the waiting block sets the error
// word and returns false, and every other block leaves at its next poll, so
// a launch that lost a block ends with an error status instead of hanging.
#pragma once

#include "gsls_internal.cuh"

namespace gsls {

struct GridBar {
  unsigned count;  // arrivals, monotonic within one launch (zeroed before it)
  unsigned pad;
  int err, pad2;
};
constexpr unsigned kBarSpin = 1u << 24;

// Barrier number `epoch` (1, 2, ...) of the launch: every block adds one
// arrival and waits until all nblk * epoch arrivals are in; no reset, so
// the last arriver has nothing more to publish.
__device__ __forceinline__ bool grid_bar(GridBar *b, unsigned nblk, unsigned &epoch) {
  __shared__ int s_ok;
  __syncthreads();
  epoch += 1;
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned target = epoch * nblk;
    __threadfence();
    atomicAdd(&b->count, 1u);
    unsigned it = 0;
    while (*(volatile unsigned *)&b->count < target) {
      if (*(volatile int *)&b->err) {
        ok = 0;
        break;
      }
      if (++it > kBarSpin) {
        atomicExch(&b->err, 1);
        ok = 0;
        break;
      }
      __nanosleep(20);
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// sum of nblk block partials in block order, broadcast to the block
__device__ __forceinline__ double sum_partials(const double *part, unsigned nblk, double *sh) {
  double v = 0.0;
  for (unsigned k = threadIdx.x; k < nblk; k += blockDim.x) v += __ldcg(part + k);
  v = block_sum(v, sh);
  __shared__ double s_tot;
  if (threadIdx.x == 0) s_tot = v;
  __syncthreads();
  const double r = s_tot;
  __syncthreads();
  return r;
}

}  // namespace gsls
