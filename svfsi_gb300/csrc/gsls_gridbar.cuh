// Grid-wide barrier and reductions of the persistent (cooperative) Krylov
// kernels.  Every wait is bounded: after `limit` polls (kBarSpinDefault
// unless set, each a 20 ns sleep plus an L2 round trip: seconds at most; the
// host can lower it with gsls_set_wait_limit) the waiting block sets the
// error word and returns false, and every other block leaves at its next
// poll or at its own limit, so a launch that lost a block ends with an
// error status instead of hanging.
#pragma once

#include "gsls_internal.cuh"

namespace gsls {

struct GridBar {
  unsigned count;  // arrivals, monotonic within one launch (zeroed before it)
  unsigned pad;
  int err, pad2;
};

// Barrier number `epoch` (1, 2, ...) of the launch: every block adds one
// arrival (release at GPU scope) and thread 0 polls the count with acquire
// loads until all nblk * epoch arrivals are in, then releases its block
// with a block barrier; no reset, so the last arriver has nothing more to
// publish.  The error word is polled every 32 iterations.
__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ bool grid_bar(GridBar *b, unsigned nblk, unsigned &epoch,
                                         unsigned limit) {
  __shared__ int s_ok;
  __syncthreads();
  epoch += 1;
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned target = epoch * nblk;
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(&b->count), "r"(1u) : "memory");
    unsigned it = 0;
    while (ld_acquire_gpu(&b->count) < target) {
      ++it;
      if ((it & 31u) == 0u && *(volatile int *)&b->err) {
        ok = 0;
        break;
      }
      if (it > limit) {
        atomicExch(&b->err, 1);
        ok = 0;
        break;
      }
      if (it > 64u) __nanosleep(20);
    }
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
