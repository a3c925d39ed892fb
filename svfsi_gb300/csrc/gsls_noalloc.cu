// Dot product of two device vectors that allocates no device memory.
//
// For callers that cannot call cudaMalloc: drivers that hand the whole
// device heap to their own pool at start-up, or code running where no new
// allocation may be made.  The reduction scratch -- one partial sum per
// block, the group sums of the two-level reduction, the result slot and the
// arrival counters -- lives in a file-scope __device__ array of fixed size
// (137,476 bytes), which every GPU that loads this translation unit's
// module holds until the process exits.  CUDA loads modules lazily by
// default, so the array is placed on a device when its address is first
// resolved: gsls_init does that for the device it selects, so that a
// caller whose pool then takes the whole heap still finds the array in
// place.  Host code cannot use the array's name as a device address; its
// address is resolved with cudaGetSymbolAddress once per device, with that
// device current (in gsls_init, or else on the first call on the device),
// and kept for the life of the process: after a cudaDeviceReset, call
// gsls_init again, which resolves it anew.
#include <mutex>

#include "gsls_internal.cuh"

namespace gsls {

constexpr int kNaThreads = 256;
constexpr long long kNaChunk = 4096;    // elements summed by one block
constexpr int kNaMaxBlocks = 16384;     // => n <= 67,108,864
constexpr long long kNaMaxN = kNaChunk * kNaMaxBlocks;
constexpr int kNaMaxGroups = (kNaMaxBlocks + kRedGroup - 1) / kRedGroup;
// layout: partials (blocks + groups) | result | counters (1 + groups)
constexpr size_t kNaResultOff = sizeof(double) * (kNaMaxBlocks + kNaMaxGroups);
constexpr size_t kNaTicketOff = kNaResultOff + 256;
constexpr size_t kNaTicketBytes = sizeof(unsigned) * (1 + kNaMaxGroups);
constexpr size_t kNaBytes = kNaTicketOff + kNaTicketBytes;
static_assert(kNaBytes == 137476, "scratch size as documented in include/gsls.h");

static __device__ __align__(256) unsigned char g_na_scratch[kNaBytes];

// One block per chunk of kNaChunk elements, then the deterministic
// two-level grid reduction of the block sums into the result slot.
__global__ void __launch_bounds__(kNaThreads) k_dot_chunked(long long n, const double *__restrict__ u,
                                                            const double *__restrict__ v,
                                                            unsigned char *scratch) {
  __shared__ double sh[32];
  const long long s = (long long)blockIdx.x * kNaChunk;
  const long long e = s + kNaChunk < n ? s + kNaChunk : n;
  double acc = 0.0;
  for (long long k = s + threadIdx.x; k < e; k += blockDim.x) acc += u[k] * v[k];
  double bs = block_sum(acc, sh);
  double tot;
  double *part = reinterpret_cast<double *>(scratch);
  unsigned *tk = reinterpret_cast<unsigned *>(scratch + kNaTicketOff);
  if (grid_reduce_last<1>(&bs, part, tk, &tot, sh) && threadIdx.x == 0)
    *reinterpret_cast<double *>(scratch + kNaResultOff) = tot;
}

static std::mutex g_na_mu;
static unsigned char *g_na_ptr[64] = {};

// Device address of the scratch array on the current device: resolved on
// the first use on a device (or always, with refresh) and kept.
static int na_scratch(unsigned char **out, bool refresh) {
  int dev = 0;
  GSLS_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    set_error("gsls_dot_noalloc: device index out of range");
    return GSLS_ERR_ARG;
  }
  std::lock_guard<std::mutex> lk(g_na_mu);
  if (refresh || !g_na_ptr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_na_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_na_scratch)", __FILE__, __LINE__);
    g_na_ptr[dev] = static_cast<unsigned char *>(p);
  }
  if (out) *out = g_na_ptr[dev];
  return GSLS_OK;
}

// Called by gsls_init with the selected device current: loads this module
// on the device (placing the scratch array) and resolves its address.
int noalloc_prepare_device() { return na_scratch(nullptr, true); }

}  // namespace gsls

using namespace gsls;

extern "C" int gsls_dot_noalloc(long long n, const double *du, const double *dv, double *result,
                                void *stream) {
  if (n < 0 || (n > 0 && (!du || !dv)) || !result) {
    set_error("gsls_dot_noalloc: bad arguments");
    return GSLS_ERR_ARG;
  }
  if (n > kNaMaxN) {
    set_error("gsls_dot_noalloc: n exceeds the maximum of 67108864 elements (4096 x 16384) "
              "that the fixed scratch array supports");
    return GSLS_ERR_ARG;
  }
  unsigned char *scratch = nullptr;
  GSLS_TRY(na_scratch(&scratch, false));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // the array keeps the previous call's contents: the arrival counters must
  // start at zero (a completed call leaves them at zero; clear regardless)
  GSLS_CUDA(cudaMemsetAsync(scratch + kNaTicketOff, 0, kNaTicketBytes, st));
  const long long nb = n > 0 ? (n + kNaChunk - 1) / kNaChunk : 1;
  k_dot_chunked<<<(unsigned)nb, kNaThreads, 0, st>>>(n, du, dv, scratch);
  GSLS_CHECK_LAUNCH();
  GSLS_CUDA(cudaMemcpyAsync(result, scratch + kNaResultOff, sizeof(double), cudaMemcpyDeviceToHost, st));
  GSLS_CUDA(cudaStreamSynchronize(st));
  return GSLS_OK;
}
