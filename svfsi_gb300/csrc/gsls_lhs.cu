// svFSILS-shaped object management: LHS (CSR + faces), BC faces, LS
// defaults, device workspace, error state, stream.
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "gsls_internal.cuh"

namespace gsls {

static thread_local std::string g_err;
static std::atomic<long long> g_launches{0};

void set_error(const std::string &msg) { g_err = msg; }

int cuda_fail(cudaError_t e, const char *what, const char *file, int line) {
  char buf[512];
  snprintf(buf, sizeof(buf), "CUDA error %d (%s) in %s at %s:%d", (int)e,
           cudaGetErrorString(e), what, file, line);
  g_err = buf;
  return GSLS_ERR_CUDA;
}

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void count_launch_n(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

struct ProfEntry {
  long long count = 0;
  double ms = 0.0;
};
static bool g_prof = false;
static std::mutex g_prof_mu;
static std::vector<std::pair<std::string, ProfEntry>> g_prof_tab;
static std::vector<cudaEvent_t> g_events;

bool prof_on() { return g_prof; }

int zigzag_on() {
  static const int on = [] {
    const char *e = getenv("GSLS_ZIGZAG");
    return (e && strcmp(e, "0") == 0) ? 0 : 1;
  }();
  return on;
}

void prof_add(const char *name, long long count, double ms) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  for (auto &kv : g_prof_tab)
    if (kv.first == name) {
      kv.second.count += count;
      kv.second.ms += ms;
      return;
    }
  ProfEntry e;
  e.count = count;
  e.ms = ms;
  g_prof_tab.emplace_back(name, e);
}

cudaEvent_t prof_event(int i) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  while ((int)g_events.size() <= i) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    g_events.push_back(e);
  }
  return g_events[i];
}

int num_sms() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
  }
  return n;
}

int DevBuf::alloc(size_t n) {
  if (n <= bytes && p) return GSLS_OK;
  release();
  if (n == 0) n = 16;
  cudaError_t e = cudaMalloc(&p, n);
  if (e != cudaSuccess) {
    p = nullptr;
    bytes = 0;
    return cuda_fail(e, "cudaMalloc", __FILE__, __LINE__);
  }
  bytes = n;
  return GSLS_OK;
}

void DevBuf::release() {
  if (p) cudaFree(p);
  p = nullptr;
  bytes = 0;
}

// Reduction grid: a fixed number of blocks (multiple of the SM count) so
// that grid reductions are reproducible for a given device.
static int pick_grid(int nNo) {
  const int sms = num_sms();
  int g = sms * 8;
  const int need = (nNo + 7) / 8;  // 8 rows per block at least
  if (need < g) g = ((need + sms - 1) / sms) * sms;
  if (g < sms) g = sms;
  return g;
}

int lhs_prepare_ws(gsls_lhs *lhs, int dof) {
  Workspace &ws = lhs->ws;
  const size_t nv = (size_t)lhs->nNo * dof;
  GSLS_TRY(ws.partials.alloc(sizeof(double) * (size_t)lhs->grid * 64));
  if (!ws.ticket.p) {
    // one group counter per kRedGroup blocks of the largest grid + 1
    GSLS_TRY(ws.ticket.alloc(sizeof(unsigned) * 256));
    GSLS_CUDA(cudaMemsetAsync(ws.ticket.p, 0, sizeof(unsigned) * 256, lhs->stream));
  }
  GSLS_TRY(ws.scal.alloc(sizeof(KrylovScalars)));
  for (int k = 0; k < 6; k++) GSLS_TRY(ws.vec[k].alloc(sizeof(double) * nv));
  GSLS_TRY(ws.W.alloc(sizeof(double) * nv));
  GSLS_TRY(ws.W2.alloc(sizeof(double) * nv));
  GSLS_TRY(ws.Wf.alloc(sizeof(float) * nv));
  if (!ws.err.p) {
    GSLS_TRY(ws.err.alloc(64));
    GSLS_CUDA(cudaMemsetAsync(ws.err.p, 0, 64, lhs->stream));
  }
  GSLS_TRY(ws.mask.alloc(sizeof(double) * nv));
  if (!ws.h_scal) {
    GSLS_CUDA(cudaMallocHost(&ws.h_scal, sizeof(KrylovScalars)));
    memset(ws.h_scal, 0, sizeof(KrylovScalars));
  }
  return GSLS_OK;
}

// incFlag / coupledFlag from incL and res, Code/Source/svFSILS/SOLVE.f:69-91
int lhs_update_faces(gsls_lhs *lhs, const int *incL, const double *res) {
  for (int f = 0; f < lhs->nFaces; f++) {
    Face &fa = lhs->faces[f];
    fa.incFlag = true;
    if (incL && incL[f] == 0) fa.incFlag = false;
  }
  bool anyNeu = false;
  for (auto &fa : lhs->faces)
    if (fa.foC && fa.bGrp == GSLS_BC_TYPE_NEU) anyNeu = true;
  if (!res && anyNeu) {
    set_error("res is required for Neu surfaces");
    return GSLS_ERR_ARG;
  }
  for (int f = 0; f < lhs->nFaces; f++) {
    Face &fa = lhs->faces[f];
    fa.coupledFlag = false;
    if (!fa.incFlag) continue;
    if (fa.bGrp == GSLS_BC_TYPE_NEU && res && res[f] != 0.0) {
      fa.res = res[f];
      fa.coupledFlag = true;
    }
  }
  return GSLS_OK;
}

// valM = val W on the coupled faces (PRECONDDIAG, Code/Source/svFSILS/
// PRECOND.f:133-143) and nS = |valM(1:dof-1,:)|^2 (BCPRE, NSSOLVER.f:307-343).
// The reference sets valM in PRECONDDIAG only (its RCS counterpart is
// commented out), so coupled faces require PRECOND_FSILS.
int cpl_prepare(gsls_lhs *lhs, int dof, const double *dW, int prec) {
  Workspace &ws = lhs->ws;
  ws.cpl_on = false;
  int nf = 0;
  for (auto &fa : lhs->faces)
    if (fa.foC && fa.coupledFlag) nf++;
  if (nf == 0) return GSLS_OK;
  if (prec != GSLS_PRECOND_FSILS) {
    set_error("coupled Neumann faces need PRECOND_FSILS (valM is set by PRECONDDIAG)");
    return GSLS_ERR_UNSUPPORTED;
  }
  if (nf > kMaxCpl) {
    set_error("at most 8 coupled Neumann faces per solve");
    return GSLS_ERR_UNSUPPORTED;
  }
  std::vector<double> W((size_t)lhs->nNo * dof);
  GSLS_CUDA(cudaMemcpyAsync(W.data(), dW, sizeof(double) * W.size(), cudaMemcpyDeviceToHost,
                            lhs->stream));
  GSLS_CUDA(cudaStreamSynchronize(lhs->stream));
  CplFaces &F = ws.cpl;
  memset(&F, 0, sizeof(F));
  std::vector<int> glob;
  std::vector<double> valM;
  for (auto &fa : lhs->faces) {
    if (!(fa.foC && fa.coupledFlag)) continue;
    const int f = F.nf++;
    F.off[f] = (int)glob.size();
    F.fdof[f] = fa.dof;
    F.voff[f] = (int)valM.size();
    const int m = fa.dof < dof ? fa.dof : dof;
    double nS = 0.0;
    for (int a = 0; a < fa.nNo; a++) {
      const int Ac = fa.glob[a];
      glob.push_back(Ac);
      for (int i = 0; i < fa.dof; i++) {
        const double v = (i < m) ? fa.val[(size_t)a * fa.dof + i] * W[(size_t)Ac * dof + i] : 0.0;
        valM.push_back(v);
        if (i < dof - 1) nS = nS + pow(v, 2.0);
      }
    }
    fa.nS = nS;
    F.cadd[f] = fa.res;
    F.cpre[f] = -fa.res / (1.0 + fa.res * nS);
  }
  F.off[F.nf] = (int)glob.size();
  GSLS_TRY(ws.cpl_glob.alloc(sizeof(int) * (glob.size() + 1)));
  GSLS_TRY(ws.cpl_valM.alloc(sizeof(double) * (valM.size() + 1)));
  GSLS_CUDA(cudaMemcpyAsync(ws.cpl_glob.p, glob.data(), sizeof(int) * glob.size(),
                            cudaMemcpyHostToDevice, lhs->stream));
  GSLS_CUDA(cudaMemcpyAsync(ws.cpl_valM.p, valM.data(), sizeof(double) * valM.size(),
                            cudaMemcpyHostToDevice, lhs->stream));
  ws.cpl_on = true;
  return GSLS_OK;
}

// One block: all face products first (from X), then the updates face by
// face, so that Y may alias X (the PRE form) as in the reference.
template <class XT>
__global__ void __launch_bounds__(1024) k_addbcmul(CplFaces F, const int *__restrict__ glob,
                                                   const double *__restrict__ valM, int op,
                                                   int vdof, const XT *X, XT *Y, const int *done) {
  if (done && *(volatile const int *)done) return;
  __shared__ double sh[32];
  __shared__ double sS[kMaxCpl];
  for (int f = 0; f < F.nf; f++) {
    const int fd = F.fdof[f], m = fd < vdof ? fd : vdof;
    double s = 0.0;
    for (int a = F.off[f] + threadIdx.x; a < F.off[f + 1]; a += blockDim.x) {
      const int Ac = glob[a];
      const double *v = valM + F.voff[f] + (size_t)(a - F.off[f]) * fd;
      for (int i = 0; i < m; i++) s += v[i] * double(X[(size_t)Ac * vdof + i]);
    }
    s = block_sum(s, sh);
    if (threadIdx.x == 0) sS[f] = (op == 0 ? F.cadd[f] : F.cpre[f]) * s;
    __syncthreads();
  }
  for (int f = 0; f < F.nf; f++) {
    const int fd = F.fdof[f], m = fd < vdof ? fd : vdof;
    const double S = sS[f];
    for (int a = F.off[f] + threadIdx.x; a < F.off[f + 1]; a += blockDim.x) {
      const int Ac = glob[a];
      const double *v = valM + F.voff[f] + (size_t)(a - F.off[f]) * fd;
      for (int i = 0; i < m; i++) {
        XT *y = Y + (size_t)Ac * vdof + i;
        *y = XT(double(*y) + v[i] * S);
      }
    }
    __syncthreads();
  }
}

template <class XT>
void launch_addbcmul(gsls_lhs *lhs, int op, int vdof, const XT *X, XT *Y, const int *done) {
  Workspace &ws = lhs->ws;
  if (!ws.cpl_on) return;
  k_addbcmul<XT><<<1, 1024, 0, lhs->stream>>>(ws.cpl, ws.cpl_glob.as<int>(),
                                              ws.cpl_valM.as<double>(), op, vdof, X, Y, done);
  count_launch();
}
template void launch_addbcmul<float>(gsls_lhs *, int, int, const float *, float *, const int *);
template void launch_addbcmul<double>(gsls_lhs *, int, int, const double *, double *,
                                      const int *);

// Dirichlet mask = product over included Dir faces of val(1:min(dof,fdof)),
// the factor PRECONDDIAG applies to W (Code/Source/svFSILS/PRECOND.f:107-117).
// Cached on the (dof, incFlag) key; built on the host, uploaded once.
int build_dir_mask(gsls_lhs *lhs, int dof) {
  Workspace &ws = lhs->ws;
  std::vector<int> key;
  key.push_back(dof);
  for (auto &fa : lhs->faces) key.push_back(fa.foC && fa.incFlag ? 1 : 0);
  if (ws.mask_dof == dof && ws.mask_key == key) return GSLS_OK;
  std::vector<double> m((size_t)lhs->nNo * dof, 1.0);
  for (auto &fa : lhs->faces) {
    if (!fa.foC || !fa.incFlag || fa.bGrp != GSLS_BC_TYPE_DIR) continue;
    const int i = fa.dof < dof ? fa.dof : dof;
    for (int a = 0; a < fa.nNo; a++) {
      const int Ac = fa.glob[a];
      for (int k = 0; k < i; k++) m[(size_t)Ac * dof + k] *= fa.val[(size_t)a * fa.dof + k];
    }
  }
  GSLS_TRY(ws.mask.alloc(sizeof(double) * m.size()));
  GSLS_CUDA(cudaMemcpyAsync(ws.mask.p, m.data(), sizeof(double) * m.size(),
                            cudaMemcpyHostToDevice, lhs->stream));
  GSLS_CUDA(cudaStreamSynchronize(lhs->stream));
  ws.mask_dof = dof;
  ws.mask_key = key;
  ws.mask_serial++;
  return GSLS_OK;
}

__global__ void k_row_of(const int *rowPtr, int nNo, int *rowOf) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nNo; i += gridDim.x * blockDim.x)
    for (int j = rowPtr[i]; j < rowPtr[i + 1]; j++) rowOf[j] = i;
}

// FP64 FMA throughput probe: 8 independent chains per thread, one store per
// thread into a buffer of exactly grid * block doubles.
__global__ void __launch_bounds__(256) k_dfma_probe(double *out, int iters) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; k++) a[k] = 1e-9 * (t + k);
  const double b = 0.9999999, c = 1e-7;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 8; k++) a[k] = fma(a[k], b, c);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += a[k];
  out[t] = s;
}

// L2 read-bandwidth probe: every block sweeps the whole L2-resident buffer
// (float4 loads, each block from its own starting offset), `passes` times;
// one sum per thread stored into out[grid * block].
__global__ void __launch_bounds__(512) k_l2_probe(const float4 *__restrict__ buf, size_t n4,
                                                  int passes, float *out) {
  float acc = 0.f;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (int p = 0; p < passes; p++)
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n4; k += stride) {
      const float4 v = __ldcg(buf + k);
      acc += v.x + v.y + v.z + v.w;
    }
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

}  // namespace gsls

namespace gsls {
static std::atomic<unsigned> g_wait_limit{kBarSpinDefault};
unsigned wait_limit() { return g_wait_limit.load(std::memory_order_relaxed); }
}  // namespace gsls

using namespace gsls;

extern "C" {

int gsls_version(void) { return GSLS_VERSION; }

int gsls_fp64_fma_rate(double *fma_per_s) {
  if (!fma_per_s) return GSLS_ERR_ARG;
  const int threads = 256, blocks = 4 * num_sms(), iters = 4000;
  const size_t n = (size_t)blocks * threads;
  double *d = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = GSLS_OK;
  float ms = 0.0f;
  if (cudaMalloc(&d, n * sizeof(double)) != cudaSuccess ||
      cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    rc = GSLS_ERR_CUDA;
  } else {
    for (int r = 0; r < 3; r++) k_dfma_probe<<<blocks, threads, 0, st>>>(d, iters);
    cudaEventRecord(e0, st);
    k_dfma_probe<<<blocks, threads, 0, st>>>(d, iters);
    cudaEventRecord(e1, st);
    count_launch_n(4);
    if (cudaGetLastError() != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
        cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess || ms <= 0.0f)
      rc = GSLS_ERR_CUDA;
  }
  if (rc == GSLS_OK) *fma_per_s = 8.0 * iters * (double)n / (ms * 1e-3);
  else set_error("gsls_fp64_fma_rate: CUDA error");
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  if (d) cudaFree(d);
  return rc;
}

int gsls_l2_read_rate(double *bytes_per_s) {
  if (!bytes_per_s) return GSLS_ERR_ARG;
  const int threads = 512, blocks = 2 * num_sms(), passes = 20;
  const size_t bytes = (size_t)48 << 20;  // 48 MiB: well inside the 129 MB L2
  const size_t n4 = bytes / 16;
  float4 *buf = nullptr;
  float *out = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = GSLS_OK;
  float ms = 0.0f;
  if (cudaMalloc(&buf, bytes) != cudaSuccess ||
      cudaMalloc(&out, sizeof(float) * (size_t)blocks * threads) != cudaSuccess ||
      cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess ||
      cudaMemsetAsync(buf, 0, bytes, st) != cudaSuccess) {
    rc = GSLS_ERR_CUDA;
  } else {
    for (int r = 0; r < 3; r++) k_l2_probe<<<blocks, threads, 0, st>>>(buf, n4, 2, out);
    cudaEventRecord(e0, st);
    k_l2_probe<<<blocks, threads, 0, st>>>(buf, n4, passes, out);
    cudaEventRecord(e1, st);
    count_launch_n(4);
    if (cudaGetLastError() != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
        cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess || ms <= 0.0f)
      rc = GSLS_ERR_CUDA;
  }
  if (rc == GSLS_OK) *bytes_per_s = (double)passes * (double)bytes / (ms * 1e-3);
  else set_error("gsls_l2_read_rate: CUDA error");
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  if (out) cudaFree(out);
  if (buf) cudaFree(buf);
  return rc;
}

const char *gsls_last_error(void) { return g_err.c_str(); }

long long gsls_launch_count(void) { return g_launches.load(); }

int gsls_profile_enable(int on) {
  g_prof = on != 0;
  return GSLS_OK;
}

int gsls_profile_reset(void) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_prof_tab.clear();
  return GSLS_OK;
}

int gsls_profile_read(const char *name, long long *count, double *total_ms) {
  if (!name) return GSLS_ERR_ARG;
  std::lock_guard<std::mutex> lk(g_prof_mu);
  for (auto &kv : g_prof_tab)
    if (kv.first == name) {
      if (count) *count = kv.second.count;
      if (total_ms) *total_ms = kv.second.ms;
      return GSLS_OK;
    }
  if (count) *count = 0;
  if (total_ms) *total_ms = 0.0;
  return GSLS_OK;
}

int gsls_set_wait_limit(unsigned polls) {
  g_wait_limit.store(polls ? polls : kBarSpinDefault, std::memory_order_relaxed);
  return GSLS_OK;
}

int gsls_init(int device) {
  GSLS_CUDA(cudaSetDevice(device));
  GSLS_CUDA(cudaFree(0));
  // place the fixed scratch array of gsls_dot_noalloc on this device now
  // (lazy module loading would otherwise place it on its first call)
  return noalloc_prepare_device();
}

int gsls_lhs_create(gsls_lhs **out, int gnNo, int nNo, int nnz, const int *gNodes,
                    const int *rowPtr, const int *colPtr, int nFaces) {
  (void)gNodes;
  if (!out || nNo <= 0 || nnz <= 0 || !rowPtr || !colPtr || nFaces < 0) {
    set_error("gsls_lhs_create: bad arguments");
    return GSLS_ERR_ARG;
  }
  if (rowPtr[0] != 1 || rowPtr[nNo] - 1 != nnz) {
    set_error("gsls_lhs_create: rowPtr must be 1-based with rowPtr(nNo+1)-1 == nnz");
    return GSLS_ERR_ARG;
  }
  gsls_lhs *lhs = new gsls_lhs();
  lhs->gnNo = gnNo;
  lhs->nNo = nNo;
  lhs->nnz = nnz;
  lhs->nFaces = nFaces;
  lhs->mynNo = nNo;
  lhs->h_rowPtr.resize(nNo + 1);
  lhs->h_colPtr.resize(nnz);
  lhs->h_diagPtr.assign(nNo, -1);
  for (int i = 0; i <= nNo; i++) lhs->h_rowPtr[i] = rowPtr[i] - 1;
  for (int j = 0; j < nnz; j++) {
    lhs->h_colPtr[j] = colPtr[j] - 1;
    if (lhs->h_colPtr[j] < 0 || lhs->h_colPtr[j] >= nNo) {
      set_error("gsls_lhs_create: column index out of range");
      delete lhs;
      return GSLS_ERR_ARG;
    }
  }
  // diagPtr search, Code/Source/svFSILS/LHS.f:93-103
  for (int Ac = 0; Ac < nNo; Ac++) {
    for (int i = lhs->h_rowPtr[Ac]; i < lhs->h_rowPtr[Ac + 1]; i++)
      if (lhs->h_colPtr[i] == Ac) {
        lhs->h_diagPtr[Ac] = i;
        break;
      }
    if (lhs->h_diagPtr[Ac] < 0) {
      set_error("gsls_lhs_create: row without a diagonal entry");
      delete lhs;
      return GSLS_ERR_ARG;
    }
  }
  lhs->faces.resize(nFaces);
  int rc;
  cudaError_t e = cudaStreamCreateWithFlags(&lhs->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete lhs;
    return cuda_fail(e, "cudaStreamCreate", __FILE__, __LINE__);
  }
  lhs->own_stream = true;
  cudaEventCreate(&lhs->ev0);
  cudaEventCreate(&lhs->ev1);
  if ((rc = lhs->d_rowPtr.alloc(sizeof(int) * (nNo + 1))) ||
      (rc = lhs->d_colPtr.alloc(sizeof(int) * nnz + 64)) ||
      (rc = lhs->d_diagPtr.alloc(sizeof(int) * nNo)) ||
      (rc = lhs->d_rowOf.alloc(sizeof(int) * nnz))) {
    gsls_lhs_free(lhs);
    return rc;
  }
  cudaMemcpyAsync(lhs->d_rowPtr.p, lhs->h_rowPtr.data(), sizeof(int) * (nNo + 1),
                  cudaMemcpyHostToDevice, lhs->stream);
  cudaMemcpyAsync(lhs->d_colPtr.p, lhs->h_colPtr.data(), sizeof(int) * nnz,
                  cudaMemcpyHostToDevice, lhs->stream);
  cudaMemcpyAsync(lhs->d_diagPtr.p, lhs->h_diagPtr.data(), sizeof(int) * nNo,
                  cudaMemcpyHostToDevice, lhs->stream);
  k_row_of<<<num_sms() * 4, 256, 0, lhs->stream>>>(lhs->d_rowPtr.as<int>(), nNo,
                                                  lhs->d_rowOf.as<int>());
  count_launch();
  lhs->grid = pick_grid(nNo);
  if ((rc = lhs_prepare_ws(lhs, 1)) != GSLS_OK) {
    gsls_lhs_free(lhs);
    return rc;
  }
  e = cudaStreamSynchronize(lhs->stream);
  if (e != cudaSuccess) {
    gsls_lhs_free(lhs);
    return cuda_fail(e, "lhs upload", __FILE__, __LINE__);
  }
  *out = lhs;
  return GSLS_OK;
}

int gsls_lhs_free(gsls_lhs *lhs) {
  if (!lhs) return GSLS_ERR_ARG;
  if (lhs->stream) cudaStreamSynchronize(lhs->stream);
  for (gsls_lhs **ref : lhs->deps) *ref = nullptr;
  if (lhs->ws.h_scal) cudaFreeHost(lhs->ws.h_scal);
  if (lhs->ws.cg_graph) cudaGraphExecDestroy(lhs->ws.cg_graph);
  if (lhs->ws.cg_graph_s) cudaGraphExecDestroy(lhs->ws.cg_graph_s);
  if (lhs->ev0) cudaEventDestroy(lhs->ev0);
  if (lhs->ev1) cudaEventDestroy(lhs->ev1);
  cudaStream_t s = lhs->own_stream ? lhs->stream : nullptr;
  delete lhs;
  if (s) cudaStreamDestroy(s);
  return GSLS_OK;
}

int gsls_bc_create(gsls_lhs *lhs, int faIn, int nNo, int dof, int BC_type,
                   const int *gNodes, const double *val) {
  if (!lhs) return GSLS_ERR_ARG;
  if (faIn > lhs->nFaces || faIn <= 0) {
    set_error("gsls_bc_create: faIn out of range (Code/Source/svFSILS/BC.f:63-71)");
    return GSLS_ERR_ARG;
  }
  Face &f = lhs->faces[faIn - 1];
  if (f.foC) {
    set_error("gsls_bc_create: face is not free");
    return GSLS_ERR_STATE;
  }
  if (nNo < 0 || dof <= 0 || (nNo > 0 && !gNodes)) return GSLS_ERR_ARG;
  f.foC = true;
  f.nNo = nNo;
  f.dof = dof;
  f.bGrp = BC_type;
  f.glob.resize(nNo);
  f.val.assign((size_t)dof * nNo, 0.0);
  for (int a = 0; a < nNo; a++) {
    const int Ac = gNodes[a] - 1;
    if (Ac < 0 || Ac >= lhs->nNo) {
      f.foC = false;
      set_error("gsls_bc_create: node out of range");
      return GSLS_ERR_ARG;
    }
    f.glob[a] = Ac;
  }
  if (val) memcpy(f.val.data(), val, sizeof(double) * (size_t)dof * nNo);
  lhs->ws.mask_dof = -1;  // invalidate cached mask
  return GSLS_OK;
}

int gsls_ls_create(gsls_ls *ls, int LS_type, const double *relTol, const double *absTol,
                   const int *maxItr, const int *dimKry, const double *relTolIn,
                   const double *absTolIn, const int *maxItrIn) {
  if (!ls) return GSLS_ERR_ARG;
  memset(ls, 0, sizeof(*ls));
  ls->foC = 1;
  ls->LS_type = LS_type;
  // defaults, Code/Source/svFSILS/LS.f:68-95
  switch (LS_type) {
    case GSLS_LS_TYPE_NS:
      ls->RI.relTol = 0.4;
      ls->GM.relTol = 1e-2;
      ls->CG.relTol = 0.2;
      ls->RI.mItr = 10;
      ls->GM.mItr = 2;
      ls->CG.mItr = 500;
      ls->GM.sD = 100;
      ls->RI.sD = 100;
      break;
    case GSLS_LS_TYPE_GMRES:
      ls->RI.relTol = 0.1;
      ls->RI.mItr = 4;
      ls->RI.sD = 250;
      break;
    case GSLS_LS_TYPE_CG:
      ls->RI.relTol = 1e-2;
      ls->RI.mItr = 1000;
      break;
    case GSLS_LS_TYPE_BICGS:
      ls->RI.relTol = 1e-2;
      ls->RI.mItr = 500;
      break;
    default:
      set_error("gsls_ls_create: LS_TYPE is not defined");
      ls->foC = 0;
      return GSLS_ERR_ARG;
  }
  ls->RI.absTol = 1e-10;
  ls->GM.absTol = 1e-10;
  ls->CG.absTol = 1e-10;
  if (relTol) ls->RI.relTol = *relTol;
  if (absTol) ls->RI.absTol = *absTol;
  if (maxItr) ls->RI.mItr = *maxItr;
  if (dimKry) {
    ls->RI.sD = *dimKry;
    ls->GM.sD = *dimKry;
  }
  if (relTolIn) {
    ls->GM.relTol = relTolIn[0];
    ls->CG.relTol = relTolIn[1];
  }
  if (absTolIn) {
    ls->GM.absTol = absTolIn[0];
    ls->CG.absTol = absTolIn[1];
  }
  if (maxItrIn) {
    ls->GM.mItr = maxItrIn[0];
    ls->CG.mItr = maxItrIn[1];
  }
  return GSLS_OK;
}

int gsls_set_stream(gsls_lhs *lhs, void *stream) {
  if (!lhs) return GSLS_ERR_ARG;
  cudaStreamSynchronize(lhs->stream);
  if (stream == nullptr) {
    if (!lhs->own_stream) {
      GSLS_CUDA(cudaStreamCreateWithFlags(&lhs->stream, cudaStreamNonBlocking));
      lhs->own_stream = true;
    }
    return GSLS_OK;
  }
  if (lhs->own_stream) cudaStreamDestroy(lhs->stream);
  lhs->stream = (cudaStream_t)stream;
  lhs->own_stream = false;
  return GSLS_OK;
}

void *gsls_get_stream(gsls_lhs *lhs) { return lhs ? (void *)lhs->stream : nullptr; }

}  // extern "C"
