// Internal definitions shared by the gsls translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/gsls.h"

namespace gsls {

// ---------------------------------------------------------------------------
// error handling
void set_error(const std::string &msg);
int cuda_fail(cudaError_t e, const char *what, const char *file, int line);

#define GSLS_CUDA(...)                                                         \
  do {                                                                         \
    cudaError_t _e = (__VA_ARGS__);                                                 \
    if (_e != cudaSuccess) return ::gsls::cuda_fail(_e, #__VA_ARGS__, __FILE__, __LINE__); \
  } while (0)

#define GSLS_CHECK_LAUNCH()                                                    \
  do {                                                                         \
    ::gsls::count_launch();                                                    \
    cudaError_t _e = cudaGetLastError();                                       \
    if (_e != cudaSuccess) return ::gsls::cuda_fail(_e, "kernel launch", __FILE__, __LINE__); \
  } while (0)

#define GSLS_TRY(...)                                                          \
  do {                                                                         \
    int _rc = (__VA_ARGS__);                                                        \
    if (_rc != GSLS_OK) return _rc;                                            \
  } while (0)

void count_launch();
void count_launch_n(int n);
int num_sms();
// gsls_noalloc.cu: place gsls_dot_noalloc's scratch array on the current
// device and resolve its address (called by gsls_init)
int noalloc_prepare_device();
// poll limit of the grid barriers of the persistent kernels (gsls_set_wait_limit)
constexpr unsigned kBarSpinDefault = 1u << 24;
unsigned wait_limit();
// Zig-zag traversal of the Krylov SpMVs: a matrix larger than L2 streamed in
// the same order every iteration leaves L2 holding its tail, which the next
// forward pass evicts before reaching it; reversing the row order every
// other iteration starts each pass on what the previous one left in L2.
// Default on; GSLS_ZIGZAG=0 keeps the forward order.
int zigzag_on();

// kernel timing registry (gsls_profile_*)
bool prof_on();
void prof_add(const char *name, long long count, double ms);
// pool of reusable CUDA events
cudaEvent_t prof_event(int i);

// ---------------------------------------------------------------------------
// device buffer (RAII, stream-ordered free)
struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }
  int alloc(size_t n);              // no-op if already >= n bytes
  void release();
  template <class T> T *as() const { return reinterpret_cast<T *>(p); }
};

// ---------------------------------------------------------------------------
// Krylov scalar block living in device memory (one per solve context).
struct KrylovScalars {
  double iNorm, eps, err, errO, alpha, dot, fNorm;
  double beta;
  int done;   // 0 running, 1 converged, 2 max iterations, 3 breakdown/NaN,
              // 4 grid barrier timed out (persistent CG)
  int itr;    // completed iterations
  int mItr;
  int suc;
  // GMRES
  double h_norm;
  double pad1[3];
};

// Face (BC) description, FSILS_faceType.
struct Face {
  bool foC = false, coupledFlag = false, sharedFlag = false, incFlag = true;
  int nNo = 0, dof = 0, bGrp = GSLS_BC_TYPE_DIR;
  std::vector<int> glob;     // 0-based
  std::vector<double> val;   // dof x nNo
  double nS = 0.0, res = 0.0;
};

// Coupled-Neumann (resistance) faces of one solve, ADDBCMUL
// (Code/Source/svFSILS/ADDBCMUL.f:53-114): face f holds entries
// off[f]..off[f+1] of the concatenated node list and valM (fdof values per
// node); cadd = res, cpre = -res/(1 + res nS).
constexpr int kMaxCpl = 8;
struct CplFaces {
  int nf;
  int off[kMaxCpl + 1];
  int fdof[kMaxCpl];
  int voff[kMaxCpl];  // offset of face f in valM
  double cadd[kMaxCpl], cpre[kMaxCpl];
};

// Identity of a captured CG batch graph (kernel arguments baked in).
struct GraphKey {
  int D, vsz, xsz;
  const void *val;
  const void *x;
  int batch, nNo;
  bool tma;
  bool fused;
  const void *part, *scal, *w;  // workspace buffers baked into the graph
  const void *sval;             // sliced copy of the matrix (null: CSR SpMV)
  bool operator==(const GraphKey &o) const {
    return D == o.D && vsz == o.vsz && xsz == o.xsz && val == o.val && x == o.x &&
           batch == o.batch && nNo == o.nNo && tma == o.tma && fused == o.fused &&
           part == o.part && scal == o.scal && w == o.w && sval == o.sval;
  }
};

// Scratch for reductions and Krylov work vectors.
struct Workspace {
  DevBuf Wf;          // float copy of W (FP32 scaling pass)
  DevBuf err;         // device error word of staged kernels
  int tma_key = -1, tma_smem = 0, tma_grid = 0;
  bool tma_ok = false;
  long long tma_info[3] = {0, 0, 0};  // TmaTiles of the cached geometry
  cudaGraphExec_t cg_graph = nullptr;      // CG batch on the CSR matrix
  GraphKey cg_key{};
  cudaGraphExec_t cg_graph_s = nullptr;    // CG batch on the sliced copy
  GraphKey cg_key_s{};
  int cg_last_itr = 0;                     // iterations of the last CG solve (first-batch size)
  // sliced block-ELL layout of the CG SpMV (structure per block size D,
  // values per solve): slice offsets, slot rows, columns, CSR block -> slot
  int sell_D = 0, sell_nS = 0, sell_vkey = 0;
  long long sell_steps = 0;
  DevBuf sell_off, sell_row, sell_col, sell_pos, sell_val;
  DevBuf partials;    // double[grid * 64]
  DevBuf ticket;      // unsigned[8]
  DevBuf scal;        // KrylovScalars
  DevBuf cgbar;       // grid barrier of the persistent CG
  DevBuf vec[6];      // Krylov work vectors (X, P, KP, R32...)
  DevBuf W;           // diag preconditioner (double dof x nNo)
  DevBuf W2;          // RCS second scaling
  DevBuf mask;        // Dirichlet mask (double dof x nNo)
  DevBuf basis;       // GMRES basis (sD+1) vectors
  DevBuf hcol;        // GMRES Hessenberg column (double)
  DevBuf io;          // host<->device staging for gsls_solve
  DevBuf io2;
  DevBuf ns_vec;      // NS solver vectors (Rm, Rc, U, P, MU, MP, Schur CG)
  DevBuf ns_mat;      // NS solver blocks (mK, mG, mD, mL, Gt)
  DevBuf rcs;         // RCS scaling state (W1, Wr, Wc, control words)
  DevBuf cpl_glob, cpl_valM;  // coupled faces of the current solve
  CplFaces cpl{};
  bool cpl_on = false;
  KrylovScalars *h_scal = nullptr;  // pinned host mirror
  int mask_dof = -1;
  std::vector<int> mask_key;
  unsigned mask_serial = 0;          // bumped by every rebuild of the Dirichlet mask
  unsigned long long pre_serial = 0; // bumped by every preconditioning (W and W Val W)
};

}  // namespace gsls

struct gsls_lhs {
  int gnNo = 0, nNo = 0, nnz = 0, nFaces = 0, mynNo = 0;
  std::vector<int> h_rowPtr, h_colPtr, h_diagPtr;  // 0-based
  gsls::DevBuf d_rowPtr, d_colPtr, d_diagPtr, d_rowOf;
  gsls::DevBuf d_tpos;   // CSR position of the transposed block (built on first use)
  bool tpos_ok = false;
  std::vector<gsls::Face> faces;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int grid = 0;          // fixed reduction grid (deterministic sums)
  gsls::Workspace ws;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // the `lhs` fields of the meshes and equations bound to this lhs:
  // gsls_lhs_free sets them to null, so that freeing those objects later
  // (in any order) touches no freed lhs
  std::vector<gsls_lhs **> deps;
};

namespace gsls {
inline void lhs_attach(gsls_lhs *lhs, gsls_lhs **ref) {
  if (lhs) lhs->deps.push_back(ref);
}
inline void lhs_detach(gsls_lhs *lhs, gsls_lhs **ref) {
  if (!lhs) return;
  for (size_t k = 0; k < lhs->deps.size(); k++)
    if (lhs->deps[k] == ref) {
      lhs->deps.erase(lhs->deps.begin() + (long)k);
      return;
    }
}
}  // namespace gsls

namespace gsls {

// ---------------------------------------------------------------------------
// kernel-side helpers
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum; result valid in thread 0. blockDim.x multiple of 32, <= 1024.
__device__ __forceinline__ double block_sum(double v, double *sh /*[32]*/) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  const int nw = blockDim.x >> 5;
  v = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
  if (wid == 0) v = warp_sum(v);
  return v;
}

// Ticket increment with acquire-release semantics at GPU scope: the
// caller's earlier writes are visible to whoever later acquires the ticket,
// and the caller sees the writes released by earlier increments.
__device__ __forceinline__ unsigned atomic_add_acq_rel(unsigned *p, unsigned v) {
  unsigned old;
  asm volatile("atom.add.acq_rel.gpu.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}

// Deterministic grid reduction of NV values per block.  Every block calls it
// with its block sums in thread 0 (vals[k]); returns true in exactly one
// block (the last to arrive), whose thread 0 holds the totals in out[k].
// The summation order depends only on gridDim.x, so results are bitwise
// reproducible for a fixed grid.
// Two levels (groups of kRedGroup blocks, then the group sums) keep the
// chain of same-address atomics short; both levels sum in a fixed order.
// ticket[0] counts groups, ticket[1 + g] counts blocks of group g (both are
// reset by their last arrival).  partials holds NV*(grid + ngroups) values.
constexpr int kRedGroup = 32;
template <int NV>
__device__ __forceinline__ bool grid_reduce_last(const double *vals, double *partials,
                                                 unsigned *ticket, double *out,
                                                 double *sh) {
  __shared__ int stage;  // 0: not last, 1: last of its group, 2: last overall
  const int G = gridDim.x, g = blockIdx.x / kRedGroup;
  const int ngroups = (G + kRedGroup - 1) / kRedGroup;
  const int gsz = min(kRedGroup, G - g * kRedGroup);
  double *gpart = partials + (size_t)NV * G;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; k++) partials[(size_t)k * G + blockIdx.x] = vals[k];
    const unsigned t = atomic_add_acq_rel(ticket + 1 + g, 1u);
    stage = (t == (unsigned)gsz - 1) ? 1 : 0;
  }
  __syncthreads();
  if (stage == 0) return false;
  // last block of group g: fixed-order sum of the group's partials
  double gs[NV];
#pragma unroll
  for (int k = 0; k < NV; k++) {
    double s = 0.0;
    for (int i = threadIdx.x; i < gsz; i += blockDim.x)
      s += __ldcg(&partials[(size_t)k * G + g * kRedGroup + i]);
    s = block_sum(s, sh);
    gs[k] = s;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; k++) gpart[(size_t)k * ngroups + g] = gs[k];
    ticket[1 + g] = 0u;
    const unsigned t = atomic_add_acq_rel(ticket, 1u);
    stage = (t == (unsigned)ngroups - 1) ? 2 : 1;
  }
  __syncthreads();
  if (stage != 2) return false;
#pragma unroll
  for (int k = 0; k < NV; k++) {
    double s = 0.0;
    for (int i = threadIdx.x; i < ngroups; i += blockDim.x)
      s += __ldcg(&gpart[(size_t)k * ngroups + i]);
    s = block_sum(s, sh);
    if (threadIdx.x == 0) out[k] = s;
    __syncthreads();
  }
  if (threadIdx.x == 0) *ticket = 0u;
  return true;
}

// Single-level form of grid_reduce_last for grids of a few hundred blocks
// (the resident grids of the CG kernels): one acquire-release ticket per
// block, and the last block sums all partials in block order -- one memory
// round trip less on the critical path than the two-level form.  The last
// block's other threads read the partials after the barrier that follows
// thread 0's acquire.  Uses ticket[0] only (reset by the last block).
template <int NV>
__device__ __forceinline__ bool grid_reduce_last1(const double *vals, double *partials,
                                                  unsigned *ticket, double *out, double *sh) {
  __shared__ int last;
  const int G = gridDim.x;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; k++) partials[(size_t)k * G + blockIdx.x] = vals[k];
    last = (atomic_add_acq_rel(ticket, 1u) == (unsigned)G - 1) ? 1 : 0;
  }
  __syncthreads();
  if (!last) return false;
#pragma unroll
  for (int k = 0; k < NV; k++) {
    double s = 0.0;
    for (int i = threadIdx.x; i < G; i += blockDim.x) s += __ldcg(&partials[(size_t)k * G + i]);
    s = block_sum(s, sh);
    if (threadIdx.x == 0) out[k] = s;
    __syncthreads();
  }
  if (threadIdx.x == 0) *ticket = 0u;
  return true;
}

template <class T> struct VecOf;

}  // namespace gsls

// internal entry points across translation units
namespace gsls {
int lhs_prepare_ws(gsls_lhs *lhs, int dof);
int lhs_update_faces(gsls_lhs *lhs, const int *incL, const double *res);
int build_dir_mask(gsls_lhs *lhs, int dof);
// padded: dVal has >= 16 bytes of slack after its end (enables staged copies)
// prescaled: dVal already holds W Val W of the diagonal preconditioner and
// ws.W its W, both from the last preconditioning on this lhs (the caller has
// checked ws.pre_serial and ws.mask_serial): only R = W R is formed
int solve_dev(gsls_lhs *lhs, gsls_ls *ls, int dof, double *dRi, void *dVal,
              int val_prec, int prec, bool padded, bool prescaled = false);
// The HEATS/CEP operator path of the assembly (R = rho M A + nu K Y - rho s
// b, Val = cM M + cK K from the mesh's cached operators).  In: a tangent key
// from an earlier call; if it matches (same operators, same coefficients)
// and skip_val is set, only R is formed and Val is left as it is.  Out:
// whether the operator path ran, its key, whether Val was skipped.
struct LinAsm {
  bool skip_val = false;
  unsigned serial = 0;
  double cM = 0.0, cK = 0.0;
  bool used = false, skipped = false;
};
int spmv_launch(gsls_lhs *lhs, int dof, const void *dVal, int val_prec,
                const void *dx, void *dy, int xprec);
// restarted GMRES on the preconditioned system (gsls_gmres.cu)
int gmres_run(gsls_lhs *lhs, gsls_sub_ls *ls, int D, bool mixed, const void *Val,
              double *R, const double *Wc);
// GMRES of the NS solver on device vectors (gsls_gmres.cu)
template <int D, class VT, class XT>
int gmres_ns(gsls_lhs *lhs, gsls_sub_ls *ls, const VT *Val, const XT *Rk, XT *X);
// coupled faces: valM, nS from the diagonal scaling W (gsls_lhs.cu)
int cpl_prepare(gsls_lhs *lhs, int dof, const double *dW, int prec);
// Y += coef_f valM_f (valM_f . X) over the coupled faces; op 0 ADD, 1 PRE;
// vectors with vdof values per node; skipped when *done is set
template <class XT>
void launch_addbcmul(gsls_lhs *lhs, int op, int vdof, const XT *X, XT *Y, const int *done);
// BiCGStab on the preconditioned system (gsls_bicgs.cu)
int bicgs_run(gsls_lhs *lhs, gsls_sub_ls *ls, int D, bool mixed, const void *Val, double *R,
              const double *W);
// RCS preconditioner and NS block solver (gsls_ns.cu)
int precond_rcs_run(gsls_lhs *lhs, int D, bool mixed, void *Val, double *R, double *W);
int ns_run(gsls_lhs *lhs, gsls_ls *ls, int D, bool mixed, const void *Val, double *R,
           const double *W);
}  // namespace gsls
