// Batched least squares of many independent, unevenly sized tall-skinny
// problems: min ||A_i x_i - b_i|| with n_i <= 128 (one panel each).
//
// The reference solves one panel at a time (hh_recon_qr,
// alg/QR/hh_recon/hh_recon.cxx:129-321); a batch of uneven problems on one GPU
// needs concurrency instead: problems are sorted by cost (m_i n_i^2) and dealt
// round-robin onto a pool of streams, so the small ones fill the SMs that the
// large ones' TSQR trees leave idle.  Per problem: TSQR-HR of A_i (A_i becomes
// Y\R), Q^T b_i in FP64 with the panel's T, and back substitution with R by
// one warp (b_i's first n_i entries become x_i, as LAPACK's dgels returns it).
// With use_graph the whole fork/join schedule is captured once into a CUDA
// graph (keyed by the sizes, pointers and tuning) and replayed afterwards.
#include <algorithm>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "kernels.cuh"

namespace candmc {

// R x = c in place on x (R upper, n x n, ld ldr), one warp.
__global__ void k_trsv_upper(const double* R, int64_t ldr, int n, double* x) {
  const int lane = threadIdx.x;
  for (int i = n - 1; i >= 0; --i) {
    double s = 0.0;
    for (int j = i + 1 + lane; j < n; j += 32) s = fma(R[(int64_t)j * ldr + i], x[j], s);
    s = warp_sum(s);
    if (lane == 0) x[i] = (x[i] - s) / R[(int64_t)i * ldr + i];
    __syncwarp();
  }
}

struct StreamPool {
  std::vector<cudaStream_t> s;
  cudaStream_t get(int i) {
    while ((int)s.size() <= i) {
      cudaStream_t t = nullptr;
      if (cudaStreamCreateWithFlags(&t, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
      s.push_back(t);
    }
    return s[i];
  }
};

static StreamPool g_pool[64];

// Per device: the status word every batched call's kernels record failures in
// (sticky until candmc_batched_status reads and clears it).  Allocated by the
// first call on the device, outside any stream capture.
static int* g_bstatus[64] = {};
static std::mutex g_bstatus_mu;

static int batched_status_word(int dev, int** out) {
  std::lock_guard<std::mutex> g(g_bstatus_mu);
  if (!g_bstatus[dev]) {
    int* p = nullptr;
    CANDMC_CK(cudaMalloc(&p, sizeof(int)));
    CANDMC_CK(cudaMemset(p, 0, sizeof(int)));
    g_bstatus[dev] = p;
  }
  *out = g_bstatus[dev];
  return CANDMC_OK;
}
// arithmetic form of the panels' own half-panel updates in batched calls
// (tuning knob "batched_form"): emulated FP64 on the tensor cores for panels
// of at least "panel_oz_min_rows" rows (the default), or FP64
int g_batched_form = CANDMC_PREC_OZAKI;
static std::mutex g_graph_mu;
struct CachedGraph {
  cudaGraphExec_t exec;
  long long kernels;   // kernel nodes: launches per replay
};
static std::map<std::vector<int64_t>, CachedGraph> g_graphs;

static long long kernel_nodes(cudaGraph_t g) {
  size_t n = 0;
  if (cudaGraphGetNodes(g, nullptr, &n) != cudaSuccess || n == 0) return 0;
  std::vector<cudaGraphNode_t> nodes(n);
  if (cudaGraphGetNodes(g, nodes.data(), &n) != cudaSuccess) return 0;
  long long k = 0;
  for (auto nd : nodes) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++k;
  }
  return k;
}

static int batched_issue(int64_t nprob, const int64_t* m, const int64_t* n, double* const* A,
                         const int64_t* lda, double* const* B, int nstreams, cudaStream_t s) {
  int dev = 0;
  CANDMC_CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return set_error(CANDMC_ERR_ARG, "device index");
  std::vector<int64_t> order(nprob);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
    return (double)m[a] * n[a] * n[a] > (double)m[b] * n[b] * n[b];
  });
  int64_t tsz = 0;
  std::vector<int64_t> toff(nprob);
  for (int64_t i = 0; i < nprob; ++i) {
    toff[i] = tsz;
    tsz += n[i] * n[i];
  }
  DevBuf tbuf;
  CANDMC_RET(tbuf.alloc(sizeof(double) * std::max<int64_t>(tsz, 1), s));
  int* stword = nullptr;
  CANDMC_RET(batched_status_word(dev, &stword));
  cudaEvent_t fork;
  CANDMC_CK(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
  CANDMC_CK(cudaEventRecord(fork, s));
  std::vector<cudaEvent_t> joins;
  const int ns = std::max(1, std::min<int>(nstreams, (int)nprob));
  int rc = CANDMC_OK;
  for (int k = 0; k < ns && rc == CANDMC_OK; ++k) {
    cudaStream_t sk = g_pool[dev].get(k);
    if (!sk) { rc = set_error(CANDMC_ERR_CUDA, "stream pool"); break; }
    if (cudaStreamWaitEvent(sk, fork, 0) != cudaSuccess) { rc = CANDMC_ERR_CUDA; break; }
    for (int64_t q = k; q < nprob; q += ns) {
      const int64_t i = order[q];
      double* T = tbuf.d() + toff[i];
      rc = hr_rec(A[i], lda[i], m[i], (int)n[i], T, n[i], stword, g_batched_form, sk);
      if (rc != CANDMC_OK) break;
      rc = apply_qt(A[i], lda[i], m[i], (int)n[i], T, n[i], B[i], m[i], 1, CANDMC_PREC_FP64, sk);
      if (rc != CANDMC_OK) break;
      {
        ProfScope ps(CANDMC_KCLASS_SMALL, (double)n[i] * n[i], sk);
        k_trsv_upper<<<1, 32, 0, sk>>>(A[i], lda[i], (int)n[i], B[i]);
      }
      if (cudaGetLastError() != cudaSuccess) { rc = CANDMC_ERR_CUDA; break; }
    }
    cudaEvent_t j;
    if (cudaEventCreateWithFlags(&j, cudaEventDisableTiming) != cudaSuccess) { rc = CANDMC_ERR_CUDA; break; }
    joins.push_back(j);
    if (cudaEventRecord(j, sk) != cudaSuccess) rc = CANDMC_ERR_CUDA;
  }
  for (auto j : joins) {
    cudaStreamWaitEvent(s, j, 0);
    cudaEventDestroy(j);
  }
  cudaEventDestroy(fork);
  return rc;
}

}  // namespace candmc

using namespace candmc;

extern "C" int candmc_batched_status(void* stream, int* status) {
  if (!status) return set_error(CANDMC_ERR_ARG, "batched_status args");
  int dev = 0, *w = nullptr;
  CANDMC_CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return set_error(CANDMC_ERR_ARG, "device index");
  CANDMC_RET(batched_status_word(dev, &w));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  CANDMC_CK(cudaMemcpyAsync(status, w, sizeof(int), cudaMemcpyDeviceToHost, s));
  CANDMC_CK(cudaStreamSynchronize(s));
  CANDMC_CK(cudaMemsetAsync(w, 0, sizeof(int), s));
  CANDMC_CK(cudaStreamSynchronize(s));
  return CANDMC_OK;
}

extern "C" int candmc_set_tuning(const char* key, int64_t value) {
  if (!key) return set_error(CANDMC_ERR_ARG, "tuning key");
  if (std::string(key) == "leaf_rows") {
    if (value < 32 || value > 256) return set_error(CANDMC_ERR_ARG, "leaf_rows in [32, 256]");
    g_leaf_rows = value;
    return CANDMC_OK;
  }
  if (std::string(key) == "oz_reserve_sms") {
    if (value < 0 || value > 144) return set_error(CANDMC_ERR_ARG, "oz_reserve_sms in [0, 144]");
    g_oz_reserve_sms = (int)value;
    return CANDMC_OK;
  }
  if (std::string(key) == "pipe_leaf_rows") {
    if (value < 32 || value > 256) return set_error(CANDMC_ERR_ARG, "pipe_leaf_rows in [32, 256]");
    g_pipe_leaf_rows = value;
    return CANDMC_OK;
  }
  if (std::string(key) == "batched_form") {
    if (value != CANDMC_PREC_FP64 && value != CANDMC_PREC_OZAKI)
      return set_error(CANDMC_ERR_ARG, "batched_form is CANDMC_PREC_FP64 or CANDMC_PREC_OZAKI");
    g_batched_form = (int)value;
    return CANDMC_OK;
  }
  if (std::string(key) == "ls_refine") {
    if (value != 0 && value != 1) return set_error(CANDMC_ERR_ARG, "ls_refine is 0 or 1");
    g_ls_refine = (int)value;
    return CANDMC_OK;
  }
  if (std::string(key) == "panel_oz_min_rows") {
    if (value < 0) return set_error(CANDMC_ERR_ARG, "panel_oz_min_rows >= 0 (0 disables)");
    g_panel_oz_min_rows = value;
    return CANDMC_OK;
  }
  if (std::string(key) == "pipe_tree") {
    if (value != 0 && value != 1) return set_error(CANDMC_ERR_ARG, "pipe_tree is 0 or 1");
    g_pipe_tree = (int)value;
    return CANDMC_OK;
  }
  return set_error(CANDMC_ERR_ARG, "unknown tuning key");
}

extern "C" int candmc_batched_ls(int64_t nprob, const int64_t* m, const int64_t* n, double* const* A,
                                 const int64_t* lda, double* const* B, int nstreams, int use_graph,
                                 void* stream) {
  if (nprob < 0 || (nprob > 0 && (!m || !n || !A || !lda || !B)))
    return set_error(CANDMC_ERR_ARG, "batched_ls args");
  for (int64_t i = 0; i < nprob; ++i)
    if (n[i] < 1 || n[i] > 128 || m[i] < n[i] || lda[i] < m[i] || !A[i] || !B[i])
      return set_error(CANDMC_ERR_ARG, "batched_ls: each problem needs 1 <= n <= 128 and m >= n");
  if (nprob == 0) return CANDMC_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  {
    int dev = 0, *w = nullptr;
    CANDMC_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return set_error(CANDMC_ERR_ARG, "device index");
    CANDMC_RET(batched_status_word(dev, &w));   // before any capture begins
  }
  if (!use_graph) return batched_issue(nprob, m, n, A, lda, B, nstreams, s);
  std::vector<int64_t> key;
  key.reserve(6 * nprob + 4);
  key.push_back(nprob);
  key.push_back(nstreams);
  key.push_back(g_leaf_rows);
  key.push_back(g_pipe_tree);
  key.push_back(g_batched_form);
  key.push_back(g_panel_oz_min_rows);
  for (int64_t i = 0; i < nprob; ++i) {
    key.push_back(m[i]);
    key.push_back(n[i]);
    key.push_back(lda[i]);
    key.push_back((int64_t)(uintptr_t)A[i]);
    key.push_back((int64_t)(uintptr_t)B[i]);
  }
  // the schedule is captured on (and replayed from) a stream of the library's
  // own, joined to the caller's stream by events, so the caller's stream may be
  // the legacy default stream (which cannot be captured)
  int dev = 0;
  CANDMC_CK(cudaGetDevice(&dev));
  cudaStream_t cs = g_pool[dev].get(63);
  if (!cs) return set_error(CANDMC_ERR_CUDA, "capture stream");
  cudaGraphExec_t exec = nullptr;
  long long nkern = 0;
  {
    std::lock_guard<std::mutex> g(g_graph_mu);
    auto it = g_graphs.find(key);
    if (it != g_graphs.end()) {
      exec = it->second.exec;
      nkern = it->second.kernels;
    }
  }
  if (!exec) {
    // kernel attributes are set by an eager run first (not a stream operation)
    cudaGraph_t graph = nullptr;
    CANDMC_CK(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    int rc = batched_issue(nprob, m, n, A, lda, B, nstreams, cs);
    cudaError_t e = cudaStreamEndCapture(cs, &graph);
    if (rc != CANDMC_OK) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    CANDMC_CK(e);
    // the capture counted its launches although nothing ran; each replay
    // counts the graph's kernel nodes instead
    nkern = kernel_nodes(graph);
    count_launches(-nkern);
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    CANDMC_CK(e);
    std::lock_guard<std::mutex> g(g_graph_mu);
    g_graphs[key] = {exec, nkern};
  }
  cudaEvent_t e0, e1;
  CANDMC_CK(cudaEventCreateWithFlags(&e0, cudaEventDisableTiming));
  CANDMC_CK(cudaEventCreateWithFlags(&e1, cudaEventDisableTiming));
  cudaError_t e = cudaEventRecord(e0, s);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(cs, e0, 0);
  if (e == cudaSuccess) e = cudaGraphLaunch(exec, cs);
  if (e == cudaSuccess) count_launches(nkern);
  if (e == cudaSuccess) e = cudaEventRecord(e1, cs);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(s, e1, 0);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  CANDMC_CK(e);
  return CANDMC_OK;
}

// ---- float32 inputs --------------------------------------------------------
// The FP32-input variant of the batched solve: A_i and b_i arrive as float32;
// they are widened into an FP64 work area on the device, solved exactly as
// candmc_batched_ls solves FP64 problems (TSQR-HR, Q^T b, back substitution,
// all FP64), and x_i is rounded back into b_i's first n_i entries.  The work
// area is kept per device and grows on demand, so repeated calls with the same
// sizes reuse it (and a captured graph of the FP64 solve stays valid).
namespace candmc {

__global__ void k_widen_batch(int64_t nprob, const float* const* src, const int64_t* ld, const int64_t* rows,
                              const int64_t* cols, const int64_t* off, double* dst) {
  const int64_t p = blockIdx.y;
  if (p >= nprob) return;
  const int64_t r = rows[p], c = cols[p], l = ld[p];
  const float* a = src[p];
  double* d = dst + off[p];
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < r * c; e += (int64_t)gridDim.x * blockDim.x)
    d[e] = (double)a[(e / r) * l + e % r];
}

__global__ void k_narrow_x(int64_t nprob, const double* src, const int64_t* off, const int64_t* n,
                           float* const* dst) {
  const int64_t p = blockIdx.x;
  if (p >= nprob) return;
  for (int64_t e = threadIdx.x; e < n[p]; e += blockDim.x) dst[p][e] = (float)src[off[p] + e];
}

struct F32Work {
  double* d = nullptr;
  size_t cap = 0;      // doubles
  void* meta = nullptr;
  size_t meta_cap = 0; // bytes
  cudaEvent_t done = nullptr;  // end of the last call that used this area
};
static F32Work g_f32[64];
static std::mutex g_f32_mu;

}  // namespace candmc

extern "C" int candmc_batched_ls_f32(int64_t nprob, const int64_t* m, const int64_t* n, float* const* A,
                                     const int64_t* lda, float* const* B, int nstreams, int use_graph,
                                     void* stream) {
  if (nprob < 0 || (nprob > 0 && (!m || !n || !A || !lda || !B)))
    return set_error(CANDMC_ERR_ARG, "batched_ls_f32 args");
  for (int64_t i = 0; i < nprob; ++i)
    if (n[i] < 1 || n[i] > 128 || m[i] < n[i] || lda[i] < m[i] || !A[i] || !B[i])
      return set_error(CANDMC_ERR_ARG, "batched_ls_f32: each problem needs 1 <= n <= 128 and m >= n");
  if (nprob == 0) return CANDMC_OK;
  if (nprob > 65535) return set_error(CANDMC_ERR_ARG, "batched_ls_f32: at most 65535 problems per call");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int dev = 0;
  CANDMC_CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return set_error(CANDMC_ERR_ARG, "device index");
  // FP64 work area: A_i (m_i x n_i, ld m_i) then b_i (m_i), 32-double aligned
  std::vector<int64_t> offA(nprob), offB(nprob), ones(nprob, 1), ldw(nprob);
  size_t tot = 0;
  for (int64_t i = 0; i < nprob; ++i) {
    offA[i] = (int64_t)tot;
    tot += ((size_t)(m[i] * n[i]) + 31) & ~(size_t)31;
  }
  for (int64_t i = 0; i < nprob; ++i) {
    offB[i] = (int64_t)tot;
    tot += ((size_t)m[i] + 31) & ~(size_t)31;
    ldw[i] = m[i];
  }
  const size_t meta_bytes = sizeof(int64_t) * 8 * (size_t)nprob + sizeof(void*) * 2 * (size_t)nprob;
  std::lock_guard<std::mutex> lock(g_f32_mu);
  F32Work& w = g_f32[dev];
  if (!w.done) CANDMC_CK(cudaEventCreateWithFlags(&w.done, cudaEventDisableTiming));
  // the previous call may have run on another stream: its solve must finish
  // before this one rewrites the work area and the tables
  CANDMC_CK(cudaEventSynchronize(w.done));
  if (w.cap < tot) {
    CANDMC_CK(cudaStreamSynchronize(s));
    if (w.d) cudaFree(w.d);
    w.d = nullptr;
    w.cap = 0;
    CANDMC_CK(cudaMalloc(&w.d, sizeof(double) * tot));
    w.cap = tot;
  }
  if (w.meta_cap < meta_bytes) {
    CANDMC_CK(cudaStreamSynchronize(s));
    if (w.meta) cudaFree(w.meta);
    w.meta = nullptr;
    w.meta_cap = 0;
    CANDMC_CK(cudaMalloc(&w.meta, meta_bytes));
    w.meta_cap = meta_bytes;
  }
  // device tables: rows, cols, ld, offsets of A and b, ones, pointers
  std::vector<unsigned char> h(meta_bytes);
  int64_t* hi = reinterpret_cast<int64_t*>(h.data());
  for (int64_t i = 0; i < nprob; ++i) {
    hi[i] = m[i];
    hi[nprob + i] = n[i];
    hi[2 * nprob + i] = lda[i];
    hi[3 * nprob + i] = offA[i];
    hi[4 * nprob + i] = offB[i];
    hi[5 * nprob + i] = 1;
    hi[6 * nprob + i] = 1;   // ld of b as a column
  }
  const float** hp = reinterpret_cast<const float**>(h.data() + sizeof(int64_t) * 8 * nprob);
  for (int64_t i = 0; i < nprob; ++i) {
    hp[i] = A[i];
    hp[nprob + i] = B[i];
  }
  CANDMC_CK(cudaMemcpyAsync(w.meta, h.data(), meta_bytes, cudaMemcpyHostToDevice, s));
  CANDMC_CK(cudaStreamSynchronize(s));   // h is pageable and goes out of scope
  const int64_t* dm = static_cast<const int64_t*>(w.meta);
  const int64_t* dn = dm + nprob;
  const int64_t* dl = dm + 2 * nprob;
  const int64_t* doA = dm + 3 * nprob;
  const int64_t* doB = dm + 4 * nprob;
  const int64_t* d1 = dm + 5 * nprob;
  const float* const* dpA = reinterpret_cast<const float* const*>(static_cast<char*>(w.meta) + sizeof(int64_t) * 8 * nprob);
  const float* const* dpB = dpA + nprob;
  {
    ProfScope ps(CANDMC_KCLASS_SMALL, 12.0 * (double)tot, s);
    k_widen_batch<<<dim3(256, (unsigned)nprob), 256, 0, s>>>(nprob, dpA, dl, dm, dn, doA, w.d);
    k_widen_batch<<<dim3(64, (unsigned)nprob), 256, 0, s>>>(nprob, dpB, dm, dm, d1, doB, w.d);
  }
  CANDMC_CK(cudaGetLastError());
  std::vector<double*> Ad(nprob), Bd(nprob);
  for (int64_t i = 0; i < nprob; ++i) {
    Ad[i] = w.d + offA[i];
    Bd[i] = w.d + offB[i];
  }
  CANDMC_RET(candmc_batched_ls(nprob, m, n, Ad.data(), ldw.data(), Bd.data(), nstreams, use_graph, s));
  {
    ProfScope ps(CANDMC_KCLASS_SMALL, 0.0, s);
    k_narrow_x<<<(unsigned)nprob, 128, 0, s>>>(nprob, w.d, doB, dn, const_cast<float* const*>(dpB));
  }
  CANDMC_CK(cudaGetLastError());
  CANDMC_CK(cudaEventRecord(w.done, s));
  return CANDMC_OK;
}
