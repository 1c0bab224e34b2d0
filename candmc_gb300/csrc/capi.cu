// C ABI and host orchestration of the QR hot path (include/candmc_gb300.h).
//
// hh_recon_qr is computed by recursive column blocking: a panel wider than
// kDirectB is split in two halves; the left half is reconstructed, the right
// half receives the left half's Q^T, the lower part of the right half is
// reconstructed, and the two compact-WY factors are merged
// (T12 = -T11 * Y1^T Y2 * T22, LAPACK dlarft's block form).  The blocked
// Householder factor equals the unblocked one in exact arithmetic (it is
// what LAPACK's blocked dgeqrf relies on), so the output is the same
// canonical (Y, T, S*R) as the reference's single-panel reconstruction
// (alg/QR/hh_recon/hh_recon.cxx:129-321), while the FP64 tree-node work stays
// at 32-column nodes.
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "kernels.cuh"

namespace candmc {

static thread_local std::string g_last_error;

int64_t g_panel_oz_min_rows = 8192;

int set_error(int code, const char* what) {
  g_last_error = what ? what : "";
  return code;
}

int cuda_status(cudaError_t e, const char* where) {
  g_last_error = std::string(where) + ": " + cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return CANDMC_ERR_ALLOC;
  return CANDMC_ERR_CUDA;
}

// Once per device: keep freed stream-ordered scratch in the device's default
// pool instead of returning it to the CUDA driver at every synchronisation, so a
// repeated factorization reuses its scratch without re-mapping memory.
static void ensure_pool() {
  static std::atomic<bool> done[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64 || done[dev].load()) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t thr = ~0ull;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  done[dev] = true;
}

int DevBuf::alloc(size_t bytes, cudaStream_t stream) {
  s = stream;
  ensure_pool();
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMallocAsync(&p, bytes, stream);
  if (e != cudaSuccess) {
    p = nullptr;
    return cuda_status(e, "cudaMallocAsync");
  }
  return CANDMC_OK;
}

DevBuf::~DevBuf() {
  if (p) cudaFreeAsync(p, s);
}

// Per-call device status word.
struct Status {
  DevBuf buf;
  int init(cudaStream_t s) {
    CANDMC_RET(buf.alloc(sizeof(int), s));
    CANDMC_CK(cudaMemsetAsync(buf.p, 0, sizeof(int), s));
    return CANDMC_OK;
  }
  int* p() { return static_cast<int*>(buf.p); }
  int check(cudaStream_t s) {
    int h = 0;
    CANDMC_CK(cudaMemcpyAsync(&h, buf.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    CANDMC_CK(cudaStreamSynchronize(s));
    return h;
  }
};

// C <- (I - Y T Y^T)^T C = C - Y * (T^T * (Y^T * C))
int apply_qt(const double* Y, int64_t ldy, int64_t m, int nb, const double* T, int64_t ldT,
             double* C, int64_t ldc, int64_t n, int precision, cudaStream_t s);

// Recursive blocked TSQR-HR (see file comment).  T (ldT) receives the b x b
// upper-triangular factor; the strictly lower part of T is zeroed.
int hr_rec(double* A, int64_t lda, int64_t m, int b, double* T, int64_t ldT, int* st,
                  int precision, cudaStream_t s) {
  if (b <= kDirectB) return hr_direct4(A, lda, m, b, T, ldT, nullptr, 0, st, s);
  const int b1 = b / 2, b2 = b - b1;
  CANDMC_RET(hr_rec(A, lda, m, b1, T, ldT, st, precision, s));
  // Q1^T on the right half.  The reflectors, norms, tree and T stay FP64;
  // this m x b/2 x b/2 product is a trailing update, so in the tensor-core
  // forms (emulated FP64, and FP32, whose panels keep FP64-class accuracy) on
  // tall panels, where its FP64 cost is on the panel's critical path, it runs
  // in emulated FP64 on the tensor cores with the panel kept in FP64 storage.
  const bool oz = precision != CANDMC_PREC_FP64 && g_panel_oz_min_rows > 0 && m >= g_panel_oz_min_rows;
  if (oz)
    CANDMC_RET(apply_qt_ozaki(A, lda, kUnitLower, m, b1, mref(T, ldT, 1, kUpper), A + (int64_t)b1 * lda,
                              lda, b2, m, st, s, true));
  else
    CANDMC_RET(apply_qt(A, lda, m, b1, T, ldT, A + (int64_t)b1 * lda, lda, b2, CANDMC_PREC_FP64, s));
  double* T22 = T + (int64_t)b1 * ldT + b1;
  CANDMC_RET(hr_rec(A + (int64_t)b1 * lda + b1, lda, m - b1, b2, T22, ldT, st, precision, s));
  // G = Y1[b1:m, :]^T * Y2   (Y2 unit-lower in A[b1:, b1:]); with the half
  // update on the tensor cores, this (m - b1) x b1 x b2 product goes there too
  DevBuf g, x;
  CANDMC_RET(g.alloc(sizeof(double) * b1 * b2, s));
  CANDMC_RET(x.alloc(sizeof(double) * b1 * b2, s));
  if (oz)
    CANDMC_RET(gram_ozaki(A + b1, lda, kDense, A + (int64_t)b1 * lda + b1, lda, kUnitLower, m - b1, b1, b2,
                          g.d(), st, s));
  else
    CANDMC_RET(gemm_tn_reduce(mref(A + b1, lda), mref(A + (int64_t)b1 * lda + b1, lda, 0, kUnitLower),
                              m - b1, b1, b2, mref(nullptr, 0), 1.0, g.d(), b1, s));
  // X = T11 * G;  T12 = -X * T22
  CANDMC_RET(small_gemm(b1, b2, b1, 1.0, mref(T, ldT, 0, kUpper), mref(g.d(), b1), 0.0, x.d(), b1, s));
  CANDMC_RET(small_gemm(b1, b2, b2, -1.0, mref(x.d(), b1), mref(T22, ldT, 0, kUpper), 0.0,
                        T + (int64_t)b1 * ldT, ldT, s));
  CANDMC_CK(cudaMemset2DAsync(T + b1, sizeof(double) * ldT, 0, sizeof(double) * b2, b1, s));
  return CANDMC_OK;
}

int apply_qt(const double* Y, int64_t ldy, int64_t m, int nb, const double* T, int64_t ldT,
             double* C, int64_t ldc, int64_t n, int precision, cudaStream_t s) {
  if (n <= 0 || m <= 0) return CANDMC_OK;
  if (precision != CANDMC_PREC_FP64) return set_error(CANDMC_ERR_ARG, "precision form not built");
  DevBuf z;
  CANDMC_RET(z.alloc(sizeof(double) * (size_t)nb * n, s));
  MatRef Ym = mref(Y, ldy, 0, kUnitLower);
  CANDMC_RET(gemm_tn_reduce(Ym, mref(C, ldc), m, nb, n, mref(T, ldT, 1, kUpper), 1.0, z.d(), nb, s));
  CANDMC_RET(gemm_nn_sub(C, ldc, Ym, z.d(), nb, m, n, nb, s));
  return CANDMC_OK;
}

// Top-level TSQR-HR with optional W = -T * Y1^T (ld ldW) and T (ld ldT).
static int hh_recon_dev(double* A, int64_t lda, int64_t m, int64_t b, double* W, int64_t ldW,
                        double* T, int64_t ldT, int* st, int precision, cudaStream_t s) {
  DevBuf tb;
  if (!T) {
    CANDMC_RET(tb.alloc(sizeof(double) * b * b, s));
    T = tb.d();
    ldT = b;
  }
  if (b <= kDirectB) return hr_direct4(A, lda, m, (int)b, T, ldT, W, ldW, st, s);
  CANDMC_RET(hr_rec(A, lda, m, (int)b, T, ldT, st, precision, s));
  if (W) {
    CANDMC_RET(small_gemm(b, b, b, -1.0, mref(T, ldT, 0, kUpper), mref(A, lda, 1, kUnitLower), 0.0,
                          W, ldW, s));
  }
  return CANDMC_OK;
}

// Tᵀ-application factor for upd_A's W conventions (qr_2d.cxx:242-253):
// returns Top (b x b lower, ld b) with Top = T^T.
static int top_from_W(const double* Y, int64_t ldy, int64_t mb, int64_t b, const double* W,
                      int W_is_T, int ymask, double* Top, cudaStream_t s) {
  DevBuf x;
  CANDMC_RET(x.alloc(sizeof(double) * b * b, s));
  if (W == nullptr) {
    // T^-T = stril(Y^T Y) with halved diagonal, T^T = (T^-T)^-1
    CANDMC_RET(gemm_tn_reduce(mref(Y, ldy, 0, ymask), mref(Y, ldy, 0, ymask), mb, (int)b, b,
                              mref(nullptr, 0), 1.0, x.d(), b, s));
    CANDMC_CK(cudaMemsetAsync(Top, 0, sizeof(double) * b * b, s));
    CANDMC_RET(invT_from_gram(x.d(), b, (int)b, Top, b, s));
    CANDMC_CK(cudaMemcpyAsync(x.d(), Top, sizeof(double) * b * b, cudaMemcpyDeviceToDevice, s));
    CANDMC_RET(tri_inv(x.d(), b, (int)b, 1, 0, Top, b, s));
  } else if (W_is_T) {
    CANDMC_RET(tri_inv(W, b, (int)b, 1, 0, Top, b, s));
  } else {
    // T^-T = -W^-T Y1  =>  T^T = -Y1^-1 W^T
    CANDMC_RET(tri_inv(Y, ldy, (int)b, 1, 1, x.d(), b, s));
    CANDMC_RET(small_gemm(b, b, b, -1.0, mref(x.d(), b, 0, kLower), mref(W, b, 1, kUpper), 0.0,
                          Top, b, s));
  }
  return CANDMC_OK;
}

static int upd_core(const double* Y, int64_t ldy, int ymask, double* A, int64_t lda, int64_t mb,
                    int64_t kb, int64_t b, const double* W, int W_is_T, int precision,
                    cudaStream_t s) {
  if (mb <= 0 || kb <= 0) return CANDMC_OK;
  if (precision != CANDMC_PREC_FP64 && precision != CANDMC_PREC_OZAKI && precision != CANDMC_PREC_FP32)
    return set_error(CANDMC_ERR_ARG, "unknown precision form");
  DevBuf top, z;
  CANDMC_RET(top.alloc(sizeof(double) * b * b, s));
  CANDMC_RET(top_from_W(Y, ldy, mb, b, W, W_is_T, ymask, top.d(), s));
  if (precision != CANDMC_PREC_FP64) {
    if (b > 128) return set_error(CANDMC_ERR_ARG, "the ozaki and fp32 forms need b <= 128");
    Status st;
    CANDMC_RET(st.init(s));
    CANDMC_RET(to_df64(A, lda, mb, kb, s));
    if (precision == CANDMC_PREC_OZAKI)
      CANDMC_RET(apply_qt_ozaki(Y, ldy, ymask, mb, (int)b, mref(top.d(), b, 0, kLower), A, lda, kb, 0,
                                st.p(), s));
    else
      CANDMC_RET(apply_qt_f32(Y, ldy, ymask, mb, (int)b, mref(top.d(), b, 0, kLower), A, lda, kb, 0,
                              st.p(), s));
    return from_df64(A, lda, mb, kb, s);
  }
  CANDMC_RET(z.alloc(sizeof(double) * b * kb, s));
  MatRef Ym = mref(Y, ldy, 0, ymask);
  CANDMC_RET(gemm_tn_reduce(Ym, mref(A, lda), mb, (int)b, kb, mref(top.d(), b, 0, kLower), 1.0,
                            z.d(), b, s));
  CANDMC_RET(gemm_nn_sub(A, lda, Ym, z.d(), b, mb, kb, (int)b, s));
  return CANDMC_OK;
}

// Trailing update of columns [c0, c0 + n) of the block whose panel starts at P
// (Y in P's Y\R, T upper), in the requested arithmetic.  In the emulated form
// the columns hold df64 pairs and their top b rows are written back as FP64.
static int update_cols(double* P, int64_t lda, int64_t mm, int64_t b, const double* T, int64_t c0,
                       int64_t n, int* st, int precision, cudaStream_t s) {
  if (n <= 0) return CANDMC_OK;
  double* C = P + c0 * lda;
  if (precision == CANDMC_PREC_OZAKI)
    return apply_qt_ozaki(P, lda, kUnitLower, mm, (int)b, mref(T, b, 1, kUpper), C, lda, n, b, st, s);
  if (precision == CANDMC_PREC_FP32)
    return apply_qt_f32(P, lda, kUnitLower, mm, (int)b, mref(T, b, 1, kUpper), C, lda, n, b, st, s);
  return apply_qt(P, lda, mm, (int)b, T, b, C, lda, n, precision, s);
}

// The ozaki and fp32 forms keep the unfactored part as df64 pairs.
static int check_form(int precision, int64_t b, bool* pair) {
  *pair = (precision == CANDMC_PREC_OZAKI || precision == CANDMC_PREC_FP32);
  if (precision != CANDMC_PREC_FP64 && !*pair) return set_error(CANDMC_ERR_ARG, "unknown precision form");
  if (*pair && b > 128) return set_error(CANDMC_ERR_ARG, "the ozaki and fp32 forms need b <= 128");
  return CANDMC_OK;
}

// High-priority, non-blocking side stream per device for the lookahead panels.
static int device_sms() {
  static std::atomic<int> n{0};
  if (n.load() == 0) {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    n = v > 0 ? v : 148;
  }
  return n.load();
}

// One lookahead stream per host thread and device, so that factorizations
// issued concurrently from several threads (the request server's workers) do
// not queue their panels behind one another.
struct PanelStreams {
  cudaStream_t sp[64] = {};
  ~PanelStreams() {
    for (auto s : sp)
      if (s) cudaStreamDestroy(s);
  }
};

static cudaStream_t panel_stream() {
  static thread_local PanelStreams ps;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  if (!ps.sp[dev]) {
    int lo = 0, hi = 0;
    cudaDeviceGetStreamPriorityRange(&lo, &hi);
    if (cudaStreamCreateWithPriority(&ps.sp[dev], cudaStreamNonBlocking, hi) != cudaSuccess)
      ps.sp[dev] = nullptr;
  }
  return ps.sp[dev];
}

struct EventRing {
  std::vector<cudaEvent_t> ev;
  ~EventRing() {
    for (auto e : ev) cudaEventDestroy(e);
  }
  int make(cudaEvent_t* out) {
    cudaEvent_t e;
    CANDMC_CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    ev.push_back(e);
    *out = e;
    return CANDMC_OK;
  }
};

// QR_2D_pipe on one GPU (alg/QR/qr_2d/qr_2d.cxx:378-635): the lookahead
// pipeline of the reference, with the process columns replaced by two
// streams.  Panel i+1 is factored on a high-priority side stream while the
// bulk of panel i's trailing update runs on the caller's stream:
//   side: HR(i); wait(A_{i-1}); U_next(i) = Q_i^T on panel i+1's columns; HR(i+1) ...
//   main: wait(HR(i)); A_i = Q_i^T on panel i+2's columns (recorded); Q_i^T on the rest
// Every column block receives Q_0^T .. Q_{i}^T in order, so the result is the
// same factorization as QR_2D.
int qr_2d_pipe_dev(double* A, int64_t lda, int64_t m, int64_t k, int64_t b, int* st, int precision,
                   cudaStream_t s, double* Tall) {
  bool oz;
  CANDMC_RET(check_form(precision, b, &oz));
  // keep some SMs free of the persistent trailing-update CTAs for the panel stream
  // and factor its panels with taller leaves (fewer CTAs compete with the update)
  struct CapScope {
    int saved;
    int64_t saved_leaf;
    CapScope(int cap, int64_t leaf) : saved(t_oz_cap), saved_leaf(t_leaf_rows) {
      t_oz_cap = cap;
      t_leaf_rows = leaf;
    }
    ~CapScope() {
      t_oz_cap = saved;
      t_leaf_rows = saved_leaf;
    }
  } cap_scope(g_oz_reserve_sms > 0 ? std::max(1, device_sms() - g_oz_reserve_sms) : 0, g_pipe_leaf_rows);
  cudaStream_t sp = panel_stream();
  if (!sp) return set_error(CANDMC_ERR_CUDA, "could not create the lookahead stream");
  EventRing evs;
  DevBuf tbuf;   // ring of three T factors, or every panel's T (Tall: b x b per panel)
  if (!Tall) CANDMC_RET(tbuf.alloc(sizeof(double) * 3 * b * b, s));
  auto tslot = [&](int64_t i) { return Tall ? Tall + i * b * b : tbuf.d() + (i % 3) * b * b; };
  cudaEvent_t e_start;
  CANDMC_RET(evs.make(&e_start));
  if (oz) CANDMC_RET(to_df64(A, lda, m, k, s));
  CANDMC_CK(cudaEventRecord(e_start, s));
  CANDMC_CK(cudaStreamWaitEvent(sp, e_start, 0));
  const int64_t npan = (k + b - 1) / b;
  cudaEvent_t e_prevA = nullptr;   // main stream finished Q_{i-1}^T on panel i+1's columns
  // panel 0 on the side stream
  {
    const int64_t bb = std::min(k, b);
    if (oz) CANDMC_RET(from_df64(A, lda, m, bb, sp));
    CANDMC_RET(hr_rec(A, lda, m, (int)bb, tslot(0), b, st, precision, sp));
  }
  for (int64_t i = 0; i < npan; ++i) {
    const int64_t r0 = i * b, mm = m - r0, kk = k - r0;
    double* P = A + r0 * lda + r0;
    double* Ti = tslot(i);
    const bool trailing = (kk - b > 0 && mm - b > 0);
    cudaEvent_t e_hr;
    CANDMC_RET(evs.make(&e_hr));
    CANDMC_CK(cudaEventRecord(e_hr, sp));   // HR(i) done (it was issued on sp)
    if (!trailing) break;
    // side stream: next panel's columns, then its factorization
    const int64_t nnext = std::min(b, kk - b);
    if (e_prevA) CANDMC_CK(cudaStreamWaitEvent(sp, e_prevA, 0));
    CANDMC_RET(update_cols(P, lda, mm, b, Ti, b, nnext, st, precision, sp));
    {
      const int64_t r1 = r0 + b;
      double* P1 = A + r1 * lda + r1;
      const int64_t bb1 = std::min(k - r1, b);
      double* T1 = tslot(i + 1);
      if (oz) CANDMC_RET(from_df64(P1, lda, m - r1, bb1, sp));
      CANDMC_RET(hr_rec(P1, lda, m - r1, (int)bb1, T1, b, st, precision, sp));
    }
    // main stream: Q_i^T on panel i+2's columns (recorded), then the rest
    CANDMC_CK(cudaStreamWaitEvent(s, e_hr, 0));
    const int64_t na = std::min(b, std::max<int64_t>(0, kk - 2 * b));
    if (na > 0) {
      CANDMC_RET(update_cols(P, lda, mm, b, Ti, 2 * b, na, st, precision, s));
      cudaEvent_t ea;
      CANDMC_RET(evs.make(&ea));
      CANDMC_CK(cudaEventRecord(ea, s));
      e_prevA = ea;
    } else {
      e_prevA = nullptr;
    }
    CANDMC_RET(update_cols(P, lda, mm, b, Ti, 3 * b, kk - 3 * b, st, precision, s));
  }
  // the caller's stream waits for the side stream's last work
  cudaEvent_t e_end;
  CANDMC_RET(evs.make(&e_end));
  CANDMC_CK(cudaEventRecord(e_end, sp));
  CANDMC_CK(cudaStreamWaitEvent(s, e_end, 0));
  return CANDMC_OK;
}

static int qr_2d_dev(double* A, int64_t lda, int64_t m, int64_t k, int64_t b, double* aggreg_Y,
                     int64_t lda_aY, int* st, int precision, cudaStream_t s) {
  DevBuf tb;
  CANDMC_RET(tb.alloc(sizeof(double) * b * b, s));
  bool oz;
  CANDMC_RET(check_form(precision, b, &oz));
  // emulated and fp32 forms: the not-yet-factored part lives as df64 pairs;
  // each panel is turned back into FP64 before its reconstruction, and the
  // trailing update writes the finished R rows as FP64.
  if (oz) CANDMC_RET(to_df64(A, lda, m, k, s));
  int64_t r0 = 0;
  for (;;) {
    const int64_t mm = m - r0, kk = k - r0;
    const int64_t bb = std::min(kk, b);
    double* P = A + r0 * lda + r0;
    if (oz) CANDMC_RET(from_df64(P, lda, mm, bb, s));
    CANDMC_RET(hr_rec(P, lda, mm, (int)bb, tb.d(), b, st, precision, s));
    if (aggreg_Y)
      CANDMC_RET(materialize(mref(P, lda, 0, kUnitLower), mm, bb, aggreg_Y + r0 * lda_aY + r0,
                             lda_aY, s));
    if (kk - b > 0 && mm - b > 0) {
      CANDMC_RET(update_cols(P, lda, mm, b, tb.d(), b, kk - b, st, precision, s));
      r0 += b;
    } else {
      break;
    }
  }
  return CANDMC_OK;
}

static int device_ok() {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) return set_error(CANDMC_ERR_NODEV, "no CUDA device");
  return CANDMC_OK;
}

// Host staging helper: device copy of a column-major m x n block with leading dimension ld.
struct HostMat {
  DevBuf d;
  int64_t ldd = 0;
  int in(const double* h, int64_t ld, int64_t m, int64_t n, cudaStream_t s) {
    ldd = std::max<int64_t>(m, 1);
    CANDMC_RET(d.alloc(sizeof(double) * (size_t)ldd * std::max<int64_t>(n, 1), s));
    if (m > 0 && n > 0)
      CANDMC_CK(cudaMemcpy2DAsync(d.p, sizeof(double) * ldd, h, sizeof(double) * ld,
                                  sizeof(double) * m, n, cudaMemcpyHostToDevice, s));
    return CANDMC_OK;
  }
  int out(double* h, int64_t ld, int64_t m, int64_t n, cudaStream_t s) {
    if (m > 0 && n > 0)
      CANDMC_CK(cudaMemcpy2DAsync(h, sizeof(double) * ld, d.p, sizeof(double) * ldd,
                                  sizeof(double) * m, n, cudaMemcpyDeviceToHost, s));
    return CANDMC_OK;
  }
};


// ------------------------------------------------------- Yamamoto's representation
// Yamamoto's basis-kernel representation (alg/QR/hh_recon/yamamoto.cxx,
// alg/QR/qr_2d/qr_y2d.cxx): Q_HH^T = I + Qm W Qm^T with Qm = [Q1 - S; Q2] and
// W = (Q1 - S)^-1 S for the first b columns [Q1; Q2] of a TSQR basis.  From
// the Householder reconstruction of the panel (Y unit lower in A, W_hr = U S)
// the basis [Q1; Q2] S satisfies Q1 S - I = L W_hr, which gives
//   Qm = Y W_hr,  W = W_hr^-1 L^-1  (and S = I for that basis).
// These equal the reference's pair up to its own sign matrix S_ref
// (Qm_ref = Qm S_ref, W_ref = S_ref W S_ref); the products the
// representation is used for (Qm W Qm^T, the updates, S R) are the same.
struct YAgg {
  double* aQm;
  int64_t ld_aqm;   // rows of aQm
  double* aT;
  int64_t ld_at;    // rows of aT, columns of aQm and aT
  int64_t n;
  int64_t shift;
};

static int yamamoto_from_hr(const double* A, int64_t lda, int64_t m, int64_t b, const double* whr,
                            double* Qm, int64_t ldq, double* W, cudaStream_t s) {
  DevBuf tmp;
  CANDMC_RET(tmp.alloc(sizeof(double) * 3 * b * b, s));
  double* eye = tmp.d();
  double* negw = eye + b * b;
  double* li = negw + b * b;
  // Qm = Y W_hr, as Qm (zeroed) -= Y (-W_hr)
  CANDMC_RET(set_identity(eye, b, b, b, s));
  CANDMC_RET(small_gemm(b, b, b, -1.0, mref(eye, b), mref(whr, b, 0, kUpper), 0.0, negw, b, s));
  CANDMC_CK(cudaMemset2DAsync(Qm, sizeof(double) * ldq, 0, sizeof(double) * m, b, s));
  CANDMC_RET(gemm_nn_sub(Qm, ldq, mref(A, lda, 0, kUnitLower), negw, b, m, b, (int)b, s));
  // W = W_hr^-1 L^-1
  CANDMC_RET(tri_inv(whr, b, (int)b, 0, 0, eye, b, s));
  CANDMC_RET(tri_inv(A, lda, (int)b, 1, 1, li, b, s));
  CANDMC_RET(small_gemm(b, b, b, 1.0, mref(eye, b, 0, kUpper), mref(li, b, 0, kLower), 0.0, W, b, s));
  return CANDMC_OK;
}

// Yamamoto on one panel (yamamoto.cxx:98-174): A becomes Y\(S R), Qm (ldq) and
// W (b x b, ld b) the representation.
static int yamamoto_panel(double* A, int64_t lda, int64_t m, int64_t b, double* Qm, int64_t ldq,
                          double* W, int* st, cudaStream_t s) {
  DevBuf whr, t;
  CANDMC_RET(whr.alloc(sizeof(double) * b * b, s));
  CANDMC_RET(t.alloc(sizeof(double) * b * b, s));
  CANDMC_RET(hh_recon_dev(A, lda, m, b, whr.d(), b, t.d(), b, st, CANDMC_PREC_FP64, s));
  return yamamoto_from_hr(A, lda, m, b, whr.d(), Qm, ldq, W, s);
}

// A (mb x kb) += Qm (W (Qm^T A)) in the requested arithmetic (qr_y2d.cxx:133-178).
static int upd_yamamoto(const double* Qm, int64_t ldq, double* A, int64_t lda, int64_t mb, int64_t kb,
                        int64_t b, const double* W, int64_t ldw, int precision, cudaStream_t s) {
  if (mb <= 0 || kb <= 0) return CANDMC_OK;
  if (precision == CANDMC_PREC_FP64) {
    DevBuf z;
    CANDMC_RET(z.alloc(sizeof(double) * b * kb, s));
    CANDMC_RET(gemm_tn_reduce(mref(Qm, ldq), mref(A, lda), mb, (int)b, kb, mref(W, ldw), -1.0, z.d(),
                              b, s));
    return gemm_nn_sub(A, lda, mref(Qm, ldq), z.d(), b, mb, kb, (int)b, s);
  }
  if (precision != CANDMC_PREC_OZAKI && precision != CANDMC_PREC_FP32)
    return set_error(CANDMC_ERR_ARG, "unknown precision form");
  if (b > 128) return set_error(CANDMC_ERR_ARG, "the ozaki and fp32 forms need b <= 128");
  // the emulated contractions apply A -= Qm Top (Qm^T A): Top = -W
  DevBuf nw;
  CANDMC_RET(nw.alloc(sizeof(double) * 2 * b * b, s));
  CANDMC_RET(set_identity(nw.d() + b * b, b, b, b, s));
  CANDMC_RET(small_gemm(b, b, b, -1.0, mref(W, ldw), mref(nw.d() + b * b, b), 0.0, nw.d(), b, s));
  Status st;
  CANDMC_RET(st.init(s));
  CANDMC_RET(to_df64(A, lda, mb, kb, s));
  if (precision == CANDMC_PREC_OZAKI)
    CANDMC_RET(apply_qt_ozaki(Qm, ldq, kDense, mb, (int)b, mref(nw.d(), b), A, lda, kb, 0, st.p(), s));
  else
    CANDMC_RET(apply_qt_f32(Qm, ldq, kDense, mb, (int)b, mref(nw.d(), b), A, lda, kb, 0, st.p(), s));
  return from_df64(A, lda, mb, kb, s);
}

// aggregator::append (qr_y2d.cxx:38-66): Qm below the previous panels, and
// the new block row of the block-lower aT: [T (Qm^T aQm) aT, T].
static int yamamoto_append(YAgg* g, int64_t mb, int64_t b, const double* Qm, int64_t ldq, const double* T,
                           int64_t ldt, cudaStream_t s) {
  const int64_t n = g->n, sh = g->shift;
  if (n + b > g->ld_at || (mb > 0 && sh + mb > g->ld_aqm))
    return set_error(CANDMC_ERR_ARG, "aggregator too small for the appended panel");
  if (mb > 0)
    CANDMC_CK(cudaMemcpy2DAsync(g->aQm + n * g->ld_aqm + sh, sizeof(double) * g->ld_aqm, Qm,
                                sizeof(double) * ldq, sizeof(double) * mb, b, cudaMemcpyDeviceToDevice, s));
  if (n > 0) {
    DevBuf x;
    CANDMC_RET(x.alloc(sizeof(double) * 2 * b * n, s));
    if (mb > 0)
      CANDMC_RET(gemm_tn_reduce(mref(Qm, ldq), mref(g->aQm + sh, g->ld_aqm), mb, (int)b, n,
                                mref(nullptr, 0), 1.0, x.d(), b, s));
    else
      CANDMC_CK(cudaMemsetAsync(x.d(), 0, sizeof(double) * b * n, s));
    CANDMC_RET(small_gemm(b, n, n, 1.0, mref(x.d(), b), mref(g->aT, g->ld_at), 0.0, x.d() + b * n, b, s));
    CANDMC_RET(small_gemm(b, n, b, 1.0, mref(T, ldt), mref(x.d() + b * n, b), 0.0, g->aT + n, g->ld_at, s));
  }
  CANDMC_CK(cudaMemcpy2DAsync(g->aT + n * g->ld_at + n, sizeof(double) * g->ld_at, T, sizeof(double) * ldt,
                              sizeof(double) * b, b, cudaMemcpyDeviceToDevice, s));
  g->n += b;
  return CANDMC_OK;
}

static int yamamoto_reset(YAgg* g, cudaStream_t s) {
  CANDMC_CK(cudaMemsetAsync(g->aQm, 0, sizeof(double) * g->ld_aqm * g->ld_at, s));
  CANDMC_CK(cudaMemsetAsync(g->aT, 0, sizeof(double) * g->ld_at * g->ld_at, s));
  g->n = 0;
  g->shift = 0;
  return CANDMC_OK;
}

// QR_Yamamoto_2D on one GPU (qr_y2d.cxx:181-263).  Y below R is the panel's
// Householder Y in both settings of compute_Y: the reference writes
// Qm U^-1 (:220-240), which is that Y, and otherwise leaves its leaf
// reflectors there, which on one process are the same vectors.
static int qr_yamamoto_2d_dev(double* A, int64_t lda, int64_t m, int64_t k, int64_t b, YAgg* agg, int* st,
                              int precision, cudaStream_t s) {
  int64_t r0 = 0;
  for (;;) {
    const int64_t mm = m - r0, kk = k - r0, bb = std::min(kk, b);
    double* P = A + r0 * lda + r0;
    DevBuf qm, w;
    CANDMC_RET(qm.alloc(sizeof(double) * mm * bb, s));
    CANDMC_RET(w.alloc(sizeof(double) * bb * bb, s));
    CANDMC_RET(yamamoto_panel(P, lda, mm, bb, qm.d(), mm, w.d(), st, s));
    const bool more = kk - b > 0 && mm - b > 0;
    if (!more) {
      if (agg && mm - b >= 0) CANDMC_RET(yamamoto_append(agg, mm, bb, qm.d(), mm, w.d(), bb, s));
      break;
    }
    CANDMC_RET(upd_yamamoto(qm.d(), mm, P + bb * lda, lda, mm, kk - b, bb, w.d(), bb, precision, s));
    if (agg) {
      CANDMC_RET(yamamoto_append(agg, mm, bb, qm.d(), mm, w.d(), bb, s));
      agg->shift += b;
    }
    r0 += b;
  }
  return CANDMC_OK;
}

// QR_Yamamoto_2D_2D (qr_y2d.cxx:265-393): a b-wide block by QR_Yamamoto_2D
// with b_sub panels aggregated into one representation, which updates the
// columns beyond the block at once; the aggregator is reset, the trailing
// block recurses.
static int qr_yamamoto_2d_2d_dev(double* A, int64_t lda, int64_t m, int64_t k, int64_t b, int64_t b_sub,
                                 YAgg* agg, int* st, int precision, cudaStream_t s) {
  DevBuf aq, at;
  YAgg own{};
  int64_t r0 = 0;
  for (;;) {
    const int64_t mm = m - r0, kk = k - r0;
    double* P = A + r0 * lda + r0;
    if (!(kk - b > 0 && mm - b > 0)) return qr_yamamoto_2d_dev(P, lda, mm, kk, b_sub, agg, st, precision, s);
    if (!agg) {
      CANDMC_RET(aq.alloc(sizeof(double) * mm * b, s));
      CANDMC_RET(at.alloc(sizeof(double) * b * b, s));
      own = YAgg{aq.d(), mm, at.d(), b, 0, 0};
      CANDMC_RET(yamamoto_reset(&own, s));
      agg = &own;
    }
    CANDMC_RET(qr_yamamoto_2d_dev(P, lda, mm, std::min(kk, b), b_sub, agg, st, precision, s));
    if (agg->n < b || agg->ld_aqm < mm) return set_error(CANDMC_ERR_ARG, "aggregator too small for the block");
    CANDMC_RET(upd_yamamoto(agg->aQm, agg->ld_aqm, P + b * lda, lda, mm, kk - b, b, agg->aT, agg->ld_at,
                            precision, s));
    CANDMC_RET(yamamoto_reset(agg, s));
    r0 += b;
  }
}
}  // namespace candmc

using namespace candmc;

#define STREAM(x) static_cast<cudaStream_t>(x)

extern "C" {

const char* candmc_status_string(int status) {
  switch (status) {
    case CANDMC_OK: return "ok";
    case CANDMC_ERR_ARG: return "invalid argument";
    case CANDMC_ERR_ALLOC: return "allocation failed";
    case CANDMC_ERR_CUDA: return "CUDA error";
    case CANDMC_ERR_TIMEOUT: return "device wait timed out";
    case CANDMC_ERR_NUMERIC: return "non-finite value or zero pivot";
    case CANDMC_ERR_NODEV: return "no usable CUDA device";
    case CANDMC_ERR_CANCELLED: return "request cancelled at server shutdown";
    default: return "unknown status";
  }
}

int candmc_version(void) { return 100; }

const char* candmc_last_error(void) { return g_last_error.c_str(); }

int candmc_hh_recon_qr(double* A, int64_t lda, int64_t m, int64_t b, double* W, double* T,
                       void* stream) {
  if (!A || !W || b < 1 || m < b || lda < m) return set_error(CANDMC_ERR_ARG, "hh_recon_qr args");
  cudaStream_t s = STREAM(stream);
  Status st;
  CANDMC_RET(st.init(s));
  return hh_recon_dev(A, lda, m, b, W, b, T, b, st.p(), CANDMC_PREC_FP64, s);
}

int candmc_hh_recon_qr_host(double* A, int64_t lda, int64_t m, int64_t b, double* W, double* T) {
  if (!A || !W || b < 1 || m < b || lda < m) return set_error(CANDMC_ERR_ARG, "hh_recon_qr args");
  CANDMC_RET(device_ok());
  cudaStream_t s = nullptr;
  int rc;
  {
    HostMat dA;
    DevBuf dW, dT;
    Status st;
    CANDMC_RET(st.init(s));
    CANDMC_RET(dA.in(A, lda, m, b, s));
    CANDMC_RET(dW.alloc(sizeof(double) * b * b, s));
    CANDMC_RET(dT.alloc(sizeof(double) * b * b, s));
    CANDMC_RET(hh_recon_dev(dA.d.d(), dA.ldd, m, b, dW.d(), b, dT.d(), b, st.p(), CANDMC_PREC_FP64, s));
    CANDMC_RET(dA.out(A, lda, m, b, s));
    CANDMC_CK(cudaMemcpyAsync(W, dW.p, sizeof(double) * b * b, cudaMemcpyDeviceToHost, s));
    if (T) CANDMC_CK(cudaMemcpyAsync(T, dT.p, sizeof(double) * b * b, cudaMemcpyDeviceToHost, s));
    rc = st.check(s);
  }
  CANDMC_CK(cudaStreamSynchronize(s));
  return rc;
}

int candmc_bitree_tsqr(double* A, int64_t lda, double* R, double* tau, int64_t m, int64_t b,
                       int output_Y, void* stream) {
  if (!A || !R || !tau || b < 1 || m < b || lda < m) return set_error(CANDMC_ERR_ARG, "bitree_tsqr args");
  cudaStream_t s = STREAM(stream);
  Status st;
  CANDMC_RET(st.init(s));
  DevBuf tb, work;
  CANDMC_RET(tb.alloc(sizeof(double) * b * b, s));
  double* P = A;
  int64_t ldp = lda;
  if (!output_Y) {
    CANDMC_RET(work.alloc(sizeof(double) * m * b, s));
    CANDMC_CK(cudaMemcpy2DAsync(work.p, sizeof(double) * m, A, sizeof(double) * lda,
                                sizeof(double) * m, b, cudaMemcpyDeviceToDevice, s));
    P = work.d();
    ldp = m;
  }
  CANDMC_RET(hh_recon_dev(P, ldp, m, b, nullptr, 0, tb.d(), b, st.p(), CANDMC_PREC_FP64, s));
  CANDMC_RET(materialize(mref(P, ldp, 0, kUpper), b, b, R, b, s));
  // tau_i = T_ii
  CANDMC_CK(cudaMemcpy2DAsync(tau, sizeof(double), tb.p, sizeof(double) * (b + 1), sizeof(double),
                              b, cudaMemcpyDeviceToDevice, s));
  return CANDMC_OK;
}

// ---- tree_tsqr: QR of two stacked upper-triangular blocks ----------------
// [R1; R2] (2b x b, ld 2b).  Only the upper triangles are read; the stage
// kernel copies them into a dense 2b x b panel with zeros below, which the
// Householder reconstruction factors; the store kernel writes R over R1's
// upper triangle, the reflector block V (upper triangular) over R2's, and
// the block-diagonal T in dtpqrt's nb x b layout, leaving every strictly-
// lower entry of the caller's buffer as it was (bitree_tsqr.cxx:20-34).
__global__ void k_tree_stage(const double* A, int64_t b, double* P) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= 2 * b * b) return;
  const int64_t i = idx % (2 * b), j = idx / (2 * b);
  const int64_t r = i < b ? i : i - b;
  P[j * 2 * b + i] = (r <= j) ? A[j * 2 * b + i] : 0.0;
}

__global__ void k_tree_store(const double* P, const double* T, int64_t b, int64_t nb, double* A,
                             double* Tout) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < 2 * b * b) {
    const int64_t i = idx % (2 * b), j = idx / (2 * b);
    const int64_t r = i < b ? i : i - b;
    if (r <= j) A[j * 2 * b + i] = P[j * 2 * b + i];
  }
  if (Tout && idx < nb * b) {
    const int64_t r = idx % nb, c = idx / nb, q0 = (c / nb) * nb;
    if (q0 + r <= c) Tout[c * nb + r] = T[c * b + q0 + r];
  }
}

int candmc_tree_tsqr(double* A, int64_t b, double* T, void* stream) {
  if (!A || b < 1) return set_error(CANDMC_ERR_ARG, "tree_tsqr args");
  cudaStream_t s = STREAM(stream);
  const int64_t nb = std::min<int64_t>(b, 16);
  Status st;
  CANDMC_RET(st.init(s));
  DevBuf P, Tf;
  CANDMC_RET(P.alloc(sizeof(double) * 2 * b * b, s));
  CANDMC_RET(Tf.alloc(sizeof(double) * b * b, s));
  const unsigned grid = (unsigned)((2 * b * b + 255) / 256);
  {
    ProfScope ps(CANDMC_KCLASS_SMALL, 16.0 * b * b, s);
    k_tree_stage<<<grid, 256, 0, s>>>(A, b, P.d());
  }
  CANDMC_CK(cudaGetLastError());
  CANDMC_RET(hh_recon_dev(P.d(), 2 * b, 2 * b, b, nullptr, 0, Tf.d(), b, st.p(), CANDMC_PREC_FP64, s));
  {
    ProfScope ps(CANDMC_KCLASS_SMALL, 16.0 * b * b, s);
    k_tree_store<<<grid, 256, 0, s>>>(P.d(), Tf.d(), b, nb, A, T);
  }
  CANDMC_CK(cudaGetLastError());
  return CANDMC_OK;
}

int candmc_construct_Q1(const double* Y, int64_t ldy, const double* tau, double* Q1, int64_t ldq,
                        int64_t m, int64_t b, int64_t k, void* stream) {
  if (!Y || !tau || !Q1 || b < 1 || k < 1 || k > b || m < b || ldy < m || ldq < m)
    return set_error(CANDMC_ERR_ARG, "construct_Q1 args");
  cudaStream_t s = STREAM(stream);
  DevBuf g, t, z;
  CANDMC_RET(g.alloc(sizeof(double) * b * b, s));
  CANDMC_RET(t.alloc(sizeof(double) * b * b, s));
  CANDMC_RET(z.alloc(sizeof(double) * b * k, s));
  MatRef Ym = mref(Y, ldy, 0, kUnitLower);
  CANDMC_RET(gemm_tn_reduce(Ym, Ym, m, (int)b, b, mref(nullptr, 0), 1.0, g.d(), b, s));
  CANDMC_RET(larft_from_gram(g.d(), b, tau, (int)b, t.d(), b, s));
  // Z = T * Y[0:k, :]^T  (b x k);  Q1 = E - Y * Z
  CANDMC_RET(small_gemm(b, k, b, 1.0, mref(t.d(), b, 0, kUpper), mref(Y, ldy, 1, kUnitLower), 0.0,
                        z.d(), b, s));
  CANDMC_RET(set_identity(Q1, ldq, m, k, s));
  CANDMC_RET(gemm_nn_sub(Q1, ldq, Ym, z.d(), b, m, k, (int)b, s));
  return CANDMC_OK;
}

int candmc_apply_tsqr_QT(const double* Y, int64_t ldy, const double* tau, double* B, int64_t ldb,
                         int64_t m, int64_t b, int64_t k, void* stream) {
  if (!Y || !tau || !B || b < 1 || m < b || ldy < m || ldb < m || k < 0)
    return set_error(CANDMC_ERR_ARG, "apply_tsqr_QT args");
  if (k == 0) return CANDMC_OK;
  cudaStream_t s = STREAM(stream);
  DevBuf g, t;
  CANDMC_RET(g.alloc(sizeof(double) * b * b, s));
  CANDMC_RET(t.alloc(sizeof(double) * b * b, s));
  MatRef Ym = mref(Y, ldy, 0, kUnitLower);
  CANDMC_RET(gemm_tn_reduce(Ym, Ym, m, (int)b, b, mref(nullptr, 0), 1.0, g.d(), b, s));
  CANDMC_RET(larft_from_gram(g.d(), b, tau, (int)b, t.d(), b, s));
  return apply_qt(Y, ldy, m, (int)b, t.d(), b, B, ldb, k, CANDMC_PREC_FP64, s);
}

// tau_i = 2 / (1 + ||y_i||^2) over the structure's part of column i (0 when
// that gives 2, an empty reflector), one warp per column; the norm is a
// scaled sum of squares (max |y| first), as LAPACK's Frobenius norm scales.
__global__ void k_tau_recon(char structure, int64_t ncol, int64_t nrow, int64_t lda, const double* Y,
                            double* tau) {
  const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= ncol) return;
  int64_t r0 = 0, r1 = nrow;
  if (structure == 'L') r0 = i + 1;
  if (structure == 'U') r1 = i + 1;
  const double* y = Y + i * lda;
  double mx = 0.0;
  for (int64_t r = r0 + lane; r < r1; r += 32) mx = fmax(mx, fabs(y[r]));
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  double ss = 0.0;
  if (mx > 0.0)
    for (int64_t r = r0 + lane; r < r1; r += 32) {
      const double t = y[r] / mx;
      ss = fma(t, t, ss);
    }
  for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
  if (lane == 0) {
    const double nrm = mx * sqrt(ss);
    const double t = 2.0 / (nrm * nrm + 1.0);
    tau[i] = (t == 2.0) ? 0.0 : t;
  }
}

int candmc_tau_recon(char structure, int64_t ncol, int64_t nrow, int64_t lda, const double* Y, double* tau,
                     void* stream) {
  if ((structure != 'R' && structure != 'L' && structure != 'U') || ncol < 0 || nrow < 0 || !tau ||
      (ncol > 0 && (!Y || lda < std::max<int64_t>(nrow, 1))))
    return set_error(CANDMC_ERR_ARG, "tau_recon args");
  if (ncol == 0) return CANDMC_OK;
  cudaStream_t s = STREAM(stream);
  {
    ProfScope ps(CANDMC_KCLASS_SMALL, 8.0 * ncol * nrow, s);
    k_tau_recon<<<(unsigned)((ncol * 32 + 255) / 256), 256, 0, s>>>(structure, ncol, nrow, lda, Y, tau);
  }
  CANDMC_CK(cudaGetLastError());
  return CANDMC_OK;
}

int candmc_compute_invT_from_W(const double* W, int64_t b, double* invT, void* stream) {
  if (!W || !invT || b < 1) return set_error(CANDMC_ERR_ARG, "compute_invT_from_W args");
  cudaStream_t s = STREAM(stream);
  DevBuf wi, y1;
  CANDMC_RET(wi.alloc(sizeof(double) * b * b, s));
  CANDMC_RET(y1.alloc(sizeof(double) * b * b, s));
  CANDMC_CK(cudaMemcpyAsync(y1.p, invT, sizeof(double) * b * b, cudaMemcpyDeviceToDevice, s));
  CANDMC_RET(tri_inv(W, b, (int)b, 0, 0, wi.d(), b, s));
  // X = -W^-T * Y1
  CANDMC_RET(small_gemm(b, b, b, -1.0, mref(wi.d(), b, 1, kUpper), mref(y1.d(), b), 0.0, invT, b, s));
  return CANDMC_OK;
}

int candmc_signed_NLU(double* A, double* R, int64_t b, int64_t lda, int64_t ldr, int64_t* signs,
                      void* stream) {
  if (!A || !R || !signs || b < 1 || lda < b || ldr < b) return set_error(CANDMC_ERR_ARG, "NLU args");
  return signed_nlu(A, R, b, lda, ldr, signs, STREAM(stream));
}

int candmc_recursive_NLU(double* A, double* R, int64_t b, int64_t lda, int64_t ldr,
                         int64_t* signs, void* stream) {
  // The recursion of hh_recon.cxx:80-110 reorders the same elimination; one
  // kernel performs it directly.
  return candmc_signed_NLU(A, R, b, lda, ldr, signs, stream);
}

int candmc_compute_invT_from_Y(const double* Y, int64_t ldy, double* T, int64_t ldt, int64_t mb,
                               int64_t b, void* stream) {
  if (!Y || !T || b < 1 || mb < 0 || ldt < b) return set_error(CANDMC_ERR_ARG, "invT_from_Y args");
  cudaStream_t s = STREAM(stream);
  DevBuf g;
  CANDMC_RET(g.alloc(sizeof(double) * b * b, s));
  if (mb > 0) {
    CANDMC_RET(gemm_tn_reduce(mref(Y, ldy), mref(Y, ldy), mb, (int)b, b, mref(nullptr, 0), 1.0,
                              g.d(), b, s));
  } else {
    CANDMC_CK(cudaMemsetAsync(g.p, 0, sizeof(double) * b * b, s));
  }
  return invT_from_gram(g.d(), b, (int)b, T, ldt, s);
}

int candmc_compute_invT_from_Y2(const double* Y1, int64_t ldy1, const double* Y2, int64_t ldy2,
                                double* T, int64_t ldt, int64_t mb, int64_t b1, int64_t b2,
                                void* stream) {
  if (!Y1 || !Y2 || !T || b1 < 1 || b2 < 1 || ldt < b1) return set_error(CANDMC_ERR_ARG, "invT_from_Y2 args");
  cudaStream_t s = STREAM(stream);
  if (mb <= 0) {
    CANDMC_CK(cudaMemset2DAsync(T, sizeof(double) * ldt, 0, sizeof(double) * b1, b2, s));
    return CANDMC_OK;
  }
  return gemm_tn_reduce(mref(Y1, ldy1), mref(Y2, ldy2), mb, (int)b1, b2, mref(nullptr, 0), 1.0, T,
                        ldt, s);
}

int candmc_upd_A(const double* Y, int64_t ldy, double* A, int64_t lda, int64_t mb, int64_t kb,
                 int64_t b, const double* W, int W_is_T, int precision, void* stream) {
  if (!Y || !A || b < 1 || mb < 0 || kb < 0 || (mb > 0 && (ldy < mb || lda < mb)))
    return set_error(CANDMC_ERR_ARG, "upd_A args");
  return upd_core(Y, ldy, kDense, A, lda, mb, kb, b, W, W_is_T, precision, STREAM(stream));
}

int candmc_update_A(const double* Y, int64_t ldy, double* A, int64_t lda, int64_t m, int64_t k,
                    int64_t b, const double* W, double* aggreg_Y, int64_t lda_aY, int W_is_T,
                    int precision, void* stream) {
  if (!Y || !A || b < 1 || m < 0 || k < 0 || (m > 0 && (ldy < m || lda < m)))
    return set_error(CANDMC_ERR_ARG, "update_A args");
  cudaStream_t s = STREAM(stream);
  CANDMC_RET(upd_core(Y, ldy, kUnitLower, A, lda, m, k, b, W, W_is_T, precision, s));
  if (aggreg_Y && m > 0) CANDMC_RET(materialize(mref(Y, ldy, 0, kUnitLower), m, b, aggreg_Y, lda_aY, s));
  return CANDMC_OK;
}

int candmc_QR_2D(double* A, int64_t lda, int64_t m, int64_t k, int64_t b, double* aggreg_Y,
                 int64_t lda_aY, int precision, void* stream) {
  if (!A || b < 1 || k < 1 || m < k || lda < m) return set_error(CANDMC_ERR_ARG, "QR_2D args");
  cudaStream_t s = STREAM(stream);
  Status st;
  CANDMC_RET(st.init(s));
  return qr_2d_dev(A, lda, m, k, b, aggreg_Y, lda_aY, st.p(), precision, s);
}

int candmc_QR_2D_host(double* A, int64_t lda, int64_t m, int64_t k, int64_t b, int precision) {
  if (!A || b < 1 || k < 1 || m < k || lda < m) return set_error(CANDMC_ERR_ARG, "QR_2D args");
  CANDMC_RET(device_ok());
  cudaStream_t s = nullptr;
  int rc;
  {
    HostMat dA;
    Status st;
    CANDMC_RET(st.init(s));
    CANDMC_RET(dA.in(A, lda, m, k, s));
    // the lookahead pipeline: the same factorization as qr_2d_dev, panels overlapped
    CANDMC_RET(qr_2d_pipe_dev(dA.d.d(), dA.ldd, m, k, b, st.p(), precision, s, nullptr));
    CANDMC_RET(dA.out(A, lda, m, k, s));
    rc = st.check(s);
  }
  CANDMC_CK(cudaStreamSynchronize(s));
  return rc;
}

// Symmetric full -> band reduction (alg/SE/full_to_band.cxx:27-295, the
// first caller of QR_2D_pipe and compute_invT_from_Y outside the QR
// directory).  Per band step, with m = n - r0 - b rows below the band:
//   P = A[r0+b:, r0:r0+b]  -> CAQR in panels of b_sub, Y aggregated (:99)
//   T from Y^T Y (compute_invT_from_Y, :105),  U = Y T^T (:177)
//   W = Y^T A22 (:121),  Z = Y^T A22 Y (:160),  V' = W - Z U^T / 2 (:186)
//   A22 -= U V' + (U V')^T (:217-242), then the next step on A22.
// A22 <- Q^T A22 Q with Q = I - Y T Y^T, so A's eigenvalues are kept; the
// band (R blocks below the diagonal blocks) and the reflectors below it are
// left in the lower triangle as the reference leaves them.  The symmetric
// updates run in FP64; `precision` is the form of the panel CAQR's own
// trailing updates.
static int sym_full2band_dev(double* A, int64_t lda, int64_t n, int64_t b, int64_t b_sub, int precision,
                             cudaStream_t s) {
  int64_t r0 = 0;
  Status st;
  CANDMC_RET(st.init(s));
  DevBuf Yb, top, Ub, Ut, Wb, Zh;
  const int64_t mmax = std::max<int64_t>(n - b, 1);
  CANDMC_RET(Yb.alloc(sizeof(double) * mmax * b, s));
  CANDMC_RET(top.alloc(sizeof(double) * b * b, s));
  CANDMC_RET(Ub.alloc(sizeof(double) * mmax * b, s));
  CANDMC_RET(Ut.alloc(sizeof(double) * mmax * b, s));
  CANDMC_RET(Wb.alloc(sizeof(double) * mmax * b, s));
  CANDMC_RET(Zh.alloc(sizeof(double) * b * b, s));
  while (n - r0 > b) {
    const int64_t m = n - r0 - b;
    double* P = A + r0 * lda + r0 + b;
    double* A22 = A + (r0 + b) * lda + r0 + b;
    const int64_t bb = std::min(b, m);
    // the panel's CAQR with its reflectors aggregated into Y (m x bb, ld m)
    CANDMC_CK(cudaMemsetAsync(Yb.p, 0, sizeof(double) * m * bb, s));
    CANDMC_RET(qr_2d_dev(P, lda, m, bb, std::min(b_sub, bb), Yb.d(), m, st.p(), precision, s));
    // fewer rows than the band: the block's remaining columns receive Q^T (R trapezoidal)
    if (bb < b)
      CANDMC_RET(upd_core(Yb.d(), m, kDense, P + bb * lda, lda, m, b - bb, bb, nullptr, 0, CANDMC_PREC_FP64, s));
    // T^T from Y^T Y, U = Y T^T, U^T
    CANDMC_RET(top_from_W(Yb.d(), m, m, bb, nullptr, 0, kDense, top.d(), s));
    CANDMC_CK(cudaMemsetAsync(Ub.p, 0, sizeof(double) * m * bb, s));
    CANDMC_CK(cudaMemsetAsync(Zh.p, 0, sizeof(double) * bb * bb, s));
    // Zh = -T^T (scratch), U -= Y Zh
    CANDMC_RET(set_identity(Zh.d(), bb, bb, bb, s));
    CANDMC_RET(small_gemm(bb, bb, bb, -1.0, mref(top.d(), bb), mref(Zh.d(), bb), 0.0, Wb.d(), bb, s));
    CANDMC_RET(gemm_nn_sub(Ub.d(), m, mref(Yb.d(), m), Wb.d(), bb, m, bb, (int)bb, s));
    CANDMC_RET(materialize(mref(Ub.d(), m, 1, kDense), bb, m, Ut.d(), bb, s));
    // W = Y^T A22 (bb x m);  Zh = Y^T W^T / 2 (= Y^T A22 Y / 2)
    CANDMC_RET(gemm_tn_reduce(mref(Yb.d(), m), mref(A22, lda), m, (int)bb, m, mref(nullptr, 0), 1.0, Wb.d(),
                              bb, s));
    CANDMC_RET(gemm_tn_reduce(mref(Yb.d(), m), mref(Wb.d(), bb, 1), m, (int)bb, bb, mref(nullptr, 0), 0.5,
                              Zh.d(), bb, s));
    // V' = W - Zh U^T  (in place in W)
    CANDMC_RET(gemm_nn_sub(Wb.d(), bb, mref(Zh.d(), bb), Ut.d(), bb, bb, m, (int)bb, s));
    // A22 -= U V' + V'^T U^T
    CANDMC_RET(gemm_nn_sub(A22, lda, mref(Ub.d(), m), Wb.d(), bb, m, m, (int)bb, s));
    CANDMC_RET(gemm_nn_sub(A22, lda, mref(Wb.d(), bb, 1), Ut.d(), bb, m, m, (int)bb, s));
    r0 += b;
  }
  return st.check(s);
}

int candmc_sym_full2band(double* A, int64_t lda, int64_t n, int64_t b, int64_t b_sub, int precision,
                         void* stream) {
  if (!A || n < 1 || b < 1 || b > 256 || b_sub < 1 || b_sub > b || b % b_sub != 0 || lda < n)
    return set_error(CANDMC_ERR_ARG, "sym_full2band args (b <= 256, a multiple of b_sub)");
  bool pair;
  CANDMC_RET(check_form(precision, b_sub, &pair));
  return sym_full2band_dev(A, lda, n, b, b_sub, precision, STREAM(stream));
}

int candmc_QR_2D_2D(double* A, int64_t lda, int64_t m, int64_t k, int64_t b, int64_t b_sub,
                    double* aggreg_Y, int64_t lda_aY, int precision, void* stream) {
  if (!A || b < 1 || b_sub < 1 || b % b_sub != 0 || k < 1 || m < k || lda < m)
    return set_error(CANDMC_ERR_ARG, "QR_2D_2D args");
  cudaStream_t s = STREAM(stream);
  Status st;
  CANDMC_RET(st.init(s));
  // qr_2d.cxx:793-896: factor a b-wide block with QR_2D(b_sub), then update the
  // rest once with the aggregated Y and T from Y^T Y (upd_A with W = NULL).
  int64_t r0 = 0;
  for (;;) {
    const int64_t mm = m - r0, kk = k - r0;
    double* P = A + r0 * lda + r0;
    if (kk - b > 0 && mm - b > 0) {
      CANDMC_RET(qr_2d_dev(P, lda, mm, b, b_sub, nullptr, 0, st.p(), precision, s));
      if (aggreg_Y)
        CANDMC_RET(materialize(mref(P, lda, 0, kUnitLower), mm, b, aggreg_Y + r0 * lda_aY + r0,
                               lda_aY, s));
      CANDMC_RET(upd_core(P, lda, kUnitLower, P + b * lda, lda, mm, kk - b, b, nullptr, 0,
                          precision, s));
      r0 += b;
    } else {
      CANDMC_RET(qr_2d_dev(P, lda, mm, kk, b_sub, aggreg_Y ? aggreg_Y + r0 * lda_aY + r0 : nullptr,
                           lda_aY, st.p(), precision, s));
      break;
    }
  }
  return CANDMC_OK;
}

int candmc_QR_2D_pipe(double* A, int64_t lda, int64_t m, int64_t k, int64_t b, int precision,
                      void* stream) {
  if (!A || b < 1 || k < 1 || m < k || lda < m) return set_error(CANDMC_ERR_ARG, "QR_2D_pipe args");
  cudaStream_t s = STREAM(stream);
  Status st;
  CANDMC_RET(st.init(s));
  return qr_2d_pipe_dev(A, lda, m, k, b, st.p(), precision, s, nullptr);
}

int candmc_Yamamoto(double* A, int64_t lda, double* Qm, int64_t ldq, int64_t m, int64_t b, double* W,
                    void* stream) {
  if (!A || !Qm || !W || b < 1 || m < b || lda < m || ldq < m) return set_error(CANDMC_ERR_ARG, "Yamamoto args");
  cudaStream_t s = STREAM(stream);
  Status st;
  CANDMC_RET(st.init(s));
  return yamamoto_panel(A, lda, m, b, Qm, ldq, W, st.p(), s);
}

int candmc_upd_Yamamoto_A(const double* Qm, int64_t ldq, double* A, int64_t lda, int64_t mb, int64_t kb,
                          int64_t b, const double* W, int precision, void* stream) {
  if (!Qm || !A || !W || b < 1 || b > 256 || mb < 0 || kb < 0 || (mb > 0 && (ldq < mb || lda < mb)))
    return set_error(CANDMC_ERR_ARG, "upd_Yamamoto_A args");
  return upd_yamamoto(Qm, ldq, A, lda, mb, kb, b, W, b, precision, STREAM(stream));
}

int candmc_yamamoto_append(double* aQm, int64_t ld_aqm, double* aT, int64_t ld_at, int64_t n, int64_t shift,
                           int64_t mb, int64_t b, const double* Qm, int64_t ldq, const double* T, void* stream) {
  if (!aQm || !aT || !Qm || !T || b < 1 || b > 256 || n < 0 || shift < 0 || mb < 0 || (mb > 0 && ldq < mb))
    return set_error(CANDMC_ERR_ARG, "aggregator append args");
  YAgg g{aQm, ld_aqm, aT, ld_at, n, shift};
  return yamamoto_append(&g, mb, b, Qm, ldq, T, b, STREAM(stream));
}

static int yagg_args(double* aQm, int64_t ld_aqm, double* aT, int64_t ld_at, int64_t* agg_n,
                     int64_t* agg_shift, YAgg* g, YAgg** out) {
  *out = nullptr;
  if (!aQm && !aT) return CANDMC_OK;
  if (!aQm || !aT || !agg_n || !agg_shift || ld_aqm < 1 || ld_at < 1 || *agg_n < 0 || *agg_shift < 0)
    return set_error(CANDMC_ERR_ARG, "aggregator args");
  *g = YAgg{aQm, ld_aqm, aT, ld_at, *agg_n, *agg_shift};
  *out = g;
  return CANDMC_OK;
}

int candmc_QR_Yamamoto_2D(double* A, int64_t lda, int64_t m, int64_t k, int64_t b, int compute_Y, double* aQm,
                          int64_t ld_aqm, double* aT, int64_t ld_at, int64_t* agg_n, int64_t* agg_shift,
                          int precision, void* stream) {
  (void)compute_Y;   // Y below R is the panel's Householder Y either way
  if (!A || b < 1 || b > 256 || k < 1 || m < k || lda < m) return set_error(CANDMC_ERR_ARG, "QR_Yamamoto_2D args");
  YAgg g, *pg;
  CANDMC_RET(yagg_args(aQm, ld_aqm, aT, ld_at, agg_n, agg_shift, &g, &pg));
  cudaStream_t s = STREAM(stream);
  Status st;
  CANDMC_RET(st.init(s));
  const int rc = qr_yamamoto_2d_dev(A, lda, m, k, b, pg, st.p(), precision, s);
  if (pg) {
    *agg_n = pg->n;
    *agg_shift = pg->shift;
  }
  return rc;
}

int candmc_QR_Yamamoto_2D_2D(double* A, int64_t lda, int64_t m, int64_t k, int64_t b, int64_t b_sub,
                             int compute_Y, double* aQm, int64_t ld_aqm, double* aT, int64_t ld_at,
                             int64_t* agg_n, int64_t* agg_shift, int precision, void* stream) {
  (void)compute_Y;
  if (!A || b < 1 || b > 256 || b_sub < 1 || b % b_sub != 0 || k < 1 || m < k || lda < m)
    return set_error(CANDMC_ERR_ARG, "QR_Yamamoto_2D_2D args");
  YAgg g, *pg;
  CANDMC_RET(yagg_args(aQm, ld_aqm, aT, ld_at, agg_n, agg_shift, &g, &pg));
  cudaStream_t s = STREAM(stream);
  Status st;
  CANDMC_RET(st.init(s));
  const int rc = qr_yamamoto_2d_2d_dev(A, lda, m, k, b, b_sub, pg, st.p(), precision, s);
  if (pg) {
    *agg_n = pg->n;
    *agg_shift = pg->shift;
  }
  return rc;
}

}  // extern "C"
