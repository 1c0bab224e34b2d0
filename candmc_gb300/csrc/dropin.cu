// C++ drop-in of CANDMC's QR entry points (include/CANDMC.h) on one GPU.
//
// Same signatures, argument meanings and host-pointer conventions as the
// reference; each call stages its operands to the current CUDA device, runs
// the C ABI (include/candmc_gb300.h) on the legacy default stream and copies
// the results back.  The reference's void functions abort on errors; these
// record the status (candmc_dropin_last_status) and leave the outputs
// untouched instead.  Process grids larger than 1 x 1 are rejected.
#include <cuda_runtime.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "../../include/CANDMC.h"

namespace {

thread_local int g_status = CANDMC_OK;
int g_precision = CANDMC_PREC_FP64;

struct DMat {
  double* p = nullptr;
  int64_t ld = 0;
  int64_t m = 0, n = 0;
  ~DMat() {
    if (p) cudaFree(p);
  }
  bool alloc(int64_t rows, int64_t cols) {
    m = rows;
    n = cols;
    ld = std::max<int64_t>(rows, 1);
    return cudaMalloc(&p, sizeof(double) * (size_t)ld * std::max<int64_t>(cols, 1)) == cudaSuccess;
  }
  bool in(const double* h, int64_t ldh) {
    if (!h || m == 0 || n == 0) return true;
    return cudaMemcpy2D(p, sizeof(double) * ld, h, sizeof(double) * ldh, sizeof(double) * m, n,
                        cudaMemcpyHostToDevice) == cudaSuccess;
  }
  bool out(double* h, int64_t ldh) const {
    if (!h || m == 0 || n == 0) return true;
    return cudaMemcpy2D(h, sizeof(double) * ldh, p, sizeof(double) * ld, sizeof(double) * m, n,
                        cudaMemcpyDeviceToHost) == cudaSuccess;
  }
};

bool stage(DMat& d, const double* h, int64_t ldh, int64_t m, int64_t n) {
  if (!d.alloc(m, n)) return false;
  return d.in(h, ldh);
}

int finish(int rc) {
  if (rc == CANDMC_OK && cudaDeviceSynchronize() != cudaSuccess) rc = CANDMC_ERR_CUDA;
  g_status = rc;
  return rc;
}

bool one_rank(int64_t numPes, int64_t myRank) { return numPes == 1 && myRank == 0; }

bool one_grid(const pview* pv) {
  return pv && pv->crow.np == 1 && pv->ccol.np == 1 && pv->crow.rank == 0 && pv->ccol.rank == 0;
}

}  // namespace

int candmc_dropin_last_status(void) { return g_status; }

void candmc_dropin_set_precision(int precision) { g_precision = precision; }

// ------------------------------------------------------------------ TSQR
void bitree_tsqr(double* A, int64_t const lda_A, double* R, double* tau, int64_t const m,
                 int64_t const b, int64_t const myRank, int64_t const numPes, int64_t const root,
                 int64_t const req_id, CommData_t cdt, int64_t const output_Y, double* tree_data) {
  (void)root; (void)req_id; (void)cdt; (void)tree_data;   // single rank: no tree, no messages
  if (!one_rank(numPes, myRank) || !A || !R || !tau) { g_status = CANDMC_ERR_ARG; return; }
  DMat dA, dR, dt;
  if (!stage(dA, A, lda_A, m, b) || !dR.alloc(b, b) || !dt.alloc(b, 1)) { g_status = CANDMC_ERR_ALLOC; return; }
  int rc = candmc_bitree_tsqr(dA.p, dA.ld, dR.p, dt.p, m, b, (int)output_Y, nullptr);
  if (finish(rc) != CANDMC_OK) return;
  if (output_Y) dA.out(A, lda_A);
  dR.out(R, b);
  dt.out(tau, b);
}

void local_tsqr(double* A, double* R, int64_t const m, int64_t const b, int64_t const lda_A,
                double* tau) {
  (void)R;   // the reference uses this argument as dgeqrf workspace
  std::vector<double> rbuf((size_t)b * b), tbuf(tau ? 0 : (size_t)b);
  CommData_t c;
  SET_COMM(MPI_COMM_WORLD, 0, 1, c);
  bitree_tsqr(A, lda_A, rbuf.data(), tau ? tau : tbuf.data(), m, b, 0, 1, 0, 0, c, 1, nullptr);
}

void tree_tsqr(double* A, double* buf, int64_t const b, double* tau) {
  (void)buf;   // the reference's dtpqrt workspace
  // QR of the stacked [R1; R2] (2b x b, ld 2b) with dtpqrt's contract: the
  // upper triangles are read and overwritten (R over V), the strictly-lower
  // entries are left alone, and tau receives the block-diagonal T.
  const int64_t m = 2 * b, nbk = std::min<int64_t>(b, TAU_BLK);
  DMat dA, dT;
  if (!stage(dA, A, m, m, b) || (tau && !stage(dT, tau, nbk, nbk, b))) {
    g_status = CANDMC_ERR_ALLOC;
    return;
  }
  int rc = candmc_tree_tsqr(dA.p, b, tau ? dT.p : nullptr, nullptr);
  if (finish(rc) != CANDMC_OK) return;
  dA.out(A, m);
  if (tau) dT.out(tau, nbk);
}

void construct_Q1(double const* Y, int64_t const lda_Y, double const* tau, double* Q1,
                  int64_t const lda_Q, int64_t const m, int64_t const b, int64_t const k,
                  int64_t const myRank, int64_t const numPes, int64_t const root, CommData_t cdt,
                  double* tree_data, double* ID) {
  (void)root; (void)cdt; (void)tree_data;
  if (!one_rank(numPes, myRank) || ID != nullptr) { g_status = CANDMC_ERR_ARG; return; }
  DMat dY, dt, dQ;
  if (!stage(dY, Y, lda_Y, m, b) || !stage(dt, tau, b, b, 1) || !dQ.alloc(m, k)) {
    g_status = CANDMC_ERR_ALLOC;
    return;
  }
  int rc = candmc_construct_Q1(dY.p, dY.ld, dt.p, dQ.p, dQ.ld, m, b, k, nullptr);
  if (finish(rc) == CANDMC_OK) dQ.out(Q1, lda_Q);
}

void apply_tsqr_QT(double const* Y, int64_t const lda_Y, double const* tau, double* B,
                   int64_t const lda_B, int64_t const m, int64_t const b, int64_t const k,
                   int64_t const myRank, int64_t const numPes, int64_t const root, CommData_t cdt,
                   double* tree_data) {
  (void)root; (void)cdt; (void)tree_data;
  if (!one_rank(numPes, myRank)) { g_status = CANDMC_ERR_ARG; return; }
  DMat dY, dt, dB;
  if (!stage(dY, Y, lda_Y, m, b) || !stage(dt, tau, b, b, 1) || !stage(dB, B, lda_B, m, k)) {
    g_status = CANDMC_ERR_ALLOC;
    return;
  }
  int rc = candmc_apply_tsqr_QT(dY.p, dY.ld, dt.p, dB.p, dB.ld, m, b, k, nullptr);
  if (finish(rc) == CANDMC_OK) dB.out(B, lda_B);
}

// ------------------------------------------------------------------ reconstruction
void tau_recon(const char structure, const int ncol, const int nrow, const int lda, double const* Y,
               double* tau) {
  if (ncol <= 0) return;
  DMat dY, dt;
  if (!stage(dY, Y, lda, nrow, ncol) || !dt.alloc(ncol, 1)) {
    g_status = CANDMC_ERR_ALLOC;
    return;
  }
  int rc = candmc_tau_recon(structure, ncol, nrow, dY.ld, dY.p, dt.p, nullptr);
  if (finish(rc) == CANDMC_OK) dt.out(tau, ncol);
}

void compute_invT_from_W(double const* W, int64_t b, double* invT) {
  DMat dW, dX;
  if (!stage(dW, W, b, b, b) || !stage(dX, invT, b, b, b)) { g_status = CANDMC_ERR_ALLOC; return; }
  int rc = candmc_compute_invT_from_W(dW.p, b, dX.p, nullptr);
  if (finish(rc) == CANDMC_OK) dX.out(invT, b);
}

static void nlu(int (*fn)(double*, double*, int64_t, int64_t, int64_t, int64_t*, void*), double* A,
                double* R, int64_t b, int64_t lda_A, int64_t lda_R, int64_t* signs) {
  DMat dA, dR;
  int64_t* ds = nullptr;
  if (!stage(dA, A, lda_A, b, b) || !stage(dR, R, lda_R, b, b) ||
      cudaMalloc(&ds, sizeof(int64_t) * b) != cudaSuccess) {
    g_status = CANDMC_ERR_ALLOC;
    return;
  }
  int rc = fn(dA.p, dR.p, b, dA.ld, dR.ld, ds, nullptr);
  if (finish(rc) == CANDMC_OK) {
    dA.out(A, lda_A);
    dR.out(R, lda_R);
    if (signs) cudaMemcpy(signs, ds, sizeof(int64_t) * b, cudaMemcpyDeviceToHost);
  }
  cudaFree(ds);
}

void signed_NLU(double* A, double* R, int64_t b, int64_t lda_A, int64_t lda_R, int64_t* signs) {
  nlu(candmc_signed_NLU, A, R, b, lda_A, lda_R, signs);
}

void recursive_NLU(double* A, double* R, int64_t b, int64_t lda_A, int64_t lda_R, int64_t* signs) {
  nlu(candmc_recursive_NLU, A, R, b, lda_A, lda_R, signs);
}

void hh_recon_qr(double* A, int64_t lda_A, int64_t m, int64_t b, double* W, int64_t myRank,
                 int64_t numPes, int64_t root, int64_t req_id, CommData_t cdt) {
  (void)root; (void)req_id; (void)cdt;
  if (!one_rank(numPes, myRank)) { g_status = CANDMC_ERR_ARG; return; }
  g_status = candmc_hh_recon_qr_host(A, lda_A, m, b, W, nullptr);
}

// ------------------------------------------------------------------ T factor and CAQR
void compute_invT_from_Y(double const* Y, int64_t lda_Y, double* T, int64_t lda_T, int64_t mb,
                         int64_t b, pview* pv) {
  if (!one_grid(pv)) { g_status = CANDMC_ERR_ARG; return; }
  DMat dY, dT;
  if (!stage(dY, Y, lda_Y, mb, b) || !stage(dT, T, lda_T, b, b)) { g_status = CANDMC_ERR_ALLOC; return; }
  int rc = candmc_compute_invT_from_Y(dY.p, dY.ld, dT.p, dT.ld, mb, b, nullptr);
  if (finish(rc) == CANDMC_OK) dT.out(T, lda_T);
}

void compute_invT_from_Y(double const* Y1, int64_t lda_Y1, double const* Y2, int64_t lda_Y2,
                         double* T, int64_t lda_T, int64_t mb, int64_t b1, int64_t b2, pview* pv) {
  if (!one_grid(pv)) { g_status = CANDMC_ERR_ARG; return; }
  DMat d1, d2, dT;
  if (!stage(d1, Y1, lda_Y1, mb, b1) || !stage(d2, Y2, lda_Y2, mb, b2) || !dT.alloc(b1, b2)) {
    g_status = CANDMC_ERR_ALLOC;
    return;
  }
  int rc = candmc_compute_invT_from_Y2(d1.p, d1.ld, d2.p, d2.ld, dT.p, dT.ld, mb, b1, b2, nullptr);
  if (finish(rc) == CANDMC_OK) dT.out(T, lda_T);
}

void upd_A(double const* Ybuf, int64_t lda_Y, double* A, int64_t lda_A, int64_t mb, int64_t kb,
           int64_t b, double const* W, pview* pv, bool W_is_T) {
  if (!one_grid(pv)) { g_status = CANDMC_ERR_ARG; return; }
  DMat dY, dA, dW;
  if (!stage(dY, Ybuf, lda_Y, mb, b) || !stage(dA, A, lda_A, mb, kb) ||
      (W && !stage(dW, W, b, b, b))) {
    g_status = CANDMC_ERR_ALLOC;
    return;
  }
  int rc = candmc_upd_A(dY.p, dY.ld, dA.p, dA.ld, mb, kb, b, W ? dW.p : nullptr, W_is_T ? 1 : 0,
                        g_precision, nullptr);
  if (finish(rc) == CANDMC_OK) dA.out(A, lda_A);
}

void update_A(double const* Y, int64_t lda_Y, double* A, int64_t lda_A, int64_t m, int64_t k,
              int64_t b, double const* W, pview* pv, double* aggreg_Y, int64_t lda_aY, bool W_is_T) {
  if (!one_grid(pv)) { g_status = CANDMC_ERR_ARG; return; }
  // local sizes of qr_2d.cxx:140-147 on a 1 x 1 grid: whole b-blocks only
  const int64_t mb = (m / b) * b, kb = (k / b) * b;
  DMat dY, dA, dW, dG;
  if (!stage(dY, Y, lda_Y, mb, b) || !stage(dA, A, lda_A, mb, kb) ||
      (W && !stage(dW, W, b, b, b)) || (aggreg_Y && !dG.alloc(mb, b))) {
    g_status = CANDMC_ERR_ALLOC;
    return;
  }
  int rc = candmc_update_A(dY.p, dY.ld, dA.p, dA.ld, mb, kb, b, W ? dW.p : nullptr,
                           aggreg_Y ? dG.p : nullptr, dG.ld, W_is_T ? 1 : 0, g_precision, nullptr);
  if (finish(rc) != CANDMC_OK) return;
  dA.out(A, lda_A);
  if (aggreg_Y) dG.out(aggreg_Y, lda_aY);
}

void QR_2D(double* A, int64_t lda_A, int64_t m, int64_t k, int64_t b, pview* pv, double* aggreg_Y,
           int64_t lda_aY) {
  if (!one_grid(pv)) { g_status = CANDMC_ERR_ARG; return; }
  DMat dA, dG;
  if (!stage(dA, A, lda_A, m, k) || (aggreg_Y && !stage(dG, aggreg_Y, lda_aY, m, k))) {
    g_status = CANDMC_ERR_ALLOC;
    return;
  }
  int rc = candmc_QR_2D(dA.p, dA.ld, m, k, b, aggreg_Y ? dG.p : nullptr, dG.ld, g_precision, nullptr);
  if (finish(rc) != CANDMC_OK) return;
  dA.out(A, lda_A);
  if (aggreg_Y) dG.out(aggreg_Y, lda_aY);
}

void QR_2D_pipe(double* A, int64_t lda_A, int64_t m, int64_t k, int64_t b, pview* pv,
                double* last_Y, int64_t lda_lY, double* last_W, double* my_last_W) {
  (void)last_Y; (void)lda_lY; (void)last_W; (void)my_last_W;   // pipeline state of the MPI version
  if (!one_grid(pv)) { g_status = CANDMC_ERR_ARG; return; }
  DMat dA;
  if (!stage(dA, A, lda_A, m, k)) { g_status = CANDMC_ERR_ALLOC; return; }
  int rc = candmc_QR_2D_pipe(dA.p, dA.ld, m, k, b, g_precision, nullptr);
  if (finish(rc) == CANDMC_OK) dA.out(A, lda_A);
}

void QR_2D_2D(double* A, int64_t lda_A, int64_t m, int64_t k, int64_t b, int64_t b_sub, pview* pv,
              double* aggreg_Y, int64_t lda_aY, int* desc_A, double* org_A, int64_t IA, int64_t JA) {
  (void)org_A; (void)IA; (void)JA;
  if (!one_grid(pv) || desc_A != nullptr) { g_status = CANDMC_ERR_ARG; return; }   // no ScaLAPACK panel
  DMat dA, dG;
  if (!stage(dA, A, lda_A, m, k) || (aggreg_Y && !stage(dG, aggreg_Y, lda_aY, m, k))) {
    g_status = CANDMC_ERR_ALLOC;
    return;
  }
  int rc = candmc_QR_2D_2D(dA.p, dA.ld, m, k, b, b_sub, aggreg_Y ? dG.p : nullptr, dG.ld,
                           g_precision, nullptr);
  if (finish(rc) != CANDMC_OK) return;
  dA.out(A, lda_A);
  if (aggreg_Y) dG.out(aggreg_Y, lda_aY);
}

// ------------------------------------------------------------------ Yamamoto
void Yamamoto(double* A, int64_t lda_A, double* Qm, int64_t lda_Qm, int64_t m, int64_t b, double* W,
              int64_t myRank, int64_t numPes, int64_t root, int64_t req_id, CommData_t cdt) {
  (void)root; (void)req_id; (void)cdt;
  if (!one_rank(numPes, myRank) || !A || !Qm || !W) { g_status = CANDMC_ERR_ARG; return; }
  DMat dA, dQ, dW;
  if (!stage(dA, A, lda_A, m, b) || !dQ.alloc(m, b) || !dW.alloc(b, b)) { g_status = CANDMC_ERR_ALLOC; return; }
  int rc = candmc_Yamamoto(dA.p, dA.ld, dQ.p, dQ.ld, m, b, dW.p, nullptr);
  if (finish(rc) != CANDMC_OK) return;
  dA.out(A, lda_A);
  dQ.out(Qm, lda_Qm);
  dW.out(W, b);
}

aggregator::aggregator(int64_t lda_aQm_, int64_t lda_aT_) {
  lda_aQm = lda_aQm_;
  lda_aT = lda_aT_;
  aQm = static_cast<double*>(calloc((size_t)(lda_aT * lda_aQm > 0 ? lda_aT * lda_aQm : 1), sizeof(double)));
  aT = static_cast<double*>(calloc((size_t)(lda_aT > 0 ? lda_aT * lda_aT : 1), sizeof(double)));
  n = 0;
  shift = 0;
}

aggregator::~aggregator() {
  free(aQm);
  free(aT);
}

void aggregator::reset() {
  n = 0;
  shift = 0;
  std::fill(aQm, aQm + lda_aT * lda_aQm, 0.0);
  std::fill(aT, aT + lda_aT * lda_aT, 0.0);
}

void aggregator::shift_down(int64_t b) { shift += b; }

namespace {

// the aggregator's host arrays on the device for one call
struct DAgg {
  DMat q, t;
  bool in(const aggregator* a) {
    return stage(q, a->aQm, a->lda_aQm, a->lda_aQm, a->lda_aT) && stage(t, a->aT, a->lda_aT, a->lda_aT, a->lda_aT);
  }
  void out(aggregator* a) const {
    q.out(a->aQm, a->lda_aQm);
    t.out(a->aT, a->lda_aT);
  }
};

}  // namespace

void aggregator::append(int64_t mb, int64_t b, double const* Qm, int64_t lda_Qm, double const* T, pview* pv) {
  if (!one_grid(pv)) { g_status = CANDMC_ERR_ARG; return; }
  DAgg d;
  DMat dQ, dT;
  if (!d.in(this) || !stage(dQ, Qm, lda_Qm, mb, b) || !stage(dT, T, b, b, b)) { g_status = CANDMC_ERR_ALLOC; return; }
  int rc = candmc_yamamoto_append(d.q.p, d.q.ld, d.t.p, d.t.ld, n, shift, mb, b, dQ.p, dQ.ld, dT.p, nullptr);
  if (finish(rc) != CANDMC_OK) return;
  d.out(this);
  n += b;
}

void upd_Yamamoto_A(double const* Qm, int64_t lda_Qm, double* A, int64_t lda_A, int64_t mb, int64_t kb,
                    int64_t b, double const* T, pview* pv) {
  if (!one_grid(pv)) { g_status = CANDMC_ERR_ARG; return; }
  DMat dQ, dA, dT;
  if (!stage(dQ, Qm, lda_Qm, mb, b) || !stage(dA, A, lda_A, mb, kb) || !stage(dT, T, b, b, b)) {
    g_status = CANDMC_ERR_ALLOC;
    return;
  }
  int rc = candmc_upd_Yamamoto_A(dQ.p, dQ.ld, dA.p, dA.ld, mb, kb, b, dT.p, g_precision, nullptr);
  if (finish(rc) == CANDMC_OK) dA.out(A, lda_A);
}

void update_Yamamoto_A(double* Qm, int64_t lda_Qm, double* A, int64_t lda_A, int64_t m, int64_t k, int64_t b,
                       double* T, pview* pv, aggregator* agg) {
  // one process: mb = m and kb = k (qr_y2d.cxx:81-89), no broadcasts
  upd_Yamamoto_A(Qm, lda_Qm, A, lda_A, m, k, b, T, pv);
  if (g_status == CANDMC_OK && agg != nullptr) agg->append(m, b, Qm, lda_Qm, T, pv);
}

void QR_Yamamoto_2D(double* A, int64_t lda_A, int64_t m, int64_t k, int64_t b, pview* pv, aggregator* agg,
                    bool compute_Y) {
  if (!one_grid(pv)) { g_status = CANDMC_ERR_ARG; return; }
  DMat dA;
  DAgg d;
  if (!stage(dA, A, lda_A, m, k) || (agg && !d.in(agg))) { g_status = CANDMC_ERR_ALLOC; return; }
  int64_t n = agg ? agg->n : 0, sh = agg ? agg->shift : 0;
  int rc = candmc_QR_Yamamoto_2D(dA.p, dA.ld, m, k, b, compute_Y ? 1 : 0, agg ? d.q.p : nullptr, d.q.ld,
                                 agg ? d.t.p : nullptr, d.t.ld, agg ? &n : nullptr, agg ? &sh : nullptr,
                                 g_precision, nullptr);
  if (finish(rc) != CANDMC_OK) return;
  dA.out(A, lda_A);
  if (agg) {
    d.out(agg);
    agg->n = n;
    agg->shift = sh;
  }
}

void QR_Yamamoto_2D_2D(double* A, int64_t lda_A, int64_t m, int64_t k, int64_t b, int64_t b_sub, pview* pv,
                       aggregator* agg, bool compute_Y) {
  if (!one_grid(pv)) { g_status = CANDMC_ERR_ARG; return; }
  DMat dA;
  DAgg d;
  if (!stage(dA, A, lda_A, m, k) || (agg && !d.in(agg))) { g_status = CANDMC_ERR_ALLOC; return; }
  int64_t n = agg ? agg->n : 0, sh = agg ? agg->shift : 0;
  int rc = candmc_QR_Yamamoto_2D_2D(dA.p, dA.ld, m, k, b, b_sub, compute_Y ? 1 : 0, agg ? d.q.p : nullptr,
                                    d.q.ld, agg ? d.t.p : nullptr, d.t.ld, agg ? &n : nullptr,
                                    agg ? &sh : nullptr, g_precision, nullptr);
  if (finish(rc) != CANDMC_OK) return;
  dA.out(A, lda_A);
  if (agg) {
    d.out(agg);
    agg->n = n;
    agg->shift = sh;
  }
}

void sym_full2band(double* A, int64_t lda_A, int64_t n, int64_t b, int64_t b_sub, pview* pv) {
  if (!one_grid(pv)) { g_status = CANDMC_ERR_ARG; return; }
  DMat dA;
  if (!stage(dA, A, lda_A, n, n)) { g_status = CANDMC_ERR_ALLOC; return; }
  int rc = candmc_sym_full2band(dA.p, dA.ld, n, b, b_sub, g_precision, nullptr);
  if (finish(rc) == CANDMC_OK) dA.out(A, lda_A);
}
