// C entry points over the reference's own QR functions on a 1 x 1 grid.
//
// TEST INFRASTRUCTURE ONLY.  This file is compiled together with the
// reference's unmodified sources (alg/shared/*.cxx, alg/QR/tsqr,
// alg/QR/hh_recon, alg/QR/qr_2d) into oracle/_ref/libcandmc_ref.so by
// oracle/build_ref.py.  Each function below builds the single-rank
// communicator / process-grid view that the reference's own drivers build
// (bench/QR/bench_qr_2d.cxx:51-58, test/QR/test_hh_recon.cxx) and calls one
// reference function with plain pointers, so that Python (ctypes) can run the
// reference on the same bytes as the GPU path.  Nothing here computes.
#include <stdint.h>

#include "alg/shared/util.h"
#include "alg/QR/tsqr/bitree_tsqr.h"
#include "alg/QR/hh_recon/hh_recon.h"
#include "alg/QR/hh_recon/yamamoto.h"
#include "alg/QR/qr_2d/qr_2d.h"
#include "alg/QR/qr_2d/qr_y2d.h"

namespace {

CommData_t one_rank() {
  CommData_t c;
  c.cm = MPI_COMM_WORLD;
  c.np = 1;
  c.rank = 0;
  c.color = 0;
  c.alive = 1;
  return c;
}

pview one_grid() {
  pview pv;
  pv.rrow = 0;
  pv.rcol = 0;
  pv.crow = one_rank();
  pv.ccol = one_rank();
  pv.cdiag = one_rank();
  pv.cworld = one_rank();
  return pv;
}

}  // namespace

extern "C" {

// bitree_tsqr.h:16-19 (bitree_tsqr.cxx:20-34): QR of [R1; R2] by dtpqrt
void ref_tree_tsqr(double* A, double* buf, int64_t b, double* tau) { tree_tsqr(A, buf, b, tau); }

// bitree_tsqr.h:31-36 (bitree_tsqr.cxx:48-71): leaf dgeqrf
void ref_local_tsqr(double* A, double* R, int64_t m, int64_t b, int64_t lda, double* tau) {
  local_tsqr(A, R, m, b, lda, tau);
}

// bitree_tsqr.h:58-70 at numPes == 1
void ref_bitree_tsqr(double* A, int64_t lda, double* R, double* tau, int64_t m, int64_t b, int64_t output_Y,
                     double* tree_data) {
  bitree_tsqr(A, lda, R, tau, m, b, 0, 1, 0, 7, one_rank(), output_Y, tree_data);
}

// bitree_tsqr.h:91-104 at numPes == 1
void ref_construct_Q1(const double* Y, int64_t ldY, const double* tau, double* Q1, int64_t ldQ, int64_t m,
                      int64_t b, int64_t k, double* tree_data) {
  construct_Q1(Y, ldY, tau, Q1, ldQ, m, b, k, 0, 1, 0, one_rank(), tree_data, NULL);
}

// bitree_tsqr.h:126-138 at numPes == 1
void ref_apply_tsqr_QT(const double* Y, int64_t ldY, const double* tau, double* B, int64_t ldB, int64_t m,
                       int64_t b, int64_t k, double* tree_data) {
  apply_tsqr_QT(Y, ldY, tau, B, ldB, m, b, k, 0, 1, 0, one_rank(), tree_data);
}

// util.h:675-680 (util.cxx:437-466)
void ref_tau_recon(char structure, int64_t ncol, int64_t nrow, int64_t lda, const double* Y, double* tau) {
  tau_recon(structure, (int)ncol, (int)nrow, (int)lda, Y, tau);
}

// hh_recon.h:13-15
void ref_compute_invT_from_W(const double* W, int64_t b, double* invT) { compute_invT_from_W(W, b, invT); }

// hh_recon.h:27-32, 43-48
void ref_signed_NLU(double* A, double* R, int64_t b, int64_t lda_A, int64_t lda_R, int64_t* signs) {
  signed_NLU(A, R, b, lda_A, lda_R, signs);
}
void ref_recursive_NLU(double* A, double* R, int64_t b, int64_t lda_A, int64_t lda_R, int64_t* signs) {
  recursive_NLU(A, R, b, lda_A, lda_R, signs);
}

// hh_recon.h:66-75 at numPes == 1
void ref_hh_recon_qr(double* A, int64_t lda, int64_t m, int64_t b, double* W) {
  hh_recon_qr(A, lda, m, b, W, 0, 1, 0, 42, one_rank());
}

// yamamoto.h (yamamoto.cxx:98-174) at numPes == 1
void ref_Yamamoto(double* A, int64_t lda, double* Qm, int64_t ldQm, int64_t m, int64_t b, double* W) {
  Yamamoto(A, lda, Qm, ldQm, m, b, W, 0, 1, 0, 42, one_rank());
}

// qr_2d.h:25-56
void ref_compute_invT_from_Y(const double* Y, int64_t ldY, double* T, int64_t ldT, int64_t mb, int64_t b) {
  pview pv = one_grid();
  compute_invT_from_Y(Y, ldY, T, ldT, mb, b, &pv);
}
void ref_compute_invT_from_Y2(const double* Y1, int64_t ldY1, const double* Y2, int64_t ldY2, double* T,
                              int64_t ldT, int64_t mb, int64_t b1, int64_t b2) {
  pview pv = one_grid();
  compute_invT_from_Y(Y1, ldY1, Y2, ldY2, T, ldT, mb, b1, b2, &pv);
}

// qr_2d.h:74-85 (no aggregation)
void ref_update_A(const double* Y, int64_t ldY, double* A, int64_t ldA, int64_t m, int64_t k, int64_t b,
                  const double* W, int64_t W_is_T) {
  pview pv = one_grid();
  update_A(Y, ldY, A, ldA, m, k, b, W, &pv, NULL, 0, W_is_T != 0);
}

// qr_2d.h:99-108
void ref_upd_A(const double* Ybuf, int64_t ldY, double* A, int64_t ldA, int64_t mb, int64_t kb, int64_t b,
               const double* W, int64_t W_is_T) {
  pview pv = one_grid();
  upd_A(Ybuf, ldY, A, ldA, mb, kb, b, W, &pv, W_is_T != 0);
}

// qr_2d.h:124-131, 293-302, 176-188 on a 1 x 1 grid
void ref_QR_2D(double* A, int64_t lda, int64_t m, int64_t k, int64_t b) {
  pview pv = one_grid();
  QR_2D(A, lda, m, k, b, &pv, NULL, 0);
}
void ref_QR_2D_pipe(double* A, int64_t lda, int64_t m, int64_t k, int64_t b) {
  pview pv = one_grid();
  QR_2D_pipe(A, lda, m, k, b, &pv);
}
void ref_QR_2D_2D(double* A, int64_t lda, int64_t m, int64_t k, int64_t b, int64_t b_sub) {
  pview pv = one_grid();
  QR_2D_2D(A, lda, m, k, b, b_sub, &pv, NULL, 0);
}

// qr_y2d.h:108-145 on a 1 x 1 grid, without an aggregator
void ref_QR_Yamamoto_2D(double* A, int64_t lda, int64_t m, int64_t k, int64_t b, int64_t compute_Y) {
  pview pv = one_grid();
  QR_Yamamoto_2D(A, lda, m, k, b, &pv, NULL, compute_Y != 0);
}
void ref_QR_Yamamoto_2D_2D(double* A, int64_t lda, int64_t m, int64_t k, int64_t b, int64_t b_sub,
                           int64_t compute_Y) {
  pview pv = one_grid();
  QR_Yamamoto_2D_2D(A, lda, m, k, b, b_sub, &pv, NULL, compute_Y != 0);
}

// qr_y2d.h:59-94
void ref_upd_Yamamoto_A(const double* Qm, int64_t ldQm, double* A, int64_t ldA, int64_t mb, int64_t kb,
                        int64_t b, const double* T) {
  pview pv = one_grid();
  upd_Yamamoto_A(Qm, ldQm, A, ldA, mb, kb, b, T, &pv);
}

}  // extern "C"
