// Reference-style driver for the C++ drop-in (include/CANDMC.h) on one GPU.
//
// Mirrors the reference's own QR tests: the decomposition-independent srand48
// fixture (test/QR/test_hh_recon.cxx:70-85, test_qr_2d.cxx:87-103), the same
// entry points with a single-rank CommData_t / 1 x 1 pview, and the same pass
// criteria (sum_j ||(A - QR) e_j|| / ||A e_j|| <= 1e-9; ||Q^T Q - I|| <= 1e-6).
// Q is applied with the drop-in's apply_tsqr_QT, tau is rebuilt from Y as the
// reference's tau_recon does (alg/shared/util.cxx:437-466).  Prints
// "Test successful." or "TEST FAILED!!!" per test and exits non-zero on a failure.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include <algorithm>
#include <vector>

#include "CANDMC.h"

static double fixture(int64_t row, int64_t col, int64_t m, double shift) {
  srand48(99900 + (row + col * m) * 61);
  return drand48() - shift;
}

// tau_i = 2 / (1 + ||Y[i+1:, i]||^2), the reconstruction convention (tau = 2 for an empty tail)
static std::vector<double> tau_from_y(const std::vector<double>& YR, int64_t m, int64_t b) {
  std::vector<double> tau(b);
  for (int64_t i = 0; i < b; ++i) {
    double s = 0;
    for (int64_t r = i + 1; r < m; ++r) s += YR[i * m + r] * YR[i * m + r];
    tau[i] = 2.0 / (1.0 + s);
  }
  return tau;
}

// sum_j ||(Q^T A - R) e_j|| / ||A e_j|| over the first b columns (== the reference's ||A - QR|| form)
static double column_residual(const std::vector<double>& A, const std::vector<double>& YR, int64_t m,
                              int64_t b, int64_t ncols) {
  std::vector<double> tau = tau_from_y(YR, m, b);
  std::vector<double> B(A);
  CommData_t c;
  SET_COMM(MPI_COMM_WORLD, 0, 1, c);
  apply_tsqr_QT(YR.data(), m, tau.data(), B.data(), m, m, b, ncols, 0, 1, 0, c);
  double sum = 0;
  for (int64_t j = 0; j < ncols; ++j) {
    double num = 0, den = 0;
    for (int64_t r = 0; r < m; ++r) {
      const double rr = (r <= j) ? YR[j * m + r] : 0.0;
      num += (B[j * m + r] - rr) * (B[j * m + r] - rr);
      den += A[j * m + r] * A[j * m + r];
    }
    sum += sqrt(num / den);
  }
  return sum;
}

static int report(const char* name, double value, double bound) {
  const bool ok = value <= bound && candmc_dropin_last_status() == CANDMC_OK;
  printf("%s: %.3e (bound %.0e) %s\n", name, value, bound, ok ? "Test successful." : "TEST FAILED!!!");
  return ok ? 0 : 1;
}

int main() {
  int fails = 0;
  CommData_t cdt;
  SET_COMM(MPI_COMM_WORLD, 0, 1, cdt);
  // test_hh_recon at np = 1: b = 17, m = 34 (defaults), plus a taller panel
  for (int64_t mm : {34, 1700}) {
    const int64_t m = mm, b = 17;
    std::vector<double> A(m * b), W(b * b);
    for (int64_t c = 0; c < b; ++c)
      for (int64_t r = 0; r < m; ++r) A[c * m + r] = fixture(r, c, m, 0.0);
    std::vector<double> YR(A);
    hh_recon_qr(YR.data(), m, m, b, W.data(), 0, 1, 0, 0, cdt);
    char name[64];
    snprintf(name, sizeof name, "hh_recon_qr m=%ld b=%ld ||A-QR||", (long)m, (long)b);
    fails += report(name, column_residual(A, YR, m, b, b), 1e-9);
  }
  // test_construct_tsqr_Q: bitree_tsqr + construct_Q1, ||Q^T Q - I||_F <= 1e-6
  {
    const int64_t m = 84, b = 21;
    std::vector<double> A(m * b), R(b * b), tau(b), Q1(m * b);
    for (int64_t c = 0; c < b; ++c)
      for (int64_t r = 0; r < m; ++r) A[c * m + r] = fixture(r, c, m, 0.0);
    bitree_tsqr(A.data(), m, R.data(), tau.data(), m, b, 0, 1, 0, 0, cdt, 1);
    construct_Q1(A.data(), m, tau.data(), Q1.data(), m, m, b, b, 0, 1, 0, cdt);
    double e = 0;
    for (int64_t i = 0; i < b; ++i)
      for (int64_t j = 0; j < b; ++j) {
        double s = (i == j) ? -1.0 : 0.0;
        for (int64_t r = 0; r < m; ++r) s += Q1[i * m + r] * Q1[j * m + r];
        e += s * s;
      }
    fails += report("bitree_tsqr + construct_Q1 ||Q^TQ-I||", sqrt(e), 1e-6);
  }
  // test_qr_2d at a 1 x 1 grid with the pipelined variant (its default): drand48 - 0.5
  for (int prec : {CANDMC_PREC_FP64, CANDMC_PREC_OZAKI}) {
    const int64_t m = 256, k = 192, b = 64;
    std::vector<double> A(m * k);
    for (int64_t c = 0; c < k; ++c)
      for (int64_t r = 0; r < m; ++r) A[c * m + r] = fixture(r, c, m, 0.5);
    std::vector<double> YR(A);
    pview pv = candmc_single_gpu_view();
    candmc_dropin_set_precision(prec);
    QR_2D_pipe(YR.data(), m, m, k, b, &pv);
    // apply Q^T panel by panel with update_A (T from Y^T Y) and compare with R
    std::vector<double> B(A);
    for (int64_t r0 = 0; r0 < k; r0 += b) {
      pview pv2 = candmc_single_gpu_view();
      update_A(YR.data() + r0 * m + r0, m, B.data() + r0, m, m - r0, k, b, NULL, &pv2, NULL, 0);
    }
    double num = 0, den = 0;
    for (int64_t c = 0; c < k; ++c)
      for (int64_t r = 0; r < m; ++r) {
        const double rr = (r <= c) ? YR[c * m + r] : 0.0;
        num += (B[c * m + r] - rr) * (B[c * m + r] - rr);
        den += A[c * m + r] * A[c * m + r];
      }
    char name[64];
    snprintf(name, sizeof name, "QR_2D_pipe %s ||A-QR||/||A||", prec == CANDMC_PREC_FP64 ? "fp64" : "ozaki");
    fails += report(name, sqrt(num / den), 1e-13);
  }
  candmc_dropin_set_precision(CANDMC_PREC_FP64);
  // test_qr_y2d at a 1 x 1 grid: QR_Yamamoto_2D_2D with compute_Y (test/QR/test_qr_y2d.cxx:116),
  // Q^T applied panel by panel from the Y it leaves below R
  for (int prec : {CANDMC_PREC_FP64, CANDMC_PREC_OZAKI}) {
    const int64_t m = 256, k = 192, b2 = 64, b = 32;
    std::vector<double> A(m * k);
    for (int64_t c = 0; c < k; ++c)
      for (int64_t r = 0; r < m; ++r) A[c * m + r] = fixture(r, c, m, 0.5);
    std::vector<double> YR(A);
    pview pv = candmc_single_gpu_view();
    candmc_dropin_set_precision(prec);
    QR_Yamamoto_2D_2D(YR.data(), m, m, k, b2, b, &pv, NULL, true);
    candmc_dropin_set_precision(CANDMC_PREC_FP64);
    std::vector<double> B(A);
    for (int64_t r0 = 0; r0 < k; r0 += b) {
      pview pv2 = candmc_single_gpu_view();
      update_A(YR.data() + r0 * m + r0, m, B.data() + r0, m, m - r0, k, b, NULL, &pv2, NULL, 0);
    }
    double num = 0, den = 0;
    for (int64_t c = 0; c < k; ++c)
      for (int64_t r = 0; r < m; ++r) {
        const double rr = (r <= c) ? YR[c * m + r] : 0.0;
        num += (B[c * m + r] - rr) * (B[c * m + r] - rr);
        den += A[c * m + r] * A[c * m + r];
      }
    char name[64];
    snprintf(name, sizeof name, "QR_Yamamoto_2D_2D %s ||A-QR||/||A||", prec == CANDMC_PREC_FP64 ? "fp64" : "ozaki");
    fails += report(name, sqrt(num / den), 1e-13);
  }
  // Yamamoto's representation of a 128 x 64 block aggregated over two 32-column panels:
  // A + aQm aT aQm^T A is [S R; 0]
  {
    const int64_t m = 128, k = 64, b = 32;
    std::vector<double> A(m * k);
    for (int64_t c = 0; c < k; ++c)
      for (int64_t r = 0; r < m; ++r) A[c * m + r] = fixture(r, c, m, 0.5);
    std::vector<double> YR(A);
    pview pv = candmc_single_gpu_view();
    aggregator agg(m, k);
    QR_Yamamoto_2D(YR.data(), m, m, k, b, &pv, &agg, false);
    std::vector<double> B(A);
    upd_Yamamoto_A(agg.aQm, agg.lda_aQm, B.data(), m, m, k, k, agg.aT, &pv);
    double num = 0, den = 0;
    for (int64_t c = 0; c < k; ++c)
      for (int64_t r = 0; r < m; ++r) {
        const double rr = (r <= c) ? YR[c * m + r] : 0.0;
        num += (B[c * m + r] - rr) * (B[c * m + r] - rr);
        den += A[c * m + r] * A[c * m + r];
      }
    const bool n_ok = agg.n == k;
    fails += report(n_ok ? "aggregator ||A + aQm aT aQm^T A - R||/||A||" : "aggregator count wrong",
                    n_ok ? sqrt(num / den) : 1.0, 1e-13);
  }
  // tree_tsqr (dtpqrt's contract): [R1; R2] from the fixture's upper triangles
  // with the fixture's values left below them; R over R1's triangle, V over
  // R2's, nothing else written.  R*R^T-independent check: R^T R = R1^T R1 + R2^T R2.
  {
    const int64_t b = 21;
    std::vector<double> A(2 * b * b), A0;
    for (int64_t c = 0; c < b; ++c)
      for (int64_t r = 0; r < 2 * b; ++r) A[c * 2 * b + r] = fixture(r, c, 2 * b, 0.5);
    A0 = A;
    std::vector<double> buf(2 * b * b), T(16 * b, -7.0);
    tree_tsqr(A.data(), buf.data(), b, T.data());
    bool lower_ok = true;
    double num = 0, den = 0;
    for (int64_t c = 0; c < b; ++c) {
      for (int64_t r = 0; r < b; ++r)
        if (r > c) lower_ok = lower_ok && A[c * 2 * b + r] == A0[c * 2 * b + r] &&
                              A[c * 2 * b + b + r] == A0[c * 2 * b + b + r];
      for (int64_t d = 0; d < b; ++d) {   // (R^T R - R1^T R1 - R2^T R2)(c, d)
        double g = 0, g0 = 0;
        for (int64_t r = 0; r <= std::min(c, d); ++r) {
          g += A[c * 2 * b + r] * A[d * 2 * b + r];
          g0 += A0[c * 2 * b + r] * A0[d * 2 * b + r] + A0[c * 2 * b + b + r] * A0[d * 2 * b + b + r];
        }
        num += (g - g0) * (g - g0);
        den += g0 * g0;
      }
    }
    fails += report(lower_ok ? "tree_tsqr ||R^TR - R1^TR1 - R2^TR2||/||.||" : "tree_tsqr wrote below a diagonal",
                    lower_ok ? sqrt(num / den) : 1.0, 1e-13);
    // tau_recon('U') of the V block gives the node reflectors' tau = T's diagonal
    std::vector<double> tau(b);
    tau_recon('U', (int)b, (int)b, (int)(2 * b), A.data() + b, tau.data());
    double tdiff = 0;
    for (int64_t c = 0; c < b; ++c) tdiff = std::max(tdiff, fabs(tau[c] - T[c * 16 + (c % 16)]));
    fails += report("tree_tsqr T diagonal vs tau_recon('U')", tdiff, 1e-13);
  }
  // sym_full2band (the eigensolver's caller of the 2D QR): an orthogonal
  // similarity onto a band of width b keeps the trace and the Frobenius norm
  {
    const int64_t n = 96, b = 16;
    std::vector<double> A(n * n);
    for (int64_t c = 0; c < n; ++c)
      for (int64_t r = 0; r <= c; ++r) A[c * n + r] = A[r * n + c] = fixture(r, c, n, 0.5);
    double tr0 = 0, f0 = 0;
    for (int64_t i = 0; i < n * n; ++i) f0 += A[i] * A[i];
    for (int64_t i = 0; i < n; ++i) tr0 += A[i * n + i];
    pview pv = candmc_single_gpu_view();
    sym_full2band(A.data(), n, n, b, 8, &pv);
    // band matrix from the lower triangle: diagonal blocks and the R blocks below them
    double tr = 0, f = 0;
    for (int64_t c = 0; c < n; ++c)
      for (int64_t r = c; r < n; ++r) {
        const int64_t blk = c / b, rb = r / b;
        double v = 0;
        if (rb == blk) v = A[c * n + r];
        else if (rb == blk + 1 && (r - (blk + 1) * b) <= (c - blk * b)) v = A[c * n + r];
        f += (r == c ? 1.0 : 2.0) * v * v;
        if (r == c) tr += v;
      }
    const double d = fabs(tr - tr0) / fabs(tr0) + fabs(sqrt(f) - sqrt(f0)) / sqrt(f0);
    fails += report("sym_full2band trace + Frobenius norm kept", d, 1e-13);
  }
  // a grid larger than 1 x 1 is rejected without touching the data
  {
    pview pv = candmc_single_gpu_view();
    pv.ccol.np = 2;
    std::vector<double> A(64 * 64, 1.0);
    QR_2D(A.data(), 64, 64, 64, 16, &pv, NULL, 0);
    const bool ok = candmc_dropin_last_status() == CANDMC_ERR_ARG && A[5] == 1.0;
    printf("2x1 grid rejected: %s\n", ok ? "Test successful." : "TEST FAILED!!!");
    fails += ok ? 0 : 1;
  }
  return fails ? 1 : 0;
}
