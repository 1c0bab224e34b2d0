// Host-side launchers shared between the translation units of the library.
#pragma once
#include <atomic>

#include "common.cuh"

namespace candmc {

// prof.cu: every launch goes through a ProfScope (launch count + optional
// CUDA-event timing of its class on the launching stream).  Class ids are the
// CANDMC_KCLASS_* values of the public header.
constexpr int kProfClasses = 16;
void count_launch();
void count_launches(long long n);   // kernels of a replayed CUDA graph
long long launch_total();
bool prof_on(int cls);
class ProfScope {
 public:
  ProfScope(int cls, double work, cudaStream_t s);
  ~ProfScope();
 private:
  int cls_;
  double work_;
  cudaStream_t s_;
  cudaEvent_t e0_{}, e1_{};
};

// panel.cu: direct TSQR-HR of an m x b panel, b <= kDirectB (binary tree,
// explicit Q factors; used by the fixed-scratch entry point).
int hr_direct(double* A, int64_t lda, int64_t m, int b, double* T, int64_t ldT, double* W,
              int64_t ldW, int* d_status, cudaStream_t s);
// tsqr4.cu: direct TSQR-HR with a fan-in-4 tree and compact-WY Q blocks.
extern int64_t g_leaf_rows;
extern int g_pipe_tree;
// leaf height of the panels factored by the lookahead (tuning knob
// "pipe_leaf_rows"), and the per-host-thread override it sets (0: none)
extern int64_t g_pipe_leaf_rows;
extern thread_local int64_t t_leaf_rows;
// SMs left free of persistent Ozaki CTAs while a lookahead factorization runs,
// so the panel stream is not starved (tuning knob "oz_reserve_sms")
extern int g_oz_reserve_sms;
// per host thread: > 0 caps the persistent Ozaki grid (set for the duration
// of a lookahead factorization)
extern thread_local int t_oz_cap;
int hr_direct4(double* A, int64_t lda, int64_t m, int b, double* T, int64_t ldT, double* W,
               int64_t ldW, int* d_status, cudaStream_t s);

// gemm_f64.cu
int small_gemm(int64_t M, int64_t N, int64_t K, double alpha, MatRef A, MatRef B, double beta,
               double* C, int64_t ldc, cudaStream_t s);
int gemm_tn_reduce(MatRef Y, MatRef C, int64_t m, int nb, int64_t n, MatRef Top, double alpha,
                   double* Z, int64_t ldz, cudaStream_t s);
int gemm_nn_sub(double* C, int64_t ldc, MatRef Y, const double* Z, int64_t ldz, int64_t m,
                int64_t n, int nb, cudaStream_t s);
int tri_inv(const double* X, int64_t ldx, int n, int lower, int unit, double* Xi, int64_t ldi,
            cudaStream_t s);
int materialize(MatRef X, int64_t n, int64_t k, double* out, int64_t ldo, cudaStream_t s);
int set_identity(double* out, int64_t ld, int64_t n, int64_t k, cudaStream_t s);
int invT_from_gram(const double* G, int64_t ldg, int b, double* T, int64_t ldt, cudaStream_t s);

// small.cu: signed LU and the dlarft recurrence.
int signed_nlu(double* A, double* R, int64_t b, int64_t lda, int64_t ldr, int64_t* signs,
               cudaStream_t s);
int larft_from_gram(const double* G, int64_t ldg, const double* tau, int b, double* T,
                    int64_t ldt, cudaStream_t s);

// ozaki.cu: emulated-FP64 trailing update on tcgen05.  C holds df64 pairs
// (float hi, float lo in each 8-byte slot); rows < fp64_rows are written back
// as FP64.  Top is the operator T^T applied to Y^T C.
// With c_fp64, C is FP64 storage (a panel's own columns) instead.
int apply_qt_ozaki(const double* Y, int64_t ldy, int ymask, int64_t m, int nb, MatRef Top,
                   double* C, int64_t ldc, int64_t n, int64_t fp64_rows, int* status,
                   cudaStream_t s, bool c_fp64 = false);
// rows from which hr_rec applies a half panel's Q^T to the other half, and
// forms the Gram product of its T merge, with the emulated-FP64 contraction
// when the factorization runs in a tensor-core form (emulated FP64 or FP32;
// tuning knob "panel_oz_min_rows"; 0 disables)
extern int64_t g_panel_oz_min_rows;
// least-squares refinement: 0 corrected semi-normal equations (default), 1
// augmented system (tuning knob "ls_refine")
extern int g_ls_refine;
// ozaki.cu: the same update in the FP32 form (3 BF16 slices on tcgen05, FP32
// accumulation; df64 storage of C).
int apply_qt_f32(const double* Y, int64_t ldy, int ymask, int64_t m, int nb, MatRef Top, double* C,
                 int64_t ldc, int64_t n, int64_t fp64_rows, int* status, cudaStream_t s);
// G (nb x n, ld nb) = Y^T C for FP64 operands read through masks, in emulated FP64
int gram_ozaki(const double* Y, int64_t ldy, int ymask, const double* C, int64_t ldc, int cmask, int64_t m,
               int nb, int64_t n, double* G, int* status, cudaStream_t s);
int to_df64(double* X, int64_t ld, int64_t m, int64_t n, cudaStream_t s);
int from_df64(double* X, int64_t ld, int64_t m, int64_t n, cudaStream_t s);

// capi.cu: TSQR-HR of one m x b panel (recursive blocking), T (ldT) out.
int hr_rec(double* A, int64_t lda, int64_t m, int b, double* T, int64_t ldT, int* st, int precision,
           cudaStream_t s);
// capi.cu: lookahead CAQR; Tall (nullable) receives every panel's T (b x b, ld b, panel i at i b^2).
int qr_2d_pipe_dev(double* A, int64_t lda, int64_t m, int64_t k, int64_t b, int* st, int precision,
                   cudaStream_t s, double* Tall);

// trailing update C <- (I - Y T Y^T)^T C in the requested arithmetic
// (Y: unit-lower-trapezoidal m x nb read from a Y\R buffer; T upper nb x nb).
int apply_qt(const double* Y, int64_t ldy, int64_t m, int nb, const double* T, int64_t ldT,
             double* C, int64_t ldc, int64_t n, int precision, cudaStream_t s);

}  // namespace candmc
