// Least squares min ||A X - B||_F (m >= n, full column rank) on the CAQR
// factorization, with FP64 iterative refinement.
//
// The reference has no least-squares solver; this composes its pieces:
// QR_2D_pipe (any arithmetic form) -> Q^T B by applying every panel's compact
// WY factor in FP64 (the update_A step of qr_2d.cxx:124-177 on the right-hand
// sides) -> X0 = R^-1 (Q^T B)[0:n] -> iterative refinement of the augmented
// system [I A; A^T 0][r; x] = [B; 0] (Bjorck, "Iterative refinement of linear
// least squares solutions I", BIT 7, 1967), all residuals in FP64 with A kept
// resident:
//   f = B - r - A x,  g = -A^T r          (FP64 residuals of both equations)
//   h = R^-T g,  d = Q^T f
//   dx = R^-1 (d[0:n] - h),  dr = Q [h; d[n:m]]
//   x += dx,  r += dr
// Q and Q^T are the panels' compact-WY factors applied in FP64.  The fixed
// point is the exact least-squares solution whatever R's accuracy; with R from
// a backward-stable QR of A itself the iteration contracts by about
// kappa(A) * u_R per step, so the FP32 form reaches FP64 accuracy up to
// kappa ~ 1e6, and it stops at the FP64 data's own forward-error level,
// about kappa(A) * u (for kappa = 1e10, 1e-6: no FP64 solver does better on
// FP64 inputs).  By default (tuning knob "ls_refine" = 0) the refinement is
// the cheaper corrected semi-normal equations, r = B - A x, dx = R^-1 R^-T A^T r:
// with R from A's own QR it contracts as fast and reaches the same level
// (measured on the benchmark's least-squares cases), at two passes over A
// per step instead of two over A and two over Y; "ls_refine" = 1 selects the
// augmented system, which also refines r.
#include <math.h>

#include <algorithm>
#include <vector>

#include "kernels.cuh"

namespace candmc {

constexpr int TS_M = 128;   // output rows per CTA
constexpr int TS_R = 16;    // right-hand sides per CTA
constexpr int TS_K = 32;

// part[z] (r x M, ld M) = op(A)[rows of the tile, K chunk z] * X[K chunk, cols]
// op(A) = A (M x K, ld lda) or A^T (A is K x M).
template <int TRANS>
__global__ void __launch_bounds__(256) k_ts_gemm(const double* A, int64_t lda, const double* X,
                                                 int64_t ldx, int64_t M, int64_t K, int64_t r,
                                                 int64_t kchunk, double* part) {
  __shared__ double sA[TS_K][TS_M + 1];
  __shared__ double sX[TS_K][TS_R];
  const int tid = threadIdx.x;
  const int row = tid % TS_M, half = tid / TS_M;      // 2 x 8 columns
  const int64_t i0 = (int64_t)blockIdx.x * TS_M, c0 = (int64_t)blockIdx.y * TS_R;
  const int64_t k0 = (int64_t)blockIdx.z * kchunk;
  const int64_t k1 = (k0 + kchunk < K) ? k0 + kchunk : K;
  double acc[8];
#pragma unroll
  for (int v = 0; v < 8; ++v) acc[v] = 0.0;
  for (int64_t kb = k0; kb < k1; kb += TS_K) {
    for (int idx = tid; idx < TS_K * TS_M; idx += 256) {
      int kk, ii;
      if (TRANS) { kk = idx % TS_K; ii = idx / TS_K; } else { ii = idx % TS_M; kk = idx / TS_M; }
      const int64_t gi = i0 + ii, gk = kb + kk;
      double v = 0.0;
      if (gi < M && gk < k1) v = TRANS ? A[gi * lda + gk] : A[gk * lda + gi];
      sA[kk][ii] = v;
    }
    for (int idx = tid; idx < TS_K * TS_R; idx += 256) {
      const int kk = idx % TS_K, cc = idx / TS_K;
      const int64_t gk = kb + kk, gc = c0 + cc;
      sX[kk][cc] = (gk < k1 && gc < r) ? X[gc * ldx + gk] : 0.0;
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < TS_K; ++kk) {
      const double a = sA[kk][row];
#pragma unroll
      for (int v = 0; v < 8; ++v) acc[v] = fma(a, sX[kk][half * 8 + v], acc[v]);
    }
    __syncthreads();
  }
  const int64_t gi = i0 + row;
  if (gi >= M) return;
  double* out = part + (int64_t)blockIdx.z * r * M;
#pragma unroll
  for (int v = 0; v < 8; ++v) {
    const int64_t gc = c0 + half * 8 + v;
    if (gc < r) out[gc * M + gi] = acc[v];
  }
}

// One right-hand side: a 16-column tile would spend 15 of every 16 DFMAs on
// padding, so r = 1 runs one FMA per element of A (the FP64 pipe's bound for
// a matrix-vector product).
// part[z * M + i] = sum over k in chunk z of A[k * lda + i] * x[k]   (A x, A: M x K)
__global__ void __launch_bounds__(256) k_gemv_n(const double* A, int64_t lda, const double* x, int64_t M,
                                                int64_t K, int64_t kchunk, double* part) {
  __shared__ double sx[256];
  const int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x;
  const int64_t k0 = (int64_t)blockIdx.y * kchunk;
  const int64_t k1 = (k0 + kchunk < K) ? k0 + kchunk : K;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int64_t kb = k0; kb < k1; kb += 256) {
    const int kn = (int)((k1 - kb < 256) ? k1 - kb : 256);
    __syncthreads();
    if (threadIdx.x < kn) sx[threadIdx.x] = x[kb + threadIdx.x];
    __syncthreads();
    if (i < M) {
      int k = 0;
      for (; k + 4 <= kn; k += 4) {
#pragma unroll
        for (int u = 0; u < 4; ++u) acc[u] = fma(A[(kb + k + u) * lda + i], sx[k + u], acc[u]);
      }
      for (; k < kn; ++k) acc[0] = fma(A[(kb + k) * lda + i], sx[k], acc[0]);
    }
  }
  if (i < M) part[(int64_t)blockIdx.y * M + i] = (acc[0] + acc[1]) + (acc[2] + acc[3]);
}

// part[z * M + j] = sum over k in chunk z of A[j * lda + k] * x[k]   (A^T x, A: K x M):
// one warp per column j, lanes stride the rows
__global__ void __launch_bounds__(256) k_gemv_t(const double* A, int64_t lda, const double* x, int64_t M,
                                                int64_t K, int64_t kchunk, double* part) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t j = (int64_t)blockIdx.x * 8 + warp;
  if (j >= M) return;   // warp-uniform
  const int64_t k0 = (int64_t)blockIdx.y * kchunk;
  const int64_t k1 = (k0 + kchunk < K) ? k0 + kchunk : K;
  const double* a = A + j * lda;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  int64_t k = k0 + lane;
  for (; k + 96 < k1; k += 128) {
#pragma unroll
    for (int u = 0; u < 4; ++u) acc[u] = fma(a[k + 32 * u], x[k + 32 * u], acc[u]);
  }
  for (; k < k1; k += 32) acc[0] = fma(a[k], x[k], acc[0]);
  const double sum = warp_sum((acc[0] + acc[1]) + (acc[2] + acc[3]));
  if (lane == 0) part[(int64_t)blockIdx.y * M + j] = sum;
}

// out (M x r, ld ldo) = beta * Cin + alpha * sum_z part[z]
__global__ void k_ts_reduce(const double* part, int nsplit, int64_t M, int64_t r, double alpha,
                            double beta, const double* Cin, int64_t ldc, double* out, int64_t ldo) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= M * r) return;
  const int64_t i = idx % M, c = idx / M;
  double s = 0.0;
  for (int z = 0; z < nsplit; ++z) s += part[(int64_t)z * M * r + c * M + i];
  double v = alpha * s;
  if (beta != 0.0) v = fma(beta, Cin[c * ldc + i], v);
  out[c * ldo + i] = v;
}

// Inverses of the diagonal blocks of the upper triangle of R (w x w each; the
// last block may be smaller), all blocks at once: block q, one column per thread.
__global__ void k_diag_inv(const double* R, int64_t ldr, int64_t n, int w, double* Dinv) {
  const int64_t q = blockIdx.x;
  const int64_t j0 = q * w;
  const int bw = (int)((n - j0 < w) ? n - j0 : w);
  const int j = threadIdx.x;
  double* col = Dinv + q * (int64_t)w * w + (int64_t)j * w;
  if (j >= w) return;
  for (int i = w - 1; i >= 0; --i) {
    double acc = 0.0;
    if (j < bw && i < bw && i <= j) {
      acc = (i == j) ? 1.0 : 0.0;
      for (int k = i + 1; k <= j; ++k) acc = fma(-R[(j0 + k) * ldr + j0 + i], col[k], acc);
      acc /= R[(j0 + i) * ldr + j0 + i];
    }
    col[i] = acc;
  }
}

__global__ void k_add(double* Z, int64_t ldz, const double* C, int64_t ldc, int64_t m, int64_t n) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= m * n) return;
  const int64_t i = idx % m, j = idx / m;
  Z[j * ldz + i] += C[j * ldc + i];
}

// Z = Z + alpha * C (m x n)
__global__ void k_axpy(double* Z, int64_t ldz, const double* C, int64_t ldc, int64_t m, int64_t n,
                       double alpha) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= m * n) return;
  const int64_t i = idx % m, j = idx / m;
  Z[j * ldz + i] = fma(alpha, C[j * ldc + i], Z[j * ldz + i]);
}

// per column: max |D| / max |X| reported as one number (max over columns)
__global__ void k_rel_change(const double* D, int64_t ldd, const double* X, int64_t ldx, int64_t n,
                             double* out) {
  __shared__ double sd[256], sx[256];
  const int64_t c = blockIdx.x;
  double md = 0.0, mx = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    md = fmax(md, fabs(D[c * ldd + i]));
    mx = fmax(mx, fabs(X[c * ldx + i]));
  }
  sd[threadIdx.x] = md;
  sx[threadIdx.x] = mx;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      sd[threadIdx.x] = fmax(sd[threadIdx.x], sd[threadIdx.x + o]);
      sx[threadIdx.x] = fmax(sx[threadIdx.x], sx[threadIdx.x + o]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) out[c] = sx[0] > 0.0 ? sd[0] / sx[0] : sd[0];
}

static int ls_sms() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 148;
  }
  return n;
}

// out (M x r) = beta * Cin + alpha * op(A) X, FP64, op(A) M x K
static int ts_gemm(bool trans, const double* A, int64_t lda, const double* X, int64_t ldx, int64_t M,
                   int64_t K, int64_t r, double alpha, double beta, const double* Cin, int64_t ldc,
                   double* out, int64_t ldo, cudaStream_t s) {
  if (M <= 0 || r <= 0) return CANDMC_OK;
  if (r == 1 && K > 0) {
    // about 8 CTAs per SM: row (or column) blocks times K chunks
    const int64_t blk = trans ? (M + 7) / 8 : (M + 255) / 256;
    int64_t nsplit = std::max<int64_t>(1, std::min<int64_t>((8 * ls_sms() + blk - 1) / blk,
                                                            (K + 255) / 256));
    int64_t kchunk = (K + nsplit - 1) / nsplit;
    nsplit = std::max<int64_t>(1, (K + kchunk - 1) / kchunk);
    DevBuf part;
    CANDMC_RET(part.alloc(sizeof(double) * nsplit * M, s));
    {
      ProfScope ps(CANDMC_KCLASS_GEMM_TN, 2.0 * M * K, s);
      const dim3 g((unsigned)blk, (unsigned)nsplit);
      if (trans)
        k_gemv_t<<<g, 256, 0, s>>>(A, lda, X, M, K, kchunk, part.d());
      else
        k_gemv_n<<<g, 256, 0, s>>>(A, lda, X, M, K, kchunk, part.d());
      CANDMC_CK(cudaGetLastError());
    }
    ProfScope ps(CANDMC_KCLASS_REDUCE, 8.0 * nsplit * M, s);
    k_ts_reduce<<<(unsigned)((M + 255) / 256), 256, 0, s>>>(part.d(), (int)nsplit, M, 1, alpha, beta, Cin, ldc,
                                                            out, ldo);
    CANDMC_CK(cudaGetLastError());
    return CANDMC_OK;
  }
  const int64_t tiles = ((M + TS_M - 1) / TS_M) * ((r + TS_R - 1) / TS_R);
  int64_t nsplit = std::max<int64_t>(1, std::min<int64_t>((4 * ls_sms() + tiles - 1) / tiles, (K + 127) / 128));
  int64_t kchunk = ((K + nsplit - 1) / nsplit + TS_K - 1) / TS_K * TS_K;
  if (kchunk <= 0) kchunk = TS_K;
  nsplit = std::max<int64_t>(1, (K + kchunk - 1) / kchunk);
  DevBuf part;
  CANDMC_RET(part.alloc(sizeof(double) * nsplit * M * r, s));
  if (K > 0) {
    ProfScope ps(CANDMC_KCLASS_GEMM_TN, 2.0 * M * K * r, s);
    dim3 g((unsigned)((M + TS_M - 1) / TS_M), (unsigned)((r + TS_R - 1) / TS_R), (unsigned)nsplit);
    if (trans)
      k_ts_gemm<1><<<g, 256, 0, s>>>(A, lda, X, ldx, M, K, r, kchunk, part.d());
    else
      k_ts_gemm<0><<<g, 256, 0, s>>>(A, lda, X, ldx, M, K, r, kchunk, part.d());
    CANDMC_CK(cudaGetLastError());
  } else {
    CANDMC_CK(cudaMemsetAsync(part.p, 0, sizeof(double) * M * r, s));
  }
  ProfScope ps(CANDMC_KCLASS_REDUCE, 8.0 * nsplit * M * r, s);
  k_ts_reduce<<<(unsigned)((M * r + 255) / 256), 256, 0, s>>>(part.d(), (int)nsplit, M, r, alpha, beta,
                                                              Cin, ldc, out, ldo);
  CANDMC_CK(cudaGetLastError());
  return CANDMC_OK;
}

// X (n x r) <- op(R)^-1 X for the upper triangle of R (ld ldr); Dinv from k_diag_inv.
static int trsm_upper(const double* R, int64_t ldr, int64_t n, const double* Dinv, int w, double* X,
                      int64_t ldx, int64_t r, bool trans, cudaStream_t s) {
  const int64_t nblk = (n + w - 1) / w;
  DevBuf tmp;
  CANDMC_RET(tmp.alloc(sizeof(double) * w * r, s));
  for (int64_t qq = 0; qq < nblk; ++qq) {
    const int64_t q = trans ? qq : nblk - 1 - qq;
    const int64_t j0 = q * w, bw = std::min<int64_t>(w, n - j0);
    double* Xj = X + j0;
    if (!trans) {
      // tmp = X_j - R[j0:j0+bw, j0+bw:n] X[j0+bw:n]
      CANDMC_RET(ts_gemm(false, R + (j0 + bw) * ldr + j0, ldr, X + j0 + bw, ldx, bw, n - j0 - bw, r, -1.0,
                         1.0, Xj, ldx, tmp.d(), w, s));
      CANDMC_RET(small_gemm(bw, r, bw, 1.0, mref(Dinv + q * w * w, w), mref(tmp.d(), w), 0.0, Xj, ldx, s));
    } else {
      // tmp = X_j - R[0:j0, j0:j0+bw]^T X[0:j0]
      CANDMC_RET(ts_gemm(true, R + j0 * ldr, ldr, X, ldx, bw, j0, r, -1.0, 1.0, Xj, ldx, tmp.d(), w, s));
      CANDMC_RET(small_gemm(bw, r, bw, 1.0, mref(Dinv + q * w * w, w, 1), mref(tmp.d(), w), 0.0, Xj,
                            ldx, s));
    }
  }
  return CANDMC_OK;
}

// C (m x r) <- Q C or Q^T C for the factored F (Y\R, ld ldf) with every
// panel's T (b x b each), in FP64: Q^T applies the panels first to last with
// T^T, Q applies them last to first with T.
static int apply_all_q(const double* F, int64_t ldf, int64_t m, int64_t n, int64_t b, const double* Tall,
                       double* C, int64_t ldc, int64_t r, bool trans, cudaStream_t s) {
  const int64_t npan = (n + b - 1) / b;
  DevBuf z;
  CANDMC_RET(z.alloc(sizeof(double) * b * r, s));
  for (int64_t k = 0; k < npan; ++k) {
    const int64_t i = trans ? k : npan - 1 - k;
    const int64_t r0 = i * b, bb = std::min(b, n - r0);
    MatRef Ym = mref(F + r0 * ldf + r0, ldf, 0, kUnitLower);
    CANDMC_RET(gemm_tn_reduce(Ym, mref(C + r0, ldc), m - r0, (int)bb, r,
                              mref(Tall + i * b * b, b, trans ? 1 : 0, kUpper), 1.0, z.d(), bb, s));
    CANDMC_RET(gemm_nn_sub(C + r0, ldc, Ym, z.d(), bb, m - r0, r, (int)bb, s));
  }
  return CANDMC_OK;
}

int g_ls_refine = 0;

static int axpy(double* Z, int64_t ldz, const double* C, int64_t ldc, int64_t m, int64_t n, double alpha,
                cudaStream_t s) {
  if (m <= 0 || n <= 0) return CANDMC_OK;
  ProfScope ps(CANDMC_KCLASS_SMALL, 24.0 * m * n, s);
  k_axpy<<<(unsigned)((m * n + 255) / 256), 256, 0, s>>>(Z, ldz, C, ldc, m, n, alpha);
  CANDMC_CK(cudaGetLastError());
  return CANDMC_OK;
}

}  // namespace candmc

using namespace candmc;

extern "C" int candmc_ls_solve(const double* A, int64_t lda, int64_t m, int64_t n, const double* B,
                               int64_t ldb, int64_t nrhs, double* X, int64_t ldx, int64_t b,
                               int precision, int max_refine, double tol, double* stats,
                               void* stream) {
  if (!A || !B || !X || n < 1 || m < n || nrhs < 1 || b < 1 || lda < m || ldb < m || ldx < n)
    return set_error(CANDMC_ERR_ARG, "ls_solve args");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int64_t npan = (n + b - 1) / b;
  const int w = 128;
  DevBuf F, Tall, st, Bq, Dinv, Rres, Sv, D, rel;
  CANDMC_RET(F.alloc(sizeof(double) * m * n, s));
  CANDMC_RET(Tall.alloc(sizeof(double) * npan * b * b, s));
  CANDMC_RET(st.alloc(sizeof(int), s));
  CANDMC_CK(cudaMemsetAsync(st.p, 0, sizeof(int), s));
  CANDMC_CK(cudaMemcpy2DAsync(F.p, sizeof(double) * m, A, sizeof(double) * lda, sizeof(double) * m, n,
                              cudaMemcpyDeviceToDevice, s));
  // 1. factor (the caller's A stays untouched and resident for the residuals)
  CANDMC_RET(qr_2d_pipe_dev(F.d(), m, m, n, b, static_cast<int*>(st.p), precision, s, Tall.d()));
  // 2. Q^T B in FP64, panel by panel
  CANDMC_RET(Bq.alloc(sizeof(double) * m * nrhs, s));
  CANDMC_CK(cudaMemcpy2DAsync(Bq.p, sizeof(double) * m, B, sizeof(double) * ldb, sizeof(double) * m,
                              nrhs, cudaMemcpyDeviceToDevice, s));
  CANDMC_RET(apply_all_q(F.d(), m, m, n, b, Tall.d(), Bq.d(), m, nrhs, true, s));
  // 3. X0 = R^-1 (Q^T B)[0:n]
  const int64_t nblk = (n + w - 1) / w;
  CANDMC_RET(Dinv.alloc(sizeof(double) * nblk * w * w, s));
  {
    ProfScope ps(CANDMC_KCLASS_SMALL, 0.0, s);
    k_diag_inv<<<(unsigned)nblk, w, 0, s>>>(F.d(), m, n, w, Dinv.d());
    CANDMC_CK(cudaGetLastError());
  }
  CANDMC_CK(cudaMemcpy2DAsync(X, sizeof(double) * ldx, Bq.p, sizeof(double) * m, sizeof(double) * n, nrhs,
                              cudaMemcpyDeviceToDevice, s));
  CANDMC_RET(trsm_upper(F.d(), m, n, Dinv.d(), w, X, ldx, nrhs, false, s));
  // 4. refinement; r0 = B - A X0 (the augmented system refines r as well)
  CANDMC_RET(Rres.alloc(sizeof(double) * m * nrhs, s));   // r
  CANDMC_RET(Sv.alloc(sizeof(double) * n * nrhs, s));     // dx
  CANDMC_RET(D.alloc(sizeof(double) * m * nrhs, s));      // f, then d = Q^T f, then dr
  CANDMC_RET(rel.alloc(sizeof(double) * nrhs, s));
  if (g_ls_refine != 0)
    CANDMC_RET(ts_gemm(false, A, lda, X, ldx, m, n, nrhs, -1.0, 1.0, B, ldb, Rres.d(), m, s));
  DevBuf H;                                               // g, then h
  CANDMC_RET(H.alloc(sizeof(double) * n * nrhs, s));
  std::vector<double> hrel(nrhs);
  int it = 0;
  double first = -1.0, last = 0.0, prev = HUGE_VAL;
  for (; it < max_refine; ++it) {
    if (g_ls_refine == 0) {
      // corrected semi-normal equations: r = B - A x, dx = R^-1 R^-T A^T r
      CANDMC_RET(ts_gemm(false, A, lda, X, ldx, m, n, nrhs, -1.0, 1.0, B, ldb, Rres.d(), m, s));
      CANDMC_RET(ts_gemm(true, A, lda, Rres.d(), m, n, m, nrhs, 1.0, 0.0, nullptr, 0, Sv.d(), n, s));
      CANDMC_RET(trsm_upper(F.d(), m, n, Dinv.d(), w, Sv.d(), n, nrhs, true, s));
      CANDMC_RET(trsm_upper(F.d(), m, n, Dinv.d(), w, Sv.d(), n, nrhs, false, s));
    } else {
      // f = B - r - A x ;  g = -A^T r
      CANDMC_RET(ts_gemm(false, A, lda, X, ldx, m, n, nrhs, -1.0, 1.0, B, ldb, D.d(), m, s));
      CANDMC_RET(axpy(D.d(), m, Rres.d(), m, m, nrhs, -1.0, s));
      CANDMC_RET(ts_gemm(true, A, lda, Rres.d(), m, n, m, nrhs, -1.0, 0.0, nullptr, 0, H.d(), n, s));
      // h = R^-T g ;  d = Q^T f
      CANDMC_RET(trsm_upper(F.d(), m, n, Dinv.d(), w, H.d(), n, nrhs, true, s));
      CANDMC_RET(apply_all_q(F.d(), m, m, n, b, Tall.d(), D.d(), m, nrhs, true, s));
      // dx = R^-1 (d[0:n] - h)
      CANDMC_CK(cudaMemcpy2DAsync(Sv.p, sizeof(double) * n, D.p, sizeof(double) * m, sizeof(double) * n,
                                  nrhs, cudaMemcpyDeviceToDevice, s));
      CANDMC_RET(axpy(Sv.d(), n, H.d(), n, n, nrhs, -1.0, s));
      CANDMC_RET(trsm_upper(F.d(), m, n, Dinv.d(), w, Sv.d(), n, nrhs, false, s));
      // dr = Q [h; d[n:m]]
      CANDMC_CK(cudaMemcpy2DAsync(D.p, sizeof(double) * m, H.p, sizeof(double) * n, sizeof(double) * n,
                                  nrhs, cudaMemcpyDeviceToDevice, s));
      CANDMC_RET(apply_all_q(F.d(), m, m, n, b, Tall.d(), D.d(), m, nrhs, false, s));
    }
    {
      ProfScope ps(CANDMC_KCLASS_SMALL, 0.0, s);
      k_rel_change<<<(unsigned)nrhs, 256, 0, s>>>(Sv.d(), n, X, ldx, n, rel.d());
      CANDMC_CK(cudaGetLastError());
    }
    CANDMC_CK(cudaMemcpyAsync(hrel.data(), rel.p, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, s));
    CANDMC_CK(cudaStreamSynchronize(s));
    last = *std::max_element(hrel.begin(), hrel.end());
    if (first < 0.0) first = last;
    // a correction that is not smaller than the previous one (or not finite)
    // is dropped and the refinement ends with the current X: the iteration has
    // reached the FP64 data's forward-error level, or kappa(A) u_R >= 1
    if (!(last == last) || (last >= prev && last > tol)) break;
    CANDMC_RET(axpy(X, ldx, Sv.d(), n, n, nrhs, 1.0, s));
    if (g_ls_refine != 0) CANDMC_RET(axpy(Rres.d(), m, D.d(), m, m, nrhs, 1.0, s));
    prev = last;
    if (last <= tol) {
      ++it;
      break;
    }
  }
  int hst = 0;
  CANDMC_CK(cudaMemcpyAsync(&hst, st.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  CANDMC_CK(cudaStreamSynchronize(s));
  if (stats) {
    stats[0] = it;
    stats[1] = last;
    stats[2] = first;
    stats[3] = hst;
  }
  return hst;
}
