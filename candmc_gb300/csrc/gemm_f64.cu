// FP64 contractions of the CAQR trailing update and the small b x b products.
//
// Reference: upd_A (alg/QR/qr_2d/qr_2d.cxx:224-282) computes Z = Y^T*A with
// dgemm (:259), all-reduces Z over the process column (:265), applies T^T by
// dtrsm with T^-T (:271) and finishes with A -= Y*Z by dgemm (:275).  On one
// GPU the all-reduce becomes a deterministic split-K reduction: each CTA of
// gemm_tn owns a slice of rows and writes a partial Z, and reduce_apply sums
// the partials in a fixed order and multiplies by T^T in the same pass.
//
// GB300 note: FP64 runs at ~1.2 TFLOP/s chip-wide (about 2 DFMA/clk/SM), so
// these kernels are bound by the FP64 pipe, not by HBM (a 64x64 tile with
// 4x4 register blocking needs only 8 shared loads per 16 DFMA).
#include <algorithm>

#include "common.cuh"
#include "kernels.cuh"

namespace candmc {

constexpr int TK = 16;

// out(i, j) = sum_{k in [k0, k1)} opA(i, k) * opB(k, j), a (16 U) x (16 U)
// tile per CTA (U = 4: 64 x 64; U = 2: 32 x 32 for the narrow products
// inside a panel, where a 64 x 64 tile would be three quarters padding).
// mode 0: store into out + split * split_stride (partials), ld ldo.
// mode 1: out(i, j) -= result (out is the trailing matrix itself).
template <int U>
__global__ void __launch_bounds__(kThreads)
k_gemm_f64(MatRef A, MatRef B, int64_t M, int64_t N, int64_t K, int64_t kchunk, double* out,
           int64_t ldo, int64_t split_stride, int mode) {
  constexpr int TM = 16 * U, TN = 16 * U;
  __shared__ double sA[TK][TM + 1];
  __shared__ double sB[TK][TN + 1];
  const int tid = threadIdx.x;
  const int ti = tid % 16, tj = tid / 16;
  const int64_t i0 = (int64_t)blockIdx.x * TM, j0 = (int64_t)blockIdx.y * TN;
  const int64_t k0 = (int64_t)blockIdx.z * kchunk;
  const int64_t k1 = (k0 + kchunk < K) ? k0 + kchunk : K;
  double acc[U][U];
#pragma unroll
  for (int u = 0; u < U; ++u)
#pragma unroll
    for (int v = 0; v < U; ++v) acc[u][v] = 0.0;

  for (int64_t kb = k0; kb < k1; kb += TK) {
    // A tile: TM x TK.  Coalesce along the stored row index.
    for (int idx = tid; idx < TM * TK; idx += kThreads) {
      int ii, kk;
      if (A.trans) { kk = idx % TK; ii = idx / TK; } else { ii = idx % TM; kk = idx / TM; }
      int64_t gi = i0 + ii, gk = kb + kk;
      sA[kk][ii] = (gi < M && gk < k1) ? mat_at(A, gi, gk) : 0.0;
    }
    for (int idx = tid; idx < TK * TN; idx += kThreads) {
      int jj, kk;
      if (B.trans) { jj = idx % TN; kk = idx / TN; } else { kk = idx % TK; jj = idx / TK; }
      int64_t gj = j0 + jj, gk = kb + kk;
      sB[kk][jj] = (gj < N && gk < k1) ? mat_at(B, gk, gj) : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; ++kk) {
      double a[U], bb[U];
#pragma unroll
      for (int u = 0; u < U; ++u) a[u] = sA[kk][ti + 16 * u];
#pragma unroll
      for (int v = 0; v < U; ++v) bb[v] = sB[kk][tj + 16 * v];
#pragma unroll
      for (int u = 0; u < U; ++u)
#pragma unroll
        for (int v = 0; v < U; ++v) acc[u][v] = fma(a[u], bb[v], acc[u][v]);
    }
    __syncthreads();
  }
  double* o = out + (mode == 0 ? (int64_t)blockIdx.z * split_stride : 0);
#pragma unroll
  for (int u = 0; u < U; ++u) {
    int64_t gi = i0 + ti + 16 * u;
    if (gi >= M) continue;
#pragma unroll
    for (int v = 0; v < U; ++v) {
      int64_t gj = j0 + tj + 16 * v;
      if (gj >= N) continue;
      if (mode == 0) o[gj * ldo + gi] = acc[u][v];
      else o[gj * ldo + gi] -= acc[u][v];
    }
  }
}

// Single-column forms (one right-hand side: Q^T b, Q b).  A 16 x 16 tile for
// one column would spend 15 of every 16 DFMAs on padding, so these run one
// FMA per element of Y, which is what bounds a matrix-vector product on the
// FP64 pipe.
//
// part[z * nb + i] = sum over the rows r of chunk z of Y(r, i) * c(r): one warp
// per column i of Y (lanes stride the rows, four accumulators), warp-reduced.
__global__ void __launch_bounds__(kThreads)
k_gemv_tn(MatRef Y, MatRef C, int64_t m, int nb, int64_t kchunk, double* part) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t i = (int64_t)blockIdx.x * (kThreads / 32) + warp;
  if (i >= nb) return;   // warp-uniform
  const int64_t k0 = (int64_t)blockIdx.y * kchunk;
  const int64_t k1 = (k0 + kchunk < m) ? k0 + kchunk : m;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  int64_t r = k0 + lane;
  for (; r + 96 < k1; r += 128) {
#pragma unroll
    for (int u = 0; u < 4; ++u) acc[u] = fma(mat_at(Y, r + 32 * u, i), mat_at(C, r + 32 * u, 0), acc[u]);
  }
  for (; r < k1; r += 32) acc[0] = fma(mat_at(Y, r, i), mat_at(C, r, 0), acc[0]);
  const double sum = warp_sum((acc[0] + acc[1]) + (acc[2] + acc[3]));
  if (lane == 0) part[(int64_t)blockIdx.y * nb + i] = sum;
}

// c(r) -= sum_k Y(r, k) z(k), one thread per row r (z staged in shared memory)
__global__ void __launch_bounds__(kThreads)
k_gemv_nn_sub(double* C, MatRef Y, const double* Z, int64_t m, int nb) {
  __shared__ double sz[256];
  for (int k = threadIdx.x; k < nb; k += kThreads) sz[k] = Z[k];
  __syncthreads();
  const int64_t r = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  if (r >= m) return;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  int k = 0;
  for (; k + 4 <= nb; k += 4) {
#pragma unroll
    for (int u = 0; u < 4; ++u) acc[u] = fma(mat_at(Y, r, k + u), sz[k + u], acc[u]);
  }
  for (; k < nb; ++k) acc[0] = fma(mat_at(Y, r, k), sz[k], acc[0]);
  C[r] -= (acc[0] + acc[1]) + (acc[2] + acc[3]);
}

// Small-matrix product, 16 x 16 outputs per CTA, one per thread:
// C(i,j) = alpha * sum_k opA(i,k) opB(k,j) + beta * C(i,j)   (beta == 0: C not read).
__global__ void __launch_bounds__(kThreads)
k_small_gemm(MatRef A, MatRef B, int64_t M, int64_t N, int64_t K, double alpha, double beta,
             double* C, int64_t ldc) {
  __shared__ double sA[16][65];
  __shared__ double sB[64][17];
  const int ti = threadIdx.x % 16, tj = threadIdx.x / 16;
  const int64_t i0 = (int64_t)blockIdx.x * 16, j0 = (int64_t)blockIdx.y * 16;
  double acc = 0.0;
  for (int64_t kb = 0; kb < K; kb += 64) {
    for (int idx = threadIdx.x; idx < 16 * 64; idx += kThreads) {
      int ii = idx % 16, kk = idx / 16;
      int64_t gi = i0 + ii, gk = kb + kk;
      sA[ii][kk] = (gi < M && gk < K) ? mat_at(A, gi, gk) : 0.0;
      int jj = idx / 64, k2 = idx % 64;
      int64_t gj = j0 + jj, gk2 = kb + k2;
      sB[k2][jj] = (gj < N && gk2 < K) ? mat_at(B, gk2, gj) : 0.0;
    }
    __syncthreads();
#pragma unroll 16
    for (int kk = 0; kk < 64; ++kk) acc = fma(sA[ti][kk], sB[kk][tj], acc);
    __syncthreads();
  }
  int64_t gi = i0 + ti, gj = j0 + tj;
  if (gi < M && gj < N) {
    double v = alpha * acc;
    if (beta != 0.0) v += beta * C[gj * ldc + gi];
    C[gj * ldc + gi] = v;
  }
}

// Z(i,j) = alpha * sum_k opT(i,k) * (sum_s Zp[s](k,j))   with Zp[s] nb x n (ld nb);
// opT == nullptr: identity.  One CTA per output column j; thread (i, g) of the
// (nbp rows) x (256 / nbp groups) layout sums every G-th partial of row i, the
// groups are combined in shared memory, and the product with opT splits its k
// range over the groups the same way, so every dependent FP64 chain is about
// nsplit / G + nb / G long instead of nsplit + nb.  The summation order is
// fixed, so the result is deterministic.
__global__ void __launch_bounds__(kThreads)
k_reduce_apply(const double* Zp, int nsplit, int64_t split_stride, int nb, int nbp, int64_t n,
               MatRef Top, double alpha, double* Z, int64_t ldz) {
  __shared__ double part[kThreads];
  __shared__ double col[256];
  const int G = kThreads / nbp;
  const int i = threadIdx.x % nbp, g = threadIdx.x / nbp;
  const int64_t jc = blockIdx.x;
  double sacc = 0.0;
  if (i < nb)
    for (int sp = g; sp < nsplit; sp += G) sacc += Zp[sp * split_stride + jc * nb + i];
  part[g * nbp + i] = sacc;
  __syncthreads();
  if (g == 0) {
    double t = 0.0;
    for (int h = 0; h < G; ++h) t += part[h * nbp + i];
    col[i] = t;
  }
  __syncthreads();
  double z;
  if (Top.p == nullptr) {
    z = (g == 0 && i < nb) ? col[i] : 0.0;
  } else {
    z = 0.0;
    if (i < nb)
      for (int k = g; k < nb; k += G) z = fma(mat_at(Top, i, k), col[k], z);
  }
  __syncthreads();
  part[g * nbp + i] = z;
  __syncthreads();
  if (g == 0 && i < nb) {
    double t = 0.0;
    for (int h = 0; h < G; ++h) t += part[h * nbp + i];
    Z[jc * ldz + i] = alpha * t;
  }
}

// Triangular inverse of an n x n matrix (ld), one column per thread.
// lower != 0: lower triangular; unit != 0: unit diagonal implied.
__global__ void k_tri_inv(const double* X, int64_t ldx, int n, int lower, int unit, double* Xi,
                          int64_t ldi) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  double* col = Xi + (int64_t)j * ldi;
  if (lower) {
    for (int i = 0; i < n; ++i) {
      double acc;
      if (i < j) {
        acc = 0.0;
      } else {
        acc = (i == j) ? 1.0 : 0.0;
        for (int k = j; k < i; ++k) acc -= X[(int64_t)k * ldx + i] * col[k];
        if (!unit) acc /= X[(int64_t)i * ldx + i];
      }
      col[i] = acc;
    }
  } else {
    for (int i = n - 1; i >= 0; --i) {
      double acc;
      if (i > j) {
        acc = 0.0;
      } else {
        acc = (i == j) ? 1.0 : 0.0;
        for (int k = i + 1; k <= j; ++k) acc -= X[(int64_t)k * ldx + i] * col[k];
        if (!unit) acc /= X[(int64_t)i * ldx + i];
      }
      col[i] = acc;
    }
  }
}

// Copy op(X) (masked) into a dense n x k buffer (ld ldo).
__global__ void k_materialize(MatRef X, int64_t n, int64_t k, double* out, int64_t ldo) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * k) return;
  int64_t i = idx % n, j = idx / n;
  out[j * ldo + i] = mat_at(X, i, j);
}

// T^-T from a Gram matrix: lower part of G with halved diagonal (qr_2d.cxx:46-51);
// only the lower triangle (incl. diagonal) of T is written, as unpack_lower does.
__global__ void k_invT_from_gram(const double* G, int64_t ldg, int b, double* T, int64_t ldt) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= b * b) return;
  int i = idx % b, j = idx / b;
  if (i < j) return;
  double g = G[(int64_t)j * ldg + i];
  T[(int64_t)j * ldt + i] = (i == j) ? 0.5 * g : g;
}

// out (n x k, ld) = identity (ones on the leading diagonal, zeros elsewhere)
__global__ void k_set_identity(double* out, int64_t ld, int64_t n, int64_t k) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * k) return;
  int64_t i = idx % n, j = idx / n;
  out[j * ld + i] = (i == j) ? 1.0 : 0.0;
}

// ---------------------------------------------------------------- host side

static int num_sms() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 148;
  }
  return n;
}

int small_gemm(int64_t M, int64_t N, int64_t K, double alpha, MatRef A, MatRef B, double beta,
               double* C, int64_t ldc, cudaStream_t s) {
  if (M <= 0 || N <= 0) return CANDMC_OK;
  dim3 grid((unsigned)((M + 15) / 16), (unsigned)((N + 15) / 16));
  ProfScope ps(CANDMC_KCLASS_SMALL, 2.0 * M * N * K, s);
  k_small_gemm<<<grid, kThreads, 0, s>>>(A, B, M, N, K, alpha, beta, C, ldc);
  CANDMC_CK(cudaGetLastError());
  return CANDMC_OK;
}

// Tile width 16 U of the FP64 products (U = 4, 2, 1): the widest tile whose
// grid still gives every SM work and that is not much wider than the product
// (a product with a single right-hand side takes 16 x 16 tiles).  Each CTA's FP64 work is serial on its SM
// (about 2 DFMA/clk), so a narrow product (a panel's own b/2-wide updates,
// with 64 x 64 outputs or fewer) on a handful of 64 x 64 tiles leaves most of
// the GPU idle and takes ~60 us; the same product on 16 x 16 tiles spreads
// over the whole chip.
static int tile_u(int64_t M, int64_t N, int64_t kparts) {
  const int64_t want = 2 * (int64_t)num_sms();
  const int64_t narrow = std::min(M, N);   // no tile much wider than the product itself
  for (int U : {4, 2}) {
    if (16 * U > 2 * std::max<int64_t>(narrow, 8)) continue;
    const int64_t t = ((M + 16 * U - 1) / (16 * U)) * ((N + 16 * U - 1) / (16 * U));
    if (t * kparts >= want) return U;
  }
  return 1;
}

template <int U>
static void launch_gemm(dim3 grid, MatRef A, MatRef B, int64_t M, int64_t N, int64_t K, int64_t kchunk,
                        double* out, int64_t ldo, int64_t stride, int mode, cudaStream_t s) {
  k_gemm_f64<U><<<grid, kThreads, 0, s>>>(A, B, M, N, K, kchunk, out, ldo, stride, mode);
}

static void launch_gemm_u(int U, dim3 grid, MatRef A, MatRef B, int64_t M, int64_t N, int64_t K,
                          int64_t kchunk, double* out, int64_t ldo, int64_t stride, int mode, cudaStream_t s) {
  if (U == 4) launch_gemm<4>(grid, A, B, M, N, K, kchunk, out, ldo, stride, mode, s);
  else if (U == 2) launch_gemm<2>(grid, A, B, M, N, K, kchunk, out, ldo, stride, mode, s);
  else launch_gemm<1>(grid, A, B, M, N, K, kchunk, out, ldo, stride, mode, s);
}

// Z (nb x n, ldz) = alpha * opT * (opY^T * opC), Y and C with m rows.
// opT.p == nullptr means no triangular factor.
int gemm_tn_reduce(MatRef Y, MatRef C, int64_t m, int nb, int64_t n, MatRef Top, double alpha,
                   double* Z, int64_t ldz, cudaStream_t s) {
  if (nb <= 0 || n <= 0) return CANDMC_OK;
  if (nb > 256) return CANDMC_ERR_ARG;
  if (n == 1) {
    // one column: a warp per column of Y over row slices, about 8 CTAs per SM
    const int64_t cblk = (nb + kThreads / 32 - 1) / (kThreads / 32);
    int64_t nsplit = std::max<int64_t>(1, std::min<int64_t>((8 * (int64_t)num_sms() + cblk - 1) / cblk,
                                                            (m + 255) / 256));
    int64_t kchunk = (m + nsplit - 1) / nsplit;
    nsplit = std::max<int64_t>(1, (m + kchunk - 1) / kchunk);
    DevBuf part;
    CANDMC_RET(part.alloc(sizeof(double) * (size_t)nb * nsplit, s));
    {
      ProfScope ps(CANDMC_KCLASS_GEMM_TN, 2.0 * nb * m, s);
      k_gemv_tn<<<dim3((unsigned)cblk, (unsigned)nsplit), kThreads, 0, s>>>(Y, C, m, nb, kchunk, part.d());
    }
    CANDMC_CK(cudaGetLastError());
    int nbp = 1;
    while (nbp < nb) nbp <<= 1;
    ProfScope ps(CANDMC_KCLASS_REDUCE, 8.0 * nb * nsplit, s);
    k_reduce_apply<<<1u, kThreads, 0, s>>>(part.d(), (int)nsplit, nb, nb, nbp, 1, Top, alpha, Z, ldz);
    CANDMC_CK(cudaGetLastError());
    return CANDMC_OK;
  }
  // the widest tile that, split over 64-row slices, still fills the GPU; for
  // narrow products 16 x 16 tiles over slices down to TK rows
  const int U = tile_u(nb, n, std::max<int64_t>(1, m / 64));
  const int TM = 16 * U, TN = TM;
  const int64_t tiles = ((nb + TM - 1) / TM) * ((n + TN - 1) / TN);
  // FP64 work per CTA is what bounds these kernels: aim at ~4 CTAs per SM
  const int64_t target = 4 * (int64_t)num_sms();
  const int64_t min_rows = U == 4 ? 64 : (U == 2 ? 32 : TK);
  int64_t nsplit = std::max<int64_t>(1, std::min<int64_t>((target + tiles - 1) / tiles,
                                                          (m + min_rows - 1) / min_rows));
  nsplit = std::min<int64_t>(nsplit, 1024);
  int64_t kchunk = (m + nsplit - 1) / nsplit;
  kchunk = ((kchunk + TK - 1) / TK) * TK;
  nsplit = std::max<int64_t>(1, (m + kchunk - 1) / kchunk);
  const int64_t stride = (int64_t)nb * n;
  DevBuf part;
  CANDMC_RET(part.alloc(sizeof(double) * (size_t)stride * nsplit, s));
  MatRef Yt = Y;
  Yt.trans = !Y.trans;   // element (i, r) of Y^T is Y(r, i)
  dim3 grid((unsigned)((nb + TM - 1) / TM), (unsigned)((n + TN - 1) / TN), (unsigned)nsplit);
  {
    ProfScope ps(CANDMC_KCLASS_GEMM_TN, 2.0 * nb * n * m, s);
    launch_gemm_u(U, grid, Yt, C, nb, n, m, kchunk, part.d(), nb, stride, 0, s);
  }
  CANDMC_CK(cudaGetLastError());
  int nbp = 1;
  while (nbp < nb) nbp <<= 1;
  {
    ProfScope ps(CANDMC_KCLASS_REDUCE, 8.0 * stride * nsplit, s);
    k_reduce_apply<<<(unsigned)n, kThreads, 0, s>>>(part.d(), (int)nsplit, stride, nb, nbp, n, Top, alpha,
                                                    Z, ldz);
  }
  CANDMC_CK(cudaGetLastError());
  return CANDMC_OK;
}

// C (m x n, ldc) -= opY (m x nb) * Z (nb x n, ldz)
int gemm_nn_sub(double* C, int64_t ldc, MatRef Y, const double* Z, int64_t ldz, int64_t m, int64_t n,
                int nb, cudaStream_t s) {
  if (m <= 0 || n <= 0 || nb <= 0) return CANDMC_OK;
  if (n == 1 && nb <= 256) {
    ProfScope ps(CANDMC_KCLASS_GEMM_NN, 2.0 * m * nb, s);
    k_gemv_nn_sub<<<(unsigned)((m + kThreads - 1) / kThreads), kThreads, 0, s>>>(C, Y, Z, m, nb);
    CANDMC_CK(cudaGetLastError());
    return CANDMC_OK;
  }
  const int U = tile_u(m, n, 1);
  const int T = 16 * U;
  dim3 grid((unsigned)((m + T - 1) / T), (unsigned)((n + T - 1) / T), 1);
  ProfScope ps(CANDMC_KCLASS_GEMM_NN, 2.0 * m * n * nb, s);
  launch_gemm_u(U, grid, Y, mref(Z, ldz), m, n, nb, nb, C, ldc, 0, 1, s);
  CANDMC_CK(cudaGetLastError());
  return CANDMC_OK;
}

int tri_inv(const double* X, int64_t ldx, int n, int lower, int unit, double* Xi, int64_t ldi,
            cudaStream_t s) {
  if (n <= 0) return CANDMC_OK;
  ProfScope ps(CANDMC_KCLASS_SMALL, 0.0, s);
  k_tri_inv<<<(n + 127) / 128, 128, 0, s>>>(X, ldx, n, lower, unit, Xi, ldi);
  CANDMC_CK(cudaGetLastError());
  return CANDMC_OK;
}

int materialize(MatRef X, int64_t n, int64_t k, double* out, int64_t ldo, cudaStream_t s) {
  if (n <= 0 || k <= 0) return CANDMC_OK;
  int64_t tot = n * k;
  ProfScope ps(CANDMC_KCLASS_SMALL, 16.0 * tot, s);
  k_materialize<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(X, n, k, out, ldo);
  CANDMC_CK(cudaGetLastError());
  return CANDMC_OK;
}

int set_identity(double* out, int64_t ld, int64_t n, int64_t k, cudaStream_t s) {
  if (n <= 0 || k <= 0) return CANDMC_OK;
  int64_t tot = n * k;
  ProfScope ps(CANDMC_KCLASS_SMALL, 8.0 * tot, s);
  k_set_identity<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(out, ld, n, k);
  CANDMC_CK(cudaGetLastError());
  return CANDMC_OK;
}

int invT_from_gram(const double* G, int64_t ldg, int b, double* T, int64_t ldt, cudaStream_t s) {
  if (b <= 0) return CANDMC_OK;
  ProfScope ps(CANDMC_KCLASS_SMALL, 0.0, s);
  k_invT_from_gram<<<(b * b + 255) / 256, 256, 0, s>>>(G, ldg, b, T, ldt);
  CANDMC_CK(cudaGetLastError());
  return CANDMC_OK;
}

}  // namespace candmc
