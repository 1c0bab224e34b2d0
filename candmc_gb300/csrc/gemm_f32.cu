// FP32 form of the CAQR trailing update: C <- C - Y (T^T (Y^T C)) with both
// contractions in FP32 arithmetic (inputs rounded to FP32, FP32 accumulation
// on the SIMT FFMA pipe, ~74 TFLOP/s on GB300).  The trailing matrix uses the
// same df64 storage as the emulated form (float hi, float lo per 8-byte
// slot), so panels, lookahead and the FP64 write-back of finished R rows are
// shared; the contraction reads hi only and the subtraction is done on the
// pair.  The result is an FP32-accurate factorization (backward error ~1e-7),
// the form the least-squares solver refines back to FP64 accuracy.
//
// Tiles: 128 x 128 outputs per CTA, 8 x 8 per thread, K steps of 8 staged in
// shared memory (double-buffered through registers).
#include "kernels.cuh"

namespace candmc {

constexpr int F_TM = 128, F_TN = 128, F_TK = 8;

struct LdY {   // element (i, k) of op(Y) from an FP64 source
  MatRef X;
  __device__ __forceinline__ float at(int64_t i, int64_t k) const { return (float)mat_at(X, i, k); }
};
struct LdHi {  // element (k, j) of a df64 column-major matrix (hi part)
  const float2* p;
  int64_t ld;
  __device__ __forceinline__ float at(int64_t k, int64_t j) const { return p[j * ld + k].x; }
};
struct LdF {   // element (k, j) of an FP32 column-major matrix
  const float* p;
  int64_t ld;
  __device__ __forceinline__ float at(int64_t k, int64_t j) const { return p[j * ld + k]; }
};

// out(i, j) = sum_{k in CTA's K range} opA(i, k) opB(k, j).
// MODE 0: store FP32 partials out0 + split * stride (ld ldo).
// MODE 1: C (df64, ld ldc) -= result; rows i < fp64_rows are written as FP64.
template <int MODE, class LA, class LB>
__global__ void __launch_bounds__(256)
k_gemm_f32(LA A, LB B, int64_t M, int64_t N, int64_t K, int64_t kchunk, float* out0, int64_t ldo,
           int64_t stride, float2* C, int64_t ldc, int64_t fp64_rows) {
  __shared__ __align__(16) float sA[2][F_TK][F_TM];
  __shared__ __align__(16) float sB[2][F_TK][F_TN];
  const int tid = threadIdx.x;
  const int ti = tid % 16, tj = tid / 16;
  const int64_t i0 = (int64_t)blockIdx.x * F_TM, j0 = (int64_t)blockIdx.y * F_TN;
  const int64_t k0 = (int64_t)blockIdx.z * kchunk;
  const int64_t k1 = (k0 + kchunk < K) ? k0 + kchunk : K;
  float acc[8][8];
#pragma unroll
  for (int u = 0; u < 8; ++u)
#pragma unroll
    for (int v = 0; v < 8; ++v) acc[u][v] = 0.0f;
  // each thread stages 4 A and 4 B elements per K step
  float ra[4], rb[4];
  // A: MODE 0 reads Y^T (K runs down Y's columns: k fastest); MODE 1 reads Y
  // itself (i runs down the columns: i fastest).  B: k fastest.
  auto a_idx = [&](int idx, int& kk, int& ii) {
    if (MODE == 0) { kk = idx % F_TK; ii = idx / F_TK; } else { ii = idx % F_TM; kk = idx / F_TM; }
  };
  auto fetch = [&](int64_t kb) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int idx = tid + q * 256;   // 0 .. 1023
      int kk, ii;
      a_idx(idx, kk, ii);
      const int64_t gi = i0 + ii, gk = kb + kk;
      ra[q] = (gi < M && gk < k1) ? A.at(gi, gk) : 0.0f;
      const int kb2 = idx % F_TK, jj = idx / F_TK;
      const int64_t gj = j0 + jj, gk2 = kb + kb2;
      rb[q] = (gj < N && gk2 < k1) ? B.at(gk2, gj) : 0.0f;
    }
  };
  auto stash = [&](int buf) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int idx = tid + q * 256;
      int kk, ii;
      a_idx(idx, kk, ii);
      sA[buf][kk][ii] = ra[q];
      sB[buf][idx % F_TK][idx / F_TK] = rb[q];
    }
  };
  int buf = 0;
  if (k0 < k1) {
    fetch(k0);
    stash(0);
  }
  __syncthreads();
  for (int64_t kb = k0; kb < k1; kb += F_TK) {
    const bool more = kb + F_TK < k1;
    if (more) fetch(kb + F_TK);
#pragma unroll
    for (int kk = 0; kk < F_TK; ++kk) {
      float a[8], bv[8];
      const float4 a0 = *reinterpret_cast<const float4*>(&sA[buf][kk][ti * 4]);
      const float4 a1 = *reinterpret_cast<const float4*>(&sA[buf][kk][64 + ti * 4]);
      const float4 b0 = *reinterpret_cast<const float4*>(&sB[buf][kk][tj * 4]);
      const float4 b1 = *reinterpret_cast<const float4*>(&sB[buf][kk][64 + tj * 4]);
      a[0] = a0.x; a[1] = a0.y; a[2] = a0.z; a[3] = a0.w;
      a[4] = a1.x; a[5] = a1.y; a[6] = a1.z; a[7] = a1.w;
      bv[0] = b0.x; bv[1] = b0.y; bv[2] = b0.z; bv[3] = b0.w;
      bv[4] = b1.x; bv[5] = b1.y; bv[6] = b1.z; bv[7] = b1.w;
#pragma unroll
      for (int u = 0; u < 8; ++u)
#pragma unroll
        for (int v = 0; v < 8; ++v) acc[u][v] = fmaf(a[u], bv[v], acc[u][v]);
    }
    if (more) stash(buf ^ 1);
    __syncthreads();
    buf ^= 1;
  }
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    const int64_t gi = i0 + (u < 4 ? ti * 4 + u : 64 + ti * 4 + (u - 4));
    if (gi >= M) continue;
#pragma unroll
    for (int v = 0; v < 8; ++v) {
      const int64_t gj = j0 + (v < 4 ? tj * 4 + v : 64 + tj * 4 + (v - 4));
      if (gj >= N) continue;
      if (MODE == 0) {
        out0[(int64_t)blockIdx.z * stride + gj * ldo + gi] = acc[u][v];
      } else {
        const int64_t ci = gj * ldc + gi;
        const float2 c = C[ci];
        // (hi, lo) - p, TwoSum on the high parts
        const float s = c.x - acc[u][v];
        const float bb = s - c.x;
        const float e = (c.x - (s - bb)) + (-acc[u][v] - bb) + c.y;
        const float h = s + e;
        const float l = e - (h - s);
        if (gi < fp64_rows) reinterpret_cast<double*>(C)[ci] = (double)h + (double)l;
        else C[ci] = make_float2(h, l);
      }
    }
  }
}

// Z (nb x n, FP32) = opT (FP64) * sum_s partials[s] (nb x n, ld nb)
__global__ void k_f32_reduce_T(const float* part, int nsplit, int64_t stride, int nb, int64_t n,
                               MatRef Top, float* Z) {
  extern __shared__ float shz[];   // nb x 16
  const int ti = threadIdx.x % 16, tj = threadIdx.x / 16;
  const int64_t j0 = (int64_t)blockIdx.y * 16;
  for (int idx = threadIdx.x; idx < nb * 16; idx += blockDim.x) {
    const int k = idx % nb, jj = idx / nb;
    const int64_t gj = j0 + jj;
    float s = 0.0f;
    if (gj < n)
      for (int sp = 0; sp < nsplit; ++sp) s += part[sp * stride + gj * nb + k];
    shz[jj * nb + k] = s;
  }
  __syncthreads();
  const int64_t gi = (int64_t)blockIdx.x * 16 + ti, gj = j0 + tj;
  if (gi >= nb || gj >= n) return;
  float acc = 0.0f;
  for (int k = 0; k < nb; ++k) acc = fmaf((float)mat_at(Top, gi, k), shz[tj * nb + k], acc);
  Z[gj * nb + gi] = acc;
}

static int f32_sms() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 148;
  }
  return n;
}

// C (df64, m x n) <- C - Y (Top (Y^T C)) in FP32 arithmetic; rows < fp64_rows
// of C are written back as FP64.
int apply_qt_f32(const double* Y, int64_t ldy, int ymask, int64_t m, int nb, MatRef Top, double* C,
                 int64_t ldc, int64_t n, int64_t fp64_rows, cudaStream_t s) {
  if (m <= 0 || n <= 0) return CANDMC_OK;
  if (nb > 256) return set_error(CANDMC_ERR_ARG, "fp32 form needs b <= 256");
  const int64_t tiles = ((nb + F_TM - 1) / F_TM) * ((n + F_TN - 1) / F_TN);
  int64_t nsplit = std::max<int64_t>(1, std::min<int64_t>((2 * f32_sms() + tiles - 1) / tiles, m / 256));
  int64_t kchunk = ((m + nsplit - 1) / nsplit + F_TK - 1) / F_TK * F_TK;
  nsplit = (m + kchunk - 1) / kchunk;
  const int64_t stride = (int64_t)nb * n;
  DevBuf part, z;
  CANDMC_RET(part.alloc(sizeof(float) * stride * nsplit, s));
  CANDMC_RET(z.alloc(sizeof(float) * stride, s));
  MatRef Ym = mref(Y, ldy, 0, ymask);
  MatRef Yt = Ym;
  Yt.trans = 1;
  float2* Cd = reinterpret_cast<float2*>(C);
  {
    ProfScope ps(CANDMC_KCLASS_F32, 2.0 * nb * n * m, s);
    dim3 g((unsigned)((nb + F_TM - 1) / F_TM), (unsigned)((n + F_TN - 1) / F_TN), (unsigned)nsplit);
    k_gemm_f32<0, LdY, LdHi><<<g, 256, 0, s>>>(LdY{Yt}, LdHi{Cd, ldc}, nb, n, m, kchunk,
                                                static_cast<float*>(part.p), nb, stride, nullptr, 0, 0);
    CANDMC_CK(cudaGetLastError());
  }
  {
    ProfScope ps(CANDMC_KCLASS_REDUCE, 4.0 * stride * nsplit, s);
    dim3 g((unsigned)((nb + 15) / 16), (unsigned)((n + 15) / 16));
    k_f32_reduce_T<<<g, 256, sizeof(float) * nb * 16, s>>>(static_cast<float*>(part.p), (int)nsplit,
                                                           stride, nb, n, Top, static_cast<float*>(z.p));
    CANDMC_CK(cudaGetLastError());
  }
  {
    ProfScope ps(CANDMC_KCLASS_F32, 2.0 * m * n * nb, s);
    dim3 g((unsigned)((m + F_TM - 1) / F_TM), (unsigned)((n + F_TN - 1) / F_TN), 1);
    k_gemm_f32<1, LdY, LdF><<<g, 256, 0, s>>>(LdY{Ym}, LdF{static_cast<float*>(z.p), nb}, m, n, nb, nb,
                                               nullptr, 0, 0, Cd, ldc, fp64_rows);
    CANDMC_CK(cudaGetLastError());
  }
  return CANDMC_OK;
}

}  // namespace candmc
