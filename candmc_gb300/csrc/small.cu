// Small b x b kernels: the signed LU of hh_recon and the dlarft recurrence.
#include "kernels.cuh"

namespace candmc {

// Sign-choice unpivoted LU of (A - S) in place (alg/QR/hh_recon/hh_recon.cxx:43-68):
// S_ii = -1 if A_ii > 0 else +1; A_ii -= S_ii; column scaled by the pivot;
// rank-1 update.  Row i of R is negated from column i on when S_ii = -1.
// One CTA; the matrix is staged in shared memory when it fits (use_smem).
__global__ void __launch_bounds__(kThreads)
k_signed_nlu(double* A, double* R, int b, int64_t lda, int64_t ldr, int64_t* signs, int use_smem,
             int* status) {
  extern __shared__ double sh[];
  __shared__ int s_sign;
  const int tid = threadIdx.x;
  double* M = use_smem ? sh : A;
  const int64_t ldm = use_smem ? b : lda;
  if (use_smem) {
    for (int idx = tid; idx < b * b; idx += blockDim.x) sh[idx] = A[(idx / b) * lda + idx % b];
    __syncthreads();
  }
  int bad = 0;
  for (int i = 0; i < b; ++i) {
    if (tid == 0) {
      double d = M[i * ldm + i];
      s_sign = d > 0.0 ? -1 : 1;
      M[i * ldm + i] = d - (double)s_sign;
      signs[i] = s_sign;
      if (M[i * ldm + i] == 0.0 || !isfinite(M[i * ldm + i])) bad = 1;
    }
    __syncthreads();
    const int s = s_sign;
    if (s == -1)
      for (int c = i + tid; c < b; c += blockDim.x) R[c * ldr + i] = -R[c * ldr + i];
    const double piv = M[i * ldm + i];
    for (int r = i + 1 + tid; r < b; r += blockDim.x) M[i * ldm + r] /= piv;
    __syncthreads();
    const int n = b - i - 1;
    for (int idx = tid; idx < n * n; idx += blockDim.x) {
      int r = i + 1 + idx % n, c = i + 1 + idx / n;
      M[c * ldm + r] -= M[i * ldm + r] * M[c * ldm + i];
    }
    __syncthreads();
  }
  if (use_smem) {
    for (int idx = tid; idx < b * b; idx += blockDim.x) A[(idx / b) * lda + idx % b] = sh[idx];
  }
  if (bad) atomicExch(status, CANDMC_ERR_NUMERIC);
}

int signed_nlu(double* A, double* R, int64_t b, int64_t lda, int64_t ldr, int64_t* signs,
               cudaStream_t s) {
  if (b <= 0) return CANDMC_OK;
  DevBuf st;
  CANDMC_RET(st.alloc(sizeof(int), s));
  CANDMC_CK(cudaMemsetAsync(st.p, 0, sizeof(int), s));
  size_t sm = sizeof(double) * (size_t)b * b;
  int use_smem = sm <= 200 * 1024;
  if (use_smem) {
    CANDMC_CK(cudaFuncSetAttribute(k_signed_nlu, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)sm));
  } else {
    sm = 0;
  }
  ProfScope ps(CANDMC_KCLASS_SMALL, 0.0, s);
  k_signed_nlu<<<1, kThreads, sm, s>>>(A, R, (int)b, lda, ldr, signs, use_smem,
                                        static_cast<int*>(st.p));
  CANDMC_CK(cudaGetLastError());
  return CANDMC_OK;
}

// LAPACK dlarft ('F','C') from a Gram matrix G = Y^T Y:
// T_ii = tau_i, T[0:i, i] = -tau_i * T[0:i, 0:i] * G[0:i, i].  One CTA; column
// i depends on the columns before it, rows of each column run in parallel.
__global__ void __launch_bounds__(kThreads)
k_larft(const double* G, int64_t ldg, const double* tau, int b, double* T, int64_t ldt) {
  for (int i = 0; i < b; ++i) {
    const double ti = tau[i];
    for (int r = threadIdx.x; r < b; r += blockDim.x) {
      double v;
      if (r < i) {
        double acc = 0.0;
        for (int k = r; k < i; ++k) acc += T[(int64_t)k * ldt + r] * G[(int64_t)i * ldg + k];
        v = -ti * acc;
      } else {
        v = (r == i) ? ti : 0.0;
      }
      T[(int64_t)i * ldt + r] = v;
    }
    __syncthreads();
  }
}

int larft_from_gram(const double* G, int64_t ldg, const double* tau, int b, double* T,
                    int64_t ldt, cudaStream_t s) {
  if (b <= 0) return CANDMC_OK;
  ProfScope ps(CANDMC_KCLASS_SMALL, 0.0, s);
  k_larft<<<1, kThreads, 0, s>>>(G, ldg, tau, b, T, ldt);
  CANDMC_CK(cudaGetLastError());
  return CANDMC_OK;
}

}  // namespace candmc
