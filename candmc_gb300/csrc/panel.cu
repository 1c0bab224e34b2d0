// Direct TSQR + Householder reconstruction of a panel at most kDirectB (32)
// columns wide, all in FP64.
//
// Reference path (alg/QR/hh_recon/hh_recon.cxx:129-321 at numPes == 1 and the
// binary tree of alg/QR/tsqr/bitree_tsqr.cxx:172-232): leaf Householder QR,
// tree of [R1; R2] combines, explicit Q1 by tree descent, sign-choice LU of
// (Q1_top - S), Y2 = Q2 * U^-1, W = U * S.
//
// GPU design.  The panel's rows are split into P leaves (one CTA each).
//  kernel 1 (hr_leaf_tree): each CTA factors its leaf in shared memory
//    (Householder QR, LAPACK dlarfg convention), forms the leaf's explicit Q
//    in place and writes it to scratch.  CTAs then climb the binary tree with
//    the last-arriver rule: the second child to finish a node combines the two
//    R factors ([R1; R2] Householder QR that skips the structural zeros) and
//    stores the node's explicit Q blocks Q11, Q21 (both upper triangular).
//    Nobody waits on anybody, so no spin loop exists.  The CTA that completes
//    the root multiplies the leftmost Q11 chain, forms Q1_top, runs the signed
//    LU and writes L\(S*R) into the panel's top block, T, W and U^-1.
//  kernel 2 (hr_form_y): each leaf CTA multiplies its root-to-leaf chain of
//    Q11/Q21 blocks into U^-1 and writes Y = Q_leaf * (chain * U^-1).
// The result is the canonical Householder factor (independent of the tree
// shape), which is what makes it comparable with the reference.
#include <math.h>

#include <algorithm>

#include "kernels.cuh"

namespace candmc {

// One Householder step on a column-major shared-memory matrix S (leading
// dimension ld): reflector j is generated from head row j and tail rows
// [t0, t1) of column j and applied to columns j+1 .. ncols-1.  LAPACK dlarfg:
// beta = -sign(alpha)*hypot(alpha, ||x||), tau = (beta-alpha)/beta,
// v = x/(alpha-beta); tau = 0 when ||x|| == 0.
__device__ void house_step(double* S, int ld, int j, int t0, int t1, int ncols, double* tau_out,
                           double* red) {
  __shared__ double h_tau, h_scal;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  for (int c = j + warp; c < ncols; c += nw) {
    double acc = 0.0;
    for (int r = t0 + lane; r < t1; r += 32) acc += S[j * ld + r] * S[c * ld + r];
    acc = warp_sum(acc);
    if (lane == 0) red[c] = acc;
  }
  __syncthreads();
  if (tid == 0) {
    double alpha = S[j * ld + j];
    double xn2 = red[j];
    if (xn2 == 0.0) {
      h_tau = 0.0;
      h_scal = 0.0;
    } else {
      double beta = -copysign(hypot(alpha, sqrt(xn2)), alpha);
      h_tau = (beta - alpha) / beta;
      h_scal = 1.0 / (alpha - beta);
      S[j * ld + j] = beta;
    }
    tau_out[j] = h_tau;
  }
  __syncthreads();
  const double tau = h_tau, scal = h_scal;
  if (tau == 0.0) return;
  for (int c = j + 1 + tid; c < ncols; c += blockDim.x) red[c] = S[c * ld + j] + scal * red[c];
  __syncthreads();
  const int nt = t1 - t0, nc = ncols - j - 1;
  for (int c = j + 1 + tid; c < ncols; c += blockDim.x) S[c * ld + j] -= tau * red[c];
  for (int idx = tid; idx < nt * nc; idx += blockDim.x) {
    int r = t0 + idx % nt, c = j + 1 + idx / nt;
    S[c * ld + r] -= tau * (scal * S[j * ld + r]) * red[c];
  }
  __syncthreads();
  for (int r = t0 + tid; r < t1; r += blockDim.x) S[j * ld + r] *= scal;
  __syncthreads();
}

// Explicit-Q step (LAPACK dorg2r, applied in place): for reflector i (head i,
// tail [t0, t1)), apply H_i to columns i+1..ncols-1, then turn column i into
// H_i e_i.  Called for i = ncols-1 down to 0 after the factorization.
__device__ void orgq_step(double* S, int ld, int i, int t0, int t1, int ncols, const double* tau,
                          double* red) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const double ti = tau[i];
  if (ti != 0.0 && i + 1 < ncols) {
    for (int c = i + 1 + warp; c < ncols; c += nw) {
      double acc = 0.0;
      for (int r = t0 + lane; r < t1; r += 32) acc += S[i * ld + r] * S[c * ld + r];
      acc = warp_sum(acc);
      if (lane == 0) red[c] = acc + S[c * ld + i];
    }
    __syncthreads();
    const int nt = t1 - t0, nc = ncols - i - 1;
    for (int c = i + 1 + tid; c < ncols; c += blockDim.x) S[c * ld + i] -= ti * red[c];
    for (int idx = tid; idx < nt * nc; idx += blockDim.x) {
      int r = t0 + idx % nt, c = i + 1 + idx / nt;
      S[c * ld + r] -= ti * S[i * ld + r] * red[c];
    }
    __syncthreads();
  }
  for (int r = t0 + tid; r < t1; r += blockDim.x) S[i * ld + r] *= -ti;
  for (int r = tid; r < i; r += blockDim.x) S[i * ld + r] = 0.0;
  if (tid == 0) S[i * ld + i] = 1.0 - ti;
  __syncthreads();
}

// C = A * B for b x b shared-memory matrices (ld b); C must not alias A or B.
__device__ void smem_mm(const double* A, const double* B, double* C, int b) {
  for (int idx = threadIdx.x; idx < b * b; idx += blockDim.x) {
    int i = idx % b, j = idx / b;
    double acc = 0.0;
    for (int k = 0; k < b; ++k) acc += A[k * b + i] * B[j * b + k];
    C[j * b + i] = acc;
  }
  __syncthreads();
}

__device__ void load_bxb(double* dst, const double* src, int64_t ld, int b) {
  for (int idx = threadIdx.x; idx < b * b; idx += blockDim.x) {
    int i = idx % b, j = idx / b;
    dst[j * b + i] = __ldcg(src + j * ld + i);
  }
  __syncthreads();
}

struct HrArgs {
  double* A;        // panel, m x b, lda
  int64_t lda;
  int64_t m;
  int b;
  double* Qw;       // scratch m x b (ld m): explicit leaf Q factors
  double* Rn;       // scratch nnodes x b x b: R of every tree node
  double* Q11;      // scratch nnodes x b x b: node Q blocks (internal nodes)
  double* Q21;
  unsigned* cnt;    // nnodes arrival counters, zeroed before launch
  double* T;        // out b x b (ldT), upper
  int64_t ldT;
  double* W;        // out b x b (ldW) or nullptr
  int64_t ldW;
  double* Uinv;     // scratch b x b: U^-1
  int* status;      // device status word (0 = ok)
  TreeDesc tree;
};

// first row of leaf i when m rows are split into P nearly equal leaves: floor(m*i/P)
__host__ __device__ __forceinline__ int64_t leaf_row0(int64_t m, int P, int i) {
  return (m / P) * i + (m % P) * i / P;
}

// Signed LU, R scaling, and the T / W / U^-1 / top-block outputs.  One CTA.
__device__ void hr_root_finalize(const HrArgs& a, double* smem) {
  const int b = a.b, tid = threadIdx.x;
  double* sR = smem;
  double* sM = sR + b * b;
  double* sQ = sM + b * b;
  double* sX = sQ + b * b;
  __shared__ int s_sign[kDirectB];
  const TreeDesc& t = a.tree;

  load_bxb(sR, a.Rn + (size_t)t.base[t.depth] * b * b, b, b);
  for (int idx = tid; idx < b * b; idx += blockDim.x) sM[idx] = (idx % b == idx / b) ? 1.0 : 0.0;
  __syncthreads();
  for (int lvl = t.depth; lvl >= 1; --lvl) {
    if (t.nlev[lvl - 1] > 1) {
      load_bxb(sX, a.Q11 + (size_t)t.base[lvl] * b * b, b, b);
      smem_mm(sX, sM, sQ, b);
      for (int idx = tid; idx < b * b; idx += blockDim.x) sM[idx] = sQ[idx];
      __syncthreads();
    }
  }
  // Q1_top = Q_leaf0[0:b, :] * chain
  load_bxb(sX, a.Qw, a.m, b);
  smem_mm(sX, sM, sQ, b);

  // signed LU of (Q1_top - S), hh_recon.cxx:43-68
  for (int i = 0; i < b; ++i) {
    if (tid == 0) {
      double d = sQ[i * b + i];
      int s = d > 0.0 ? -1 : 1;
      s_sign[i] = s;
      sQ[i * b + i] = d - (double)s;
    }
    __syncthreads();
    double piv = sQ[i * b + i];
    for (int r = i + 1 + tid; r < b; r += blockDim.x) sQ[i * b + r] /= piv;
    __syncthreads();
    int n = b - i - 1;
    for (int idx = tid; idx < n * n; idx += blockDim.x) {
      int r = i + 1 + idx % n, c = i + 1 + idx / n;
      sQ[c * b + r] -= sQ[i * b + r] * sQ[c * b + i];
    }
    __syncthreads();
  }
  // top block of the panel: L strictly below, S*R on/above the diagonal; W = U*S
  for (int idx = tid; idx < b * b; idx += blockDim.x) {
    int r = idx % b, c = idx / b;
    a.A[c * a.lda + r] = (r > c) ? sQ[c * b + r] : (double)s_sign[r] * sR[c * b + r];
    if (a.W) a.W[c * a.ldW + r] = (r <= c) ? sQ[c * b + r] * (double)s_sign[c] : 0.0;
  }
  // T = -W * L^-T: row i by forward substitution (T upper since W is)
  for (int i = tid; i < b; i += blockDim.x) {
    for (int k = 0; k < b; ++k) {
      double w = (i <= k) ? sQ[k * b + i] * (double)s_sign[k] : 0.0;
      double acc = -w;
      for (int j = 0; j < k; ++j) acc -= sQ[j * b + k] * sX[j * b + i];
      sX[k * b + i] = acc;   // sX reused as T (row i is owned by this thread)
    }
  }
  __syncthreads();
  for (int idx = tid; idx < b * b; idx += blockDim.x) {
    int r = idx % b, c = idx / b;
    a.T[c * a.ldT + r] = (r <= c) ? sX[c * b + r] : 0.0;
  }
  // U^-1 by back substitution, one column per thread
  for (int j = tid; j < b; j += blockDim.x) {
    for (int i = b - 1; i >= 0; --i) {
      double acc;
      if (i > j) {
        acc = 0.0;
      } else {
        acc = (i == j) ? 1.0 : 0.0;
        for (int k = i + 1; k <= j; ++k) acc -= sQ[k * b + i] * sM[j * b + k];
        acc /= sQ[i * b + i];
      }
      sM[j * b + i] = acc;   // sM reused as U^-1 (column j owned by this thread)
    }
  }
  __syncthreads();
  int bad = 0;
  for (int idx = tid; idx < b * b; idx += blockDim.x) {
    double v = sM[idx];
    if (!isfinite(v)) bad = 1;
    a.Uinv[idx] = v;
  }
  if (bad) atomicExch(a.status, CANDMC_ERR_NUMERIC);
}

__global__ void __launch_bounds__(kThreads) hr_leaf_tree(HrArgs a) {
  extern __shared__ double smem[];
  __shared__ double s_tau[kDirectB];
  __shared__ double s_red[kDirectB + 1];
  __shared__ int s_second;
  const int b = a.b, tid = threadIdx.x;
  const TreeDesc& t = a.tree;
  const int leaf = blockIdx.x;
  const int64_t r0 = leaf_row0(a.m, t.P, leaf);
  const int L = (int)(leaf_row0(a.m, t.P, leaf + 1) - r0);

  // ---- leaf: load, Householder QR, R out, explicit Q out ----
  double* S = smem;
  for (int c = 0; c < b; ++c)
    for (int r = tid; r < L; r += blockDim.x) S[c * L + r] = a.A[c * a.lda + r0 + r];
  __syncthreads();
  for (int j = 0; j < b; ++j) house_step(S, L, j, j + 1, L, b, s_tau, s_red);
  double* Rleaf = a.Rn + (size_t)(t.base[0] + leaf) * b * b;
  for (int idx = tid; idx < b * b; idx += blockDim.x) {
    int r = idx % b, c = idx / b;
    Rleaf[idx] = (r <= c) ? S[c * L + r] : 0.0;
  }
  for (int i = b - 1; i >= 0; --i) orgq_step(S, L, i, i + 1, L, b, s_tau, s_red);
  for (int c = 0; c < b; ++c)
    for (int r = tid; r < L; r += blockDim.x) a.Qw[c * a.m + r0 + r] = S[c * L + r];

  // ---- climb the tree (last arriver combines) ----
  int node = leaf;
  for (int lvl = 0; lvl < t.depth; ++lvl) {
    const int parent = node >> 1;
    double* Rpar = a.Rn + (size_t)(t.base[lvl + 1] + parent) * b * b;
    const bool has_pair = (2 * parent + 1) < t.nlev[lvl];
    if (!has_pair) {
      // pass-through node: R moves up unchanged (this CTA is its only child)
      const double* Rme = a.Rn + (size_t)(t.base[lvl] + node) * b * b;
      __syncthreads();
      for (int idx = tid; idx < b * b; idx += blockDim.x) Rpar[idx] = __ldcg(Rme + idx);
      __syncthreads();
      node = parent;
      continue;
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) s_second = atomicAdd(a.cnt + t.base[lvl + 1] + parent, 1u) == 1u;
    __syncthreads();
    if (!s_second) return;
    __threadfence();
    // [R_left; R_right] as a dense 2b x b matrix in shared memory (ld 2b)
    double* S2 = smem;
    const int ld2 = 2 * b;
    const double* Rl = a.Rn + (size_t)(t.base[lvl] + 2 * parent) * b * b;
    const double* Rr = a.Rn + (size_t)(t.base[lvl] + 2 * parent + 1) * b * b;
    for (int idx = tid; idx < b * b; idx += blockDim.x) {
      int r = idx % b, c = idx / b;
      S2[c * ld2 + r] = (r <= c) ? __ldcg(Rl + idx) : 0.0;
      S2[c * ld2 + b + r] = (r <= c) ? __ldcg(Rr + idx) : 0.0;
    }
    __syncthreads();
    // reflector j: head row j, tail rows b .. b+j (structure of two triangles)
    for (int j = 0; j < b; ++j) house_step(S2, ld2, j, b, b + j + 1, b, s_tau, s_red);
    for (int idx = tid; idx < b * b; idx += blockDim.x) {
      int r = idx % b, c = idx / b;
      Rpar[idx] = (r <= c) ? S2[c * ld2 + r] : 0.0;
    }
    for (int i = b - 1; i >= 0; --i) orgq_step(S2, ld2, i, b, b + i + 1, b, s_tau, s_red);
    double* q11 = a.Q11 + (size_t)(t.base[lvl + 1] + parent) * b * b;
    double* q21 = a.Q21 + (size_t)(t.base[lvl + 1] + parent) * b * b;
    for (int idx = tid; idx < b * b; idx += blockDim.x) {
      int r = idx % b, c = idx / b;
      q11[idx] = S2[c * ld2 + r];
      q21[idx] = S2[c * ld2 + b + r];
    }
    __syncthreads();
    node = parent;
  }
  // only the CTA that completed the root (or the single leaf) gets here
  __threadfence();
  __syncthreads();
  hr_root_finalize(a, smem);
}

__global__ void __launch_bounds__(kThreads) hr_form_y(HrArgs a) {
  extern __shared__ double smem[];
  const int b = a.b, tid = threadIdx.x;
  const TreeDesc& t = a.tree;
  const int leaf = blockIdx.x;
  const int64_t r0 = leaf_row0(a.m, t.P, leaf);
  const int64_t r1 = leaf_row0(a.m, t.P, leaf + 1);
  double* sM = smem;
  double* sX = sM + b * b;
  double* sY = sX + b * b;
  load_bxb(sM, a.Uinv, b, b);
  for (int lvl = t.depth; lvl >= 1; --lvl) {
    const int nd = leaf >> lvl;
    if (2 * nd + 1 < t.nlev[lvl - 1]) {
      const int child = leaf >> (lvl - 1);
      const double* q = ((child & 1) ? a.Q21 : a.Q11) + (size_t)(t.base[lvl] + nd) * b * b;
      load_bxb(sX, q, b, b);
      smem_mm(sX, sM, sY, b);
      for (int idx = tid; idx < b * b; idx += blockDim.x) sM[idx] = sY[idx];
      __syncthreads();
    }
  }
  // Y rows below the top block: Y[r, :] = Q_leaf[r, :] * M   (M upper triangular)
  for (int64_t r = r0 + tid; r < r1; r += blockDim.x) {
    if (r < b) continue;
    double q[kDirectB];
#pragma unroll
    for (int k = 0; k < kDirectB; ++k) q[k] = (k < b) ? a.Qw[(int64_t)k * a.m + r] : 0.0;
    for (int c = 0; c < b; ++c) {
      double acc = 0.0;
#pragma unroll
      for (int k = 0; k < kDirectB; ++k)
        if (k <= c) acc += q[k] * sM[c * b + k];
      a.A[c * a.lda + r] = acc;
    }
  }
}

// Host launcher of the direct TSQR-HR (b <= kDirectB).  T (ldT) and W (ldW,
// nullable) receive the compact-WY factor and U*S.
int hr_direct(double* A, int64_t lda, int64_t m, int b, double* T, int64_t ldT, double* W,
              int64_t ldW, int* d_status, cudaStream_t s) {
  if (b < 1 || b > kDirectB || m < b) return CANDMC_ERR_ARG;
  // leaves of ~64 rows (at least b rows each), at most m/b leaves
  int64_t P64 = m / 64;
  int64_t Pmax = m / b;
  int64_t P = P64 < 1 ? 1 : P64;
  if (P > Pmax) P = Pmax;
  if (P < 1) P = 1;
  if (P > (1 << 24)) return CANDMC_ERR_ARG;
  TreeDesc tree = make_tree((int)P);
  const int64_t Lmax = (m + P - 1) / P;
  size_t sm_leaf = sizeof(double) * (size_t)std::max<int64_t>(Lmax * b, 4 * (int64_t)b * b);
  sm_leaf = std::max(sm_leaf, sizeof(double) * (size_t)(2 * b * b));
  if (sm_leaf > 200 * 1024) return CANDMC_ERR_ARG;

  const size_t nb2 = (size_t)b * b;
  DevBuf qw, rn, q11, q21, cnt, uinv;
  CANDMC_RET(qw.alloc(sizeof(double) * (size_t)m * b, s));
  CANDMC_RET(rn.alloc(sizeof(double) * nb2 * tree.nnodes, s));
  CANDMC_RET(q11.alloc(sizeof(double) * nb2 * tree.nnodes, s));
  CANDMC_RET(q21.alloc(sizeof(double) * nb2 * tree.nnodes, s));
  CANDMC_RET(cnt.alloc(sizeof(unsigned) * tree.nnodes, s));
  CANDMC_RET(uinv.alloc(sizeof(double) * nb2, s));
  CANDMC_CK(cudaMemsetAsync(cnt.p, 0, sizeof(unsigned) * tree.nnodes, s));

  HrArgs a;
  a.A = A; a.lda = lda; a.m = m; a.b = b;
  a.Qw = qw.d(); a.Rn = rn.d(); a.Q11 = q11.d(); a.Q21 = q21.d();
  a.cnt = static_cast<unsigned*>(cnt.p);
  a.T = T; a.ldT = ldT; a.W = W; a.ldW = ldW; a.Uinv = uinv.d();
  a.status = d_status; a.tree = tree;
  CANDMC_CK(cudaFuncSetAttribute(hr_leaf_tree, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sm_leaf));
  {
    // algorithmic work: leaf QR + explicit leaf Q (~4 m b^2) and the tree nodes
    ProfScope ps(CANDMC_KCLASS_PANEL_LEAF, 4.0 * m * b * b, s);
    hr_leaf_tree<<<(unsigned)P, kThreads, sm_leaf, s>>>(a);
  }
  CANDMC_CK(cudaGetLastError());
  size_t sm_y = sizeof(double) * 3 * nb2;
  {
    ProfScope ps(CANDMC_KCLASS_PANEL_Y, 1.0 * m * b * b, s);
    hr_form_y<<<(unsigned)P, kThreads, sm_y, s>>>(a);
  }
  CANDMC_CK(cudaGetLastError());
  return CANDMC_OK;
}

// Same two kernels as hr_direct, on scratch the caller provides (no
// allocation here).  P leaves of at most 256 rows.  The caller zeroes cnt and
// the status word before the launch and guarantees the scratch sizes of
// hr_prealloc_sizes().
void hr_prealloc_sizes(int64_t m, int b, int64_t* P, int64_t* nnodes) {
  int64_t p = (m + 255) / 256;
  if (p > m / b) p = m / b;
  if (p < 1) p = 1;
  *P = p;
  *nnodes = make_tree((int)p).nnodes;
}

int hr_direct_prealloc(double* A, int64_t lda, int64_t m, int b, double* T, int64_t ldT, double* W,
                       int64_t ldW, double* Qw, double* Rn, double* Q11, double* Q21,
                       unsigned* cnt, double* Uinv, int* d_status, cudaStream_t s) {
  if (b < 1 || b > kDirectB || m < b) return CANDMC_ERR_ARG;
  int64_t P, nn;
  hr_prealloc_sizes(m, b, &P, &nn);
  TreeDesc tree = make_tree((int)P);
  const int64_t Lmax = (m + P - 1) / P;
  size_t sm_leaf = sizeof(double) * (size_t)std::max<int64_t>(Lmax * b, 4 * (int64_t)b * b);
  if (sm_leaf > 200 * 1024) return CANDMC_ERR_ARG;
  HrArgs a;
  a.A = A; a.lda = lda; a.m = m; a.b = b;
  a.Qw = Qw; a.Rn = Rn; a.Q11 = Q11; a.Q21 = Q21; a.cnt = cnt;
  a.T = T; a.ldT = ldT; a.W = W; a.ldW = ldW; a.Uinv = Uinv;
  a.status = d_status; a.tree = tree;
  {
    ProfScope ps(CANDMC_KCLASS_PANEL_LEAF, 4.0 * m * b * b, s);
    hr_leaf_tree<<<(unsigned)P, kThreads, sm_leaf, s>>>(a);
  }
  CANDMC_CK(cudaGetLastError());
  {
    ProfScope ps(CANDMC_KCLASS_PANEL_Y, 1.0 * m * b * b, s);
    hr_form_y<<<(unsigned)P, kThreads, sizeof(double) * 3 * (size_t)b * b, s>>>(a);
  }
  CANDMC_CK(cudaGetLastError());
  return CANDMC_OK;
}

// Raise the leaf kernel's dynamic shared-memory limit (no allocation).
int hr_prealloc_setup() {
  CANDMC_CK(cudaFuncSetAttribute(hr_leaf_tree, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 200 * 1024));
  return CANDMC_OK;
}

}  // namespace candmc
