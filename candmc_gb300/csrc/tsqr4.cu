// Direct TSQR + Householder reconstruction of a panel at most kDirectB (32)
// columns wide, FP64, with a fan-in-4 reduction tree and compact-WY Q blocks.
//
// Reference path: alg/QR/hh_recon/hh_recon.cxx:129-321 with the TSQR of
// alg/QR/tsqr/bitree_tsqr.cxx:91-248 and the Q1 construction of
// alg/QR/tsqr/construct_tsqr_Q.cxx:34-242.  The reference pairs ranks in a
// binary tree and forms Q1 by applying every node's reflectors (dtprfb) and
// every leaf's reflectors (dormqr) to [I; 0].  On GB300 the FP64 pipe is
// narrow (about 2 DFMA/clk/SM) and every Householder step is a chain of
// dependent FP64 operations and block barriers, so the design minimises the
// number of sequential steps on the critical path:
//  * leaves of ~64 rows, one CTA each: b Householder steps, then the leaf's
//    compact-WY T (LAPACK dlarft from the Gram matrix V^T V, an independent
//    recurrence per row of T);
//  * a fan-in-4 tree (last arriver combines, no waiting): the node stacks up
//    to four R factors and runs b Householder steps on the stacked matrix (the
//    zeros below the children's diagonals stay zero); with V = [I; V_2..V_4]
//    the node's Q blocks are Q_1 = I - T and Q_k = -V_k T (all upper
//    triangular), so no explicit-Q pass is needed;
//  * the CTA that completes the root forms Q1_top = C0 - V0 (T0 (V0^T C0)),
//    C0 the chain of Q_1 blocks, runs the sign-choice LU and writes L\(S R),
//    T, W and U^-1;
//  * kernel 2: each leaf multiplies its root-to-leaf chain of Q blocks into
//    U^-1 (M) and writes Y = [M; 0] - V (T (V_top^T M)).
// The Householder factor is canonical, so the result equals the binary-tree
// reconstruction and LAPACK's dgeqrf up to rounding.
#include <math.h>

#include <algorithm>

#include "kernels.cuh"

namespace candmc {

constexpr int kFan = 4;

// Target rows per TSQR leaf (tuning knob, candmc_set_tuning("leaf_rows", v)).
int64_t g_leaf_rows = 64;
constexpr int kTriScratch = 512 + kDirectB * kDirectB;   // h4_tri_inv workspace (doubles)

__device__ __forceinline__ int64_t t4_leaf_row0(int64_t m, int P, int i) {
  return (m / P) * i + (m % P) * i / P;
}

// FP64 reciprocal and reciprocal square root by Newton-Raphson refinement of
// an FP32 seed (Newton's iteration y <- y (2 - x y) and y <- y (3 - x y^2)/2;
// each step squares the relative error, so two steps take the ~2^-23 seed
// below FP64 rounding).  On this GPU an FP64 divide or square root costs
// about ten dependent FP64 operations, which these replace on the reflector's
// critical path.  Values outside FP32's range fall back to the FP64 operation.
__device__ __forceinline__ double nr_rcp(double x) {
  const float xf = (float)x;
  if (!(fabsf(xf) > 1e-37f && fabsf(xf) < 1e37f)) return 1.0 / x;
  double y = (double)(1.0f / xf);
  double e = fma(-x, y, 1.0);
  y = fma(y, e, y);
  e = fma(-x, y, 1.0);
  return fma(y, e, y);
}

__device__ __forceinline__ double nr_rsqrt(double q) {
  const float qf = (float)q;
  if (!(qf > 1e-37f && qf < 1e37f)) return 1.0 / sqrt(q);
  double y = (double)rsqrtf(qf);
  const double hq = 0.5 * q;
#pragma unroll
  for (int it = 0; it < 2; ++it) {
    const double t = y * y;
    y = y * fma(-hq, t, 1.5);
  }
  return y;
}

// One Householder step on the column-major shared matrix S (ld): head row j,
// tail rows {r < nrows : tail(r, j)}, columns j..ncols-1 (ncols <= 32).
// beta = -sign(alpha) sqrt(q), q = alpha^2 + ||x||^2:  with r = q^-1/2,
// beta = -sign(alpha) q r, 1/beta = -sign(alpha) r, tau = 1 - alpha / beta,
// scal = 1 / (alpha - beta) (LAPACK dlarfg).  An all-zero tail takes the
// reconstruction's convention tau = 2 (H = I - 2 e_j e_j^T, beta = -alpha)
// rather than LAPACK's tau = 0, so that T^-1 = striu(V^T V) + diag(V^T V)/2
// holds for every reflector.
// Phase A (all warps): each thread owns rows and forms x_r S[r, c] for the 32
// columns; a warp transpose-reduction (16+8+4+2+1 exchanges) leaves the sum
// of column l in lane l.  Phase B (warp 0): column sums, scalars, head row.
// Phase C: row owners update their tail rows and store v.  Three barriers.
// part: 8 x 32 doubles, wsm: 32 doubles of shared scratch.
template <class Tail>
__device__ void h4_step(double* S, int ld, int nrows, int j, int ncols, Tail tail, double* tau,
                        double* part, double* wsm) {
  __shared__ double s_tau, s_scal;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nwarp_rows = (nrows + 31) >> 5;
  if (warp < nwarp_rows) {
    double p[32];
#pragma unroll
    for (int c = 0; c < 32; ++c) p[c] = 0.0;
    for (int r = tid; r < nrows; r += blockDim.x) {
      if (!tail(r, j)) continue;
      const double x = S[j * ld + r];
#pragma unroll
      for (int c = 0; c < 32; ++c)
        if (c >= j && c < ncols) p[c] = fma(x, S[c * ld + r], p[c]);
    }
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
      const bool up = (lane & off) != 0;
#pragma unroll
      for (int k = 0; k < off; ++k) {
        const double send = up ? p[k] : p[k + off];
        const double keep = up ? p[k + off] : p[k];
        p[k] = keep + __shfl_xor_sync(0xffffffffu, send, off);
      }
    }
    part[warp * 32 + lane] = p[0];   // sum over this warp's rows of column `lane`
  }
  __syncthreads();
  if (warp == 0) {
    double s = 0.0;
    const int nw = nwarp_rows < 8 ? nwarp_rows : 8;
    for (int w = 0; w < nw; ++w) s += part[w * 32 + lane];
    const double xn2 = __shfl_sync(0xffffffffu, s, j);
    const double alpha = S[j * ld + j];
    double tj, sc, beta;
    if (xn2 == 0.0) {
      tj = 2.0;
      sc = 0.0;
      beta = -alpha;
    } else {
      const double q = fma(alpha, alpha, xn2);
      const double r = nr_rsqrt(q);
      const double sg = alpha >= 0.0 ? -1.0 : 1.0;   // -sign(alpha), sign(0) = +
      beta = sg * q * r;
      tj = fma(-alpha, sg * r, 1.0);
      sc = nr_rcp(alpha - beta);
    }
    // head row: w_c = S[j,c] + scal * s_c;  S[j,c] -= tau * w_c
    if (lane > j && lane < ncols) {
      const double w = fma(sc, s, S[lane * ld + j]);
      wsm[lane] = w;
      S[lane * ld + j] -= tj * w;
    }
    if (lane == 0) {
      S[j * ld + j] = beta;
      tau[j] = tj;
      s_tau = tj;
      s_scal = sc;
    }
  }
  __syncthreads();
  const double tj = s_tau, sc = s_scal;
  // tail rows: v_r = scal * x_r;  S[r,c] -= tau * v_r * w_c;  column j <- v
  for (int r = tid; r < nrows; r += blockDim.x) {
    if (!tail(r, j)) continue;
    const double v = sc * S[j * ld + r];
    const double tv = tj * v;
    for (int c = j + 1; c < ncols; ++c) S[c * ld + r] = fma(-tv, wsm[c], S[c * ld + r]);
    S[j * ld + r] = v;
  }
  __syncthreads();
}

// Inverse of the upper triangle of X (b x b, ld b, b <= 32; unit: diagonal
// taken as 1) into Xi, by recursive 2 x 2 block inversion done bottom-up:
// inv([[A, B], [0, C]]) = [[A^-1, -A^-1 B C^-1], [0, C^-1]].  Every level is
// two small products computed in parallel, so the dependent FP64 chain is
// about 2 (1 + 2 + 4 + 8 + 16) operations instead of the b^2 / 2 of a
// substitution.  The size is padded to a power of two with identity rows.
// scratch: >= kTriScratch doubles.
__device__ void h4_tri_inv(const double* X, int b, bool unit, double* Xi, double* scratch) {
  int bp = 1;
  while (bp < b) bp <<= 1;
  auto xat = [&](int i, int k) -> double {
    if (i >= b || k >= b) return (i == k) ? 1.0 : 0.0;
    return X[k * b + i];
  };
  // Xi is bp x bp here (ld bp); the caller's layout (ld b) is restored at the end
  for (int idx = threadIdx.x; idx < bp * bp; idx += blockDim.x) {
    const int i = idx % bp, k = idx / bp;
    double v = 0.0;
    if (i == k) v = (unit || i >= b) ? 1.0 : 1.0 / X[i * b + i];
    scratch[512 + idx] = v;
  }
  __syncthreads();
  double* Z = scratch + 512;
  for (int h = 1; h < bp; h <<= 1) {
    const int npair = bp / (2 * h);
    // M = B C^-1 (h x h per pair)
    for (int idx = threadIdx.x; idx < npair * h * h; idx += blockDim.x) {
      const int p = idx / (h * h), e = idx % (h * h), i = e % h, j = e / h;
      const int i0 = p * 2 * h, c0 = i0 + h;
      double acc = 0.0;
      for (int k = 0; k <= j; ++k) acc = fma(xat(i0 + i, c0 + k), Z[(c0 + j) * bp + c0 + k], acc);
      scratch[p * h * h + e] = acc;
    }
    __syncthreads();
    // top-right block = -A^-1 M
    for (int idx = threadIdx.x; idx < npair * h * h; idx += blockDim.x) {
      const int p = idx / (h * h), e = idx % (h * h), i = e % h, j = e / h;
      const int i0 = p * 2 * h, c0 = i0 + h;
      double acc = 0.0;
      for (int k = i; k < h; ++k) acc = fma(Z[(i0 + k) * bp + i0 + i], scratch[p * h * h + j * h + k], acc);
      Z[(c0 + j) * bp + i0 + i] = -acc;
    }
    __syncthreads();
  }
  for (int idx = threadIdx.x; idx < b * b; idx += blockDim.x) {
    const int i = idx % b, k = idx / b;
    Xi[k * b + i] = Z[k * bp + i];
  }
  __syncthreads();
}

// Compact-WY T (b x b, ld b) of the reflectors whose vectors are
// V(r, i) = vget(r, i) over rows [0, rows): with G = V^T V, T^-1 =
// striu(G) + diag(G) / 2 (the identity the reference uses in
// compute_invT_from_Y, alg/QR/qr_2d/qr_2d.cxx:22-60; it is the T that makes
// I - V T V^T orthogonal for the computed V).  The Gram dots are split into
// four partial sums to shorten their dependent chains.
template <class VGet>
__device__ void h4_larft(VGet vget, int rows, int b, double* G, double* T, double* scratch) {
  for (int idx = threadIdx.x; idx < b * b; idx += blockDim.x) {
    const int i = idx % b, j = idx / b;
    double acc = 0.0;
    if (i <= j) {
      double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
      int r = 0;
      for (; r + 3 < rows; r += 4) {
        a0 = fma(vget(r, i), vget(r, j), a0);
        a1 = fma(vget(r + 1, i), vget(r + 1, j), a1);
        a2 = fma(vget(r + 2, i), vget(r + 2, j), a2);
        a3 = fma(vget(r + 3, i), vget(r + 3, j), a3);
      }
      for (; r < rows; ++r) a0 = fma(vget(r, i), vget(r, j), a0);
      acc = (a0 + a1) + (a2 + a3);
      if (i == j) acc *= 0.5;
    }
    G[j * b + i] = acc;
  }
  __syncthreads();
  h4_tri_inv(G, b, false, T, scratch);
}

// C = A * B for b x b shared matrices (ld b), A and B upper triangular.
__device__ void h4_mm_upper(const double* A, const double* B, double* C, int b) {
  for (int idx = threadIdx.x; idx < b * b; idx += blockDim.x) {
    const int i = idx % b, j = idx / b;
    double acc = 0.0;
    for (int k = i; k <= j; ++k) acc = fma(A[k * b + i], B[j * b + k], acc);
    C[j * b + i] = (i <= j) ? acc : 0.0;
  }
  __syncthreads();
}

__device__ void h4_load(double* dst, const double* src, int b) {
  for (int idx = threadIdx.x; idx < b * b; idx += blockDim.x) dst[idx] = __ldcg(src + idx);
  __syncthreads();
}

struct Hr4Args {
  double* A;
  int64_t lda;
  int64_t m;
  int b;
  double* Vw;       // m x b (ld m): leaf reflector vectors (strictly lower part; unit diagonal implied)
  double* Tl;       // P x b x b: leaf T factors
  double* Rn;       // nnodes x b x b: R of every node
  double* Qn;       // nnodes x kFan x b x b: node Q blocks
  unsigned* cnt;    // nnodes arrival counters (zeroed)
  double* T;        // out
  int64_t ldT;
  double* W;        // out or nullptr
  int64_t ldW;
  double* Uinv;     // scratch b x b
  int* status;
  int P;
  int depth;
  int nlev[kMaxLevels + 1];
  int base[kMaxLevels + 1];
};

__device__ __forceinline__ int h4_children(const Hr4Args& a, int lvl, int node) {
  // children of node (lvl, node) at level lvl-1
  const int first = node * kFan;
  const int n = a.nlev[lvl - 1] - first;
  return n < kFan ? n : kFan;
}

__device__ void h4_root(const Hr4Args& a, double* sm) {
  const int b = a.b, tid = threadIdx.x;
  double* sR = sm;
  double* sM = sR + b * b;
  double* sQ = sM + b * b;
  double* sX = sQ + b * b;
  double* sY = sX + b * b;
  double* sT = sY + b * b;
  __shared__ int s_sign[kDirectB];
  h4_load(sR, a.Rn + (size_t)a.base[a.depth] * b * b, b);
  for (int idx = tid; idx < b * b; idx += blockDim.x) sM[idx] = (idx % b == idx / b) ? 1.0 : 0.0;
  __syncthreads();
  for (int lvl = a.depth; lvl >= 1; --lvl) {
    if (h4_children(a, lvl, 0) > 1) {
      h4_load(sX, a.Qn + ((size_t)a.base[lvl] * kFan + 0) * b * b, b);
      h4_mm_upper(sX, sM, sQ, b);
      for (int idx = tid; idx < b * b; idx += blockDim.x) sM[idx] = sQ[idx];
      __syncthreads();
    }
  }
  // Q1_top = C0 - V0 (T0 (V0^T C0)), V0 = unit-lower top block of leaf 0
  for (int idx = tid; idx < b * b; idx += blockDim.x) {
    const int r = idx % b, c = idx / b;
    sY[idx] = (r > c) ? __ldcg(a.Vw + (int64_t)c * a.m + r) : (r == c ? 1.0 : 0.0);
  }
  h4_load(sT, a.Tl, b);
  for (int idx = tid; idx < b * b; idx += blockDim.x) {     // sX = V0^T C0
    const int i = idx % b, j = idx / b;
    double acc = 0.0;
    for (int k = i; k < b; ++k) acc = fma(sY[i * b + k], sM[j * b + k], acc);
    sX[idx] = acc;
  }
  __syncthreads();
  for (int idx = tid; idx < b * b; idx += blockDim.x) {     // sQ = T0 sX
    const int i = idx % b, j = idx / b;
    double acc = 0.0;
    for (int k = i; k < b; ++k) acc = fma(sT[k * b + i], sX[j * b + k], acc);
    sQ[idx] = acc;
  }
  __syncthreads();
  for (int idx = tid; idx < b * b; idx += blockDim.x) {     // sX = C0 - V0 sQ
    const int i = idx % b, j = idx / b;
    double acc = sM[idx];
    for (int k = 0; k <= i; ++k) acc = fma(-sY[k * b + i], sQ[j * b + k], acc);
    sX[idx] = acc;
  }
  __syncthreads();
  double* sL = sX;   // Q1_top, becomes L\U
  for (int i = 0; i < b; ++i) {
    if (tid == 0) {
      const double d = sL[i * b + i];
      const int s = d > 0.0 ? -1 : 1;
      s_sign[i] = s;
      sL[i * b + i] = d - (double)s;
    }
    __syncthreads();
    const double piv = sL[i * b + i];
    for (int r = i + 1 + tid; r < b; r += blockDim.x) sL[i * b + r] /= piv;
    __syncthreads();
    const int n = b - i - 1;
    for (int idx = tid; idx < n * n; idx += blockDim.x) {
      const int r = i + 1 + idx % n, c = i + 1 + idx / n;
      sL[c * b + r] = fma(-sL[i * b + r], sL[c * b + i], sL[c * b + r]);
    }
    __syncthreads();
  }
  for (int idx = tid; idx < b * b; idx += blockDim.x) {
    const int r = idx % b, c = idx / b;
    a.A[c * a.lda + r] = (r > c) ? sL[c * b + r] : (double)s_sign[r] * sR[c * b + r];
    if (a.W) a.W[c * a.ldW + r] = (r <= c) ? sL[c * b + r] * (double)s_sign[c] : 0.0;
  }
  // T = -W L^-T: W (upper) into sQ, L^T (unit upper) into sY, (L^T)^-1 into sM
  double* scratch = sm + 6 * b * b;
  for (int idx = tid; idx < b * b; idx += blockDim.x) {
    const int i = idx % b, k = idx / b;
    sQ[idx] = (i <= k) ? sL[k * b + i] * (double)s_sign[k] : 0.0;
    sY[idx] = (i < k) ? sL[i * b + k] : (i == k ? 1.0 : 0.0);
  }
  __syncthreads();
  h4_tri_inv(sY, b, true, sM, scratch);
  h4_mm_upper(sQ, sM, sT, b);
  for (int idx = tid; idx < b * b; idx += blockDim.x) {
    const int r = idx % b, c = idx / b;
    a.T[c * a.ldT + r] = (r <= c) ? -sT[c * b + r] : 0.0;
  }
  // U^-1 (the upper triangle of L\U); sM holds it
  h4_tri_inv(sL, b, false, sM, scratch);
  int bad = 0;
  for (int idx = tid; idx < b * b; idx += blockDim.x) {
    const double v = sM[idx];
    if (!isfinite(v)) bad = 1;
    a.Uinv[idx] = v;
  }
  if (bad) atomicExch(a.status, CANDMC_ERR_NUMERIC);
}

__global__ void __launch_bounds__(kThreads) k_hr4_leaf_tree(Hr4Args a) {
  extern __shared__ double sm4[];
  __shared__ double s_tau[kDirectB];
  __shared__ double s_part[8 * 32];
  __shared__ double s_w[32];
  __shared__ int s_last;
  const int b = a.b, tid = threadIdx.x;
  const int leaf = blockIdx.x;
  const int64_t r0 = t4_leaf_row0(a.m, a.P, leaf);
  const int L = (int)(t4_leaf_row0(a.m, a.P, leaf + 1) - r0);
  double* S = sm4;
  double* G = sm4 + (size_t)(L > kFan * b ? L : kFan * b) * b;
  double* Tt = G + b * b;
  double* scratch = Tt + b * b;

  // ---- leaf: Householder QR, R, V and T out
  for (int c = 0; c < b; ++c)
    for (int r = tid; r < L; r += blockDim.x) S[c * L + r] = a.A[c * a.lda + r0 + r];
  __syncthreads();
  for (int j = 0; j < b; ++j)
    h4_step(S, L, L, j, b, [](int r, int jj) { return r > jj; }, s_tau, s_part, s_w);
  double* Rl = a.Rn + (size_t)(a.base[0] + leaf) * b * b;
  for (int idx = tid; idx < b * b; idx += blockDim.x) {
    const int r = idx % b, c = idx / b;
    Rl[idx] = (r <= c) ? S[c * L + r] : 0.0;
  }
  for (int c = 0; c < b; ++c)
    for (int r = tid; r < L; r += blockDim.x) a.Vw[(int64_t)c * a.m + r0 + r] = (r > c) ? S[c * L + r] : 0.0;
  h4_larft([&](int r, int i) { return r > i ? S[i * L + r] : (r == i ? 1.0 : 0.0); }, L, b, G, Tt,
           scratch);
  double* Tleaf = a.Tl + (size_t)leaf * b * b;
  for (int idx = tid; idx < b * b; idx += blockDim.x) Tleaf[idx] = Tt[idx];

  // ---- climb the fan-in-4 tree
  int node = leaf;
  for (int lvl = 0; lvl < a.depth; ++lvl) {
    const int parent = node / kFan;
    const int nch = h4_children(a, lvl + 1, parent);
    double* Rpar = a.Rn + (size_t)(a.base[lvl + 1] + parent) * b * b;
    if (nch == 1) {
      const double* Rme = a.Rn + (size_t)(a.base[lvl] + node) * b * b;
      __syncthreads();
      for (int idx = tid; idx < b * b; idx += blockDim.x) Rpar[idx] = __ldcg(Rme + idx);
      __syncthreads();
      node = parent;
      continue;
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) s_last = (atomicAdd(a.cnt + a.base[lvl + 1] + parent, 1u) == (unsigned)(nch - 1));
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    // stack the children's R factors: rows [k b, k b + b) hold child k (ld = nch * b)
    const int ld2 = nch * b;
    for (int k = 0; k < nch; ++k) {
      const double* Rk = a.Rn + (size_t)(a.base[lvl] + parent * kFan + k) * b * b;
      for (int idx = tid; idx < b * b; idx += blockDim.x) {
        const int r = idx % b, c = idx / b;
        S[c * ld2 + k * b + r] = (r <= c) ? __ldcg(Rk + idx) : 0.0;
      }
    }
    __syncthreads();
    // reflector j: head row j, tail = rows 0..j of every other child (the
    // children are upper triangular, so nothing below their diagonals is touched)
    const int bb = b;
    for (int j = 0; j < b; ++j)
      h4_step(S, ld2, ld2, j, b, [bb](int r, int jj) { return r >= bb && (r % bb) <= jj; }, s_tau,
              s_part, s_w);
    for (int idx = tid; idx < b * b; idx += blockDim.x) {
      const int r = idx % b, c = idx / b;
      Rpar[idx] = (r <= c) ? S[c * ld2 + r] : 0.0;
    }
    // V = [I; V_1; ..; V_{nch-1}], V_k upper triangular: G = I + sum_k V_k^T V_k,
    // with the diagonal halved, is T^-1
    for (int idx = tid; idx < b * b; idx += blockDim.x) {
      const int i = idx % b, j = idx / b;
      double acc = 0.0;
      if (i <= j) {
        acc = (i == j) ? 1.0 : 0.0;
        for (int k = 1; k < nch; ++k)
          for (int r = 0; r <= i; ++r) acc = fma(S[i * ld2 + k * b + r], S[j * ld2 + k * b + r], acc);
        if (i == j) acc *= 0.5;
      }
      G[j * b + i] = acc;
    }
    __syncthreads();
    h4_tri_inv(G, b, false, Tt, scratch);
    double* Qp = a.Qn + (size_t)(a.base[lvl + 1] + parent) * kFan * b * b;
    // Q_1 = I - T;  Q_k = -V_k T  (V_k = rows [k b, k b + b) of the tail, upper triangular)
    for (int idx = tid; idx < b * b; idx += blockDim.x) {
      const int r = idx % b, c = idx / b;
      Qp[idx] = ((r == c) ? 1.0 : 0.0) - ((r <= c) ? Tt[c * b + r] : 0.0);
    }
    for (int k = 1; k < nch; ++k) {
      for (int idx = tid; idx < b * b; idx += blockDim.x) {
        const int r = idx % b, c = idx / b;
        double acc = 0.0;
        for (int kk = r; kk <= c; ++kk) acc = fma(S[kk * ld2 + k * b + r], Tt[c * b + kk], acc);
        Qp[(size_t)k * b * b + idx] = (r <= c) ? -acc : 0.0;
      }
    }
    __syncthreads();
    node = parent;
  }
  __threadfence();
  __syncthreads();
  h4_root(a, sm4);
}

__global__ void __launch_bounds__(kThreads) k_hr4_form_y(Hr4Args a) {
  extern __shared__ double sm4[];
  const int b = a.b, tid = threadIdx.x;
  const int leaf = blockIdx.x;
  const int64_t r0 = t4_leaf_row0(a.m, a.P, leaf);
  const int64_t r1 = t4_leaf_row0(a.m, a.P, leaf + 1);
  double* sM = sm4;
  double* sX = sM + b * b;
  double* sY = sX + b * b;
  double* sT = sY + b * b;
  h4_load(sM, a.Uinv, b);
  for (int lvl = a.depth; lvl >= 1; --lvl) {
    int nd = leaf;
    for (int l = 0; l < lvl; ++l) nd /= kFan;
    int child = leaf;
    for (int l = 0; l < lvl - 1; ++l) child /= kFan;
    if (h4_children(a, lvl, nd) > 1) {
      const int k = child - nd * kFan;
      h4_load(sX, a.Qn + ((size_t)(a.base[lvl] + nd) * kFan + k) * b * b, b);
      h4_mm_upper(sX, sM, sY, b);
      for (int idx = tid; idx < b * b; idx += blockDim.x) sM[idx] = sY[idx];
      __syncthreads();
    }
  }
  // Z = T (V_top^T M);  Y = [M; 0] - V Z
  for (int idx = tid; idx < b * b; idx += blockDim.x) {
    const int r = idx % b, c = idx / b;
    sY[idx] = (r > c) ? a.Vw[(int64_t)c * a.m + r0 + r] : (r == c ? 1.0 : 0.0);
  }
  h4_load(sT, a.Tl + (size_t)leaf * b * b, b);
  for (int idx = tid; idx < b * b; idx += blockDim.x) {
    const int i = idx % b, j = idx / b;
    double acc = 0.0;
    for (int k = i; k < b; ++k) acc = fma(sY[i * b + k], sM[j * b + k], acc);
    sX[idx] = acc;
  }
  __syncthreads();
  for (int idx = tid; idx < b * b; idx += blockDim.x) {
    const int i = idx % b, j = idx / b;
    double acc = 0.0;
    for (int k = i; k < b; ++k) acc = fma(sT[k * b + i], sX[j * b + k], acc);
    sY[idx] = acc;   // sY now holds Z (V_top no longer needed)
  }
  __syncthreads();
  for (int64_t r = r0 + tid; r < r1; r += blockDim.x) {
    if (r < b) continue;
    const int rl = (int)(r - r0);
    double v[kDirectB];
#pragma unroll
    for (int k = 0; k < kDirectB; ++k)
      v[k] = (k < b) ? (rl > k ? a.Vw[(int64_t)k * a.m + r] : (rl == k ? 1.0 : 0.0)) : 0.0;
    for (int c = 0; c < b; ++c) {
      double acc = (rl < b) ? sM[c * b + rl] : 0.0;
#pragma unroll
      for (int k = 0; k < kDirectB; ++k)
        if (k < b) acc = fma(-v[k], sY[c * b + k], acc);
      a.A[c * a.lda + r] = acc;
    }
  }
}

int hr_direct4(double* A, int64_t lda, int64_t m, int b, double* T, int64_t ldT, double* W,
               int64_t ldW, int* d_status, cudaStream_t s) {
  if (b < 1 || b > kDirectB || m < b) return CANDMC_ERR_ARG;
  const int64_t leaf_rows = std::max<int64_t>(32, std::min<int64_t>(g_leaf_rows, 256));
  int64_t P = std::max<int64_t>(1, std::min<int64_t>(m / leaf_rows, m / b));
  if (P > (1 << 24)) return CANDMC_ERR_ARG;
  Hr4Args a{};
  a.P = (int)P;
  a.nlev[0] = (int)P;
  a.base[0] = 0;
  int total = (int)P, l = 0;
  while (a.nlev[l] > 1) {
    a.nlev[l + 1] = (a.nlev[l] + kFan - 1) / kFan;
    a.base[l + 1] = total;
    total += a.nlev[l + 1];
    ++l;
  }
  a.depth = l;
  const int nnodes = total;
  const int64_t Lmax = (m + P - 1) / P;
  const size_t nb2 = (size_t)b * b;
  // leaf/node matrix + G + T + tri-inverse workspace; the root reuses the
  // front of the same area for six b x b buffers plus the workspace
  const size_t sm = sizeof(double) * ((size_t)std::max<int64_t>(Lmax, kFan * b) * b + 6 * nb2 +
                                      kTriScratch);
  if (sm > 200 * 1024) return CANDMC_ERR_ARG;
  DevBuf vw, tl, rn, qn, cnt, uinv;
  CANDMC_RET(vw.alloc(sizeof(double) * (size_t)m * b, s));
  CANDMC_RET(tl.alloc(sizeof(double) * nb2 * P, s));
  CANDMC_RET(rn.alloc(sizeof(double) * nb2 * nnodes, s));
  CANDMC_RET(qn.alloc(sizeof(double) * nb2 * kFan * nnodes, s));
  CANDMC_RET(cnt.alloc(sizeof(unsigned) * nnodes, s));
  CANDMC_RET(uinv.alloc(sizeof(double) * nb2, s));
  CANDMC_CK(cudaMemsetAsync(cnt.p, 0, sizeof(unsigned) * nnodes, s));
  a.A = A; a.lda = lda; a.m = m; a.b = b;
  a.Vw = vw.d(); a.Tl = tl.d(); a.Rn = rn.d(); a.Qn = qn.d();
  a.cnt = static_cast<unsigned*>(cnt.p);
  a.T = T; a.ldT = ldT; a.W = W; a.ldW = ldW; a.Uinv = uinv.d(); a.status = d_status;
  static std::atomic<bool> attr{false};
  if (!attr) {
    CANDMC_CK(cudaFuncSetAttribute(k_hr4_leaf_tree, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   200 * 1024));
    attr = true;
  }
  {
    ProfScope ps(CANDMC_KCLASS_PANEL_LEAF, 2.0 * m * b * b, s);
    k_hr4_leaf_tree<<<(unsigned)P, kThreads, sm, s>>>(a);
  }
  CANDMC_CK(cudaGetLastError());
  {
    ProfScope ps(CANDMC_KCLASS_PANEL_Y, 2.0 * m * b * b, s);
    k_hr4_form_y<<<(unsigned)P, kThreads, sizeof(double) * 4 * nb2, s>>>(a);
  }
  CANDMC_CK(cudaGetLastError());
  return CANDMC_OK;
}

}  // namespace candmc
