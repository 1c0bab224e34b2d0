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
//  * leaves of at most leaf_rows rows, one CTA each: b Householder steps in
//    the column-owner schedule below, which also yields the leaf's
//    compact-WY T (T^-1 from the Gram matrix V^T V);
//  * a fan-in-4 tree: the node stacks up to four R factors and runs b
//    Householder steps on the stacked matrix (the zeros below the children's
//    diagonals stay zero); with V = [I; V_2..V_4] the node's Q blocks are
//    Q_1 = I - T and Q_k = -V_k T (all upper triangular), so no explicit-Q
//    pass is needed.  Two schedules: k_hr6_pipe, where every node is a CTA
//    that starts column j as soon as its children have published it (the
//    levels overlap; roles by atomic ticket, bounded waits), and
//    k_hr4_leaf_tree, where the last CTA to arrive combines a node;
//  * the root: Q1_top = (I - V0 T0 V0^T) Q_1^(1) ... Q_1^(depth) on the top
//    b rows, then the sign-choice LU of Q1_top - S, and L\(S R), T, W and
//    U^-1.  In k_hr6_pipe leaf 0 and the nodes on its path build Q1_top as a
//    prefix product while they finish, and one extra CTA solves the root;
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
int64_t g_pipe_leaf_rows = 128;
thread_local int64_t t_leaf_rows = 0;
// Pipelined tree on/off (tuning knob, candmc_set_tuning("pipe_tree", 0|1)).
int g_pipe_tree = 1;
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

// ---- Householder QR of a shared-memory block, column-owner schedule.
//
// The block S (column-major, ld rows, b <= 32 columns) is worked by 4 warps;
// warp w owns the columns c with c % 4 == w for every row, and lane l owns the
// rows l + 32 t.  Step j applies reflector j (vector v_j: 1 at the head row j,
// S[j][r] on the tail rows) to every other column and computes reflector j+1:
//  * the owner of column j+1 updates that column first, then forms reflector
//    j+1 from it with warp-only reductions (nothing else waits for it but the
//    next step);
//  * every warp forms d_c = v_j^T S[c] for its other columns (one transposed
//    warp reduction for all of them), updates the columns c > j and records
//    d_c = v_c^T v_j for c < j: these are the strictly upper entries of
//    T^-1 = striu(V^T V) + diag(V^T V) / 2 (the identity of the reference's
//    compute_invT_from_Y, alg/QR/qr_2d/qr_2d.cxx:22-60), so T costs no extra
//    pass over the rows;
//  * one block barrier per step.
// On GB300 every warp-wide FP64 instruction holds its SMSP's FP64 pipe for 64
// cycles, so the schedule keeps one warp per SMSP and the per-step chain of
// the owner short.  The reflector follows LAPACK dlarfg: beta = -sign(alpha)
// sqrt(alpha^2 + |x|^2), tau = 1 - alpha / beta, v = x / (alpha - beta); an
// all-zero tail takes tau = 2, beta = -alpha (a sign flip), the convention of
// the reconstruction, so that the T^-1 identity holds for every reflector.
constexpr int kLeafThreads = 128;   // 4 warps, one per SMSP
constexpr int kMaxR = 8;            // rows per lane: leaves of up to 256 rows, nodes of 4 x 32
// leaves from which the Y formation takes its path products from a top-down
// pass over the nodes instead of multiplying each leaf's whole path itself
constexpr int kNodeMinLeaves = 256;
// rows from which the lookahead's panels take 256-row leaves
constexpr int64_t kTallPanelRows = 32768;

// Sum over the warp of eight values per lane; every lane receives all eight sums.
__device__ __forceinline__ void warp_sum8(const double (&d)[8], double (&out)[8]) {
  const int lane = threadIdx.x & 31;
  const bool u16 = (lane & 16) != 0, u8 = (lane & 8) != 0, u4 = (lane & 4) != 0;
  double p[4], q[2];
#pragma unroll
  for (int k = 0; k < 4; ++k)
    p[k] = (u16 ? d[k + 4] : d[k]) + __shfl_xor_sync(0xffffffffu, u16 ? d[k] : d[k + 4], 16);
#pragma unroll
  for (int k = 0; k < 2; ++k)
    q[k] = (u8 ? p[k + 2] : p[k]) + __shfl_xor_sync(0xffffffffu, u8 ? p[k] : p[k + 2], 8);
  double s = (u4 ? q[1] : q[0]) + __shfl_xor_sync(0xffffffffu, u4 ? q[0] : q[1], 4);
  s += __shfl_xor_sync(0xffffffffu, s, 2);
  s += __shfl_xor_sync(0xffffffffu, s, 1);
  // lane l now holds sum number 4 (l & 16 != 0) + 2 (l & 8 != 0) + (l & 4 != 0)
#pragma unroll
  for (int k = 0; k < 8; ++k)
    out[k] = __shfl_sync(0xffffffffu, s, (((k >> 2) & 1) << 4) | (((k >> 1) & 1) << 3) | ((k & 1) << 2));
}

// The same reduction without the final broadcast: lane l returns sum number
// 4 (l & 16 != 0) + 2 (l & 8 != 0) + (l & 4 != 0); the four lanes l with equal
// bits 2..4 hold the same sum.
__device__ __forceinline__ double warp_sum8_held(const double (&d)[8]) {
  const int lane = threadIdx.x & 31;
  const bool u16 = (lane & 16) != 0, u8 = (lane & 8) != 0, u4 = (lane & 4) != 0;
  double p[4], q[2];
#pragma unroll
  for (int k = 0; k < 4; ++k)
    p[k] = (u16 ? d[k + 4] : d[k]) + __shfl_xor_sync(0xffffffffu, u16 ? d[k] : d[k + 4], 16);
#pragma unroll
  for (int k = 0; k < 2; ++k)
    q[k] = (u8 ? p[k + 2] : p[k]) + __shfl_xor_sync(0xffffffffu, u8 ? p[k] : p[k + 2], 8);
  double s = (u4 ? q[1] : q[0]) + __shfl_xor_sync(0xffffffffu, u4 ? q[0] : q[1], 4);
  s += __shfl_xor_sync(0xffffffffu, s, 2);
  s += __shfl_xor_sync(0xffffffffu, s, 1);
  return s;
}

__device__ __forceinline__ int warp_sum8_index(int lane) {
  return ((lane >> 4) & 1) * 4 + ((lane >> 3) & 1) * 2 + ((lane >> 2) & 1);
}

// Sixteen sums at once, without the broadcast: lane l returns sum number
// 8 (l & 16 != 0) + 4 (l & 8 != 0) + 2 (l & 4 != 0) + (l & 2 != 0); lanes l and
// l ^ 1 hold the same sum.
__device__ __forceinline__ double warp_sum16_held(const double (&d)[16]) {
  const int lane = threadIdx.x & 31;
  const bool u16 = (lane & 16) != 0, u8 = (lane & 8) != 0, u4 = (lane & 4) != 0, u2 = (lane & 2) != 0;
  double p[8], q[4], r[2];
#pragma unroll
  for (int k = 0; k < 8; ++k)
    p[k] = (u16 ? d[k + 8] : d[k]) + __shfl_xor_sync(0xffffffffu, u16 ? d[k] : d[k + 8], 16);
#pragma unroll
  for (int k = 0; k < 4; ++k)
    q[k] = (u8 ? p[k + 4] : p[k]) + __shfl_xor_sync(0xffffffffu, u8 ? p[k] : p[k + 4], 8);
#pragma unroll
  for (int k = 0; k < 2; ++k)
    r[k] = (u4 ? q[k + 2] : q[k]) + __shfl_xor_sync(0xffffffffu, u4 ? q[k] : q[k + 2], 4);
  double s = (u2 ? r[1] : r[0]) + __shfl_xor_sync(0xffffffffu, u2 ? r[0] : r[1], 2);
  s += __shfl_xor_sync(0xffffffffu, s, 1);
  return s;
}

__device__ __forceinline__ int warp_sum16_index(int lane) {
  return ((lane >> 4) & 1) * 8 + ((lane >> 3) & 1) * 4 + ((lane >> 2) & 1) * 2 + ((lane >> 1) & 1);
}

// Reflector j from column j of S, by one warp: alpha = S[j][j], x = the tail
// rows (lane l owns rows l + 32 t).  Writes beta to S[j][j],
// v = x / (alpha - beta) to the tail rows, tau to s_tau[j] and v^T v / 2
// (with the unit head) to g[j][j] (ld b).
template <int R, class Tail>
__device__ void h5_reflector(double* S, int ld, int rows, int j, int b, Tail tail, double* s_tau,
                             double* g) {
  const int lane = threadIdx.x & 31;
  double* col = S + (size_t)j * ld;
  double x[R];
  double xn2 = 0.0;
#pragma unroll
  for (int t = 0; t < R; ++t) {
    const int r = lane + 32 * t;
    x[t] = (r < rows && tail(r, j)) ? col[r] : 0.0;
    xn2 = fma(x[t], x[t], xn2);
  }
  xn2 = warp_sum(xn2);
  const double alpha = col[j];
  double tj, sc, beta;
  if (xn2 == 0.0) {
    tj = 2.0;
    sc = 0.0;
    beta = -alpha;
  } else {
    const double q = fma(alpha, alpha, xn2);
    const double rq = nr_rsqrt(q);
    const double sg = alpha >= 0.0 ? -1.0 : 1.0;   // -sign(alpha), sign(0) = +
    beta = sg * q * rq;
    tj = fma(-alpha, sg * rq, 1.0);
    sc = nr_rcp(alpha - beta);
  }
#pragma unroll
  for (int t = 0; t < R; ++t) {
    const int r = lane + 32 * t;
    if (r < rows && tail(r, j)) col[r] = x[t] * sc;
  }
  __syncwarp();
  if (lane == 0) {
    col[j] = beta;
    s_tau[j] = tj;
    g[j * b + j] = 0.5 * fma(sc * sc, xn2, 1.0);
  }
}

// Householder QR of S (rows x b, ld >= 32 R, R = ceil(rows / 32) rows per
// lane); all kLeafThreads threads call it.  Afterwards S holds R (upper
// triangle) and the reflector tails, s_tau the taus and g (b x b, ld b,
// zeroed by the caller) T^-1.
// Step j: warp (j+1) % 4 is the critical warp: it applies reflector j to
// column j+1 and forms reflector j+1, and does nothing else, because a warp's
// dependent FP64 chain occupies its SMSP's FP64 pipe.  The other three warps
// share every other column c: d_c = v_j^T S[c] (a transposed reduction per 8
// columns), then S[c] -= tau_j v_j d_c for c > j+1, or T^-1[c][j] = d_c for
// c < j.  After the last reflector all four warps share the work.  The
// updates load all of a group's rows before the first store, so that
// independent columns are not serialised through shared memory.
struct NoPublish {
  __device__ void operator()(const double*, int, int) const {}
};

template <int R, class Tail, class Pub = NoPublish>
__device__ void h5_factor(double* S, int ld, int rows, int b, Tail tail, double* s_tau, double* g,
                          Pub pub = Pub()) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (warp == 0) h5_reflector<R>(S, ld, rows, 0, b, tail, s_tau, g);
  __syncthreads();
  for (int j = 0; j < b; ++j) {
    // column j of R is final now (its last update was step j-1): a warp
    // other than this step's critical one may publish it
    if (warp == ((j + 2) & 3)) pub(S, ld, j);
    const double* vj = S + (size_t)j * ld;
    double vv[R];
#pragma unroll
    for (int t = 0; t < R; ++t) {
      const int r = lane + 32 * t;
      double v = 0.0;
      if (r == j) v = 1.0;
      else if (r < rows && tail(r, j)) v = vj[r];
      vv[t] = v;
    }
    const double tj = s_tau[j];
    const int nxt = j + 1;
    const bool has_crit = nxt < b;
    const int crit = nxt & 3;
    if (has_crit && warp == crit) {
      // the next pivot column: apply reflector j, then form reflector j+1
      double* cn = S + (size_t)nxt * ld;
      double x[R];
      double d = 0.0;
#pragma unroll
      for (int t = 0; t < R; ++t) {
        x[t] = cn[lane + 32 * t];
        d = fma(vv[t], x[t], d);
      }
      d = warp_sum(d) * tj;
#pragma unroll
      for (int t = 0; t < R; ++t) cn[lane + 32 * t] = fma(-vv[t], d, x[t]);
      __syncwarp();
      h5_reflector<R>(S, ld, rows, nxt, b, tail, s_tau, g);
    } else {
      // bulk: this warp's share q of the columns other than j and j+1
      const int nq = has_crit ? 3 : 4;
      const int q = has_crit ? ((warp - crit + 3) & 3) : warp;   // 0 .. nq-1
      for (int base = q; base < b; base += 8 * nq) {
        double dd[8], D[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          dd[k] = 0.0;
          const int c = base + k * nq;
          if (c < b && c != j && c != nxt) {
            const double* sc = S + (size_t)c * ld;
#pragma unroll
            for (int t = 0; t < R; ++t) dd[k] = fma(vv[t], sc[lane + 32 * t], dd[k]);
          }
        }
        warp_sum8(dd, D);
        // T^-1 entries for the columns before j
        if (lane == 0) {
#pragma unroll
          for (int k = 0; k < 8; ++k) {
            const int c = base + k * nq;
            if (c < j) g[j * b + c] = D[k];   // (V^T V)[c][j]
          }
        }
        // updates of the columns after j+1, four columns per load group
#pragma unroll
        for (int h = 0; h < 8; h += 4) {
          double xs[4][R];
          bool act[4];
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const int c = base + (h + k) * nq;
            act[k] = c < b && c > nxt;
            if (act[k]) {
              const double* sc = S + (size_t)c * ld;
#pragma unroll
              for (int t = 0; t < R; ++t) xs[k][t] = sc[lane + 32 * t];
            }
          }
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            if (!act[k]) continue;
            const double dk = D[h + k] * tj;
            double* sc = S + (size_t)(base + (h + k) * nq) * ld;
#pragma unroll
            for (int t = 0; t < R; ++t) sc[lane + 32 * t] = fma(-vv[t], dk, xs[k][t]);
          }
        }
      }
    }
    __syncthreads();
  }
}

// Structure of an operand of h5_mm, on op(X): entries outside it read as 0
// (and the unit diagonals as 1).
enum : int { kSDense = 0, kSUpper = 1, kSUnitUpper = 2, kSUnitLower = 3 };

__device__ __forceinline__ double h5_at(const double* X, int ld, bool tr, int st, int i, int k) {
  if ((st == kSUpper || st == kSUnitUpper) && k < i) return 0.0;
  if (st == kSUnitLower && k > i) return 0.0;
  if ((st == kSUnitUpper || st == kSUnitLower) && k == i) return 1.0;
  return tr ? X[i * ld + k] : X[k * ld + i];
}

// C = C0 + alpha op(A) op(B) for b x b shared-memory matrices (b <= 32; C0
// may be nullptr, or C itself; C must not alias A or B).
// The 32 x 32 output is cut into 8 x 8 tiles, each owned by one warp (lane l:
// row l % 8, columns l / 8 and l / 8 + 4), and a tile's k loop only covers
// the structural nonzeros of its row and column blocks (empty for the zero
// tiles of a product of two upper-triangular operands), and the tiles are
// dealt to the warps in order of decreasing work.  A warp-wide FP64 instruction is the unit of cost on this
// GPU (about 4 per 77 cycles per SM), so this bounds the product by the
// nonzero tile work instead of by the longest k range of any lane.
__device__ void h5_mm(const double* A, int lda, bool at, int as, const double* B, int ldb, bool bt,
                      int bs, double* C, int ldc, int b, double alpha, const double* C0) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  const int nt = (b + 7) >> 3;
  // tiles in order of decreasing k extent: the diagonal distance d = tj - ti
  // runs from nt - 1 down to -(nt - 1); tile number p walks that order
  int p = 0;
  for (int d = nt - 1; d >= -(nt - 1); --d) {
    for (int ti = 0; ti < nt; ++ti) {
      const int tj = ti + d;
      if (tj < 0 || tj >= nt) continue;
      const int i0 = ti * 8, j0 = tj * 8;
      // k range of the tile from the operands' structure
      int klo = 0, khi = b - 1;
      if (as == kSUpper || as == kSUnitUpper) klo = i0;
      if (as == kSUnitLower) khi = khi < i0 + 7 ? khi : i0 + 7;
      if (bs == kSUpper || bs == kSUnitUpper) khi = khi < j0 + 7 ? khi : j0 + 7;
      if (bs == kSUnitLower) klo = klo > j0 ? klo : j0;
      // (an empty range still writes C = C0, or zero)
      if ((p++ % nwarp) != warp) continue;
      const int i = i0 + (lane & 7), jA = j0 + (lane >> 3), jB = jA + 4;
      double acc0 = 0.0, acc1 = 0.0;
#pragma unroll 4
      for (int k = klo; k <= khi; ++k) {
        const double a = (i < b) ? h5_at(A, lda, at, as, i, k) : 0.0;
        const double b0 = (jA < b) ? h5_at(B, ldb, bt, bs, k, jA) : 0.0;
        const double b1 = (jB < b) ? h5_at(B, ldb, bt, bs, k, jB) : 0.0;
        acc0 = fma(a, b0, acc0);
        acc1 = fma(a, b1, acc1);
      }
      if (i < b) {
        if (jA < b) C[jA * ldc + i] = fma(alpha, acc0, C0 ? C0[jA * ldc + i] : 0.0);
        if (jB < b) C[jB * ldc + i] = fma(alpha, acc1, C0 ? C0[jB * ldc + i] : 0.0);
      }
    }
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

__device__ void h4_load(double* dst, const double* src, int b) {
  for (int idx = threadIdx.x; idx < b * b; idx += blockDim.x) dst[idx] = __ldcg(src + idx);
  __syncthreads();
}

// Rows [0, L) of b columns of a column-major block (ld lda) into S (ld ldS),
// zero below row L: sixteen columns' loads in flight per thread before any
// store, so the block costs two memory latencies rather than b.
__device__ void h4_load_block(double* S, int ldS, const double* A, int64_t lda, int L, int b) {
  for (int r = threadIdx.x; r < ldS; r += blockDim.x) {
    for (int c0 = 0; c0 < b; c0 += 16) {
      double t[16];
#pragma unroll
      for (int u = 0; u < 16; ++u) t[u] = (r < L && c0 + u < b) ? A[(int64_t)(c0 + u) * lda + r] : 0.0;
#pragma unroll
      for (int u = 0; u < 16; ++u)
        if (c0 + u < b) S[(c0 + u) * ldS + r] = t[u];
    }
  }
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
  unsigned* prog;   // pipelined tree: columns of R published by each node
  unsigned* done;   // pipelined tree: node finished (T, Q blocks, V written)
  unsigned* ticket; // pipelined tree: role counter
  int* fail;        // pipelined tree: a wait gave up
  double* Pc;       // pipelined tree: prefix products of Q1_top along leaf 0's path, (depth + 1) x b x b
  double* Mn;       // many leaves: per node, the product of the Q blocks from the root down to it
                    // times U^-1 (nnodes x b x b, by flat id), or nullptr
  int P;
  int ldS;          // leading dimension of the shared block (>= 32 * ceil(leaf rows / 32), >= 128)
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
  if (a.Pc) {
    // the pipelined tree multiplied Q1_top up leaf 0's path as its nodes finished
    h4_load(sX, a.Pc + (size_t)a.depth * b * b, b);
  } else {
    // chain M = Q1^(1) ... Q1^(depth) of the first-child Q blocks (upper triangular)
    for (int idx = tid; idx < b * b; idx += blockDim.x) sM[idx] = (idx % b == idx / b) ? 1.0 : 0.0;
    __syncthreads();
    for (int lvl = a.depth; lvl >= 1; --lvl) {
      if (h4_children(a, lvl, 0) > 1) {
        h4_load(sX, a.Qn + ((size_t)a.base[lvl] * kFan + 0) * b * b, b);
        h5_mm(sX, b, false, kSUpper, sM, b, false, kSUpper, sQ, b, b, 1.0, nullptr);
        for (int idx = tid; idx < b * b; idx += blockDim.x) sM[idx] = sQ[idx];
        __syncthreads();
      }
    }
    // Q1_top = C0 - V0 (T0 (V0^T C0)), V0 = unit-lower top block of leaf 0, C0 = M
    for (int idx = tid; idx < b * b; idx += blockDim.x) {
      const int r = idx % b, c = idx / b;
      sY[idx] = (r > c) ? __ldcg(a.Vw + (int64_t)c * a.m + r) : (r == c ? 1.0 : 0.0);
    }
    h4_load(sT, a.Tl, b);
    h5_mm(sY, b, true, kSUnitUpper, sM, b, false, kSUpper, sX, b, b, 1.0, nullptr);   // sX = V0^T C0 (upper)
    h5_mm(sT, b, false, kSUpper, sX, b, false, kSUpper, sQ, b, b, 1.0, nullptr);      // sQ = T0 sX (upper)
    h5_mm(sY, b, false, kSUnitLower, sQ, b, false, kSUpper, sX, b, b, -1.0, sM);      // sX = C0 - V0 sQ
  }
  double* sL = sX;   // Q1_top, becomes L\U
  __shared__ double s_rpiv;
  // Sign-choice LU without pivoting, with a one-column lookahead: in step i,
  // warp 0 applies column i to column i + 1 and finishes it (pivot, sign,
  // multipliers) while the other warps apply column i to the columns beyond;
  // one barrier per column.
  const int warp = tid >> 5, lane = tid & 31;
  auto pivot = [&](int c) {   // warp 0: the diagonal of column c, then its multipliers
    if (lane == 0) {
      const double d = sL[c * b + c];
      const int sg = d > 0.0 ? -1 : 1;
      s_sign[c] = sg;
      sL[c * b + c] = d - (double)sg;
      s_rpiv = nr_rcp(d - (double)sg);   // |d - s| >= 1: the sign choice keeps the pivot away from 0
    }
    __syncwarp();
    const double rp = s_rpiv;
    for (int r = c + 1 + lane; r < b; r += 32) sL[c * b + r] *= rp;
  };
  if (warp == 0) pivot(0);
  __syncthreads();
  for (int i = 0; i + 1 < b; ++i) {
    const int c1 = i + 1;
    if (warp == 0) {
      for (int r = c1 + lane; r < b; r += 32) sL[c1 * b + r] = fma(-sL[i * b + r], sL[c1 * b + i], sL[c1 * b + r]);
      __syncwarp();
      pivot(c1);
    } else {
      const int n = b - c1, nc = b - c1 - 1;   // rows i + 1 .., columns i + 2 ..
      for (int idx = tid - 32; idx < n * nc; idx += blockDim.x - 32) {
        const int r = c1 + idx % n, c = c1 + 1 + idx / n;
        sL[c * b + r] = fma(-sL[i * b + r], sL[c * b + i], sL[c * b + r]);
      }
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
  h5_mm(sQ, b, false, kSUpper, sM, b, false, kSUpper, sT, b, b, 1.0, nullptr);
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

__global__ void __launch_bounds__(kLeafThreads) k_hr4_leaf_tree(Hr4Args a) {
  extern __shared__ double sm4[];
  __shared__ double s_tau[kDirectB];
  __shared__ int s_last;
  const int b = a.b, tid = threadIdx.x;
  const int leaf = blockIdx.x;
  const int64_t r0 = t4_leaf_row0(a.m, a.P, leaf);
  const int L = (int)(t4_leaf_row0(a.m, a.P, leaf + 1) - r0);
  const int ldS = a.ldS;
  double* S = sm4;
  double* G = S + (size_t)ldS * b;
  double* Tt = G + b * b;
  double* scratch = Tt + b * b;

  // ---- leaf: Householder QR of rows [r0, r0 + L); rows L..ldS-1 are zero
  h4_load_block(S, ldS, a.A + r0, a.lda, L, b);
  for (int idx = tid; idx < b * b; idx += blockDim.x) G[idx] = 0.0;
  __syncthreads();
  {
    auto tail = [](int r, int j) { return r > j; };
    switch ((L + 31) >> 5) {
      case 1: h5_factor<1>(S, ldS, L, b, tail, s_tau, G); break;
      case 2: h5_factor<2>(S, ldS, L, b, tail, s_tau, G); break;
      case 3: h5_factor<3>(S, ldS, L, b, tail, s_tau, G); break;
      case 4: h5_factor<4>(S, ldS, L, b, tail, s_tau, G); break;
      default: h5_factor<8>(S, ldS, L, b, tail, s_tau, G); break;
    }
  }
  double* Rl = a.Rn + (size_t)(a.base[0] + leaf) * b * b;
  for (int idx = tid; idx < b * b; idx += blockDim.x) {
    const int r = idx % b, c = idx / b;
    Rl[idx] = (r <= c) ? S[c * ldS + r] : 0.0;
  }
  for (int c = 0; c < b; ++c)
    for (int r = tid; r < L; r += blockDim.x)
      a.Vw[(int64_t)c * a.m + r0 + r] = (r > c) ? S[c * ldS + r] : 0.0;
  h4_tri_inv(G, b, false, Tt, scratch);
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
    // stack the children's R factors: child k occupies rows [32 k, 32 k + b)
    // (rows b..31 of every child stay zero)
    const int rows = nch * 32;
    for (int c = 0; c < b; ++c)
      for (int r = tid; r < rows; r += blockDim.x) {
        const int k = r >> 5, i = r & 31;
        const double* Rk = a.Rn + (size_t)(a.base[lvl] + parent * kFan + k) * b * b;
        S[c * ldS + r] = (i <= c) ? __ldcg(Rk + c * b + i) : 0.0;
      }
    for (int idx = tid; idx < b * b; idx += blockDim.x) G[idx] = 0.0;
    __syncthreads();
    // reflector j: head row j (child 0), tail = rows 0..j of every other child
    // (the children are upper triangular, so nothing below their diagonals is touched)
    // (rows 32 k .. 32 k + j of children k >= 1 form the tail of reflector j)
    h5_factor<4>(S, ldS, rows, b, [](int r, int j) { return r >= 32 && (r & 31) <= j; }, s_tau, G);
    for (int idx = tid; idx < b * b; idx += blockDim.x) {
      const int r = idx % b, c = idx / b;
      Rpar[idx] = (r <= c) ? S[c * ldS + r] : 0.0;
    }
    h4_tri_inv(G, b, false, Tt, scratch);
    double* Qp = a.Qn + (size_t)(a.base[lvl + 1] + parent) * kFan * b * b;
    // V = [I; V_1; ..; V_{nch-1}] (V_k upper triangular):
    // Q_1 = I - T;  Q_k = -V_k T
    for (int idx = tid; idx < b * b; idx += blockDim.x) {
      const int r = idx % b, c = idx / b;
      Qp[idx] = ((r == c) ? 1.0 : 0.0) - ((r <= c) ? Tt[c * b + r] : 0.0);
    }
    for (int k = 1; k < nch; ++k) {
      double* Qk = G;   // G is free once T is formed
      h5_mm(S + 32 * k, ldS, false, kSUpper, Tt, b, false, kSUpper, Qk, b, b, -1.0, nullptr);
      for (int idx = tid; idx < b * b; idx += blockDim.x) Qp[(size_t)k * b * b + idx] = Qk[idx];
      __syncthreads();
    }
    node = parent;
  }
  __threadfence();
  __syncthreads();
  h4_root(a, sm4);
}

// ---- pipelined tree: one launch for the leaves and every internal node.
//
// The levels of the tree above do not overlap: a node starts when its
// children have finished all b columns, so a panel costs (1 + depth) b
// sequential Householder steps.  Here a node starts column j as soon as its
// children have published column j of their R: leaves run the right-looking
// steps above and publish each column of R when it becomes final; internal
// nodes run left-looking, applying their earlier reflectors to the arriving
// column through the compact-WY factor T they build as they go (LAPACK
// dlarft's column recurrence T[0:j, j] = -tau_j T[0:j, 0:j] V^T v_j), so the
// panel costs about b + depth steps.  Roles come from an atomic ticket
// (leaves first, then the nodes level by level), so a node only waits for
// CTAs that took a lower ticket and are already running, whatever the
// scheduling order.  Every wait is bounded: a wait that runs out records
// CANDMC_ERR_TIMEOUT, and the CTA releases its own flags and returns, so no
// other CTA is left waiting on it.
constexpr long kSpinLimit = 1L << 22;

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// One thread: wait until *p >= v.  False when the wait gave up or another CTA
// of this launch did.
__device__ bool h6_wait(const Hr4Args& a, const unsigned* p, unsigned v) {
  for (long it = 0; it < kSpinLimit; ++it) {
    if (ld_acquire(p) >= v) return true;
    if (*(volatile int*)a.fail) return false;
    __nanosleep(100);
  }
  atomicExch(a.fail, 1);
  atomicExch(a.status, CANDMC_ERR_TIMEOUT);
  return false;
}

__device__ void h6_release_all(const Hr4Args& a, int f) {
  if (threadIdx.x == 0) {
    __threadfence();
    st_release(a.prog + f, (unsigned)a.b);
    st_release(a.done + f, 1u);
  }
}

struct LeafPublish {
  double* Rcol;
  int b;
  unsigned* prog;
  __device__ void operator()(const double* S, int ld, int j) const {
    const int lane = threadIdx.x & 31;
    if (lane <= j) Rcol[j * b + lane] = S[j * ld + lane];
    __threadfence();
    __syncwarp();
    if (lane == 0) st_release(prog, (unsigned)(j + 1));
  }
};

__device__ void h6_leaf(const Hr4Args& a, int leaf, double* sm, double* s_tau) {
  const int b = a.b, tid = threadIdx.x;
  const int64_t r0 = t4_leaf_row0(a.m, a.P, leaf);
  const int L = (int)(t4_leaf_row0(a.m, a.P, leaf + 1) - r0);
  const int ldS = a.ldS;
  double* S = sm;
  double* G = S + (size_t)ldS * b;
  double* Tt = G + b * b;
  double* scratch = Tt + b * b;
  h4_load_block(S, ldS, a.A + r0, a.lda, L, b);
  for (int idx = tid; idx < b * b; idx += blockDim.x) G[idx] = 0.0;
  __syncthreads();
  const LeafPublish pub{a.Rn + (size_t)leaf * b * b, b, a.prog + leaf};
  auto tail = [](int r, int j) { return r > j; };
  switch ((L + 31) >> 5) {
    case 1: h5_factor<1>(S, ldS, L, b, tail, s_tau, G, pub); break;
    case 2: h5_factor<2>(S, ldS, L, b, tail, s_tau, G, pub); break;
    case 3: h5_factor<3>(S, ldS, L, b, tail, s_tau, G, pub); break;
    case 4: h5_factor<4>(S, ldS, L, b, tail, s_tau, G, pub); break;
    default: h5_factor<8>(S, ldS, L, b, tail, s_tau, G, pub); break;
  }
  for (int c = 0; c < b; ++c)
    for (int r = tid; r < L; r += blockDim.x)
      a.Vw[(int64_t)c * a.m + r0 + r] = (r > c) ? S[c * ldS + r] : 0.0;
  h4_tri_inv(G, b, false, Tt, scratch);
  double* Tleaf = a.Tl + (size_t)leaf * b * b;
  for (int idx = tid; idx < b * b; idx += blockDim.x) Tleaf[idx] = Tt[idx];
  if (leaf == 0 && a.Pc) {
    // P_0 = I - V0 T0 V0^T on the top b rows (V0 unit lower): the first factor
    // of Q1_top, multiplied by the path nodes' Q1 blocks as they finish
    h5_mm(Tt, b, false, kSUpper, S, ldS, true, kSUnitUpper, G, b, b, 1.0, nullptr);        // G = T0 V0^T
    h5_mm(S, ldS, false, kSUnitLower, G, b, false, kSUpper, scratch, b, b, 1.0, nullptr);  // V0 G
    for (int idx = tid; idx < b * b; idx += blockDim.x)
      a.Pc[idx] = ((idx % b == idx / b) ? 1.0 : 0.0) - scratch[idx];
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) {
    if (leaf == 0) st_release(a.prog + 0, (unsigned)b + 1u);
    st_release(a.done + leaf, 1u);
  }
}

__device__ void h6_node(const Hr4Args& a, int f, double* sm, double* s_tau, int* s_ok) {
  const int b = a.b, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int lvl = 1;
  while (lvl < a.depth && f >= a.base[lvl + 1]) ++lvl;
  const int idx = f - a.base[lvl];
  const int nch = h4_children(a, lvl, idx);
  const int child0 = a.base[lvl - 1] + idx * kFan;   // flat id of child 0
  double* Rme = a.Rn + (size_t)f * b * b;
  constexpr int ld = kFan * 32;   // child k at rows [32 k, 32 k + b)
  double* S = sm;
  double* Tn = S + ld * b;
  double* Qk = Tn + b * b;
  double* zv = Qk + b * b;
  double* wv = zv + 32;
  double* yv = wv + 32;
  double* part = yv + 32;    // 3 x 128 partial sums
  double* Pb = part + 384;   // prefix product of Q1_top (nodes on leaf 0's path)
  for (int i = tid; i < ld * b; i += blockDim.x) S[i] = 0.0;
  for (int i = tid; i < b * b; i += blockDim.x) Tn[i] = 0.0;
  __syncthreads();
  auto tail = [](int r, int j) { return r >= 32 && (r & 31) <= j; };
  // column c of R (head rows 0..c), published to the parent by warp 0
  auto publish = [&](int c) {
    if (lane <= c) Rme[c * b + lane] = S[c * ld + lane];
    __threadfence();
    __syncwarp();
    if (lane == 0) st_release(a.prog + f, (unsigned)(c + 1));
  };
  for (int j = 0; j < b; ++j) {
    // (1) column j of every child: lane k of warp 1 waits for child k, while
    //     warp 0 publishes column j - 1 (finished in the last step)
    if (warp == 0 && j > 0 && nch > 1) publish(j - 1);
    if (warp == 1) {
      bool ok = true;
      if (lane < nch) ok = h6_wait(a, a.prog + child0 + lane, (unsigned)(j + 1));
      ok = __all_sync(0xffffffffu, ok);
      if (lane == 0) *s_ok = ok;
    }
    __syncthreads();
    if (!*s_ok) {
      h6_release_all(a, f);
      return;
    }
    if (nch == 1) {   // a pass-through node: its R is its child's
      if (warp == 0) {
        if (lane <= j) Rme[j * b + lane] = __ldcg(a.Rn + (size_t)child0 * b * b + j * b + lane);
        __threadfence();
        __syncwarp();
        if (lane == 0) st_release(a.prog + f, (unsigned)(j + 1));
      }
      continue;
    }
    // (2) stack the children's column j
    if (warp < nch && lane <= j)
      S[j * ld + 32 * warp + lane] = __ldcg(a.Rn + (size_t)(child0 + warp) * b * b + j * b + lane);
    __syncthreads();
    if (j > 0) {
      // (3) one reduction for two sets of dot products over the children's
      //     rows: z_p = v_p^T s_j (p < j; the head adds row p of s_j) and
      //     y_p = v_p^T v_(j-1) (p < j - 1), which give column j - 1 of T
      double dd[16];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int pp = warp + 4 * q;
        dd[q] = 0.0;
        dd[8 + q] = 0.0;
        if (pp < j)
          for (int k = 1; k < nch; ++k) {
            const double vp = S[pp * ld + 32 * k + lane];
            dd[q] = fma(vp, S[j * ld + 32 * k + lane], dd[q]);
            if (pp < j - 1) dd[8 + q] = fma(vp, S[(j - 1) * ld + 32 * k + lane], dd[8 + q]);
          }
      }
      {
        const double sq = warp_sum16_held(dd);
        const int id = warp_sum16_index(lane);
        const int pp = warp + 4 * (id & 7);
        if ((lane & 1) == 0) {
          if (id < 8) {
            if (pp < j) zv[pp] = S[j * ld + pp] + sq;
          } else if (pp < j - 1) {
            yv[pp] = sq;
          }
        }
      }
      __syncthreads();
      // (4) column c = j - 1 of T: T[p][c] = -tau_c sum_{q=p}^{c-1} T[p][q] y_q
      const int c = j - 1;
      if (c > 0) {
        double acc = 0.0;
        if (lane < c)
          for (int q = warp; q < c; q += 4)
            if (q >= lane) acc = fma(Tn[q * b + lane], yv[q], acc);
        part[warp * 32 + lane] = acc;
        __syncthreads();
        if (warp == 0 && lane < c)
          Tn[c * b + lane] = -s_tau[c] * ((part[lane] + part[32 + lane]) + (part[64 + lane] + part[96 + lane]));
        __syncthreads();
      }
      // (5) w = T^T z
      {
        double acc = 0.0;
        if (lane < j)
          for (int pp = warp; pp <= lane; pp += 4) acc = fma(Tn[lane * b + pp], zv[pp], acc);
        part[warp * 32 + lane] = acc;
      }
      __syncthreads();
      if (warp == 0 && lane < j) wv[lane] = (part[lane] + part[32 + lane]) + (part[64 + lane] + part[96 + lane]);
      __syncthreads();
      // (6) s_j -= V w: the head rows p < j directly; child k's rows r < j by
      //     sum_{p<j} V_k[r][p] w_p (V_k[r][p] = 0 for r > p), p split over the warps
      {
        double acc[kFan - 1];
#pragma unroll
        for (int k = 0; k < kFan - 1; ++k) acc[k] = 0.0;
        for (int pp = warp; pp < j; pp += 4) {
          const double wp = wv[pp];
#pragma unroll
          for (int k = 1; k < kFan; ++k)
            if (k < nch) acc[k - 1] = fma(S[pp * ld + 32 * k + lane], wp, acc[k - 1]);
        }
#pragma unroll
        for (int k = 0; k < kFan - 1; ++k) part[k * 128 + warp * 32 + lane] = acc[k];
      }
      __syncthreads();
      if (warp == 0) {
        if (lane < j) S[j * ld + lane] -= wv[lane];
      } else if (warp < nch && lane < j) {
        const double* pk = part + (warp - 1) * 128;
        S[j * ld + 32 * warp + lane] -= (pk[lane] + pk[32 + lane]) + (pk[64 + lane] + pk[96 + lane]);
      }
      __syncthreads();
    }
    // (7) reflector j; T[j][j] = tau_j (read from the next step on)
    if (warp == 0) h5_reflector<kFan>(S, ld, nch * 32, j, b, tail, s_tau, Qk);
    __syncthreads();
    if (tid == 0) Tn[j * b + j] = s_tau[j];
  }
  if (nch > 1 && b > 1) {
    // the last column of T: y_p = v_p^T v_(b-1), p < b - 1
    const int c = b - 1;
    double dd[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      dd[q] = 0.0;
      const int pp = warp + 4 * q;
      if (pp < c)
        for (int k = 1; k < nch; ++k) dd[q] = fma(S[pp * ld + 32 * k + lane], S[c * ld + 32 * k + lane], dd[q]);
    }
    {
      const double sq = warp_sum8_held(dd);
      const int pp = warp + 4 * warp_sum8_index(lane);
      if ((lane & 3) == 0 && pp < c) yv[pp] = sq;
    }
    __syncthreads();
    {
      double acc = 0.0;
      if (lane < c)
        for (int q = warp; q < c; q += 4)
          if (q >= lane) acc = fma(Tn[q * b + lane], yv[q], acc);
      part[warp * 32 + lane] = acc;
    }
    __syncthreads();
    if (warp == 0 && lane < c)
      Tn[c * b + lane] = -s_tau[c] * ((part[lane] + part[32 + lane]) + (part[64 + lane] + part[96 + lane]));
  }
  __syncthreads();
  if (nch > 1 && warp == 0) publish(b - 1);
  if (idx == 0) {
    // on leaf 0's path: P_lvl = P_(lvl-1) Q1 = P_(lvl-1) (I - T), as soon as the
    // child on the path has its prefix (it then sets its progress to b + 1).
    // The root's solver waits for this node's prefix the same way.
    if (tid == 0) *s_ok = h6_wait(a, a.prog + child0, (unsigned)b + 1u);
    __syncthreads();
    if (!*s_ok) {
      h6_release_all(a, f);
      return;
    }
    h4_load(Qk, a.Pc + (size_t)(lvl - 1) * b * b, b);
    double* Pl = a.Pc + (size_t)lvl * b * b;
    if (nch > 1) {
      h5_mm(Qk, b, false, kSDense, Tn, b, false, kSUpper, Pb, b, b, -1.0, Qk);
      for (int i = tid; i < b * b; i += blockDim.x) Pl[i] = Pb[i];
    } else {
      for (int i = tid; i < b * b; i += blockDim.x) Pl[i] = Qk[i];
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) st_release(a.prog + f, (unsigned)b + 1u);
  }
  if (nch > 1) {
    // Q blocks of the node (for forming Y): Q_1 = I - T;  Q_k = -V_k T
    double* Qp = a.Qn + (size_t)f * kFan * b * b;
    for (int i = tid; i < b * b; i += blockDim.x) {
      const int r = i % b, c = i / b;
      Qp[i] = ((r == c) ? 1.0 : 0.0) - ((r <= c) ? Tn[c * b + r] : 0.0);
    }
    for (int k = 1; k < nch; ++k) {
      h5_mm(S + 32 * k, ld, false, kSUpper, Tn, b, false, kSUpper, Qk, b, b, -1.0, nullptr);
      for (int i = tid; i < b * b; i += blockDim.x) Qp[(size_t)k * b * b + i] = Qk[i];
      __syncthreads();
    }
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) st_release(a.done + f, 1u);
}

// The root's solver (one extra CTA): once the top node has published its R
// and the full prefix Q1_top, the sign-choice LU, T, W and U^-1, while the
// top node still writes its Q blocks.
__device__ void h6_root_solver(const Hr4Args& a, double* sm, int* s_ok) {
  const int top = a.base[a.depth];
  if (threadIdx.x == 0) *s_ok = h6_wait(a, a.prog + top, (unsigned)a.b + 1u);
  __syncthreads();
  if (!*s_ok) return;
  __threadfence();
  h4_root(a, sm);
}

__global__ void __launch_bounds__(kLeafThreads) k_hr6_pipe(Hr4Args a) {
  extern __shared__ double sm6[];
  __shared__ double s_tau[kDirectB];
  __shared__ int s_role, s_ok;
  if (threadIdx.x == 0) s_role = (int)atomicAdd(a.ticket, 1u);
  __syncthreads();
  const int f = s_role;   // flat tree id: leaves 0 .. P-1, the nodes level by level, the root's solver
  if (f < a.P)
    h6_leaf(a, f, sm6, s_tau);
  else if (f <= a.base[a.depth])
    h6_node(a, f, sm6, s_tau, &s_ok);
  else
    h6_root_solver(a, sm6, &s_ok);
}

// The product of the Q blocks along the root-to-node path times U^-1, for
// every node of level lvl (1 <= lvl < depth), from the parents' products:
// M(node) = Q(parent, child index) M(parent), or M(parent) for an only child,
// with M(root) = U^-1.  Run level by level from the top, this forms every
// path product once (about P / 3 products) instead of once per leaf and
// level (P x depth) in k_hr4_form_y.
__global__ void __launch_bounds__(kLeafThreads) k_hr4_node_m(Hr4Args a, int lvl) {
  extern __shared__ double sm4[];
  const int b = a.b, tid = threadIdx.x;
  const int c = blockIdx.x;                 // node index within level lvl
  const int nd = c / kFan;                  // parent at level lvl + 1
  const size_t nb2 = (size_t)b * b;
  const double* Mp = (lvl + 1 == a.depth) ? a.Uinv : a.Mn + (size_t)(a.base[lvl + 1] + nd) * nb2;
  double* Mo = a.Mn + (size_t)(a.base[lvl] + c) * nb2;
  double* sQ = sm4;
  double* sM = sQ + nb2;
  double* sO = sM + nb2;
  if (h4_children(a, lvl + 1, nd) > 1) {
    h4_load(sQ, a.Qn + ((size_t)(a.base[lvl + 1] + nd) * kFan + (c - nd * kFan)) * nb2, b);
    h4_load(sM, Mp, b);
    h5_mm(sQ, b, false, kSUpper, sM, b, false, kSUpper, sO, b, b, 1.0, nullptr);
    for (int idx = tid; idx < b * b; idx += blockDim.x) Mo[idx] = sO[idx];
  } else {
    for (int idx = tid; idx < b * b; idx += blockDim.x) Mo[idx] = __ldcg(Mp + idx);
  }
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
  // the levels above 1 come from k_hr4_node_m when it ran (a.Mn)
  const int top = (a.Mn && a.depth >= 2) ? 1 : a.depth;
  if (top < a.depth)
    h4_load(sM, a.Mn + (size_t)(a.base[1] + leaf / kFan) * b * b, b);
  else
    h4_load(sM, a.Uinv, b);
  for (int lvl = top; lvl >= 1; --lvl) {
    int nd = leaf;
    for (int l = 0; l < lvl; ++l) nd /= kFan;
    int child = leaf;
    for (int l = 0; l < lvl - 1; ++l) child /= kFan;
    if (h4_children(a, lvl, nd) > 1) {
      const int k = child - nd * kFan;
      h4_load(sX, a.Qn + ((size_t)(a.base[lvl] + nd) * kFan + k) * b * b, b);
      h5_mm(sX, b, false, kSUpper, sM, b, false, kSUpper, sY, b, b, 1.0, nullptr);
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
  h5_mm(sY, b, true, kSUnitUpper, sM, b, false, kSUpper, sX, b, b, 1.0, nullptr);   // sX = V_top^T M
  h5_mm(sT, b, false, kSUpper, sX, b, false, kSUpper, sY, b, b, 1.0, nullptr);      // sY = Z = T sX
  // Z is upper triangular: Y[r][c] = M[r][c] - sum_{k<=c} V[r][k] Z[k][c], eight
  // columns at a time with independent accumulators (the loops unroll fully,
  // so the triangle is cut at compile time)
  for (int64_t r = r0 + tid; r < r1; r += blockDim.x) {
    if (r < b) continue;
    const int rl = (int)(r - r0);
    double v[kDirectB];
#pragma unroll
    for (int k = 0; k < kDirectB; ++k)
      v[k] = (k < b) ? (rl > k ? a.Vw[(int64_t)k * a.m + r] : (rl == k ? 1.0 : 0.0)) : 0.0;
#pragma unroll
    for (int cb = 0; cb < kDirectB; cb += 8) {
      if (cb < b) {
        double acc[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) acc[u] = (rl < b && cb + u < b) ? sM[(cb + u) * b + rl] : 0.0;
#pragma unroll
        for (int k = 0; k < cb + 8; ++k) {
#pragma unroll
          for (int u = 0; u < 8; ++u)
            if (k <= cb + u) {
              const double z = (cb + u < b) ? sY[(cb + u) * b + k] : 0.0;
              acc[u] = fma(-v[k], z, acc[u]);
            }
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (cb + u < b) a.A[(int64_t)(cb + u) * a.lda + r] = acc[u];
      }
    }
  }
}

int hr_direct4(double* A, int64_t lda, int64_t m, int b, double* T, int64_t ldT, double* W,
               int64_t ldW, int* d_status, cudaStream_t s) {
  if (b < 1 || b > kDirectB || m < b) return CANDMC_ERR_ARG;
  int64_t want = t_leaf_rows > 0 ? t_leaf_rows : g_leaf_rows;
  // the lookahead's tall panels (thousands of leaves: throughput, not the
  // latency of one leaf, sets the time) take 256-row leaves
  if (t_leaf_rows > 0 && m >= kTallPanelRows) want = std::max<int64_t>(want, 256);
  const int64_t leaf_rows = std::max<int64_t>(32, std::min<int64_t>(want, 256));
  // leaves of at most leaf_rows rows and at least b rows
  int64_t P = std::max<int64_t>(1, std::min<int64_t>((m + leaf_rows - 1) / leaf_rows, m / b));
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
  // shared block: rows padded to the row slots of the factor instantiation
  // that runs (1..4 slots of 32 rows, or 8 for leaves of more than 128 rows),
  // and at least the 4 x 32 rows of a tree node
  const int64_t slots = (Lmax + 31) / 32;
  const int64_t ldS = std::max<int64_t>(32 * (slots <= 4 ? slots : 8), kFan * 32);
  if (ldS > 32 * kMaxR) return CANDMC_ERR_ARG;
  a.ldS = (int)ldS;
  // block + G + T + tri-inverse workspace; the root reuses the front of the
  // same area for six b x b buffers plus the workspace
  const size_t sm = sizeof(double) * std::max<size_t>((size_t)ldS * b + 2 * nb2 + kTriScratch,
                                                      6 * nb2 + kTriScratch);
  if (sm > 200 * 1024) return CANDMC_ERR_ARG;
  // the pipelined tree while the whole tree is a modest number of CTAs (a
  // latency-bound panel); the level-by-level tree for many leaves, where the
  // leaves dominate and the pipeline would only add synchronisation
  const bool pipe = a.depth >= 1 && g_pipe_tree && nnodes <= 4096;
  // one workspace, carved in 256-byte aligned pieces; the counters and the
  // node R blocks (read before all their entries are written) lead it, so
  // one memset clears both
  // counters: cnt (last arriver) or prog + done + ticket + fail (pipelined)
  const size_t ncnt = pipe ? 2 * (size_t)nnodes + 2 : (size_t)nnodes;
  auto rup256 = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t o_cnt = 0;
  const size_t o_rn = o_cnt + rup256(sizeof(unsigned) * ncnt);
  const size_t o_vw = o_rn + rup256(sizeof(double) * nb2 * nnodes);
  const size_t o_tl = o_vw + rup256(sizeof(double) * (size_t)m * b);
  const size_t o_qn = o_tl + rup256(sizeof(double) * nb2 * P);
  const size_t o_uinv = o_qn + rup256(sizeof(double) * nb2 * kFan * nnodes);
  const size_t o_pc = o_uinv + rup256(sizeof(double) * nb2);
  // many leaves: the path products are formed once per node, top down
  const bool node_m = P >= kNodeMinLeaves && a.depth >= 2;
  const size_t o_mn = o_pc + (pipe ? rup256(sizeof(double) * nb2 * (a.depth + 1)) : 0);
  const size_t total_bytes = o_mn + (node_m ? rup256(sizeof(double) * nb2 * nnodes) : 0);
  DevBuf ws;
  CANDMC_RET(ws.alloc(total_bytes, s));
  char* base = static_cast<char*>(ws.p);
  CANDMC_CK(cudaMemsetAsync(base, 0, pipe ? o_vw : o_rn, s));
  a.A = A; a.lda = lda; a.m = m; a.b = b;
  a.Vw = reinterpret_cast<double*>(base + o_vw);
  a.Tl = reinterpret_cast<double*>(base + o_tl);
  a.Rn = reinterpret_cast<double*>(base + o_rn);
  a.Qn = reinterpret_cast<double*>(base + o_qn);
  a.cnt = reinterpret_cast<unsigned*>(base + o_cnt);
  if (pipe) {
    a.prog = a.cnt;
    a.done = a.cnt + nnodes;
    a.ticket = a.cnt + 2 * nnodes;
    a.fail = reinterpret_cast<int*>(a.cnt + 2 * nnodes + 1);
    a.Pc = reinterpret_cast<double*>(base + o_pc);
  }
  a.T = T; a.ldT = ldT; a.W = W; a.ldW = ldW;
  a.Uinv = reinterpret_cast<double*>(base + o_uinv);
  a.Mn = node_m ? reinterpret_cast<double*>(base + o_mn) : nullptr;
  a.status = d_status;
  static std::atomic<bool> attr{false};
  if (!attr) {
    CANDMC_CK(cudaFuncSetAttribute(k_hr4_leaf_tree, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   200 * 1024));
    CANDMC_CK(cudaFuncSetAttribute(k_hr6_pipe, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    attr = true;
  }
  {
    ProfScope ps(CANDMC_KCLASS_PANEL_LEAF, 2.0 * m * b * b, s);
    if (pipe)
      k_hr6_pipe<<<(unsigned)nnodes + 1u, kLeafThreads, sm, s>>>(a);
    else
      k_hr4_leaf_tree<<<(unsigned)P, kLeafThreads, sm, s>>>(a);
  }
  CANDMC_CK(cudaGetLastError());
  if (node_m) {
    for (int lvl = a.depth - 1; lvl >= 1; --lvl) {
      ProfScope ps(CANDMC_KCLASS_PANEL_Y, 2.0 * a.nlev[lvl] * (double)nb2 * b / 3.0, s);
      k_hr4_node_m<<<(unsigned)a.nlev[lvl], kLeafThreads, sizeof(double) * 3 * nb2, s>>>(a, lvl);
      CANDMC_CK(cudaGetLastError());
    }
  }
  {
    // with several waves of leaves, one thread per leaf row: leaves of at most
    // 128 rows take 128-thread CTAs, so two of them (252 registers a thread)
    // share an SM; a single wave keeps 256 threads for the path products
    const unsigned ythreads = (Lmax <= 128 && P >= kNodeMinLeaves) ? 128u : (unsigned)kThreads;
    ProfScope ps(CANDMC_KCLASS_PANEL_Y, 2.0 * m * b * b, s);
    k_hr4_form_y<<<(unsigned)P, ythreads, sizeof(double) * 4 * nb2, s>>>(a);
  }
  CANDMC_CK(cudaGetLastError());
  return CANDMC_OK;
}

}  // namespace candmc
