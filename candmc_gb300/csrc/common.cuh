// Shared device helpers and host plumbing for the CANDMC QR hot path on sm_103a.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/candmc_gb300.h"

namespace candmc {

constexpr int kThreads = 256;   // threads of every FP64 kernel
constexpr int kDirectB = 32;    // widest sub-panel factored by the direct TSQR-HR kernels
constexpr int kMaxLevels = 40;  // tree levels (2^40 leaves is far beyond any m)

// Matrix operand view: element (i, j) of op(X), with op = transpose or not,
// and an optional structural mask applied on the STORED indices (r, c).
enum Mask : int {
  kDense = 0,
  kUnitLower = 1,    // r > c + off: X[r,c];  r == c + off: 1;  else 0   (Y of a Y\R buffer)
  kUpper = 2,        // r <= c + off: X[r,c]; else 0
  kLower = 3,        // r >= c + off: X[r,c]; else 0
};

struct MatRef {
  const double* p;
  int64_t ld;
  int trans;   // 1: element (i,j) of the operand is X[j,i]
  int mask;
  int64_t off;
};

__host__ __device__ inline MatRef mref(const double* p, int64_t ld, int trans = 0, int mask = kDense,
                                       int64_t off = 0) {
  MatRef r;
  r.p = p; r.ld = ld; r.trans = trans; r.mask = mask; r.off = off;
  return r;
}

__device__ __forceinline__ double mat_at(const MatRef& X, int64_t i, int64_t j) {
  int64_t r = X.trans ? j : i;
  int64_t c = X.trans ? i : j;
  switch (X.mask) {
    case kUnitLower:
      if (r > c + X.off) return X.p[c * X.ld + r];
      return r == c + X.off ? 1.0 : 0.0;
    case kUpper:
      return r <= c + X.off ? X.p[c * X.ld + r] : 0.0;
    case kLower:
      return r >= c + X.off ? X.p[c * X.ld + r] : 0.0;
    default:
      return X.p[c * X.ld + r];
  }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Binary reduction tree over P leaves: level 0 holds the leaves, level l has
// nlev[l] = ceil(nlev[l-1] / 2) nodes; node i of level l has children 2i and
// 2i+1 of level l-1 (only 2i when 2i+1 == nlev[l-1]: a pass-through node).
struct TreeDesc {
  int P;
  int depth;
  int nlev[kMaxLevels + 1];
  int base[kMaxLevels + 1];   // flat index of node 0 of each level
  int nnodes;
};

inline TreeDesc make_tree(int P) {
  TreeDesc t{};
  t.P = P;
  t.nlev[0] = P;
  t.base[0] = 0;
  int l = 0, total = P;
  while (t.nlev[l] > 1) {
    t.nlev[l + 1] = (t.nlev[l] + 1) / 2;
    t.base[l + 1] = total;
    total += t.nlev[l + 1];
    ++l;
  }
  t.depth = l;
  t.nnodes = total;
  return t;
}

// Host-side status helpers.
int set_error(int code, const char* what);
int cuda_status(cudaError_t e, const char* where);

#define CANDMC_CK(expr)                                      \
  do {                                                       \
    cudaError_t _e = (expr);                                 \
    if (_e != cudaSuccess) return ::candmc::cuda_status(_e, #expr); \
  } while (0)

#define CANDMC_RET(expr)               \
  do {                                 \
    int _s = (expr);                   \
    if (_s != CANDMC_OK) return _s;    \
  } while (0)

// Stream-ordered device scratch, released on the same stream.
struct DevBuf {
  void* p = nullptr;
  cudaStream_t s = nullptr;
  int alloc(size_t bytes, cudaStream_t stream);
  ~DevBuf();
  double* d() const { return static_cast<double*>(p); }
};

}  // namespace candmc
