// Emulated-FP64 contractions of the CAQR trailing update on the 5th-generation
// tensor cores (tcgen05, BF16 inputs, FP32 accumulation in TMEM).
//
// Ozaki-style splitting (Ozaki, Ogita, Oishi, Rump, "Error-free transformations
// of matrix multiplication by using fast routines of matrix multiplication and
// its applications", Numer. Algorithms 59, 2012): every operand element x of a
// scale group with |x| < 2^e is written as x = 2^(e-8) * sum_{i<7} d_i 2^(-8i)
// with balanced integer digits |d_0| <= 256, |d_i| <= 128 (i >= 1).  Slice i
// holds d_i * 2^(-8i), exact in BF16 (<= 8 significant bits).  A product of
// two slices has <= 16 significant bits, so a K = 128 sum of one "level"
// L = i + j is an exact FP32 integer (at its weight); levels 0..3 get one TMEM
// accumulator each and levels 4..6 share a fifth (their rounding sits below
// 2^-56 of the result).  28 slice pairs (i + j <= 6) are issued per K step.
//
// The trailing matrix is held as float pairs (hi, lo) ("df64", ~48 bits)
// during the emulated factorization, so no epilogue needs the GB300's slow
// FP64 pipe: the five accumulators are combined exactly (integer/fraction
// split, fast TwoSum), scaled by a power of two and accumulated or subtracted
// in df64.  Finished rows (the panel's R block) are written back as FP64.
//
// Kernel layout (k_oz_mma): persistent CTAs (at most one per SM) over work
// items of one 128 x 96 output tile and K range each; 14 warps.  Operand
// slices are pre-sliced in global memory in the UMMA "K-major, no swizzle"
// core-matrix order, so each K16 step of a tile is a contiguous 4 KB (A, 128
// rows) and 3 KB (B, 96 rows) block per slice: a producer warp streams them
// with bulk asynchronous copies into a 4-stage shared-memory ring, an MMA
// warp issues the 28 tcgen05.mma of a step and commits them to the stage's
// "empty" mbarrier (and, at the end of an exact-accumulation group, to the
// epilogue's "full" mbarrier), and twelve epilogue warps drain and combine
// the accumulators and release them; the df64 read-modify-write of C (MODE
// 1) then overlaps the next group's MMAs.  Every wait is bounded; a wait that
// runs out sets the status word, the roles stop, the MMA warp waits for its
// last MMAs, and the CTA frees its TMEM and returns.
#include <cuda_bf16.h>
#include <math.h>

#include <algorithm>

#include "kernels.cuh"

namespace candmc {

constexpr int OZ_S = 7;           // slices per operand of the emulated-FP64 form
constexpr int OZ_S32 = 3;         // slices per operand of the FP32 form
constexpr int OZ_M = 128;         // tile rows (TMEM lanes)
constexpr int OZ_N = 96;          // tile columns
constexpr int OZ_STAGES = 4;
constexpr int OZ_ABYTES = OZ_M * 16 * 2;               // one slice, one K16 step
constexpr int OZ_BBYTES = OZ_N * 16 * 2;
// Per slice count S: TMEM accumulator groups G (levels 0..3 exact each, the
// rest shared, for S = 7; one per level for S <= 5), bytes of one ring stage
// and the dynamic shared memory of the kernel.
template <int S>
struct OzCfg {
  static constexpr int G = S >= 5 ? 5 : S;
  static constexpr int STAGE_BYTES = S * (OZ_ABYTES + OZ_BBYTES);
  static constexpr int SMEM = OZ_STAGES * STAGE_BYTES + 1024;
};
constexpr long OZ_WAIT_LIMIT = 1L << 22;                // bounded mbarrier polls

// element (r, k) of an R x K operand slice plane in core-matrix K-major order
__host__ __device__ __forceinline__ int64_t cm_off(int64_t r, int64_t k, int64_t R) {
  return (k >> 4) * (R * 16) + (r >> 3) * 128 + ((k & 15) >> 3) * 64 + (r & 7) * 8 + (k & 7);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// ------------------------------------------------------------------ df64
struct f2 {
  float h, l;
};

__device__ __forceinline__ f2 two_sum(float a, float b) {
  float s = a + b;
  float bb = s - a;
  float e = (a - (s - bb)) + (b - bb);
  return {s, e};
}

__device__ __forceinline__ f2 fast_two_sum(float a, float b) {
  float s = a + b;
  return {s, b - (s - a)};
}

// (h, l) + g
__device__ __forceinline__ f2 df_add_f(f2 x, float g) {
  f2 s = two_sum(x.h, g);
  return fast_two_sum(s.h, s.l + x.l);
}

// x + y
__device__ __forceinline__ f2 df_add(f2 x, f2 y) {
  f2 s = two_sum(x.h, y.h);
  f2 t = two_sum(x.l, y.l);
  s.l += t.h;
  s = fast_two_sum(s.h, s.l);
  s.l += t.l;
  return fast_two_sum(s.h, s.l);
}

__device__ __forceinline__ f2 df_from_double(double x) {
  float h = (float)x;
  float l = (float)(x - (double)h);
  return {h, l};
}

__device__ __forceinline__ double df_to_double(f2 x) { return (double)x.h + (double)x.l; }

// ------------------------------------------------------------------ slicing
// 2^e for -126 <= e <= 127 (a normal float): x * pow2f(e) rounds once, as
// ldexpf(x, e) does
__device__ __forceinline__ float pow2f(int e) { return __int_as_float((e + 127) << 23); }

// x * 2^k rounded once: one multiplication when 2^k is a normal float
__device__ __forceinline__ float scale_pow2(float x, int k) {
  return (k >= -126 && k <= 127) ? __fmul_rn(x, pow2f(k)) : ldexpf(x, k);
}

// Scale exponent of a group maximum: smallest e with max < 2^e (0 for 0).
__device__ __forceinline__ int scale_exp(float mx) {
  if (!(mx > 0.0f)) return 0;
  int e;
  frexpf(mx, &e);   // mx = f * 2^e, f in [0.5, 1)
  return e;
}

// Write the S natural-weight digits of v = (h + l) * 2^(8 - e) to slices.
template <int S>
__device__ __forceinline__ void slice_value(f2 v, int e, __nv_bfloat16* out, int64_t plane,
                                            int64_t off) {
  float p = scale_pow2(v.h, 8 - e), q = scale_pow2(v.l, 8 - e);
  float w = 1.0f;
#pragma unroll
  for (int i = 0; i < S; ++i) {
    f2 s = two_sum(p, q);
    float d = rintf(s.h);
    out[i * plane + off] = __float2bfloat16_rn(d * w);
    p = (s.h - d) * 256.0f;
    q = s.l * 256.0f;
    w *= 0.00390625f;
  }
}

struct SliceSrc {
  const double* d;     // FP64 source (mask applies), or nullptr
  const float2* df;    // df64 source, or nullptr
  int64_t ld;
  int mask;            // kDense / kUnitLower / kUpper (FP64 source)
  int64_t off;         // diagonal offset of the mask
};

__device__ __forceinline__ f2 src_at(const SliceSrc& s, int64_t r, int64_t c) {
  if (s.df) {
    float2 v = s.df[c * s.ld + r];
    return {v.x, v.y};
  }
  double x;
  switch (s.mask) {
    case kUnitLower: x = (r > c + s.off) ? s.d[c * s.ld + r] : (r == c + s.off ? 1.0 : 0.0); break;
    case kUpper: x = (r <= c + s.off) ? s.d[c * s.ld + r] : 0.0; break;
    case kLower: x = (r >= c + s.off) ? s.d[c * s.ld + r] : 0.0; break;
    default: x = s.d[c * s.ld + r];
  }
  return df_from_double(x);
}

// Operand element (n, k) = src(k, n): K runs down the columns of a column-major
// source (rows k0 .. k0 + K).  One warp per (n, K group of G); n in [0, Nvalid)
// are data, rows beyond are zero padding up to Rpad; k beyond Kvalid are zero.
// Slices: S planes of Rpad x Kpad (cm order); exponents e[(k/G) * Rpad + n].
template <int S>
__global__ void k_slice_kcol(SliceSrc src, int64_t k0, int64_t Kvalid, int64_t Nvalid, int64_t Rpad,
                             int64_t Kpad, int G, __nv_bfloat16* out, int* eout) {
  const int lane = threadIdx.x & 31;
  const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t ngroups = Kpad / G;
  if (wid >= Rpad * ngroups) return;
  const int64_t n = wid % Rpad, g = wid / Rpad;
  const int64_t plane = Rpad * Kpad;
  float mx = 0.0f;
  if (n < Nvalid) {
    for (int64_t k = g * G + lane; k < (g + 1) * G && k < Kvalid; k += 32) {
      f2 v = src_at(src, k0 + k, n);
      mx = fmaxf(mx, fabsf(v.h));
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  // the lo part can push |x| just above |hi|'s bound; leave one ulp of room
  const int e = scale_exp(mx * (1.0f + 1.0e-6f));
  if (lane == 0) eout[g * Rpad + n] = e;
  for (int64_t k = g * G + lane; k < (g + 1) * G; k += 32) {
    f2 v = {0.0f, 0.0f};
    if (n < Nvalid && k < Kvalid) v = src_at(src, k0 + k, n);
    slice_value<S>(v, e, out, plane, cm_off(n, k, Rpad));
  }
}

// The same slicing with coalesced stores: one CTA per 8 rows n of the operand
// (one core-matrix row block) and one K group of G <= 128 (a multiple of 16).
// Warp w reads column n0 + w of the source into shared memory and finds its
// scale exponent; then, for every K16 block, the 8 x 16 elements of a slice
// plane are one contiguous 256-byte run of the core-matrix order, which a
// warp writes with 8-byte stores (4 elements per lane).
template <int S>
__global__ void __launch_bounds__(256) k_slice_kcol8(SliceSrc src, int64_t k0, int64_t Kvalid,
                                                     int64_t Nvalid, int64_t Rpad, int64_t Kpad, int G,
                                                     __nv_bfloat16* out, int* eout) {
  __shared__ float2 tile[8][128];
  __shared__ int s_e[8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t n0 = (int64_t)blockIdx.x * 8;
  const int64_t g = blockIdx.y;
  const int64_t kb0 = g * G;
  {
    const int64_t n = n0 + warp;
    float mx = 0.0f;
    for (int k = lane; k < G; k += 32) {
      f2 v = {0.0f, 0.0f};
      if (n < Nvalid && kb0 + k < Kvalid) v = src_at(src, k0 + kb0 + k, n);
      tile[warp][k] = make_float2(v.h, v.l);
      mx = fmaxf(mx, fabsf(v.h));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    // the lo part can push |x| just above |hi|'s bound; leave one ulp of room
    const int e = scale_exp(mx * (1.0f + 1.0e-6f));
    if (lane == 0) {
      s_e[warp] = e;
      if (n < Rpad) eout[g * Rpad + n] = e;
    }
  }
  __syncthreads();
  const int64_t plane = Rpad * Kpad;
  // lane u of a warp: elements 4u .. 4u+3 of a 128-element core-matrix run:
  // k-half (u / 16), row (u % 16) / 2, k & 7 = 4 (u % 2) .. +3
  const int u = lane;
  const int khalf = u >> 4, r = (u & 15) >> 1, k7 = (u & 1) * 4;
  const int e = s_e[r];
  for (int blk = warp; blk < G / 16; blk += 8) {
    float p[4], q[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float2 t = tile[r][blk * 16 + khalf * 8 + k7 + i];
      p[i] = scale_pow2(t.x, 8 - e);
      q[i] = scale_pow2(t.y, 8 - e);
    }
    const int64_t base = ((kb0 >> 4) + blk) * (Rpad * 16) + (n0 >> 3) * 128 + 4 * u;
    float w = 1.0f;
#pragma unroll
    for (int sl = 0; sl < S; ++sl) {
      __align__(8) __nv_bfloat16 d4[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const f2 sv = two_sum(p[i], q[i]);
        const float d = rintf(sv.h);
        d4[i] = __float2bfloat16_rn(d * w);
        p[i] = (sv.h - d) * 256.0f;
        q[i] = sv.l * 256.0f;
      }
      *reinterpret_cast<uint2*>(out + sl * plane + base) = *reinterpret_cast<const uint2*>(d4);
      w *= 0.00390625f;
    }
  }
}

// Operand element (n, k) = src(n, k): K runs along the rows of a column-major
// source (rows n0 + n, columns 0 .. K).  Scale group = the whole row (G = Kpad).
// A CTA stages 32 rows x Kpad columns through shared memory.
template <int S>
__global__ void k_slice_krow(SliceSrc src, int64_t n0, int64_t Nvalid, int64_t Kvalid, int64_t Rpad,
                             int64_t Kpad, __nv_bfloat16* out, int* eout) {
  extern __shared__ float2 tile[];   // [32][Kpad]
  const int64_t nb = (int64_t)blockIdx.x * 32;
  for (int64_t idx = threadIdx.x; idx < 32 * Kpad; idx += blockDim.x) {
    int64_t rr = idx % 32, k = idx / 32;
    int64_t n = nb + rr;
    f2 v = {0.0f, 0.0f};
    if (n < Nvalid && k < Kvalid) v = src_at(src, n0 + n, k);
    tile[rr * Kpad + k] = make_float2(v.h, v.l);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int64_t plane = Rpad * Kpad;
  for (int rr = warp; rr < 32; rr += nw) {
    const int64_t n = nb + rr;
    if (n >= Rpad) continue;
    float mx = 0.0f;
    for (int64_t k = lane; k < Kpad; k += 32) mx = fmaxf(mx, fabsf(tile[rr * Kpad + k].x));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    const int e = scale_exp(mx * (1.0f + 1.0e-6f));
    if (lane == 0) eout[n] = e;
    for (int64_t k = lane; k < Kpad; k += 32) {
      float2 t = tile[rr * Kpad + k];
      slice_value<S>({t.x, t.y}, e, out, plane, cm_off(n, k, Rpad));
    }
  }
}

// ------------------------------------------------------------------ tcgen05 kernel
struct OzArgs {
  const __nv_bfloat16* As;   // A-operand slices: S planes of AR x Kpad
  int64_t AR;
  const __nv_bfloat16* Bs;   // B-operand slices: S planes of BR x Kpad
  int64_t BR;
  int64_t Kpad;              // multiple of 16
  int64_t k_per_cta;         // K extent of one CTA (multiple of kgroup)
  int64_t kgroup;            // K rows per scale group / accumulator readout
  const int* eA;             // [Kpad / kgroup][AR]
  const int* eB;             // [Kpad / kgroup][BR]
  int mode;                  // 0: partial sums (df64) over the CTA's K range; 1: C -= product
  float2* part;              // mode 0: [split][Nvalid][AR] (ld AR per column)
  float2* C;                 // mode 1: df64 matrix (ld ldc)
  double* C64;               // mode 1: same storage viewed as FP64
  int64_t ldc;
  int64_t Mvalid, Nvalid;
  int64_t fp64_rows;         // mode 1: rows < fp64_rows are written as FP64 (final)
  int c_fp64;                // mode 1: C is stored as FP64 (read and written in FP64)
  int c_assign;              // mode 1 with c_fp64: C = product (C is not read)
  int* status;
  int64_t n_mt, n_nt, n_ks;  // work items: M tiles x N tiles x K splits
};

__device__ __forceinline__ uint64_t make_desc(uint32_t saddr) {
  // K-major, no swizzle: LBO = 128 B (next 8 K elements), SBO = 256 B (next 8 rows)
  return (uint64_t)((saddr & 0x3FFFF) >> 4) | ((uint64_t)(128 >> 4) << 16) |
         ((uint64_t)(256 >> 4) << 32) | (1ull << 46);
}

// tcgen05.ld writes its registers asynchronously: they hold the TMEM values
// only after tcgen05.wait::ld.  The compiler sees no dependence between the
// two, so the loaded registers are passed through tmem_regs_ready (an empty
// asm ordered after the wait) before any use.
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t* r) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                 "=r"(r[7])
               : "r"(taddr));
}

__device__ __forceinline__ void tmem_regs_ready(uint32_t* r) {
  asm volatile("" : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]),
               "+r"(r[7]));
}


constexpr int OZ_EPI_WARPS = 12;                     // epilogue warps: 4 TMEM lane quarters x column parts
constexpr int OZ_EPI_COLS = OZ_N * 4 / OZ_EPI_WARPS;  // accumulator columns per epilogue warp
constexpr int OZ_WARPS = 2 + OZ_EPI_WARPS;             // producer, MMA issuer, epilogue
constexpr int OZ_THREADS = OZ_WARPS * 32;
static_assert(OZ_EPI_WARPS % 4 == 0 && OZ_EPI_COLS % 16 == 0, "epilogue split");

// The five accumulators of one output element as one df64 value.  Groups 0..3
// hold the diagonals i + j = g of the slice products, exact multiples of
// 2^-8g with |g0| <= 2^23, |g1| <= 2^15, |g2| <= 2^8, |g3| < 1 (digits of at
// most 8 bits over a 128-row group); group 4 holds the rest, down to about
// 2^-40.  Rounding g1 and g2 to integers and g3 to a multiple of 2^-16 (the
// 1.5 * 2^23 and 1.5 * 2^7 shifts) splits them exactly: H = g0 + [g1] + [g2]
// is an integer below 2^24, M = frac(g1) + frac(g2) + [g3] a multiple of 2^-16
// below 2 in magnitude, both exact, and only L = (g3 - [g3]) + g4 rounds.  The
// two fast TwoSums are exact here (H is zero or at least 1 in magnitude), so
// the result carries about 2^-47 relative error, as a df64 sum of the five.
// The operations are round-to-nearest intrinsics, which the compiler neither
// contracts into FMAs nor reorders.
__device__ __forceinline__ f2 combine_groups(float g0, float g1, float g2, float g3, float g4) {
  const float kShift = 12582912.0f;   // 1.5 * 2^23: rounds to an integer
  const float kShift3 = 192.0f;       // 1.5 * 2^7: rounds to a multiple of 2^-16
  const float r1 = __fsub_rn(__fadd_rn(g1, kShift), kShift);
  const float r2 = __fsub_rn(__fadd_rn(g2, kShift), kShift);
  const float r3 = __fsub_rn(__fadd_rn(g3, kShift3), kShift3);
  const float H = __fadd_rn(__fadd_rn(g0, r1), r2);
  const float M = __fadd_rn(__fadd_rn(__fsub_rn(g1, r1), __fsub_rn(g2, r2)), r3);
  const float L = __fadd_rn(__fsub_rn(g3, r3), g4);
  const float s = __fadd_rn(H, M);
  const float e = __fsub_rn(M, __fsub_rn(s, H));
  const float l = __fadd_rn(e, L);
  const float h = __fadd_rn(s, l);
  return {h, __fsub_rn(l, __fsub_rn(h, s))};
}

// The accumulators of one output element as one value: the exact five-group
// combine of the emulated-FP64 form, or, for the FP32 form (one group per
// level, FP32 accuracy wanted), their FP32 sum.
template <int G>
__device__ __forceinline__ f2 combine_g(const float (&gv)[G][8], int j) {
  if constexpr (G == 5) {
    return combine_groups(gv[0][j], gv[1][j], gv[2][j], gv[3][j], gv[4][j]);
  } else {
    float h = gv[G - 1][j];
#pragma unroll
    for (int g = G - 2; g >= 0; --g) h = __fadd_rn(gv[g][j], h);
    return {h, 0.0f};
  }
}

// x + y without the lo-part TwoSum: relative error of order 2^-46 of |x| + |y|
__device__ __forceinline__ f2 df_add_sloppy(f2 x, f2 y) {
  const float s = __fadd_rn(x.h, y.h);
  const float bb = __fsub_rn(s, x.h);
  const float e = __fadd_rn(__fsub_rn(x.h, __fsub_rn(s, bb)), __fsub_rn(y.h, bb));
  const float l = __fadd_rn(e, __fadd_rn(x.l, y.l));
  const float h = __fadd_rn(s, l);
  return {h, __fsub_rn(l, __fsub_rn(h, s))};
}

// Accumulation of the epilogue: df64 for the emulated-FP64 form (G = 5); for
// the FP32 form (G < 5, products accurate to FP32) plain FP32, which keeps C
// in the df64 slots with a zero low word.
template <int G>
__device__ __forceinline__ f2 oz_accumulate(f2 x, f2 y) {
  if constexpr (G == 5) return df_add_sloppy(x, y);
  else return {__fadd_rn(x.h, y.h), 0.0f};
}

// C - p for the read-modify-write of MODE 1 (same split by form)
template <int G>
__device__ __forceinline__ f2 oz_subtract(f2 c, f2 p) {
  if constexpr (G == 5) return df_add(c, {-p.h, -p.l});
  else return {__fsub_rn(__fadd_rn(c.h, c.l), p.h), 0.0f};
}

__device__ __forceinline__ void mbar_init(uint64_t* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count));
}

__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes)
               : "memory");
}

// bulk global -> shared copy (16-byte aligned, multiple of 16 bytes) that
// signals the byte count on the stage's mbarrier
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, unsigned bytes, uint64_t* b) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
      "l"(src), "r"(bytes), "r"(smem_u32(b))
      : "memory");
}

// bounded wait; gives up early when another role of the CTA failed
__device__ __forceinline__ bool oz_wait(uint64_t* b, uint32_t parity, volatile int* fail) {
  const uint32_t addr = smem_u32(b);
  for (long it = 0; it < OZ_WAIT_LIMIT; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred q;\n\tmbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(done)
        : "r"(addr), "r"(parity)
        : "memory");
    if (done) return true;
    if ((it & 63) == 63 && *fail) return false;
  }
  *fail = 1;
  return false;
}

// One 128 x 96 x 16 BF16 MMA into the accumulator at TMEM column address dt;
// accum = 0 overwrites it.
__device__ __forceinline__ void umma_bf16(uint32_t dt, uint64_t ad, uint64_t bd, uint32_t idesc,
                                          uint32_t accum) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dt),
      "l"(ad), "l"(bd), "r"(idesc), "r"(accum));
}

// The slice-pair MMAs of one K16 step.  da / db: descriptors of the stage's
// first A and B slice (the slices follow at fixed byte strides, and a
// descriptor's address field is the shared-memory address / 16, so slice
// descriptors are the base plus a constant).  In loop order the first product
// of accumulator group g is (0, g): in a group's first step (FIRST) those
// overwrite their accumulator, every other product adds to it.
template <int S, int G, bool FIRST>
__device__ __forceinline__ void oz_issue_step(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc) {
#pragma unroll
  for (int i = 0; i < S; ++i) {
#pragma unroll
    for (int j = 0; j < S; ++j) {
      if (i + j >= S) continue;
      const int g = (i + j < G - 1) ? i + j : G - 1;
      const bool first = FIRST && i == 0 && j < G;
      umma_bf16(tmem + (uint32_t)(g * OZ_N), da + (uint64_t)(i * (OZ_ABYTES >> 4)),
                db + (uint64_t)(j * (OZ_BBYTES >> 4)), idesc, first ? 0u : 1u);
    }
  }
}

// Work item w of a launch: (M tile, N tile, K range).  M tiles run fastest so
// that consecutive items of a CTA share the B operand's slices in L2.
struct OzItem {
  int64_t m0, n0, kbeg, kend;
  int split;
};

__device__ __forceinline__ OzItem oz_item(const OzArgs& a, int64_t w) {
  OzItem it;
  const int64_t mt = w % a.n_mt, rest = w / a.n_mt;
  const int64_t nt = rest % a.n_nt, ks = rest / a.n_nt;
  it.m0 = mt * OZ_M;
  it.n0 = nt * OZ_N;
  it.kbeg = ks * a.k_per_cta;
  it.kend = (it.kbeg + a.k_per_cta < a.Kpad) ? it.kbeg + a.k_per_cta : a.Kpad;
  it.split = (int)ks;
  return it;
}

// Persistent, warp-specialised emulated-FP64 contraction.  Warp 0 streams the
// operands' pre-sliced K16 blocks into a ring of OZ_STAGES stages with bulk
// copies; warp 1 issues the 28 slice-pair MMAs of a stage into the five TMEM
// accumulator groups and commits them (freeing the stage, and at the end of
// an exact-accumulation group, handing the accumulators to the epilogue);
// the epilogue warps 2.. read the accumulators (warp w owns TMEM lanes
// 32 (w % 4) .. +31 and column part (w - 2) / 4), release them, and combine
// them in df64.
template <int MODE, int S>
__global__ void __launch_bounds__(OZ_THREADS, 1) k_oz_mma(OzArgs a) {
  constexpr int G = OzCfg<S>::G;
  constexpr int STAGE_BYTES = OzCfg<S>::STAGE_BYTES;
  extern __shared__ __align__(1024) unsigned char oz_smem[];
  __shared__ __align__(8) uint64_t full_b[OZ_STAGES], empty_b[OZ_STAGES], acc_full, acc_empty, fin;
  __shared__ uint32_t tmem_base_s;
  __shared__ volatile int s_fail;
  __shared__ int s_eb[OZ_EPI_WARPS][OZ_EPI_COLS];   // per epilogue warp: its columns' exponents
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  unsigned char* ring = (unsigned char*)(((uintptr_t)oz_smem + 1023) & ~(uintptr_t)1023);
  const int64_t nitems = a.n_mt * a.n_nt * a.n_ks;
  const int steps_per_group = (int)(a.kgroup / 16);

  if (tid == 0) {
    for (int st = 0; st < OZ_STAGES; ++st) {
      mbar_init(&full_b[st], 1);
      mbar_init(&empty_b[st], 1);
    }
    mbar_init(&acc_full, 1);
    mbar_init(&acc_empty, OZ_EPI_WARPS);
    mbar_init(&fin, 1);
    s_fail = 0;
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base_s)),
                 "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  // An A operand of fewer than 128 rows (a narrow Y^T, stored with AR rows)
  // fills only the first AR x 32 bytes of each slice block; the rest of every
  // stage's A blocks is zeroed once here and never written again, so the
  // 128-row MMA reads zeros there.
  if (MODE == 0 && a.AR < OZ_M) {
    const int abytes = (int)a.AR * 32;
    const int tail = (OZ_ABYTES - abytes) / 16;
    for (int idx = tid; idx < OZ_STAGES * S * tail; idx += blockDim.x) {
      const int blk = idx / tail, q = idx % tail;
      *reinterpret_cast<uint4*>(ring + (size_t)(blk / S) * STAGE_BYTES + (size_t)(blk % S) * OZ_ABYTES + abytes +
                                16 * q) = make_uint4(0u, 0u, 0u, 0u);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base_s;

  if (warp == 0) {
    // ---------------- producer
    if (lane == 0) {
      int64_t gs = 0;   // stage fills issued by this CTA
      for (int64_t w = blockIdx.x; w < nitems && !s_fail; w += gridDim.x) {
        const OzItem it = oz_item(a, w);
        for (int64_t kb = it.kbeg >> 4; kb < (it.kend >> 4); ++kb, ++gs) {
          const int st = (int)(gs % OZ_STAGES);
          if (!oz_wait(&empty_b[st], (uint32_t)(((gs / OZ_STAGES) & 1) ^ 1), &s_fail)) break;
          const int abytes = (MODE == 0 && a.AR < OZ_M) ? (int)a.AR * 32 : OZ_ABYTES;
          mbar_expect_tx(&full_b[st], (unsigned)(S * (abytes + OZ_BBYTES)));
          unsigned char* sb = ring + (size_t)st * STAGE_BYTES;
#pragma unroll 1
          for (int sl = 0; sl < S; ++sl) {
            bulk_g2s(smem_u32(sb + sl * OZ_ABYTES),
                     a.As + (int64_t)sl * a.AR * a.Kpad + kb * a.AR * 16 + (it.m0 >> 3) * 128,
                     (unsigned)abytes, &full_b[st]);
            bulk_g2s(smem_u32(sb + S * OZ_ABYTES + sl * OZ_BBYTES),
                     a.Bs + (int64_t)sl * a.BR * a.Kpad + kb * a.BR * 16 + (it.n0 >> 3) * 128,
                     (unsigned)OZ_BBYTES, &full_b[st]);
          }
        }
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer
    if (lane == 0) {
      const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(OZ_N >> 3) << 17) |
                             ((uint32_t)(OZ_M >> 4) << 24);
      // ring stages are 1024-byte aligned and the ring ends below 256 KB, so
      // base + offset / 16 stays inside the descriptor's 14-bit address field
      const uint64_t ring_desc = make_desc(smem_u32(ring));
      static_assert((OZ_STAGES * STAGE_BYTES + 2048) < (1 << 18), "ring within the descriptor's range");
      static_assert(STAGE_BYTES % 16 == 0 && OZ_ABYTES % 16 == 0 && OZ_BBYTES % 16 == 0, "16-byte strides");
      int64_t gs = 0, ngroups = 0;
      for (int64_t w = blockIdx.x; w < nitems && !s_fail; w += gridDim.x) {
        const OzItem it = oz_item(a, w);
        const int nsteps = (int)((it.kend - it.kbeg) >> 4);
        for (int t = 0; t < nsteps && !s_fail; ++t, ++gs) {
          const int sig = t % steps_per_group;
          if (sig == 0) {
            // the epilogue has read the previous group's accumulators
            if (!oz_wait(&acc_empty, (uint32_t)((ngroups & 1) ^ 1), &s_fail)) break;
          }
          const int st = (int)(gs % OZ_STAGES);
          if (!oz_wait(&full_b[st], (uint32_t)((gs / OZ_STAGES) & 1), &s_fail)) break;
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint64_t da = ring_desc + (uint64_t)(st * (STAGE_BYTES >> 4));
          const uint64_t db = da + (uint64_t)((S * OZ_ABYTES) >> 4);
          if (sig == 0)
            oz_issue_step<S, G, true>(tmem, da, db, idesc);
          else
            oz_issue_step<S, G, false>(tmem, da, db, idesc);
          // the stage is free once these MMAs have read it
          asm volatile(
              "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                  smem_u32(&empty_b[st]))
              : "memory");
          if (sig == steps_per_group - 1 || t == nsteps - 1) {
            asm volatile(
                "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                    smem_u32(&acc_full))
                : "memory");
            ++ngroups;
          }
        }
      }
      // every MMA this thread issued has completed before TMEM is released
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(&fin))
                   : "memory");
      volatile int dummy = 0;
      oz_wait(&fin, 0u, &dummy);
    }
  } else {
    // ---------------- epilogue: warps 2 .. 2 + OZ_EPI_WARPS - 1
    const int q = warp & 3;                // TMEM lane quarter this warp may access
    const int part = (warp - 2) >> 2;      // column part
    const int row = q * 32 + lane;
    int64_t ngroups = 0;
    f2 acc[OZ_EPI_COLS];   // MODE 0: sums over the item's K range; MODE 1: this group's product
    for (int64_t w = blockIdx.x; w < nitems && !s_fail; w += gridDim.x) {
      const OzItem it = oz_item(a, w);
      const int nsteps = (int)((it.kend - it.kbeg) >> 4);
      const int64_t gm = it.m0 + row;
      if (MODE == 1 && w + gridDim.x < nitems) {
        // the next item's C tile streams into L2 while this one is computed
        const OzItem nx = oz_item(a, w + gridDim.x);
        const int64_t pm = nx.m0 + row;
        if (pm < a.Mvalid) {
          for (int j = 0; j < OZ_EPI_COLS; ++j) {
            const int64_t gn = nx.n0 + part * OZ_EPI_COLS + j;
            if (gn < a.Nvalid && (lane & 15) == 0)
              asm volatile("prefetch.global.L2 [%0];" ::"l"(a.C + gn * a.ldc + pm));
          }
        }
      }
#pragma unroll
      for (int j = 0; j < OZ_EPI_COLS; ++j) acc[j] = {0.0f, 0.0f};
      for (int t0 = 0; t0 < nsteps; t0 += steps_per_group) {
        // the group's exponents are loaded while its MMAs run
        const int64_t grp = (it.kbeg + (int64_t)t0 * 16) / a.kgroup;
        const int eA = (gm < a.AR) ? a.eA[grp * a.AR + gm] : 0;
        int* eb = s_eb[warp - 2];
        for (int c = lane; c < OZ_EPI_COLS; c += 32) {
          const int64_t gn = it.n0 + part * OZ_EPI_COLS + c;
          eb[c] = (gn < a.BR) ? __ldg(a.eB + grp * a.BR + gn) : 0;
        }
        __syncwarp();
        if (!oz_wait(&acc_full, (uint32_t)(ngroups & 1), &s_fail)) break;
        ++ngroups;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // drain the five accumulators, 8 columns at a time
#pragma unroll
        for (int c8 = 0; c8 < OZ_EPI_COLS / 8; ++c8) {
          const int cbase = part * OZ_EPI_COLS + c8 * 8;
          int eB[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) eB[j] = eb[c8 * 8 + j];
          uint32_t gr[G][8];
#pragma unroll
          for (int g = 0; g < G; ++g)
            tmem_ld8(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(g * OZ_N + cbase), gr[g]);
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
          float gv[G][8];
#pragma unroll
          for (int g = 0; g < G; ++g) {
            tmem_regs_ready(gr[g]);
#pragma unroll
            for (int j = 0; j < 8; ++j) gv[g][j] = __uint_as_float(gr[g][j]);
          }
          // one warp-uniform test: every scale 2^(eA + eB - 16) a normal float
          bool normal = true;
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int e = eA + eB[j] - 16;
            normal = normal && e >= -126 && e <= 127;
          }
          if (__all_sync(0xffffffffu, normal)) {
#pragma unroll
            for (int j = 0; j < 8; ++j) {
              const f2 v = combine_g<G>(gv, j);
              const float f = pow2f(eA + eB[j] - 16);
              const f2 sv = {__fmul_rn(v.h, f), __fmul_rn(v.l, f)};
              if (MODE == 0) acc[c8 * 8 + j] = oz_accumulate<G>(acc[c8 * 8 + j], sv);
              else acc[c8 * 8 + j] = sv;
            }
          } else {
#pragma unroll
            for (int j = 0; j < 8; ++j) {
              const f2 v = combine_g<G>(gv, j);
              // 2^e as three normal factors (e >= -312 for float inputs): the
              // partial products stay exact unless the result leaves the range
              const int e = eA + eB[j] - 16;
              const int e1 = min(max(e, -126), 127), e2 = min(max(e - e1, -126), 127);
              const float f1 = pow2f(e1), f2v = pow2f(e2), f3 = pow2f(e - e1 - e2);
              const f2 sv = {__fmul_rn(__fmul_rn(__fmul_rn(v.h, f1), f2v), f3),
                             __fmul_rn(__fmul_rn(__fmul_rn(v.l, f1), f2v), f3)};
              if (MODE == 0) acc[c8 * 8 + j] = oz_accumulate<G>(acc[c8 * 8 + j], sv);
              else acc[c8 * 8 + j] = sv;
            }
          }
        }
        // the accumulators are free for the next group (and eb may be rewritten)
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(&acc_empty);
        if (MODE == 1 && gm < a.Mvalid) {
          // C -= product, 16 columns per batch of loads
#pragma unroll
          for (int c16 = 0; c16 < OZ_EPI_COLS / 16; ++c16) {
            if (a.c_fp64) {
              // FP64 storage (a panel's own columns): one FP64 subtraction per element
              double cd[16];
#pragma unroll
              for (int j = 0; j < 16; ++j) {
                const int64_t gn = it.n0 + part * OZ_EPI_COLS + c16 * 16 + j;
                cd[j] = (gn < a.Nvalid && !a.c_assign) ? a.C64[gn * a.ldc + gm] : 0.0;
              }
#pragma unroll
              for (int j = 0; j < 16; ++j) {
                const int64_t gn = it.n0 + part * OZ_EPI_COLS + c16 * 16 + j;
                if (gn >= a.Nvalid) continue;
                const double pv = df_to_double(acc[c16 * 16 + j]);
                a.C64[gn * a.ldc + gm] = a.c_assign ? pv : cd[j] - pv;
              }
              continue;
            }
            float2 cv[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              const int64_t gn = it.n0 + part * OZ_EPI_COLS + c16 * 16 + j;
              cv[j] = (gn < a.Nvalid) ? a.C[gn * a.ldc + gm] : make_float2(0.0f, 0.0f);
            }
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              const int64_t gn = it.n0 + part * OZ_EPI_COLS + c16 * 16 + j;
              if (gn >= a.Nvalid) continue;
              const int64_t ci = gn * a.ldc + gm;
              const f2 r = oz_subtract<G>({cv[j].x, cv[j].y}, acc[c16 * 16 + j]);
              if (gm < a.fp64_rows) a.C64[ci] = df_to_double(r);
              else a.C[ci] = make_float2(r.h, r.l);
            }
          }
        }
      }
      if (MODE == 0 && !s_fail && gm < a.AR) {
        float2* out = a.part + (int64_t)it.split * a.Nvalid * a.AR;
#pragma unroll
        for (int j = 0; j < OZ_EPI_COLS; ++j) {
          const int64_t gn = it.n0 + part * OZ_EPI_COLS + j;
          if (gn < a.Nvalid) out[gn * a.AR + gm] = make_float2(acc[j].h, acc[j].l);
        }
      }
    }
  }
  __syncthreads();
  if (s_fail && tid == 0) atomicExch(a.status, CANDMC_ERR_TIMEOUT);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 1)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
}

// ------------------------------------------------------------------ conversions and reduction
__global__ void k_to_df64(double* X, int64_t ld, int64_t m, int64_t n) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= m * n) return;
  int64_t i = idx % m, j = idx / m;
  double* p = X + j * ld + i;
  f2 v = df_from_double(*p);
  *reinterpret_cast<float2*>(p) = make_float2(v.h, v.l);
}

__global__ void k_from_df64(double* X, int64_t ld, int64_t m, int64_t n) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= m * n) return;
  int64_t i = idx % m, j = idx / m;
  double* p = X + j * ld + i;
  float2 v = *reinterpret_cast<float2*>(p);
  *p = (double)v.x + (double)v.y;
}

// Z (nb x n, FP64, ld nb) = sum over splits of the df64 partials [split][n][AR],
// added in split order.  Eight partials are loaded before they are added, so a
// narrow update's many splits (up to one per 128 rows) cost a few memory
// latencies per output instead of one per split.
__global__ void k_oz_sum_partials(const float2* part, int nsplit, int64_t AR, int nb, int64_t n,
                                  double* Z) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)nb * n) return;
  int64_t i = idx % nb, j = idx / nb;
  const float2* p = part + j * AR + i;
  const int64_t stride = n * AR;
  f2 s = {0.0f, 0.0f};
  int sp = 0;
  for (; sp + 8 <= nsplit; sp += 8) {
    float2 v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = p[(int64_t)(sp + u) * stride];
#pragma unroll
    for (int u = 0; u < 8; ++u) s = df_add(s, {v[u].x, v[u].y});
  }
  for (; sp < nsplit; ++sp) {
    const float2 v = p[(int64_t)sp * stride];
    s = df_add(s, {v.x, v.y});
  }
  Z[j * nb + i] = df_to_double(s);
}

// ------------------------------------------------------------------ host side
static inline int64_t rup(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

static int num_sms_oz() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 148;
  }
  return n;
}

int to_df64(double* X, int64_t ld, int64_t m, int64_t n, cudaStream_t s) {
  if (m <= 0 || n <= 0) return CANDMC_OK;
  ProfScope ps(CANDMC_KCLASS_OZ_SLICE, 16.0 * m * n, s);
  k_to_df64<<<(unsigned)((m * n + 255) / 256), 256, 0, s>>>(X, ld, m, n);
  CANDMC_CK(cudaGetLastError());
  return CANDMC_OK;
}

int from_df64(double* X, int64_t ld, int64_t m, int64_t n, cudaStream_t s) {
  if (m <= 0 || n <= 0) return CANDMC_OK;
  ProfScope ps(CANDMC_KCLASS_OZ_SLICE, 16.0 * m * n, s);
  k_from_df64<<<(unsigned)((m * n + 255) / 256), 256, 0, s>>>(X, ld, m, n);
  CANDMC_CK(cudaGetLastError());
  return CANDMC_OK;
}

template <int S>
static int launch_slice_kcol(SliceSrc src, int64_t k0, int64_t Kvalid, int64_t Nvalid, int64_t Rpad,
                             int64_t Kpad, int G, __nv_bfloat16* out, int* e, cudaStream_t s) {
  ProfScope ps(CANDMC_KCLASS_OZ_SLICE, 8.0 * Nvalid * Kvalid + 2.0 * S * Rpad * Kpad, s);
  if (G <= 128 && G % 16 == 0 && Rpad % 8 == 0) {
    k_slice_kcol8<S><<<dim3((unsigned)(Rpad / 8), (unsigned)(Kpad / G)), 256, 0, s>>>(src, k0, Kvalid, Nvalid,
                                                                                  Rpad, Kpad, G, out, e);
    CANDMC_CK(cudaGetLastError());
    return CANDMC_OK;
  }
  int64_t warps = Rpad * (Kpad / G);
  k_slice_kcol<S><<<(unsigned)((warps * 32 + 255) / 256), 256, 0, s>>>(src, k0, Kvalid, Nvalid, Rpad,
                                                                      Kpad, G, out, e);
  CANDMC_CK(cudaGetLastError());
  return CANDMC_OK;
}

template <int S>
static int launch_slice_krow(SliceSrc src, int64_t n0, int64_t Nvalid, int64_t Kvalid, int64_t Rpad,
                             int64_t Kpad, __nv_bfloat16* out, int* e, cudaStream_t s) {
  size_t sm = sizeof(float2) * 32 * (size_t)Kpad;
  if (sm > 48 * 1024)
    CANDMC_CK(cudaFuncSetAttribute(k_slice_krow<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  ProfScope ps(CANDMC_KCLASS_OZ_SLICE, 8.0 * Nvalid * Kvalid + 2.0 * S * Rpad * Kpad, s);
  k_slice_krow<S><<<(unsigned)((Rpad + 31) / 32), 256, sm, s>>>(src, n0, Nvalid, Kvalid, Rpad, Kpad, out, e);
  CANDMC_CK(cudaGetLastError());
  return CANDMC_OK;
}

int g_oz_reserve_sms = 32;
thread_local int t_oz_cap = 0;

// one persistent CTA per SM at most (fewer under a cap), each taking every
// gridDim-th work item
template <int S>
static int launch_oz(OzArgs a, unsigned gm, unsigned gn, unsigned gk, int cls, double flops,
                     cudaStream_t s) {
  constexpr int SMEM = OzCfg<S>::SMEM;
  static std::atomic<bool> attr{false};
  if (!attr) {
    CANDMC_CK(cudaFuncSetAttribute(k_oz_mma<0, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM));
    CANDMC_CK(cudaFuncSetAttribute(k_oz_mma<1, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM));
    attr = true;
  }
  a.n_mt = gm;
  a.n_nt = gn;
  a.n_ks = gk;
  const int64_t items = (int64_t)gm * gn * gk;
  int64_t ctas = num_sms_oz();
  if (t_oz_cap > 0 && t_oz_cap < ctas) ctas = t_oz_cap;
  const unsigned grid = (unsigned)std::min<int64_t>(items, ctas);
  ProfScope ps(cls, flops, s);
  if (a.mode == 0)
    k_oz_mma<0, S><<<grid, OZ_THREADS, SMEM, s>>>(a);
  else
    k_oz_mma<1, S><<<grid, OZ_THREADS, SMEM, s>>>(a);
  CANDMC_CK(cudaGetLastError());
  return CANDMC_OK;
}

// Z (nb x n, FP64, ld nb) = Y^T C with S-slice contractions: Y (m x nb) and C
// (m x n) read through their slice sources; split-K partials summed in df64.
template <int S>
static int oz_tn(const SliceSrc& ysrc, const SliceSrc& csrc, int64_t m, int nb, int64_t n, double* Z,
                 int* status, cudaStream_t s, int cls) {
  const int64_t KG = 128;                       // K rows per exact accumulation
  // A-op = Y^T (rows = Householder index, K = m), B-op = C (rows = columns)
  const int64_t Kp1 = rup(m, KG);
  // the A operand keeps only its nb rows (rounded to a core matrix of 8):
  // the kernel zero-fills the rest of the 128-row tile in shared memory
  const int64_t AR1 = rup(nb, 8), BR1 = rup(n, OZ_N);
  DevBuf ya, ea, cb, eb, part;
  CANDMC_RET(ya.alloc(sizeof(__nv_bfloat16) * S * AR1 * Kp1, s));
  CANDMC_RET(ea.alloc(sizeof(int) * (Kp1 / KG) * AR1, s));
  CANDMC_RET(cb.alloc(sizeof(__nv_bfloat16) * S * BR1 * Kp1, s));
  CANDMC_RET(eb.alloc(sizeof(int) * (Kp1 / KG) * BR1, s));
  auto* yas = static_cast<__nv_bfloat16*>(ya.p);
  auto* cbs = static_cast<__nv_bfloat16*>(cb.p);
  CANDMC_RET(launch_slice_kcol<S>(ysrc, 0, m, nb, AR1, Kp1, (int)KG, yas, static_cast<int*>(ea.p), s));
  CANDMC_RET(launch_slice_kcol<S>(csrc, 0, m, n, BR1, Kp1, (int)KG, cbs, static_cast<int*>(eb.p), s));
  // K split: about two waves of CTAs
  const int64_t ntiles = BR1 / OZ_N;
  int64_t ksplit = std::max<int64_t>(1, std::min<int64_t>(Kp1 / KG, (2 * num_sms_oz() + ntiles - 1) / ntiles));
  int64_t kper = rup((Kp1 + ksplit - 1) / ksplit, KG);
  ksplit = (Kp1 + kper - 1) / kper;
  CANDMC_RET(part.alloc(sizeof(float2) * ksplit * n * AR1, s));
  OzArgs g1{};
  g1.As = yas; g1.AR = AR1; g1.Bs = cbs; g1.BR = BR1; g1.Kpad = Kp1; g1.k_per_cta = kper;
  g1.kgroup = KG; g1.eA = static_cast<int*>(ea.p); g1.eB = static_cast<int*>(eb.p);
  g1.mode = 0; g1.part = static_cast<float2*>(part.p); g1.Mvalid = nb; g1.Nvalid = n;
  g1.status = status;
  CANDMC_RET(launch_oz<S>(g1, 1, (unsigned)ntiles, (unsigned)ksplit, cls, 2.0 * nb * n * m, s));
  ProfScope ps(CANDMC_KCLASS_REDUCE, 8.0 * ksplit * n * AR1, s);
  k_oz_sum_partials<<<(unsigned)((nb * n + 255) / 256), 256, 0, s>>>(static_cast<float2*>(part.p),
                                                                      (int)ksplit, AR1, nb, n, Z);
  CANDMC_CK(cudaGetLastError());
  return CANDMC_OK;
}

// Zt (nb x n, FP64, ld nb) = Top (nb x nb) * Z (nb x n, FP64, ld nb) with the
// S-slice contraction: Top is the A operand (sliced from its stored matrix,
// transposed or not), Z the B operand, and the MODE 1 epilogue stores the
// product into Zt instead of subtracting it.
template <int S>
static int oz_top_times(MatRef Top, int nb, const double* Z, int64_t n, double* Zt, int* status,
                        cudaStream_t s, int cls) {
  const int64_t Kp = rup(nb, 16), BR = rup(n, OZ_N);
  DevBuf ta, et, zb, ez;
  CANDMC_RET(ta.alloc(sizeof(__nv_bfloat16) * S * OZ_M * Kp, s));
  CANDMC_RET(et.alloc(sizeof(int) * OZ_M, s));
  CANDMC_RET(zb.alloc(sizeof(__nv_bfloat16) * S * BR * Kp, s));
  CANDMC_RET(ez.alloc(sizeof(int) * BR, s));
  auto* tas = static_cast<__nv_bfloat16*>(ta.p);
  auto* zbs = static_cast<__nv_bfloat16*>(zb.p);
  const SliceSrc tsrc{Top.p, nullptr, Top.ld, Top.mask, Top.off};
  // A operand element (i, k) = Top(i, k): X[k, i] of a transposed reference
  // (a column of X per operand row), X[i, k] otherwise (a row of X)
  if (Top.trans)
    CANDMC_RET(launch_slice_kcol<S>(tsrc, 0, nb, nb, OZ_M, Kp, (int)Kp, tas, static_cast<int*>(et.p), s));
  else
    CANDMC_RET(launch_slice_krow<S>(tsrc, 0, nb, nb, OZ_M, Kp, tas, static_cast<int*>(et.p), s));
  CANDMC_RET(launch_slice_kcol<S>(SliceSrc{Z, nullptr, nb, kDense, 0}, 0, nb, n, BR, Kp, (int)Kp, zbs,
                                  static_cast<int*>(ez.p), s));
  OzArgs g{};
  g.As = tas; g.AR = OZ_M; g.Bs = zbs; g.BR = BR;
  g.Kpad = Kp; g.k_per_cta = Kp; g.kgroup = Kp;
  g.eA = static_cast<int*>(et.p); g.eB = static_cast<int*>(ez.p);
  g.mode = 1; g.C = reinterpret_cast<float2*>(Zt); g.C64 = Zt; g.ldc = nb;
  g.Mvalid = nb; g.Nvalid = n; g.fp64_rows = 0; g.status = status;
  g.c_fp64 = 1; g.c_assign = 1;
  return launch_oz<S>(g, 1, (unsigned)(BR / OZ_N), 1, cls, 2.0 * nb * nb * n, s);
}

// Width from which the operator product T^T Z of an update runs on the
// tensor cores (below it, the FP64 small-matrix kernel is quicker).
constexpr int64_t kOzTopMinCols = 1024;

// The trailing update with S-slice contractions: C <- C - Y (Top (Y^T C)).
// C (m x n, ld ldc) holds df64 pairs; rows < fp64_rows of C are written back
// as FP64 (finished R rows).  With c_fp64, C is FP64 storage instead (read and
// written as FP64).  Y: unit-lower m x nb (read from a Y\R buffer, FP64),
// Top: the nb x nb operator applied to Y^T C.  cls_tn / cls_nn: the kernel
// classes the two contractions are counted under.
template <int S>
static int apply_qt_slices(const double* Y, int64_t ldy, int ymask, int64_t m, int nb, MatRef Top,
                           double* C, int64_t ldc, int64_t n, int64_t fp64_rows, int* status,
                           cudaStream_t s, bool c_fp64, int cls_tn, int cls_nn) {
  if (m <= 0 || n <= 0) return CANDMC_OK;
  if (nb > OZ_M) return set_error(CANDMC_ERR_ARG, "ozaki form needs b <= 128");
  // ---- GEMM1: Z = Y^T C
  SliceSrc ysrc{Y, nullptr, ldy, ymask, 0};
  SliceSrc csrc = c_fp64 ? SliceSrc{C, nullptr, ldc, kDense, 0}
                         : SliceSrc{nullptr, reinterpret_cast<const float2*>(C), ldc, kDense, 0};
  DevBuf z, zt;
  CANDMC_RET(z.alloc(sizeof(double) * nb * n, s));
  CANDMC_RET(oz_tn<S>(ysrc, csrc, m, nb, n, z.d(), status, s, cls_tn));
  // ---- Z' = T^T * Z   (FP64 storage, nb x n); counted, as on the FP64 pipe,
  // under the small-product class, apart from the two contractions with Y
  CANDMC_RET(zt.alloc(sizeof(double) * nb * n, s));
  if (n >= kOzTopMinCols)
    CANDMC_RET(oz_top_times<S>(Top, nb, z.d(), n, zt.d(), status, s, CANDMC_KCLASS_SMALL));
  else
    CANDMC_RET(small_gemm(nb, n, nb, 1.0, Top, mref(z.d(), nb), 0.0, zt.d(), nb, s));
  // ---- GEMM2: C -= Y * Z'.  A-op = Y (rows = m, K = nb), B-op = Z'^T (rows = columns, K = nb)
  const int64_t Kp2 = rup(nb, 16);
  const int64_t AR2 = rup(m, OZ_M), BR2 = rup(n, OZ_N);
  DevBuf y2, ey2, z2, ez2;
  CANDMC_RET(y2.alloc(sizeof(__nv_bfloat16) * S * AR2 * Kp2, s));
  CANDMC_RET(ey2.alloc(sizeof(int) * AR2, s));
  CANDMC_RET(z2.alloc(sizeof(__nv_bfloat16) * S * BR2 * Kp2, s));
  CANDMC_RET(ez2.alloc(sizeof(int) * BR2, s));
  CANDMC_RET(launch_slice_krow<S>(ysrc, 0, m, nb, AR2, Kp2, static_cast<__nv_bfloat16*>(y2.p),
                               static_cast<int*>(ey2.p), s));
  SliceSrc zsrc{zt.d(), nullptr, nb, kDense, 0};
  CANDMC_RET(launch_slice_kcol<S>(zsrc, 0, nb, n, BR2, Kp2, (int)Kp2, static_cast<__nv_bfloat16*>(z2.p),
                               static_cast<int*>(ez2.p), s));
  OzArgs g2{};
  g2.As = static_cast<__nv_bfloat16*>(y2.p); g2.AR = AR2;
  g2.Bs = static_cast<__nv_bfloat16*>(z2.p); g2.BR = BR2;
  g2.Kpad = Kp2; g2.k_per_cta = Kp2; g2.kgroup = Kp2;
  g2.eA = static_cast<int*>(ey2.p); g2.eB = static_cast<int*>(ez2.p);
  g2.mode = 1; g2.C = reinterpret_cast<float2*>(C); g2.C64 = C; g2.ldc = ldc;
  g2.Mvalid = m; g2.Nvalid = n; g2.fp64_rows = fp64_rows; g2.status = status;
  g2.c_fp64 = c_fp64 ? 1 : 0;
  CANDMC_RET(launch_oz<S>(g2, (unsigned)(AR2 / OZ_M), (unsigned)(BR2 / OZ_N), 1, cls_nn,
                       2.0 * m * n * nb, s));
  return CANDMC_OK;
}

// The emulated-FP64 form: 7 slices, 28 slice products per K16 step.
int apply_qt_ozaki(const double* Y, int64_t ldy, int ymask, int64_t m, int nb, MatRef Top,
                   double* C, int64_t ldc, int64_t n, int64_t fp64_rows, int* status,
                   cudaStream_t s, bool c_fp64) {
  // a panel's own half-panel updates (FP64 storage) are counted apart from
  // the trailing-matrix contractions
  return apply_qt_slices<OZ_S>(Y, ldy, ymask, m, nb, Top, C, ldc, n, fp64_rows, status, s, c_fp64,
                               c_fp64 ? CANDMC_KCLASS_OZ_PANEL : CANDMC_KCLASS_OZ_TN,
                               c_fp64 ? CANDMC_KCLASS_OZ_PANEL : CANDMC_KCLASS_OZ_NN);
}

// The FP32 form on the same tensor-core path: 3 BF16 slices (24 bits under
// each scale group's exponent, FP32-class accuracy), 6 slice products per K16
// step in 3 accumulator groups, summed in FP32.  C keeps the df64 slots of
// the emulated form, but the epilogue updates it in FP32 arithmetic (its low
// word becomes zero), so the read-modify-write costs one FP32 operation per
// element instead of a df64 addition.
int apply_qt_f32(const double* Y, int64_t ldy, int ymask, int64_t m, int nb, MatRef Top, double* C,
                 int64_t ldc, int64_t n, int64_t fp64_rows, int* status, cudaStream_t s) {
  return apply_qt_slices<OZ_S32>(Y, ldy, ymask, m, nb, Top, C, ldc, n, fp64_rows, status, s, false,
                                 CANDMC_KCLASS_F32, CANDMC_KCLASS_F32);
}

// G (nb x n, FP64, ld nb) = Y^T C for FP64 Y (m x nb, mask ymask) and C
// (m x n, mask cmask) in emulated FP64: the Gram product of a panel's
// recursive T merge.
int gram_ozaki(const double* Y, int64_t ldy, int ymask, const double* C, int64_t ldc, int cmask, int64_t m,
               int nb, int64_t n, double* G, int* status, cudaStream_t s) {
  if (m <= 0 || n <= 0 || nb <= 0) return CANDMC_OK;
  if (nb > OZ_M) return set_error(CANDMC_ERR_ARG, "gram_ozaki needs nb <= 128");
  return oz_tn<OZ_S>(SliceSrc{Y, nullptr, ldy, ymask, 0}, SliceSrc{C, nullptr, ldc, cmask, 0}, m, nb, n, G,
                     status, s, CANDMC_KCLASS_OZ_PANEL);
}

}  // namespace candmc
